"""The learned proposal on the GPU (minimumcyclebasis_gb300.learned, mcbgpu_mlp_*):
  - the network's forward pass (first layer on the tensor cores) and its gradients
    equal the CPU restatement (oracle/mlp.py) within fp32 tolerances;
  - training on traces of solved graphs lowers the loss;
  - a solve with the proposal's prefix gives the plain solve's basis (zero diffs) with
    or without a fallback, and a trained network cuts more of the candidate list than
    an untrained one on an unseen graph of the family it was trained on."""
import numpy as np
import pytest

from oracle import mlp as omlp

pytestmark = pytest.mark.gpu

# forward logits: bf16 products are exact in fp32, only the summation order differs
FWD_ATOL, FWD_RTOL = 1e-4, 1e-4
# gradients: fp32 atomics in a different order than numpy's float64 sums
GRAD_ATOL, GRAD_RTOL = 2e-5, 2e-3


def _inputs(n, seed):
    import torch
    rng = np.random.default_rng(seed)
    x = omlp.bf16_round(rng.normal(size=(n, 16)).astype(np.float32))
    y = (rng.random(n) < 0.25).astype(np.uint8)
    xd = torch.from_numpy(x).to(torch.bfloat16).cuda()
    yd = torch.from_numpy(y).cuda()
    return x, y, xd, yd


@pytest.mark.parametrize("n", [1, 127, 128, 129, 1000, 70001])
def test_forward_matches_the_cpu_restatement(n):
    import torch
    from minimumcyclebasis_gb300.learned import ProposalNet, init_params
    torch.cuda.set_device(0)
    p = init_params(7)
    net = ProposalNet(p)
    x, _, xd, _ = _inputs(n, n)
    got = net.forward(xd).cpu().numpy()
    want, _ = omlp.forward(p, x)
    assert np.allclose(got, want, atol=FWD_ATOL, rtol=FWD_RTOL), np.abs(got - want).max()
    net.close()


def test_gradients_match_the_cpu_restatement():
    import torch
    from minimumcyclebasis_gb300.learned import ProposalNet, init_params
    torch.cuda.set_device(0)
    p = init_params(11)
    net = ProposalNet(p)
    x, y, xd, yd = _inputs(5000, 5)
    loss, g = net.gradients(xd, yd, pos_weight=3.0)
    wl, wg = omlp.loss_and_grads(p, x, y, 3.0)
    assert abs(loss - wl) < 1e-4 * max(1.0, abs(wl))
    assert np.allclose(g, wg, atol=GRAD_ATOL, rtol=GRAD_RTOL), np.abs(g - wg).max()
    # gradients are recomputed, not accumulated, on a second call
    loss2, g2 = net.gradients(xd, yd, pos_weight=3.0)
    assert np.allclose(g2, g, atol=GRAD_ATOL, rtol=GRAD_RTOL)
    net.close()


def test_training_lowers_the_loss_on_a_separable_problem():
    import torch
    from minimumcyclebasis_gb300.learned import ProposalNet, train
    torch.cuda.set_device(0)
    rng = np.random.default_rng(2)
    x = omlp.bf16_round(rng.normal(size=(40000, 16)).astype(np.float32))
    y = (x[:, 0] + 0.5 * x[:, 3] > 0.3).astype(np.uint8)
    net = ProposalNet(seed=1)
    losses = train(net, [torch.from_numpy(x).to(torch.bfloat16).cuda()], [torch.from_numpy(y).cuda()], epochs=6,
                   batch=4096, lr=1e-2)
    assert losses[-1] < 0.5 * losses[0], losses
    logits = net.forward(torch.from_numpy(x).to(torch.bfloat16).cuda()).cpu().numpy()
    assert ((logits > 0) == (y == 1)).mean() > 0.95
    net.close()


def _plain(g):
    from minimumcyclebasis_gb300 import Problem, Solver
    p = Problem.from_graph(g).prepare(threads=4)
    s = Solver.from_problem(p)
    s.run()
    sel, tot = s.results()
    s.close()
    return sel, tot


def test_proposal_solve_equals_the_plain_solve_and_a_trained_net_cuts_more():
    import torch
    from minimumcyclebasis_gb300 import planar_chain_graph
    from minimumcyclebasis_gb300.learned import ProposalNet, solve_with_proposal, traces, train
    torch.cuda.set_device(0)
    xs, ys = [], []
    for seed in (41, 42, 43):
        x, y, res = traces(planar_chain_graph(1500, 30, 30, 8, 1, 1000, seed), threads=4)
        xs.append(x)
        ys.append(y)
        assert res.K_kept == res.K and not res.fallback
    trained = ProposalNet(seed=3)
    train(trained, xs, ys, epochs=30, batch=2048, lr=3e-3)
    untrained = ProposalNet(seed=3)
    g = planar_chain_graph(1500, 30, 30, 8, 1, 1000, 44)  # not among the training graphs
    want_sel, want_tot = _plain(g)
    cut = {}
    for name, net in (("trained", trained), ("untrained", untrained), ("none", None)):
        r = solve_with_proposal(g, net, margin=0.05, threads=4)
        assert np.array_equal(r.selected, want_sel) and r.total_weight == want_tot, name
        cut[name] = r.skip_rate
    assert cut["none"] == 0.0
    assert cut["trained"] > cut["untrained"] + 0.1, cut
    trained.close()
    untrained.close()


def test_a_short_prefix_falls_back_to_the_whole_list():
    import torch
    from minimumcyclebasis_gb300 import random_graph
    from minimumcyclebasis_gb300.learned import solve_with_proposal
    torch.cuda.set_device(0)
    g = random_graph(600, 1200, 1, 1000, 45)
    want_sel, want_tot = _plain(g)
    # a prefix of N / 2 candidates cannot hold a basis of N cycles: the solve runs out
    # of candidates, says so, and is run again on the whole list
    r = solve_with_proposal(g, None, threads=4, prefix=len(want_sel) // 2)
    assert r.fallback and r.K_kept < r.K
    assert r.skip_rate == 0.0 and r.proposed_skip_rate > 0.4  # the whole list was solved after all
    assert np.array_equal(r.selected, want_sel) and r.total_weight == want_tot
    # a prefix that holds the basis needs no fallback
    last = int(want_sel.max()) + 1
    r2 = solve_with_proposal(g, None, threads=4, prefix=last)
    assert not r2.fallback and r2.K_kept == last
    assert np.array_equal(r2.selected, want_sel) and r2.total_weight == want_tot
