"""The learned proposal: a small network that scores candidates, and the solve that
uses its scores to cut the candidate list, exactly.

The de Pina loop selects, at every iteration, the first odd candidate in rank order,
and rank order is ascending weight.  If the loop, run on a prefix of the rank order,
finds an odd candidate at every iteration, it selects exactly what it selects on the
whole list (a prefix's first odd candidate is the list's).  So a prefix that holds
the whole basis gives the same result for less: no coordinate lists are built,
uploaded or streamed for the candidates beyond it, and a root none of whose
candidates lies in the prefix needs no list walk at all.  The shortest such prefix
ends at the heaviest cycle of the basis; it is not known before the solve.

The network proposes it.  It scores every candidate from 16 features of its cycle
(weight against the list's median, root distances, edge weight, hop counts, list
length, rank quantile, degrees; computed on the device during the cycle walk) with a
two-layer perceptron (16 -> 64 ReLU -> 1, bf16 weights, fp32 accumulation; its first
layer on the tensor cores) trained on (candidate, selected?) traces of solved graphs.
Two rules turn scores into a prefix.  The tail rule (solve_with_proposal's default):
the shortest prefix beyond which the candidates' calibrated probabilities of
selection sum to at most eps, i.e. the expected number of selected candidates left
out is at most eps.  The top-score rule: the top ceil(N (1 + margin)) scores are the
proposals and the heaviest proposal's weight U bounds the prefix; its margin can be
calibrated on the training graphs (needed_margin, calibrate_margin), which is how
the benchmark uses it.  Either way the prefix ends at the
end of a weight class (every candidate of weight <= U, ties included).  The solver runs
on that prefix and checks itself: if some iteration finds no odd candidate in it
(the proposals did not hold a basis), the whole list is built and the solve is run
again on it.  Either way the result is the plain solve's, which stays the arbiter.  When
the prefix suffices, its heaviest selected weight is an exact upper bound of the
minimum basis's heaviest cycle (a matroid's greedy basis minimises its largest
element).
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass, field

import numpy as np

from ._native import MCBError, check_gpu, gpu_lib, ptr
from .gpu import Solver, _stream

N_FEATURES = 16
N_HIDDEN = 64


def init_params(seed: int = 0) -> np.ndarray:
    """Uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights and biases, as a linear
    layer's default initialisation."""
    rng = np.random.default_rng(seed)
    n = int(gpu_lib().mcbgpu_mlp_param_count())
    p = np.empty(n, np.float32)
    a1, a2 = 1.0 / np.sqrt(N_FEATURES), 1.0 / np.sqrt(N_HIDDEN)
    k = N_HIDDEN * N_FEATURES
    p[:k] = rng.uniform(-a1, a1, k)
    p[k:k + N_HIDDEN] = rng.uniform(-a1, a1, N_HIDDEN)
    p[k + N_HIDDEN:k + 2 * N_HIDDEN] = rng.uniform(-a2, a2, N_HIDDEN)
    p[-1] = rng.uniform(-a2, a2)
    return p


class ProposalNet:
    """The network on the device (mcbgpu_mlp_*).  Features, labels and logits are
    torch CUDA tensors: x (count, 16) bfloat16, y (count,) uint8, logits (count,)
    float32."""

    def __init__(self, params: np.ndarray | None = None, seed: int = 0):
        self.lib = gpu_lib()
        p = np.ascontiguousarray(init_params(seed) if params is None else params, np.float32)
        h = C.c_void_p()
        check_gpu(self.lib.mcbgpu_mlp_create(C.byref(h), ptr(p)), "mcbgpu_mlp_create")
        self._h = h
        self.pos_weight = 1.0  # the positive weight of the training loss (set by train)

    def params(self) -> np.ndarray:
        out = np.empty(int(self.lib.mcbgpu_mlp_param_count()), np.float32)
        check_gpu(self.lib.mcbgpu_mlp_get_params(self._h, ptr(out)), "mcbgpu_mlp_get_params")
        return out

    def forward(self, x, stream=0):
        import torch
        logits = torch.empty(x.shape[0], dtype=torch.float32, device=x.device)
        check_gpu(self.lib.mcbgpu_mlp_forward(self._h, C.c_void_p(x.data_ptr()), x.shape[0],
                                              C.c_void_p(logits.data_ptr()), _stream(stream)), "mcbgpu_mlp_forward")
        return logits

    def gradients(self, x, y, pos_weight: float = 1.0, stream=0):
        """(mean loss, gradient of every parameter) at the current parameters."""
        g = np.empty(int(self.lib.mcbgpu_mlp_param_count()), np.float32)
        loss = C.c_float()
        check_gpu(self.lib.mcbgpu_mlp_gradients(self._h, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()),
                                                x.shape[0], pos_weight, ptr(g), C.byref(loss), _stream(stream)),
                  "mcbgpu_mlp_gradients")
        return float(loss.value), g

    def train_step(self, x, y, pos_weight: float, lr: float, stream=0, want_loss: bool = False):
        loss = C.c_float()
        check_gpu(self.lib.mcbgpu_mlp_train_step(self._h, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()),
                                                 x.shape[0], pos_weight, lr,
                                                 C.byref(loss) if want_loss else None, _stream(stream)),
                  "mcbgpu_mlp_train_step")
        return float(loss.value) if want_loss else None

    def close(self) -> None:
        if getattr(self, "_h", None):
            self.lib.mcbgpu_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


def features(gen, weight_sorted, tree, edge, stream=0):
    """Walks the ranked candidates' cycles once on the device (mcbgpu_gen_rank):
    list lengths for the later list build and the (K, 16) bf16 features."""
    import torch
    K = len(weight_sorted)
    x = torch.empty((max(K, 1), N_FEATURES), dtype=torch.bfloat16, device="cuda")
    t = np.ascontiguousarray(tree, np.int32)
    e = np.ascontiguousarray(edge, np.int32)
    w = np.ascontiguousarray(weight_sorted, np.int32)
    check_gpu(gen.lib.mcbgpu_gen_rank(gen._h, K, ptr(t), ptr(e), ptr(w), C.c_void_p(x.data_ptr()), _stream(stream)),
              "mcbgpu_gen_rank")
    gen.K = K
    return x[:K]


def build_lists(gen, K_keep: int, stream=0) -> int:
    nnz = C.c_int64()
    check_gpu(gen.lib.mcbgpu_gen_build_lists(gen._h, int(K_keep), C.byref(nnz), _stream(stream)),
              "mcbgpu_gen_build_lists")
    gen.K = int(K_keep)
    gen.nnz = int(nnz.value)
    return gen.nnz


def proposal_prefix(logits_host: np.ndarray, weight_sorted: np.ndarray, N: int, margin: float):
    """(K_keep, U) by the top-score rule: the top ceil(N (1 + margin)) scores'
    heaviest weight U and the rank-order prefix of every candidate of weight <= U."""
    K = len(weight_sorted)
    k = int(min(K, np.ceil(N * (1.0 + margin))))
    if k >= K:
        return K, int(weight_sorted[-1]) if K else 0
    top = np.argpartition(-logits_host, k - 1)[:k]
    U = int(weight_sorted[top].max())
    return int(np.searchsorted(weight_sorted, U, side="right")), U


def needed_margin(logits_host: np.ndarray, weight_sorted: np.ndarray, N: int, K_needed: int) -> float:
    """The smallest top-score margin whose prefix holds the first K_needed candidates of
    the rank order: the proposals (the top ceil(N (1 + margin)) scores) must include a
    candidate at least as heavy as the last needed one, whose weight class then ends
    the prefix at or past it."""
    K = len(weight_sorted)
    if K == 0 or K_needed <= 0 or N <= 0:
        return 0.0
    w_star = weight_sorted[min(K_needed, K) - 1]
    order = np.argsort(-logits_host, kind="stable")
    heavy = np.nonzero(weight_sorted[order] >= w_star)[0]
    first = int(heavy[0]) + 1  # proposals needed to reach a heavy enough candidate
    return max(first / N - 1.0, 0.0)


def calibrate_margin(margins, scale: float = 1.25, slack: float = 0.05) -> float:
    """The top-score margin for unseen graphs: the largest margin the training graphs
    needed, scaled and padded (a margin is relative to N, so it carries over sizes)."""
    return float(max(margins, default=0.0)) * scale + slack


def calibrated(logits_host: np.ndarray, pos_weight: float) -> np.ndarray:
    """P(selected) from logits trained with positives weighted by pos_weight (the
    weighting multiplies the odds by pos_weight)."""
    z = np.clip(logits_host.astype(np.float64), -60, 60) - np.log(max(pos_weight, 1e-12))
    return 1.0 / (1.0 + np.exp(-z))


def tail_prefix(logits_host: np.ndarray, weight_sorted: np.ndarray, pos_weight: float, eps: float):
    """(K_keep, U) by the tail rule: the shortest rank-order prefix beyond which the
    expected number of selected candidates (calibrated probabilities summed) is at
    most eps (so no selected candidate lies beyond it with probability >= 1 - eps),
    extended to the end of its weight class."""
    K = len(weight_sorted)
    if K == 0:
        return 0, 0
    p = calibrated(logits_host, pos_weight)
    tail = np.cumsum(p[::-1])[::-1]  # tail[r] = sum of p over ranks >= r
    beyond = np.nonzero(tail <= eps)[0]
    K1 = int(beyond[0]) if len(beyond) else K
    if K1 >= K:
        return K, int(weight_sorted[-1])
    U = int(weight_sorted[max(K1 - 1, 0)])
    return int(np.searchsorted(weight_sorted, U, side="right")), U


def proposal_table(logits_host, weight_sorted, N: int, pos_weight: float, K_needed: int | None = None):
    """The prefix of each rule (top-score margins, tail bounds) on one graph's
    scores; with the prefix the solve needs (K_needed), whether each holds it."""
    out = []
    for rule, par in [("top", 0.05), ("top", 0.25), ("top", 1.0), ("top", 3.0), ("tail", 1.0), ("tail", 0.3),
                      ("tail", 0.1), ("tail", 0.03)]:
        if rule == "top":
            k, U = proposal_prefix(logits_host, weight_sorted, N, par)
        else:
            k, U = tail_prefix(logits_host, weight_sorted, pos_weight, par)
        row = {"rule": rule, "param": par, "K_keep": int(k), "U": int(U)}
        if K_needed is not None:
            row["holds_basis"] = bool(k >= K_needed)
        out.append(row)
    return out


@dataclass
class LearnedSolve:
    """The outcome of a solve with a proposal: the selected ranks and total weight
    (the plain solve's), how much of the list was cut, and whether the fallback ran."""
    selected: np.ndarray
    total_weight: int
    K: int
    K_kept: int
    U: int
    nnz_kept: int
    trees: int
    trees_kept: int
    fallback: bool
    times: dict = field(default_factory=dict)
    lists: tuple | None = None
    weight_sorted: np.ndarray | None = None
    compared: list = field(default_factory=list)
    logits: np.ndarray | None = None

    @property
    def K_needed(self) -> int:
        """The rank-order prefix the basis needs: up to its last selected candidate."""
        return int(np.max(self.selected)) + 1 if len(self.selected) else 0

    @property
    def proposed_skip_rate(self) -> float:
        """Share of the candidates beyond the proposal's prefix."""
        return 1.0 - self.K_kept / self.K if self.K else 0.0

    @property
    def skip_rate(self) -> float:
        """Share of the candidates the solve did without: none after a fallback to the
        whole list (the prefix did not hold the basis)."""
        return 0.0 if self.fallback else self.proposed_skip_rate


def solve_with_proposal(src, net: ProposalNet | None, margin: float = 0.05, threads: int = 0, stream=0,
                        keep_solver: bool = False, keep_features: bool = False, prefix: int | None = None,
                        host_lists: bool = False, compare=(), rule: str = "tail", eps: float = 0.1,
                        keep_logits: bool = False):
    """Graph -> basis with the device preparation and the proposal's prefix (no
    proposal: `net` None keeps the whole list; `prefix` imposes a prefix length
    instead of the proposal's).  Returns a LearnedSolve; with keep_solver also the
    Solver and the Problem, with keep_features also the candidates' features (torch
    (K, 16) bf16); with host_lists the solved lists (weights, offsets, coordinates)
    are copied to the host into LearnedSolve.lists; `compare` (networks) gets each
    one's proposal prefix on the same features, (K_keep, U), in LearnedSolve.compared
    (not solved, not timed).  `rule`: "tail" (the tail rule with bound eps, on the
    network's calibrated probabilities; the default) or "top" (the top-score rule
    with `margin`).  keep_logits stores the scores (host) in LearnedSolve.logits."""
    import torch

    from .devprep import GpuGen, generate_candidates
    from .host import Graph, Problem
    times = {}
    t0 = time.perf_counter()
    p = Problem.from_graph(src) if isinstance(src, Graph) else src
    p.prepare(threads=threads, structure_only=True)
    gen = GpuGen(p)
    offs, pis, wis, _, _ = generate_candidates(p, gen, threads, stream)
    p.rank_candidates(offs, pis, wis, threads=threads)
    _, edge, w, tree = p.candidates()
    times["generation"] = time.perf_counter() - t0
    K, N = len(w), p.N
    t1 = time.perf_counter()
    x = features(gen, w, tree, edge, stream)
    if prefix is not None:
        K_keep = int(min(max(prefix, 0), K))
        U = int(w[K_keep - 1]) if K_keep else 0
    elif net is not None:
        logits = net.forward(x, stream)
        torch.cuda.synchronize()
        lh = logits.cpu().numpy()
        if rule == "top":
            K_keep, U = proposal_prefix(lh, w, N, margin)
        else:
            K_keep, U = tail_prefix(lh, w, net.pos_weight, eps)
    else:
        K_keep, U = K, int(w[-1]) if K else 0
    times["proposal"] = time.perf_counter() - t1
    compared = []
    t_cmp = time.perf_counter()
    for other in compare:
        lg = other.forward(x, stream)
        torch.cuda.synchronize()
        lo = lg.cpu().numpy()
        compared.append(proposal_prefix(lo, w, N, margin) if rule == "top" else
                        tail_prefix(lo, w, other.pos_weight, eps))
    t_cmp = time.perf_counter() - t_cmp  # not part of the solve's time
    if not keep_features:
        del x
        x = None
    t2 = time.perf_counter()
    fallback = False
    nnz = build_lists(gen, K_keep, stream)
    dw, do, dc = gen.device_lists()
    solver = Solver.from_device_lists(N, K_keep, nnz, dw, do, dc, stream)
    times["lists"] = time.perf_counter() - t2
    t3 = time.perf_counter()
    solver.run(-1, stream)
    try:
        sel, tot = solver.results(stream=stream)
    except MCBError:
        if K_keep >= K:
            raise
        # the prefix did not hold a basis: the whole list, solved again
        fallback = True
        solver.close()
        nnz_full = build_lists(gen, K, stream)
        dw, do, dc = gen.device_lists()
        solver = Solver.from_device_lists(N, K, nnz_full, dw, do, dc, stream)
        solver.run(-1, stream)
        sel, tot = solver.results(stream=stream)
    times["solve"] = time.perf_counter() - t3
    times["total"] = time.perf_counter() - t0 - t_cmp
    trees_kept = int(len(np.unique(tree[:K_keep]))) if K_keep else 0
    lists = None
    if host_lists:
        off, co = gen.fetch_lists(stream)
        lists = (np.ascontiguousarray(w[:len(off) - 1]), off, co)
    gen.close()
    out = LearnedSolve(sel, tot, K, K_keep, U, nnz, p.F, trees_kept, fallback, times, lists, np.asarray(w),
                       compared, lh if (keep_logits and net is not None and prefix is None) else None)
    extra = []
    if keep_solver:
        extra += [solver, p]
    else:
        solver.close()
    if keep_features:
        extra.append(x)
    return (out, *extra) if extra else out


def traces(src, threads: int = 0, stream=0):
    """(features (K, 16) bf16, labels (K,) uint8, LearnedSolve) of a solved graph:
    label 1 for the candidates the plain solve selects."""
    import torch
    res, x = solve_with_proposal(src, None, threads=threads, stream=stream, keep_features=True)
    y = torch.zeros(res.K, dtype=torch.uint8, device="cuda")
    y[torch.from_numpy(np.asarray(res.selected, np.int64)).cuda()] = 1
    return x, y, res


def train(net: ProposalNet, xs, ys, epochs: int = 8, batch: int = 16384, lr: float = 3e-3,
          pos_weight: float | None = None, seed: int = 0, stream=0):
    """Adam on the mean weighted cross-entropy over the concatenated traces, shuffled
    each epoch; returns the mean loss of every epoch."""
    import torch
    x = torch.cat(list(xs))
    y = torch.cat(list(ys))
    n = x.shape[0]
    if pos_weight is None:
        pos = float(y.sum().item())
        pos_weight = max(1.0, (n - pos) / max(pos, 1.0))
    net.pos_weight = float(pos_weight)
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    losses = []
    for _ in range(epochs):
        perm = torch.randperm(n, device="cuda", generator=g)
        xp, yp = x[perm].contiguous(), y[perm].contiguous()
        tot, steps = 0.0, 0
        for i in range(0, n, batch):
            tot += net.train_step(xp[i:i + batch], yp[i:i + batch], pos_weight, lr, stream, want_loss=True)
            steps += 1
        losses.append(tot / max(steps, 1))
    return losses
