#!/usr/bin/env python3
"""Benchmark of the de Pina minimum-cycle-basis hot path on GB300.

Default workload (the scale configuration): a 1M-vertex planar-like graph, 263,000
triangulated grid points with 30% of the edges deleted (connectivity kept) and every
kept edge subdivided with probability 0.3 into a chain of 1-8 vertices, int32
weights U[1,1000], seed 1 (1,005,883 vertices; 241,787 after chain contraction;
N = 288,051 coordinates, S = 10.4 GB) - synthetic, from the repository's seeded
generator.  `--graph random --n 50000` is the 50k-vertex plain-GPU configuration.

Preparation (chain contraction, FVS and spanning tree on the host; per-root trees,
candidate test and coordinate lists on the GPU; ranking on the host) is timed once
as part of the graph-to-basis time (`e2e_with_preparation`).

One step = one complete de Pina solve (all N iterations) on the GPU: reset S to the
unit vectors, then the blocked device loop.  The rank-ordered candidates and their
coordinate lists stay resident in HBM.  The reset writes the whole support matrix
(10.4 GB at the default size), larger than the 129 MB L2, so every step starts with
a flushed L2.

  value       mean seconds per solve (CUDA events on the solver's stream)
  plain_gpu   the per-iteration device form (one odd-candidate search and one update
              per iteration, the reference loop's shape) timed on windows of
              iterations spread over the solve (each reached by the blocked run),
              integrated over all N iterations
  e2e         seconds per solve through the C ABI with pinned host buffers: upload
              (H2D of weights, offsets, coordinates) + solve + results (D2H)
  e2e_with_preparation  seconds from the graph's edge arrays in host memory to the
              basis: preparation + solve + results, once
  roofline    the kernel class with the largest time share, algorithmic bytes per
              launch / mean event-timed launch duration vs the measured HBM peak;
              the launch durations come from a second pass of the same K solves
              of the solver that gives `value`, with an event pair around every
              launch (out of the timed region); `search`: the same over the
              search kernels (streaming pass, correction, pivot search) together
  cpu_baseline  the reference's CPU main loop (oracle port of mcb/mcb_non_cpu_rd.cpp)
              on this host's cores: a label pass over a sample of the FVS trees
              and the full-width update over a sample of rows, extrapolated to the
              whole solve (N label passes over all F trees, N(N-1)/2 row updates)

`--workload batch` measures the batched configuration instead: --batch-count graphs
(n log-uniform in [50, 5000], average degree U[2.5, 5], w U[1, 255]) solved in one
BatchSolver (one persistent launch, one CTA per problem), the plain GPU form (the blocked
single-problem solver, problem after problem) on a sample beside it, and the
biconnected components of a --blocks block tree in a second batch.

`--impl reference` times only that CPU implementation and prints its own line (with
`--workload batch`: full solves of a time-bounded sample of the batch's graphs,
extrapolated by each problem's label cost N * F * n').
Under torchrun (N > 1) every rank solves its own replica (the loop does not shard).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MCB solve time (s) & search HBM GB/s: batched+learned vs plain GPU, exact"
# total basis weights of the seeded workloads (graph family, --n, --seed): the
# blocked solver's result, equal to the per-iteration form's on the same candidates
PINNED_WEIGHTS = {("planar", 263000, 1): 1008336977, ("random", 50000, 1): 180590671}
DEFAULT_N = {"planar": 263000, "random": 50000, "rgg": 20000}
BATCH_WORKLOAD = ("batched: %d random graphs, n log-uniform [50,5000], avg degree U[2.5,5], w U[1,255], seed %d; "
                  "one batched solve of all of them")


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if self.proc is None or not self.path or not os.path.exists(self.path):
            return None
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() and args.impl != "reference" else "gloo"
        dist.init_process_group(backend=backend)
        pg = dist
    return world, rank, local, pg


def max_over_ranks(x, pg):
    """The largest of every rank's `x` (the slowest rank's time), on every rank."""
    if not pg:
        return x
    import torch
    dev = "cuda" if pg.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def make_graph(args):
    from minimumcyclebasis_gb300 import planar_chain_graph, random_graph, rgg_graph
    if args.graph == "rgg":  # the learned-proposal configuration's family
        return rgg_graph(args.n, 4, args.seed)
    if args.graph == "planar":  # the scale configuration's family, --n triangulated points
        return planar_chain_graph(args.n, 30, 30, 8, 1, 1000, args.seed)
    return random_graph(args.n, 2 * args.n, 1, 1000, args.seed)


def config_of(p, args, extra=None):
    i = p.info
    names = {"random": "random sparse graph n=%d m=%d (avg degree 4), int32 w U[1,1000], seed %d"
                       % (args.n, 2 * args.n, args.seed),
             "rgg": "random geometric graph n=%d, k=4 nearest neighbours, w = round(1000 x length), seed %d"
                    % (args.n, args.seed),
             "planar": "planar-like graph from %d triangulated points, 30%% of edges deleted, 30%% subdivided into "
                       "chains of 1-8, w U[1,1000], seed %d" % (args.n, args.seed)}
    c = {"workload": names[args.graph] + "; full de Pina solve", "input_nodes": i.nodes,
         "reduced_nodes": i.reduced_nodes, "fvs": i.fvs_size, "N": i.num_coords, "K": i.num_candidates,
         "form": args.mode, "host_threads": os.cpu_count()}
    if extra:
        c.update(extra)
    return c


def cpu_baseline(p, args, threads):
    """The reference CPU main loop's cost on this host, from samples: a label pass
    (worker_thread::precompute_supportVec, the loop's per-iteration relabelling of
    every FVS tree) over `--cpu-sample-roots` trees spread over the FVS, and the
    full-width dot/XOR update over 2048 rows; extrapolated to N passes over all F
    trees and N(N-1)/2 row updates.  The list scan, which stops at the first odd
    candidate, is left out, so this is a lower bound of the loop's time."""
    import numpy as np

    import oracle
    threads = threads or os.cpu_count() or 1
    F, n, N = p.F, p.n, p.N
    step = max(1, F // max(1, args.cpu_sample_roots))
    idx = np.arange(0, F, step, dtype=np.int32)[:args.cpu_sample_roots]
    t0 = time.perf_counter()
    _, ps = p.search_trees(idx, threads=threads)
    t_trees = time.perf_counter() - t0
    lab = oracle.label_pass_seconds(p, ps, passes=3, threads=threads)
    row = oracle.update_row_seconds(N, rows=2048, passes=3, threads=threads)
    label_total = lab * F / len(idx) * N
    update_total = row * N * (N - 1) / 2.0
    value = label_total + update_total
    return {"value": value, "unit": "s", "cores": threads, "kind": "port",
            "sample": "reference CPU main loop (oracle port of mcb/mcb_non_cpu_rd.cpp:264-342) from samples: a label "
                      "pass over %d of the %d FVS trees %.4f s (x %d/%d trees x %d iterations = %.4g s), the "
                      "full-width update %.3g s per row (x N(N-1)/2 = %.4g s); list scan omitted (a lower bound); "
                      "the sampled trees searched on the host in %.1f s, untimed"
                      % (len(idx), F, lab, F, len(idx), N, label_total, row, update_total, t_trees)}


def label_cost(info):
    """Per-solve work of the reference CPU loop on one problem: every iteration
    relabels all FVS trees, N * F * n' label writes (the constant that the time
    extrapolation of a sample scales by)."""
    return float(info.num_coords) * info.fvs_size * info.reduced_nodes


def batch_cpu_baseline(graphs, costs, threads, budget_s, want=None):
    """Full solves of the reference CPU main loop (oracle port of
    mcb/mcb_non_cpu_rd.cpp:264-342) on a strided sample of the batch's graphs, taken
    in order until `budget_s` seconds of solve time are spent, skipping a problem
    whose predicted time (its cost at the rate seen so far) is above half the budget;
    extrapolated to the whole batch by the label cost N * F * n' of every problem
    (the rate per unit of cost is flat in problem size).  `costs` maps each
    graph index to its cost (graphs that are a single ring or a tree are absent);
    `want` maps graph index to the GPU's (selected ranks, total weight) to compare."""
    import numpy as np

    import oracle
    from minimumcyclebasis_gb300 import Problem
    threads = threads or os.cpu_count() or 1
    idx = sorted(costs)
    stride = 16
    order = [j for off in range(stride) for j in idx[(off * 7) % stride::stride]]
    t_sum, c_sum, solved, checked, skipped = 0.0, 0.0, 0, 0, 0
    rate0 = 1.2e-8 / threads  # seconds per unit of cost before any measurement
    for j in order:
        rate = t_sum / c_sum if c_sum > 0 and t_sum > 0.5 else rate0
        if costs[j] * rate > budget_s / 2:
            skipped += 1
            continue
        p = Problem.from_graph(graphs[j]).prepare(threads=threads, keep_trees=True)
        sel, tot, sec = oracle.solve(p, threads=threads)
        if want is not None and j in want:
            assert np.array_equal(sel, want[j][0]) and tot == want[j][1], "oracle and GPU results differ"
            checked += 1
        t_sum += sec
        c_sum += costs[j]
        solved += 1
        if t_sum >= budget_s:
            break
    total_cost = sum(costs.values())
    value = t_sum / max(c_sum, 1.0) * total_cost
    return {"value": value, "unit": "s", "cores": threads, "kind": "port",
            "sample": "full solves of %d of the %d searched problems by the reference CPU main loop (oracle port "
                      "of mcb/mcb_non_cpu_rd.cpp:264-342), %.2f s, extrapolated by the per-problem label cost "
                      "N*F*n' (sample %.3g of %.3g; %d problems predicted above half the budget skipped)%s"
                      % (solved, len(idx), t_sum, c_sum, total_cost, skipped,
                         "; %d checked equal to the GPU's" % checked if want is not None else "")}


def run_reference_batch(args, world, rank, pg):
    import numpy as np

    from minimumcyclebasis_gb300 import Problem, batch_graphs, prepare_many
    threads = args.cpu_threads or os.cpu_count() or 1
    graphs = batch_graphs(args.batch_count, seed=args.seed)
    costs, Ns = {}, []
    ps = prepare_many([Problem.from_graph(g) for g in graphs], threads=threads, cycle_lists=False)
    for j in range(len(graphs)):
        info, ps[j] = ps[j].info, None
        if not info.single_cycle and info.num_coords > 0:
            costs[j] = label_cost(info)
            Ns.append(info.num_coords)
    for _ in range(args.warmup):
        batch_cpu_baseline(graphs, costs, threads, args.cpu_budget / 8)
    vals = []
    t0 = time.time()
    for _ in range(args.steps):
        vals.append(batch_cpu_baseline(graphs, costs, threads, args.cpu_budget))
    wall = time.time() - t0
    v = statistics.mean(x["value"] for x in vals)
    cb = dict(vals[-1])
    cb["value"] = v
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": "s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": wall / max(args.steps, 1) * 1000.0, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic",
            "config": {"workload": BATCH_WORKLOAD % (args.batch_count, args.seed), "problems": len(costs),
                       "N_max": int(max(Ns, default=0)), "N_sum": int(np.sum(Ns)),
                       "form": "reference CPU loop (oracle port), bounded sample of full solves"},
            "cpu_baseline": cb, "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def run_reference(args, world, rank, pg):
    if rank != 0:
        return None
    if args.workload == "batch":
        return run_reference_batch(args, world, rank, pg)
    from minimumcyclebasis_gb300 import Problem
    threads = args.cpu_threads or os.cpu_count() or 1
    t0 = time.time()
    p = Problem.from_graph(make_graph(args)).prepare(threads=threads, structure_only=True)
    log("structure prepared in %.1fs: n'=%d F=%d N=%d" % (time.time() - t0, p.n, p.F, p.N))
    for _ in range(args.warmup):
        cpu_baseline(p, argparse.Namespace(cpu_sample_roots=max(16, args.cpu_sample_roots // 8)), threads)
    vals = []
    t0 = time.time()
    for _ in range(args.steps):
        vals.append(cpu_baseline(p, args, threads))
    wall = time.time() - t0
    v = statistics.mean(x["value"] for x in vals)
    cb = dict(vals[-1])
    cb["value"] = v
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": "s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": wall / max(args.steps, 1) * 1000.0, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic",
            "config": config_of(p, args, {"form": "reference CPU loop (oracle port), sampled",
                                          "input": "graph prepared up to its spanning tree by this repository's "
                                                   "host library (untimed); the sampled trees by its heap-ordered "
                                                   "searches (untimed)"}),
            "cpu_baseline": cb, "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def solver_words(N):
    """64-bit words of one support-vector row in the solver (ceil(N / 64) rounded up to 4)."""
    return ((N + 63) // 64 + 3) // 4 * 4


def pinned_like(a):
    """A pinned host copy of numpy array `a` (cudaMallocHost through the C ABI)."""
    import ctypes as C

    import numpy as np

    from minimumcyclebasis_gb300._native import check_gpu, gpu_lib
    lib = gpu_lib()
    ptr = C.c_void_p()
    check_gpu(lib.mcbgpu_allocate_pinned(max(a.nbytes, 1), C.byref(ptr)), "mcbgpu_allocate_pinned")
    buf = (C.c_char * max(a.nbytes, 1)).from_address(ptr.value)
    out = np.frombuffer(buf, dtype=a.dtype, count=a.size)
    out[...] = a
    return out, ptr


def plain_form(solver, N, stream, sh, windows=8, width=128):
    """The per-iteration device form (mcbgpu_select + mcbgpu_update per iteration)
    timed on `windows` windows of `width` iterations centred at (k + 1/2) N / windows,
    each reached by the blocked run; integrated over N iterations (midpoint rule).
    Each window's selections are checked against the blocked run's."""
    import numpy as np
    import torch
    full_sel, _ = solver.results(stream=sh)
    per_iter, starts = [], []
    for k in range(windows):
        e0 = int((k + 0.5) * N / windows) - width // 2
        e0 = max(0, min(N - width, e0)) // 64 * 64
        w = min(width, N - e0)
        solver.reset(sh)
        solver.run(e0, sh)
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ev0.record(stream)
        for e in range(e0, e0 + w):
            solver.select(e, sh, fetch=False)
            solver.update(e, sh)
        ev1.record(stream)
        torch.cuda.synchronize()
        sel, _ = solver.results(e0 + w, stream=sh)
        assert np.array_equal(sel[e0:e0 + w], full_sel[e0:e0 + w]), "per-iteration and blocked selections differ"
        per_iter.append(ev0.elapsed_time(ev1) / 1e3 / w)
        starts.append(e0)
    total = float(np.mean(per_iter) * N)
    return {"value": total, "unit": "s",
            "sample": "per-iteration device form (select + update per iteration) on %d windows of %d iterations "
                      "starting at %s, each reached by the blocked run; mean %.3f ms per iteration x %d iterations "
                      "(midpoint rule); every window's selections equal the blocked run's"
                      % (windows, width, starts, float(np.mean(per_iter)) * 1e3, N),
            "ms_per_iteration": [round(x * 1e3, 4) for x in per_iter]}


def forward_throughput(net, x, sh, reps: int = 10):
    """The proposal network's forward pass (mlp_forward_kernel) over the workload's
    K x 16 bf16 features, timed with CUDA events on its stream after 3 warm-up passes:
    ms per pass and GB/s of its algorithmic bytes (32 B of features read and a 4 B
    logit written per candidate; the 16 x 64 weights stay in shared memory)."""
    import torch
    stream = torch.cuda.ExternalStream(sh)
    for _ in range(3):
        net.forward(x, sh)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        net.forward(x, sh)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    K = int(x.shape[0])
    return {"candidates": K, "ms": round(ms, 4), "GBps": round(36.0 * K / ms / 1e6, 1),
            "tflops_first_layer": round(2.0 * 16 * 64 * K / ms / 1e9, 2)}


def learned_form(args, g, sel0, tot0, sh):
    """Trains the proposal network on traces of --train-graphs smaller graphs of the
    workload's family (seeds after the workload's), then solves the workload graph
    -> basis with the proposal's prefix.  Returns (the line's `learned` object, the
    solver holding the prefix lists, the prefix lists' host copies, graph-to-basis
    seconds of the learned form)."""
    import numpy as np

    from minimumcyclebasis_gb300.learned import (ProposalNet, calibrate_margin, needed_margin, solve_with_proposal,
                                                 traces, train)
    small = argparse.Namespace(**vars(args))
    small.n = args.train_n
    t0 = time.perf_counter()
    xs, ys, ks, rs = [], [], [], []
    for i in range(args.train_graphs):
        small.seed = args.seed + 1000 + i
        x, y, res = traces(make_graph(small))
        xs.append(x)
        ys.append(y)
        ks.append(res.K)
        rs.append(res)
    t_traces = time.perf_counter() - t0
    net = ProposalNet(seed=args.seed)
    t1 = time.perf_counter()
    losses = train(net, xs, ys, epochs=args.train_epochs)
    t_train = time.perf_counter() - t1
    # the top-score margin each training graph needed with the trained network, and
    # the margin calibrated from them for the unseen workload graph
    needed = [needed_margin(net.forward(x, sh).cpu().numpy(), r.weight_sorted, len(r.selected), r.K_needed)
              for x, r in zip(xs, rs)]
    margin = calibrate_margin(needed) if args.proposal_rule == "calibrated" else args.margin
    rule = "top" if args.proposal_rule == "calibrated" else args.proposal_rule
    del xs, ys, rs
    untrained = ProposalNet(seed=args.seed)
    # graph -> basis on the proposal's prefix (its lists copied to the host afterwards,
    # for the end-to-end steps; the untrained network's prefix on the same features
    # for comparison: neither is part of the timed solve)
    r, lsolver, p, x = solve_with_proposal(g, net, margin=margin, stream=sh, keep_solver=True,
                                           host_lists=True, compare=[untrained], rule=rule,
                                           eps=args.eps, keep_logits=True, keep_features=True)
    fwd = forward_throughput(net, x, sh)
    del x
    g2b = r.times["total"]
    assert np.array_equal(r.selected, sel0) and r.total_weight == tot0, "the learned form's basis differs"
    uk, _ = r.compared[0]
    from minimumcyclebasis_gb300.learned import proposal_table
    _, _, wsorted, _ = p.candidates()
    K_needed = int(np.max(sel0)) + 1  # the prefix the solve needs: up to its last selection
    table = proposal_table(r.logits, wsorted, p.N, net.pos_weight, K_needed)
    learned = {"skip_rate": r.skip_rate, "proposed_skip_rate": r.proposed_skip_rate, "diffs": 0,
               "fallback": r.fallback, "K": r.K, "K_kept": r.K_kept,
               "K_needed": K_needed, "U": r.U, "nnz_kept": r.nnz_kept, "trees": r.trees,
               "trees_kept": r.trees_kept, "rule": args.proposal_rule,
               "rule_param": args.eps if args.proposal_rule == "tail" else margin,
               "training_needed_margins": [round(m, 4) for m in needed],
               "untrained_skip_rate": 1.0 - uk / max(r.K, 1), "rules_on_this_graph": table,
               "training": {"graphs": args.train_graphs, "points": args.train_n, "candidates": int(sum(ks)),
                            "epochs": args.train_epochs, "loss_first_last": [round(losses[0], 4),
                                                                             round(losses[-1], 4)],
                            "traces_s": round(t_traces, 2), "train_s": round(t_train, 2)},
               "times_s": {k: round(v, 3) for k, v in r.times.items()}, "forward": fwd}
    untrained.close()
    return learned, lsolver, r.lists, g2b


def run_gpu(args, world, rank, local, pg):
    import numpy as np
    import torch

    from minimumcyclebasis_gb300 import Problem, Solver, prepare_on_device
    from minimumcyclebasis_gb300.build import build_all

    build_all()
    torch.cuda.set_device(local)
    want_cpu = rank == 0 and world == 1 and not args.no_cpu_baseline
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    g = make_graph(args)
    pin = PINNED_WEIGHTS.get((args.graph, args.n, args.seed))

    # graph -> basis, once: preparation + solve + results
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    tree_shapes = None
    if args.prep == "device":
        dp, gen = prepare_on_device(g, threads=0, stream=sh, keep_gen=True)
        p, solver = dp.problem, dp.solver
        prep_times = dict(dp.times)
        tree_shapes = dp.tree_shapes
    else:
        p = Problem.from_graph(g).prepare(threads=0)
        i = p.info
        prep_times = {"total": time.perf_counter() - t0, "trees": i.t_trees, "collect": i.t_collect}
        solver = Solver.from_problem(p, stream=sh)
    solver.run(args.max_iterations, sh)
    sel0, tot0 = solver.results(stream=sh)
    graph_to_basis = time.perf_counter() - t0
    log("graph to basis %.2fs (preparation %.2fs), total weight %d" % (graph_to_basis, prep_times["total"], tot0))
    if args.max_iterations < 0 and pin is not None:
        assert tot0 == pin, "total weight %d differs from the pinned %d" % (tot0, pin)
    # host copies of the lists, for the end-to-end steps from pinned host buffers
    _, _, w, _ = p.candidates()
    if args.prep == "device":
        off, co = gen.fetch_lists()
        gen.close()
        tied = dp.tied_roots
    else:
        off, co = p.cycle_lists()
        tied = None

    def solve_once():
        solver.reset(sh)
        solver.run(args.max_iterations, sh)

    def timed(s, step):
        """args.steps solves by step() after args.warmup untimed ones: CUDA events on the
        solver's stream, clocks sampled meanwhile, the results checked.  Returns (ms per
        solve, launches in the timed region, clock summary)."""
        for _ in range(args.warmup):
            step()
        r_sel, r_tot = s.results(stream=sh)
        assert np.array_equal(r_sel, sel0) and r_tot == tot0, "warm-up solve differs from the first"
        torch.cuda.synchronize()
        if pg:
            pg.barrier()
        l0 = s.launches
        with ClockSampler(local) as clk:
            torch.cuda.synchronize()
            e_a = torch.cuda.Event(enable_timing=True)
            e_b = torch.cuda.Event(enable_timing=True)
            e_a.record(stream)
            for _ in range(args.steps):
                step()
            e_b.record(stream)
            torch.cuda.synchronize()
        t_ms = e_a.elapsed_time(e_b) / args.steps
        n_l = s.launches - l0
        r_sel, r_tot = s.results(stream=sh)
        assert np.array_equal(r_sel, sel0) and r_tot == tot0, "timed solves differ from the first"
        if pg:
            t_ms = max_over_ranks(t_ms, pg)
            pg.barrier()
        return t_ms, n_l, clk.summary()

    # search shapes: one tuning solve (the candidate shapes take turns group by group;
    # each quarter of the solve keeps its fastest), checked like any other solve
    shapes = None
    if args.max_iterations < 0 and args.tune:
        shapes = solver.tune(sh)
        sel, tot = solver.results(stream=sh)
        assert np.array_equal(sel, sel0) and tot == tot0, "the tuning solve differs from the first"
    ms, launches, clocks = timed(solver, solve_once)

    # the learned proposal: a network trained on traces of smaller graphs of the same
    # family (its own kernels), then the graph -> basis solve on the proposal's
    # prefix of the rank order, checked against the full list's basis
    learned = None
    lsolver = None
    if args.learned and args.prep == "device" and args.max_iterations < 0:
        learned, lsolver, lists_l, lg2b = learned_form(args, g, sel0, tot0, sh)

    plain = None
    if not args.no_plain and args.max_iterations < 0:
        plain = plain_form(solver, p.N, stream, sh, windows=args.plain_windows, width=args.plain_width)

    full_ms = ms
    if lsolver is not None:
        # the learned form's solve on its resident prefix lists, timed as above (its
        # own tuning solve first)
        lshapes = None
        if args.tune:
            lshapes = lsolver.tune(sh)
            lsel, ltot = lsolver.results(stream=sh)
            assert np.array_equal(lsel, sel0) and ltot == tot0, "the learned form's tuning solve differs"
        def lsolve():
            lsolver.reset(sh)
            lsolver.run(-1, sh)

        lms, llaunches, lclocks = timed(lsolver, lsolve)
        learned["solve_s"] = lms / 1e3
        learned["solve_s_full_list"] = full_ms / 1e3
        if lms < ms:  # the fastest form is the line's value; its lists feed the e2e below
            ms = lms
            launches = llaunches
            clocks = lclocks
            shapes = lshapes
            solver.close()
            solver = lsolver
            w, off, co = lists_l
            learned["is_value"] = True
        else:
            lsolver.close()

    # the same solve (reset + blocked run) as one CUDA graph, captured once and
    # replayed; the faster launch form gives the value
    launch_form = {"form": "streams", "stream_ms": ms}
    use_graph = False
    if args.cuda_graph:
        from minimumcyclebasis_gb300._native import MCBError
        try:
            t_c = time.perf_counter()
            solver.run_graph(args.max_iterations, sh)
            torch.cuda.synchronize()
            capture_s = time.perf_counter() - t_c
            gms, glaunches, gclocks = timed(solver, lambda: solver.run_graph(args.max_iterations, sh))
            launch_form.update({"graph_ms": gms, "capture_and_first_replay_s": capture_s})
            if gms < ms:
                ms, launches, clocks, use_graph = gms, glaunches, gclocks, True
                launch_form["form"] = "graph"
        except MCBError as exc:
            launch_form["graph"] = "unavailable: %s" % exc

    if plain is not None:  # the per-iteration form against the fastest form
        plain["speedup"] = plain["value"] / (ms / 1e3)
        plain["speedup_vs_full_list"] = plain["value"] / (full_ms / 1e3)

    # per-kernel durations of the solver that gives `value`: K solves again, with an
    # event pair around every launch on its streams (kept out of the timed region),
    # and its search counters
    solver.diagnostics(reset=True)
    solver.set_profiling(True)
    for _ in range(args.steps):
        solver.reset(sh)
        solver.run(args.max_iterations, sh)
    torch.cuda.synchronize()
    stats = solver.kernel_stats()
    solver.set_profiling(False)
    diag = solver.diagnostics(reset=True)

    # end to end through the C ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        pw, pw_h = pinned_like(w)
        po, po_h = pinned_like(off)
        pc, pc_h = pinned_like(co)
        psel, psel_h = pinned_like(np.zeros(max(p.N, 1), np.int64))
        import ctypes as C

        from minimumcyclebasis_gb300._native import check_gpu, gpu_lib
        lib = gpu_lib()
        tot_c = C.c_int64()

        def e2e_once():
            solver.upload(sh, pw, po, pc)
            if use_graph:  # the graph reads the handle's buffers the upload refills
                solver.run_graph(args.max_iterations, sh)
            else:
                solver.run(args.max_iterations, sh)
            check_gpu(lib.mcbgpu_solver_results(solver._h, C.c_void_p(psel.ctypes.data), p.N, C.byref(tot_c),
                                                C.c_void_p(sh)), "mcbgpu_solver_results")

        e2e_once()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            e2e_once()
        e2e_s = (time.perf_counter() - t0) / args.e2e_steps
        iters = p.N if args.max_iterations < 0 else min(args.max_iterations, p.N)
        assert np.array_equal(psel[:iters], sel0[:iters]) and tot_c.value == tot0, "e2e results differ"
        e2e = {"value": e2e_s, "unit": "s", "steps": args.e2e_steps,
               "h2d_bytes_per_step": int(w.nbytes + off.nbytes + co.nbytes),
               "d2h_bytes_per_step": int(8 * p.N + 8 + 4)}
        for h in (pw_h, po_h, pc_h, psel_h):
            lib.mcbgpu_free_pinned(h)

    # roofline of the kernel class with the largest time share
    peak, peak_kind = measured_peaks()
    top = max(stats.items(), key=lambda kv: kv[1]["ms"])
    name, st = top
    per_launch_s = st["ms"] / 1e3 / max(st["launches"], 1)
    per_launch_b = st["bytes"] / max(st["launches"], 1)
    achieved = per_launch_b / per_launch_s / 1e9 if per_launch_s > 0 else 0.0
    traffic = None  # DRAM bytes per launch need an ncu capture; the ncu summaries are under profiles/
    total_ms = sum(v["ms"] for v in stats.values())
    # the search phase (streaming pass, its correction, the pivot search): the part of
    # the metric's "search HBM GB/s" -- their algorithmic bytes over their event time
    srch = [stats[k] for k in ("blk_w", "blk_wfix", "blk_pivot") if k in stats]
    s_ms = sum(v["ms"] for v in srch)
    s_b = sum(v["bytes"] for v in srch)
    blocks = max(int(diag.get("blocks", 0)), 1)
    search = {"kernels": ["blk_w", "blk_wfix", "blk_pivot"], "GBps": s_b / (s_ms / 1e3) / 1e9 if s_ms > 0 else None,
              "frac": (s_b / (s_ms / 1e3) / 1e9) / peak if s_ms > 0 else None, "ms_per_solve": s_ms / args.steps,
              "pivot_steps_per_block": diag.get("pivot_steps", 0) / blocks,
              "tiles_loaded_per_block": diag.get("tiles_loaded", 0) / blocks,
              "tiles_computed_per_block": diag.get("tiles_computed", 0) / blocks}
    far = {"dense_rows_per_block": diag.get("far_rows_gathered", 0) / blocks,
           "sparse_rows_per_block": diag.get("far_sparse_rows", 0) / blocks,
           "listed_words_per_sparse_row": diag.get("far_sparse_words", 0) / max(diag.get("far_sparse_rows", 0), 1),
           "changed_rows_per_block": diag.get("far_rows_changed", 0) / blocks,
           "touched_unit_rows_per_block": diag.get("far_rows_touched", 0) / blocks}
    roofline = {"kernel": name, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
                "bytes_per_launch": per_launch_b, "launch_ms": per_launch_s * 1e3, "share": st["ms"] / total_ms,
                "search": search, "far_update": far,
                "kernels": {k: {"launches": v["launches"], "ms": round(v["ms"], 3),
                                "GBps": (v["bytes"] / (v["ms"] / 1e3) / 1e9) if v["ms"] > 0 and v["bytes"] else None}
                            for k, v in sorted(stats.items(), key=lambda kv: -kv[1]["ms"])}}

    cb = None
    if want_cpu:
        cb = cpu_baseline(p, args, args.cpu_threads)
    if rank != 0:
        return None
    extra = {"total_weight": tot0, "total_weight_pinned": pin, "solves_per_s_all_ranks": world * 1e3 / ms,
             "search_shapes": shapes, "launch_form": launch_form,
             "cycle_nnz": int(off[-1]), "preparation": args.prep,
             "l2": ("every solve starts by writing the %.1f GB support matrix (reset to unit vectors), larger than "
                    "the 129 MB L2, which flushes it between steps; cycle lists %.2f GB"
                    % (8.0 * p.N * solver_words(p.N) / 1e9, int(off[-1]) * 4 / 1e9))}
    return {"metric": METRIC, "value": ms / 1e3, "unit": "s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "u64", "data": "synthetic", "config": config_of(p, args, extra),
            "clocks": clocks, "e2e": e2e,
            "e2e_with_preparation": {"value": graph_to_basis, "unit": "s", "runs": 1,
                                     "preparation_s": {k: round(v, 3) for k, v in prep_times.items()},
                                     "tied_roots_searched_on_host": tied, "tree_kernel_shapes": tree_shapes,
                                     "learned_form": lg2b if learned else None,
                                     "note": "graph edge arrays in host memory -> basis in host memory: "
                                             "preparation + solve + results, measured once (learned_form: the "
                                             "same with the proposal's prefix, the network trained beforehand)"},
            "plain_gpu": plain, "learned": learned, "gpu_launches": int(launches), "roofline": roofline,
            "cpu_baseline": cb}


def run_batch(args, world, rank, local, pg):
    """The batched configuration: `--batch-count` independent graphs (n log-uniform in
    [50, 5000], average degree U[2.5, 5], w U[1, 255]) in one BatchSolver, plus the
    biconnected components of a tree of `--blocks` random blocks in a second one.
    One step = one batched solve of all the graphs' problems, inputs resident."""
    import numpy as np
    import torch

    from minimumcyclebasis_gb300 import (BatchSolver, Problem, Solver, batch_graphs, bcc_split, block_tree_graph,
                                         prepare_many)
    from minimumcyclebasis_gb300.build import build_all

    build_all()
    torch.cuda.set_device(local)
    t0 = time.time()

    def problems(graphs):
        items, host_total, nsc, costs = [], 0, 0, {}
        ps = prepare_many([Problem.from_graph(g) for g in graphs])  # in parallel, one thread per graph
        for j, g in enumerate(graphs):
            p, ps[j] = ps[j], None  # each problem's host copy is freed once its arrays are taken
            if p.info.single_cycle:  # the graph is one cycle: its basis needs no search
                host_total += int(g.w.astype(np.int64).sum())
                nsc += 1
                continue
            if p.N == 0:
                continue
            _, _, w, _ = p.candidates()
            off, co = p.cycle_lists()
            items.append((p.N, w, off, co))
            costs[j] = label_cost(p.info)
        return items, host_total, nsc, costs

    graphs = batch_graphs(args.batch_count, seed=args.seed + rank)
    items, host_total, nsc, costs = problems(graphs)
    bt = block_tree_graph(args.blocks, seed=args.seed + rank)
    comps = bcc_split(bt)
    bitems, bhost_total, bnsc, _ = problems(comps)
    prep_s = time.time() - t0
    log("prepared in %.1fs: %d batch problems (%d rings), %d block-tree components (%d rings)"
        % (time.time() - t0, len(items), nsc, len(bitems), bnsc))
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    bs = BatchSolver(items, stream=sh)
    bb = BatchSolver(bitems, stream=sh)
    for _ in range(args.warmup):
        bs.run(sh)
        bb.run(sh)
    sels, tots = bs.results(sh)
    bsels, btots = bb.results(sh)
    torch.cuda.synchronize()
    if pg:
        pg.barrier()

    def timed(solver):
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(args.steps):
            solver.run(sh)
        ev1.record(stream)
        torch.cuda.synchronize()
        return ev0.elapsed_time(ev1) / args.steps

    launches0 = bs.launches
    with ClockSampler(local) as clocks:
        ms = timed(bs)
    launches = bs.launches - launches0
    ms_blocks = timed(bb)
    if pg:
        ms = max_over_ranks(ms, pg)

    # the plain GPU form: one blocked single-problem solver per problem, in sequence,
    # on every `plain_stride`-th problem (extrapolated to all)
    stride = max(1, args.plain_stride)
    plain_ms, checked = 0.0, 0
    for i in range(0, len(items), stride):
        s = Solver(*items[i], stream=sh)
        torch.cuda.synchronize()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        s.run(-1, sh)
        ev1.record(stream)
        sel, tot = s.results(stream=sh)
        plain_ms += ev0.elapsed_time(ev1)
        assert np.array_equal(sel, sels[i]) and tot == tots[i], "batched and single-problem results differ"
        checked += 1
        s.close()
    plain_est_s = plain_ms / 1e3 * len(items) / max(checked, 1)

    # per-problem profile: CTA time split and scanned candidates
    bs.set_profiling(True)
    bs.run(sh)
    prof = bs.profile()
    bs.set_profiling(False)
    cyc = prof[:, 1:6].sum(0).astype(float)
    Ns = np.array([it[0] for it in items])

    # end to end: upload from pinned host buffers, run, results
    e2e = None
    if not args.no_e2e:
        import ctypes as C

        from minimumcyclebasis_gb300._native import check_gpu, gpu_lib
        lib = gpu_lib()
        pw, pw_h = pinned_like(bs.weight)
        po, po_h = pinned_like(bs.offsets)
        pc, pc_h = pinned_like(bs.coords)
        psel, psel_h = pinned_like(np.zeros(max(int(Ns.sum()), 1), np.int64))
        ptot, ptot_h = pinned_like(np.zeros(max(len(items), 1), np.int64))

        def e2e_once():
            check_gpu(lib.mcbgpu_batch_upload(bs._h, C.c_void_p(pw.ctypes.data), C.c_void_p(po.ctypes.data),
                                              C.c_void_p(pc.ctypes.data), C.c_void_p(sh)), "mcbgpu_batch_upload")
            bs.run(sh)
            check_gpu(lib.mcbgpu_batch_results(bs._h, C.c_void_p(psel.ctypes.data), C.c_void_p(ptot.ctypes.data),
                                               None, C.c_void_p(sh)), "mcbgpu_batch_results")

        e2e_once()
        t1 = time.perf_counter()
        for _ in range(args.e2e_steps):
            e2e_once()
        e2e_s = (time.perf_counter() - t1) / args.e2e_steps
        assert np.array_equal(ptot[:len(items)], tots), "e2e results differ"
        e2e = {"value": e2e_s, "unit": "s", "steps": args.e2e_steps,
               "h2d_bytes_per_step": int(bs.weight.nbytes + bs.offsets.nbytes + bs.coords.nbytes),
               "d2h_bytes_per_step": int(8 * Ns.sum() + 8 * len(items) + 4)}
        for h in (pw_h, po_h, pc_h, psel_h, ptot_h):
            lib.mcbgpu_free_pinned(h)
    if rank != 0:
        return None
    cb = None
    if world == 1 and not args.no_cpu_baseline:
        want = {j: (sels[i], tots[i]) for i, j in enumerate(sorted(costs))}
        cb = batch_cpu_baseline(graphs, costs, args.cpu_threads, args.cpu_budget, want)
    nnz = int(bs.offsets[-1])
    scanned = int(prof[:, 6].sum())
    K = int(bs.weight.shape[0])
    # the scan reads, per scanned candidate, its two offsets and its coordinate list up
    # to the block's bound: the bytes the kernel counted as it walked them
    scan_bytes = float(prof[:, 12].sum())
    peak, peak_kind = measured_peaks()
    achieved = scan_bytes / (ms / 1e3) / 1e9
    return {"metric": METRIC, "value": ms / 1e3, "unit": "s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "u64", "data": "synthetic",
            "config": {"workload": BATCH_WORKLOAD % (args.batch_count, args.seed),
                       "problems": len(items), "rings_on_host": nsc, "N_max": int(Ns.max()), "N_sum": int(Ns.sum()),
                       "K": K, "cycle_nnz": nnz, "form": "batched (one persistent launch, one CTA per problem)",
                       "total_weight": int(tots.sum()) + host_total,
                       "l2": "inputs (%.2f GB) larger than the 129 MB L2; no flush" % ((nnz * 4 + K * 12) / 1e9),
                       "host_preparation_s": round(prep_s, 3), "host_threads": os.cpu_count()},
            "clocks": clocks.summary(), "e2e": e2e, "gpu_launches": int(launches),
            "plain_gpu": {"value": plain_est_s, "unit": "s", "speedup": plain_est_s / (ms / 1e3),
                          "sample": "blocked single-problem solver on every %d-th problem (%d solves, %.1f ms), "
                                    "extrapolated to all %d; selected ranks and weights equal the batch's"
                                    % (stride, checked, plain_ms, len(items))},
            "block_tree": {"blocks": args.blocks, "nodes": int(bt.nodes), "components_on_gpu": len(bitems),
                           "rings_on_host": bnsc, "value": ms_blocks / 1e3, "unit": "s",
                           "total_weight": int(btots.sum()) + bhost_total},
            "profile": {"cta_ms_sum": float(prof[:, 0].sum() / 1e6), "cta_ms_max": float(prof[:, 0].max() / 1e6),
                        "cycle_share": dict(zip(["transpose", "scan", "resolve", "final_rows", "update"],
                                                [round(float(c / cyc.sum()), 4) for c in cyc])),
                        "scanned_candidates": scanned},
            "roofline": {"kernel": "batch_solve", "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind, "traffic": None,
                         "bytes_per_launch": scan_bytes, "launch_ms": ms,
                         "note": "scan bytes (offsets + coordinates the list walks read, counted by the kernel) "
                                 "per batched solve; the kernel is latency-bound on the per-problem critical path"},
            "cpu_baseline": cb}


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--n", "--vertices", dest="n", type=int, default=None,
                    help="graph size: planar: triangulated points (default 263000); random: vertices, edges = 2n "
                         "(default 50000); rgg: vertices (default 20000)")
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--mode", choices=["blocked", "plain"], default="blocked")
    ap.add_argument("--max-iterations", type=int, default=-1)
    ap.add_argument("--cpu-sample-roots", type=int, default=2000,
                    help="FVS trees in the CPU baseline's label-pass sample")
    ap.add_argument("--cpu-threads", type=int, default=0)
    ap.add_argument("--cpu-budget", type=float, default=20.0,
                    help="seconds of CPU solve time in the batched workload's baseline sample")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--graph", choices=["random", "rgg", "planar"], default="planar",
                    help="graph family of the single-graph workload (planar: the 1M-vertex scale configuration; "
                         "random: the 50k plain-GPU configuration)")
    ap.add_argument("--workload", choices=["graph", "batch"], default="graph",
                    help="graph: one graph of --graph (default); batch: the batched configuration")
    ap.add_argument("--prep", choices=["device", "host"], default="device",
                    help="candidate generation on the GPU (default) or on the host")
    ap.add_argument("--no-plain", action="store_true", help="skip the per-iteration form's timing")
    ap.add_argument("--no-cuda-graph", dest="cuda_graph", action="store_false",
                    help="time the solve with stream launches only (no CUDA graph form)")
    ap.add_argument("--no-tune", dest="tune", action="store_false",
                    help="keep the default search shape (no tuning solve)")
    ap.add_argument("--no-learned", dest="learned", action="store_false",
                    help="skip the learned proposal's form")
    ap.add_argument("--train-graphs", type=int, default=3, help="graphs whose traces train the proposal")
    ap.add_argument("--train-n", type=int, default=60000, help="size (--n units) of the training graphs")
    ap.add_argument("--train-epochs", type=int, default=20)
    ap.add_argument("--proposal-rule", choices=["calibrated", "tail", "top"], default="calibrated",
                    help="top: ceil(N (1 + margin)) top scores; tail: expected selections beyond the prefix <= --eps; "
                         "calibrated (default): the top rule with the margin the training graphs needed, x 1.25 + 0.05")
    ap.add_argument("--eps", type=float, default=0.1)
    ap.add_argument("--margin", type=float, default=1.0)
    ap.add_argument("--plain-windows", type=int, default=8)
    ap.add_argument("--plain-width", type=int, default=128)
    ap.add_argument("--batch-count", type=int, default=4096)
    ap.add_argument("--blocks", type=int, default=2000)
    ap.add_argument("--plain-stride", type=int, default=16)
    args = ap.parse_args()
    if args.n is None:
        args.n = DEFAULT_N[args.graph]
    world, rank, local, pg = dist_setup(args)
    if args.impl == "reference":
        out = run_reference(args, world, rank, pg)
    elif args.workload == "batch":
        out = run_batch(args, world, rank, local, pg)
    else:
        out = run_gpu(args, world, rank, local, pg)
    if out is not None:
        print(json.dumps(out), flush=True)
    if pg:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
