"""bench.py's CPU baseline of the batched configuration: the sampled full solves of the
reference CPU loop (oracle port) and their extrapolation by label cost, on CPU."""
import json
import os
import subprocess
import sys

from conftest import ROOT

sys.path.insert(0, ROOT)


def test_batch_cpu_baseline_with_every_problem_sampled_is_the_measured_sum():
    import bench
    import oracle
    from minimumcyclebasis_gb300 import Problem, batch_graphs
    graphs = batch_graphs(12, nmin=50, nmax=400, seed=3)
    costs, want = {}, {}
    for j, g in enumerate(graphs):
        p = Problem.from_graph(g).prepare(threads=2, keep_trees=True)
        if p.info.single_cycle or p.N == 0:
            continue
        costs[j] = bench.label_cost(p.info)
        sel, tot, _ = oracle.solve(p, threads=2)
        want[j] = (sel, tot)
    assert len(costs) >= 8
    cb = bench.batch_cpu_baseline(graphs, costs, 2, 1e9, want)
    assert cb["kind"] == "port" and cb["cores"] == 2 and cb["value"] > 0
    assert "full solves of %d of the %d" % (len(costs), len(costs)) in cb["sample"]
    assert "%d checked equal" % len(costs) in cb["sample"]


def test_batch_cpu_baseline_skips_problems_above_half_the_budget():
    import bench
    from minimumcyclebasis_gb300 import Problem, batch_graphs
    graphs = batch_graphs(6, nmin=50, nmax=200, seed=4)
    costs = {}
    for j, g in enumerate(graphs):
        info = Problem.from_graph(g).prepare(threads=2).info
        if not info.single_cycle and info.num_coords > 0:
            costs[j] = bench.label_cost(info)
    # a budget below every problem's predicted time: nothing is solved, all are skipped
    cb = bench.batch_cpu_baseline(graphs, costs, 2, 1e-12)
    assert "full solves of 0 of the %d" % len(costs) in cb["sample"]
    assert "%d problems predicted above half the budget skipped" % len(costs) in cb["sample"]


def test_reference_arm_of_the_batched_workload_prints_one_line():
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "batch",
           "--batch-count", "16", "--steps", "1", "--warmup", "0", "--cpu-budget", "2", "--cpu-threads", "2"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is False
    assert d["config"]["workload"].startswith("batched: 16 random graphs")
    assert d["cpu_baseline"]["value"] == d["value"] and d["e2e"]["d2h_bytes_per_step"] == 0


def test_reference_arm_of_the_planar_workload_prints_one_line():
    # the default graph family at a small size: the sampled label pass and row update
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--n", "1500", "--steps", "1",
           "--warmup", "1", "--cpu-sample-roots", "40", "--cpu-threads", "2"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0
    assert d["config"]["workload"].startswith("planar-like graph from 1500 triangulated points")
    assert "label pass over 40 of the" in d["cpu_baseline"]["sample"]
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0


def test_sampled_cpu_baseline_tracks_a_full_oracle_solve():
    # the single-graph CPU baseline extrapolates a sampled label pass and a sampled
    # update to a whole solve; on a graph the oracle solves in a second the estimate
    # must land near the measured loop (it leaves out the list scan: slightly low)
    import argparse

    import bench
    import oracle
    from minimumcyclebasis_gb300 import Problem, planar_chain_graph
    g = planar_chain_graph(1500, 30, 30, 8, 1, 1000, 7)
    p = Problem.from_graph(g).prepare(threads=4, keep_trees=True)
    _, _, loop_s = oracle.solve(p, threads=4)
    ps = Problem.from_graph(g).prepare(threads=4, structure_only=True)
    est = bench.cpu_baseline(ps, argparse.Namespace(cpu_sample_roots=2000), 4)
    assert 0.5 < est["value"] / loop_s < 2.0, (est["value"], loop_s)
