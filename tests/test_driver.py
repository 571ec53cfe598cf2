"""The mcb_gb300 driver executable: the reference driver's command line, stats row
and cycle listing (mcb/mcb_cycle_deg_two_remove.cpp, include/stats.h:256-338,
include/cycles.h:197-207)."""
import csv
import os
import subprocess

import numpy as np
import pytest
from conftest import ROOT, load_golden

from minimumcyclebasis_gb300 import Problem

DRIVER = os.path.join(ROOT, "minimumcyclebasis_gb300", "lib", "mcb_gb300")
COUNTS = ["Total_Nodes", "Total_Edges", "New_Edges", "Fvs_size", "Initial_Cycles", "Final_cycles", "Total_Weight"]


def run(*args):
    return subprocess.run([DRIVER, *map(str, args)], capture_output=True, text=True, timeout=600)


def read_rows(path):
    with open(path) as f:
        return list(csv.DictReader(f))


def test_usage_without_arguments():
    r = run()
    assert r.returncode == 1 and "InputFile" in r.stdout


def test_single_cycle_graph(tmp_path):
    # every vertex of degree two: the basis is the graph itself, no GPU involved
    # (mcb/mcb_cycle_deg_two_remove.cpp:104-111)
    n = 7
    mtx = tmp_path / "ring.mtx"
    w = [3, 1, 4, 1, 5, 9, 2]
    mtx.write_text("%%%%MatrixMarket matrix coordinate integer symmetric\n%d %d %d\n" % (n, n, n) +
                   "".join("%d %d %d\n" % (i + 1, (i + 1) % n + 1, w[i]) for i in range(n)))
    out = tmp_path / "stats.csv"
    r = run(mtx, out, 1)
    assert r.returncode == 0, r.stderr
    row = read_rows(out)[0]
    assert int(row["Total_Nodes"]) == n and int(row["Total_Edges"]) == 2 * n
    assert int(row["Nodes_removed"]) == n - 1 and int(row["Fvs_size"]) == 1
    assert int(row["Initial_Cycles"]) == 1 and int(row["Final_cycles"]) == 1
    assert int(row["Total_Weight"]) == sum(w)
    # a second run appends a row under the same header
    assert run(mtx, out, 1).returncode == 0
    assert len(read_rows(out)) == 2


def test_tree_has_an_empty_basis(tmp_path):
    # no cycle at all: no candidate, no GPU work, weight 0; with --bcc every edge is a
    # bridge, so no component is solved and no row is written
    mtx = tmp_path / "path.mtx"
    mtx.write_text("%%MatrixMarket matrix coordinate integer symmetric\n5 5 4\n1 2 1\n2 3 2\n3 4 3\n4 5 4\n")
    out = tmp_path / "stats.csv"
    r = run(mtx, out, 1)
    assert r.returncode == 0, r.stderr
    row = read_rows(out)[0]
    assert int(row["Final_cycles"]) == 0 and int(row["Initial_Cycles"]) == 0 and int(row["Total_Weight"]) == 0
    out2 = tmp_path / "stats_bcc.csv"
    r = run(mtx, out2, 1, "--bcc")
    assert r.returncode == 0, r.stderr
    assert "0 problem(s)" in r.stdout and not out2.exists()


def expected_cycles(fx, use_input_ids):
    p = Problem.from_mtx(fx["mtx"]).prepare(threads=2, cycle_lists=False)
    root, edge, weight, _ = p.candidates()
    rows, cols = p.reduced_graph()[:2]
    vmap = p.vertex_map() if use_input_ids else np.arange(p.info.reduced_nodes)
    bar = "=" * 81
    lines = []
    for r in fx["selected_ranks"]:
        lines += [bar, "Root is %d" % (vmap[root[r]] + 1), "Edge is %d - %d" % (vmap[rows[edge[r]]] + 1,
                                                                              vmap[cols[edge[r]]] + 1),
                  "Total weight = %d" % weight[r], bar]
    lines.append("Total Weight = %d" % fx["total_weight"])
    return lines


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["grid8x8_s3", "rand300_s0", "planar300_s5", "blocktree12_s2", "batch7_g1"])
@pytest.mark.parametrize("plain", [False, True])
def test_driver_matches_reference(tmp_path, name, plain):
    fx = load_golden(name)
    out, cyc, cyc_in = tmp_path / "stats.csv", tmp_path / "c.txt", tmp_path / "ci.txt"
    args = [fx["mtx"], out, 4, 720, "--cycles", cyc, "--cycles-input", cyc_in] + (["--plain"] if plain else [])
    r = run(*args)
    assert r.returncode == 0, r.stderr
    row = read_rows(out)[0]
    ref = fx["mcb_cpu_csv"]
    for col in COUNTS:
        assert int(row[col]) == int(ref[col]), col
    assert int(row["Nodes_removed"]) == int(ref["Node_removed"])
    assert cyc.read_text().splitlines() == expected_cycles(fx, False)
    assert cyc_in.read_text().splitlines() == expected_cycles(fx, True)


def test_bcc_mode_rings_and_bridge_without_gpu(tmp_path):
    # two rings joined by a bridge: each ring is its own basis, the bridge carries none
    edges = [(1, 2, 3), (2, 3, 4), (3, 1, 5), (3, 4, 7), (4, 5, 1), (5, 6, 2), (6, 4, 6)]
    mtx = tmp_path / "g.mtx"
    mtx.write_text("%%MatrixMarket matrix coordinate integer symmetric\n6 6 7\n" +
                   "".join("%d %d %d\n" % e for e in edges))
    out, cyc = tmp_path / "stats.csv", tmp_path / "c.txt"
    r = run(mtx, out, 1, "--bcc", "--cycles", cyc, "--verify")  # rings: nothing to eliminate
    assert r.returncode == 0, r.stderr
    rows = read_rows(out)
    assert [int(x["Total_Weight"]) for x in rows] == [12, 9]
    assert cyc.read_text().splitlines()[-1] == "Total Weight = 21"


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["grid32x32_s1", "rand2000_w20_s11"])
@pytest.mark.parametrize("bcc", [False, True])
def test_driver_verify_reports_full_rank(tmp_path, name, bcc):
    # --verify: every basis re-verified over GF(2), rank N of N (the single graph by the
    # device certificate, the components by elimination on the host)
    fx = load_golden(name)
    r = run(fx["mtx"], tmp_path / "stats.csv", 4, "--verify", *(["--bcc"] if bcc else []))
    assert r.returncode == 0, r.stderr
    ranks = [ln.split() for ln in r.stderr.splitlines() if ln.startswith("GF(2) rank ")]
    assert ranks and all(x[2] == x[4] for x in ranks)
    if not bcc:
        n = str(fx["G"]["num_coords"])
        assert ranks == [["GF(2)", "rank", n, "of", n, "(device", "certificate)"]]


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["blocktree12_s2", "rand300_w3_s2", "planar300_s5"])
def test_bcc_mode_weight_matches_reference(tmp_path, name):
    # per-component solves add up to the reference's whole-graph basis
    fx = load_golden(name)
    out, cyc = tmp_path / "stats.csv", tmp_path / "c.txt"
    r = run(fx["mtx"], out, 4, "--bcc", "--cycles-input", cyc)
    assert r.returncode == 0, r.stderr
    rows = read_rows(out)
    assert sum(int(x["Total_Weight"]) for x in rows) == fx["total_weight"]
    assert sum(int(x["Final_cycles"]) for x in rows) == fx["G"]["num_coords"]
    lines = cyc.read_text().splitlines()
    assert lines[-1] == "Total Weight = %d" % fx["total_weight"]
    weights = [int(x.split("= ")[1]) for x in lines if x.startswith("Total weight = ")]
    rings = sum(int(x["Total_Weight"]) for x in rows if int(x["Initial_Cycles"]) == 1 and int(x["Fvs_size"]) == 1
                and int(x["Final_cycles"]) == 1 and int(x["New_Edges"]) == 0)
    assert sum(weights) + rings == fx["total_weight"]
