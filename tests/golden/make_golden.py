"""Generate the golden vectors under tests/golden/ from the reference itself.

Run in a container where the reference is checked out (its path from --ref or the
MCB_REFERENCE environment variable):

    python tests/golden/make_golden.py --ref /path/to/MinimumCycleBasis

It builds oracle/_ref (oracle/Makefile: the reference's own CPU drivers plus
oracle/ref_dump.cpp, a small driver over the reference's host library), generates
each graph with the repository's seeded generators, writes it as Matrix Market
next to this script, and records what the reference computes:
  - ref_dump: reduced graph size, FVS, coordinate order, the sorted candidate list
    (root, edge offset, weight) and the selected basis sequence (candidate ranks);
  - mcb_cpu / mcb_cpu_baseline: the stats CSV row (include/stats.h:256-338).
Nothing at test time reads the reference; the tests read these files.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

from minimumcyclebasis_gb300 import (batch_graphs, block_tree_graph, grid_graph, planar_chain_graph,  # noqa: E402
                                     random_graph, rgg_graph)
from minimumcyclebasis_gb300.build import build_all, build_reference  # noqa: E402

# (name, generator, args, keep full candidate list in the fixture)
CASES = [
    ("grid4x4_s7", "grid", (4, 4, 1, 100, 7), True),
    ("grid8x8_s3", "grid", (8, 8, 1, 100, 3), True),
    ("grid32x32_s1", "grid", (32, 32, 1, 100, 1), True),
    ("grid32x32_s2", "grid", (32, 32, 1, 100, 2), False),
    ("grid12x12_w5_s9", "grid", (12, 12, 1, 5, 9), True),
    ("rand300_s0", "random", (300, 600, 1, 1000, 0), True),
    ("rand300_s1", "random", (300, 600, 1, 1000, 1), True),
    ("rand300_w3_s2", "random", (300, 450, 1, 3, 2), True),
    ("rand2000_w20_s11", "random", (2000, 4000, 1, 20, 11), False),
    ("rand1000_s5", "random", (1000, 2500, 1, 1000, 5), False),
    ("tree_plus_one_s4", "random", (64, 64, 1, 50, 4), True),
    ("rgg500_s3", "rgg", (500, 4, 3), True),
    # the planar-with-chains family (triangulated grid, 30% of edges deleted,
    # 30% of edges subdivided into chains of 1..8 vertices)
    ("planar300_s5", "planar", (300, 30, 30, 8, 1, 1000, 5), True),
    ("planar2000_s2", "planar", (2000, 30, 30, 8, 1, 1000, 2), False),
    # a tree of 2-connected random blocks glued at articulation vertices
    ("blocktree12_s2", "blocktree", (12, 20, 60, 2.5, 5.0, 1, 255, 2), True),
    # members of a batch of independent graphs (n log-uniform, degree U[2.5, 5])
    ("batch7_g0", "batch", (4, 50, 600, 2.5, 5.0, 1, 255, 7, 0), True),
    ("batch7_g1", "batch", (4, 50, 600, 2.5, 5.0, 1, 255, 7, 1), True),
    ("batch7_g2", "batch", (4, 50, 600, 2.5, 5.0, 1, 255, 7, 2), True),
    ("batch7_g3", "batch", (4, 50, 600, 2.5, 5.0, 1, 255, 7, 3), True),
]


def gen(kind, args):
    if kind == "batch":
        return batch_graphs(*args[:-1])[args[-1]]
    return {"grid": grid_graph, "random": random_graph, "rgg": rgg_graph, "planar": planar_chain_graph,
            "blocktree": block_tree_graph}[kind](*args)


def parse_dump(text):
    out = {"C": [], "S": [], "V": [], "T": []}
    for line in text.splitlines():
        t = line.split()
        if not t:
            continue
        if t[0] == "G":
            out["G"] = [int(x) for x in t[1:]]
        elif t[0] == "W":
            out["W"] = int(t[1])
        elif t[0] in out:
            out[t[0]].append([int(x) for x in t[1:]])
        elif t[0] == "X":
            raise RuntimeError(line)
    return out


def csv_row(binary, mtx, threads):
    with tempfile.TemporaryDirectory() as d:
        csv = os.path.join(d, "out.csv")
        subprocess.run([binary, mtx, csv, str(threads)], check=True, capture_output=True)
        lines = open(csv).read().splitlines()
    header = [h.strip() for h in lines[0].split(",")]
    vals = [v.strip() for v in lines[1].split(",")]
    return dict(zip(header, vals))


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, np.int32).tobytes()).hexdigest()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("MCB_REFERENCE"))
    a = ap.parse_args()
    if not a.ref:
        sys.exit("name the reference checkout with --ref or MCB_REFERENCE")
    build_all()
    if not build_reference(a.ref):
        sys.exit("reference sources not found at %s" % a.ref)
    refdir = os.path.join(ROOT, "oracle", "_ref")
    index = []
    for name, kind, args, full in CASES:
        g = gen(kind, args)
        mtx = os.path.join(HERE, name + ".mtx")
        g.write_mtx(mtx)
        dump = parse_dump(subprocess.run([os.path.join(refdir, "ref_dump"), mtx, "4", "-1", "noE"], check=True,
                                         capture_output=True, text=True).stdout)
        cpu = csv_row(os.path.join(refdir, "mcb_cpu"), mtx, 4)
        base = csv_row(os.path.join(refdir, "mcb_cpu_baseline"), mtx, 4)
        C = np.array(dump["C"], np.int64).reshape(-1, 4)
        S = np.array(dump["S"], np.int64).reshape(-1, 5)
        fx = {
            "name": name, "generator": kind, "args": list(args),
            "G": dict(zip(["nodes", "edges2", "nodes_removed", "reduced_nodes", "reduced_edges2", "fvs_size",
                           "num_coords", "num_candidates"], dump["G"])),
            "fvs_vertices": [v[0] for v in dump["V"]],
            "coord_edges": [t[1] for t in dump["T"]],
            "candidates_sha256": {"root": sha(C[:, 1]), "edge": sha(C[:, 2]), "weight": sha(C[:, 3])},
            "selected_ranks": S[:, 1].tolist(),
            "selected_weights": S[:, 4].tolist(),
            "total_weight": dump["W"],
            "mcb_cpu_csv": cpu,
            "mcb_cpu_baseline_csv": base,
        }
        if full:
            fx["candidates"] = {"root": C[:, 1].tolist(), "edge": C[:, 2].tolist(), "weight": C[:, 3].tolist()}
        with open(os.path.join(HERE, name + ".json"), "w") as f:
            json.dump(fx, f, separators=(",", ":"))
        index.append(name)
        print(name, fx["G"], "W", fx["total_weight"])
    with open(os.path.join(HERE, "index.json"), "w") as f:
        json.dump(index, f, indent=1)


if __name__ == "__main__":
    main()
