"""Host-side problem preparation (the mcb driver's steps before its main loop).

Mirrors the reference driver's sequence (mcb/mcb_cycle_deg_two_remove.cpp:60-265):
read a symmetric Matrix-Market graph, contract degree-two chains, compute the MGA
feedback vertex set, the DFS spanning tree and its coordinate order, one Dijkstra
tree per FVS root with its candidate cycles, and the sorted candidate list.  The
work is done by libmcbhost.so; this module returns its arrays as numpy arrays.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from ._native import MCBHInfo, MCBHOptions, check_host, host_lib, ptr


@dataclass
class Graph:
    """An undirected weighted graph as an edge list (0-based)."""
    nodes: int
    u: np.ndarray
    v: np.ndarray
    w: np.ndarray

    @property
    def m(self) -> int:
        return int(self.u.shape[0])

    def write_mtx(self, path: str) -> None:
        check_host(host_lib().mcbh_write_mtx(path.encode(), self.nodes, self.m, ptr(self.u), ptr(self.v),
                                             ptr(self.w)), "mcbh_write_mtx")


def _edges(m: int) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    return np.empty(m, np.int32), np.empty(m, np.int32), np.empty(m, np.int32)


def grid_graph(rows: int, cols: int, wlo: int = 1, whi: int = 100, seed: int = 1) -> Graph:
    """rows x cols grid, row-major ids, right and down edges, weights U[wlo, whi]."""
    lib = host_lib()
    m = lib.mcbh_gen_grid(rows, cols, wlo, whi, seed, None, None, None)
    if m < 0:
        raise ValueError("bad grid parameters")
    u, v, w = _edges(m)
    lib.mcbh_gen_grid(rows, cols, wlo, whi, seed, ptr(u), ptr(v), ptr(w))
    return Graph(rows * cols, u, v, w)


def random_graph(n: int, m: int, wlo: int = 1, whi: int = 1000, seed: int = 1) -> Graph:
    """Connected random sparse graph: random spanning tree plus uniform extra edges."""
    lib = host_lib()
    mm = lib.mcbh_gen_random(n, m, wlo, whi, seed, None, None, None)
    if mm < 0:
        raise ValueError("bad random-graph parameters")
    u, v, w = _edges(mm)
    lib.mcbh_gen_random(n, m, wlo, whi, seed, ptr(u), ptr(v), ptr(w))
    return Graph(n, u, v, w)


def rgg_graph(n: int, k: int = 4, seed: int = 1) -> Graph:
    """Random geometric graph: k nearest neighbours in the unit square, w = round(1000*len)."""
    lib = host_lib()
    mm = lib.mcbh_gen_rgg(n, k, seed, None, None, None)
    if mm < 0:
        raise ValueError("bad rgg parameters")
    u, v, w = _edges(mm)
    lib.mcbh_gen_rgg(n, k, seed, ptr(u), ptr(v), ptr(w))
    return Graph(n, u, v, w)


def planar_chain_graph(points: int, delete_pct: int = 30, chain_pct: int = 30, chain_max: int = 8,
                       wlo: int = 1, whi: int = 1000, seed: int = 1) -> Graph:
    """Triangulated grid of about `points` vertices, delete_pct% of the edges deleted
    (connectivity kept), each kept edge subdivided with probability chain_pct% into a
    chain of 1..chain_max vertices; weights U[wlo, whi] per final edge."""
    lib = host_lib()
    nodes = C.c_int32()
    mm = lib.mcbh_gen_planar_chains(points, delete_pct, chain_pct, chain_max, wlo, whi, seed, None, None, None,
                                    C.byref(nodes))
    if mm < 0:
        raise ValueError("bad planar-chain parameters")
    u, v, w = _edges(mm)
    lib.mcbh_gen_planar_chains(points, delete_pct, chain_pct, chain_max, wlo, whi, seed, ptr(u), ptr(v), ptr(w),
                               C.byref(nodes))
    return Graph(int(nodes.value), u, v, w)


def block_tree_graph(blocks: int, nmin: int = 50, nmax: int = 150, deg_lo: float = 2.5, deg_hi: float = 5.0,
                     wlo: int = 1, whi: int = 255, seed: int = 1) -> Graph:
    """`blocks` 2-connected random blocks (size log-uniform in [nmin, nmax], average
    degree U[deg_lo, deg_hi]) glued at articulation vertices into a tree of blocks."""
    lib = host_lib()
    nodes = C.c_int32()
    lo, hi = int(round(deg_lo * 10)), int(round(deg_hi * 10))
    mm = lib.mcbh_gen_block_tree(blocks, nmin, nmax, lo, hi, wlo, whi, seed, None, None, None, C.byref(nodes))
    if mm < 0:
        raise ValueError("bad block-tree parameters")
    u, v, w = _edges(mm)
    lib.mcbh_gen_block_tree(blocks, nmin, nmax, lo, hi, wlo, whi, seed, ptr(u), ptr(v), ptr(w), C.byref(nodes))
    return Graph(int(nodes.value), u, v, w)


def _splitmix64(state: int) -> tuple[int, int]:
    state = (state + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
    z = state
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
    return state, z ^ (z >> 31)


def batch_graphs(count: int, nmin: int = 50, nmax: int = 5000, deg_lo: float = 2.5, deg_hi: float = 5.0,
                 wlo: int = 1, whi: int = 255, seed: int = 1) -> list[Graph]:
    """`count` independent connected random graphs: n log-uniform in [nmin, nmax],
    average degree U[deg_lo, deg_hi], weights U[wlo, whi]; graph i is drawn from its
    own seed, derived from `seed` by splitmix64."""
    import math
    out = []
    st = seed & 0xFFFFFFFFFFFFFFFF
    for _ in range(count):
        st, a = _splitmix64(st)
        st, b = _splitmix64(st)
        st, gseed = _splitmix64(st)
        ua, ub = (a >> 11) / float(1 << 53), (b >> 11) / float(1 << 53)
        n = int(round(math.exp(math.log(nmin) + ua * (math.log(nmax) - math.log(nmin)))))
        n = max(nmin, min(nmax, n))
        deg = deg_lo + ub * (deg_hi - deg_lo)
        m = max(n - 1, int(round(n * deg / 2)))
        m = min(m, n * (n - 1) // 2)
        out.append(random_graph(n, m, wlo, whi, gseed))
    return out


def bcc_split(g: Graph, keep_bridges: bool = False, with_ids: bool = False) -> list:
    """The biconnected components of g as graphs of their own, in order of their first
    edge, each exactly as the reference's bicc tool + Relabeller hand it to the mcb
    driver: its edges in the order the tool writes them (the input CSR's slots with
    row > column, in slot order, as (row, column); mcbh_edge_slot_order) and its
    vertices numbered in order of first appearance in that sequence
    (bicc/include/bicc.h:220-314, bicc/Relabeller.cpp:72-126), so every component's
    candidates, order and basis equal the reference's per-component run.  Components
    without a cycle (bridges) are dropped unless keep_bridges.  The minimum cycle basis
    of g is the union of the components' bases.  with_ids: (graph, input vertex of
    every component vertex) pairs."""
    comp = np.empty(max(g.m, 1), np.int32)
    lib = host_lib()
    nc = lib.mcbh_bcc_split(g.nodes, g.m, ptr(g.u), ptr(g.v), ptr(comp))
    if nc < 0:
        raise ValueError("bad graph for the biconnected split")
    comp = comp[:g.m]
    order = np.empty(max(g.m, 1), np.int64)
    k = lib.mcbh_edge_slot_order(g.nodes, g.m, ptr(g.u), ptr(g.v), ptr(order))
    if k < 0:
        raise ValueError("bad graph for the slot order")
    order = order[:k]
    # every component's edges in slot order (a stable split of the slot sequence)
    cs = comp[order]
    grouped = order[np.argsort(cs, kind="stable")]
    bounds = np.searchsorted(np.sort(cs), np.arange(nc + 1))
    hi = np.maximum(g.u, g.v).astype(np.int32)
    lo = np.minimum(g.u, g.v).astype(np.int32)
    out = []
    for c in range(nc):
        idx = grouped[bounds[c]:bounds[c + 1]]
        if idx.size == 0:
            continue
        r, q, w = hi[idx], lo[idx], g.w[idx]
        verts = np.empty(2 * idx.size, np.int32)
        verts[0::2], verts[1::2] = r, q
        uniq, first = np.unique(verts, return_index=True)
        ids = uniq[np.argsort(first, kind="stable")]  # input vertex of each component vertex
        rank = np.empty(uniq.size, np.int32)
        rank[np.argsort(first, kind="stable")] = np.arange(uniq.size, dtype=np.int32)
        cu = rank[np.searchsorted(uniq, r)]
        cv = rank[np.searchsorted(uniq, q)]
        if keep_bridges or idx.size >= uniq.size:
            cg = Graph(int(uniq.size), cu.astype(np.int32), cv.astype(np.int32), np.ascontiguousarray(w))
            out.append((cg, ids.astype(np.int32)) if with_ids else cg)
    return out


def prepare_many(problems: list, threads: int = 0, contract_chains: bool = True, keep_trees: bool = False,
                 ref_layout: bool = False, cycle_lists: bool = True) -> list:
    """Problem.prepare on independent problems at once (mcbh_prepare_many): one thread
    per problem, `threads` problems in parallel (0: all cores), largest first.  Each
    problem gets the result Problem.prepare gives it.  Raises on the first failure in
    list order, after the others are prepared."""
    n = len(problems)
    opt = MCBHOptions(threads, int(contract_chains), int(keep_trees), int(ref_layout), int(cycle_lists))
    handles = (C.c_void_p * max(n, 1))(*[p._h for p in problems])
    status = np.zeros(max(n, 1), np.int32)
    rc = host_lib().mcbh_prepare_many(C.cast(handles, C.c_void_p), n, C.byref(opt), ptr(status))
    for p, st in zip(problems, status[:n]):
        if st == 0:
            p.prepared = True
            p._opts = opt
    check_host(rc, "mcbh_prepare_many")
    return problems


class Problem:
    """A graph prepared for the de Pina main loop.

    Construct with Problem.from_mtx(path) or Problem.from_graph(graph), then
    prepare(...).  Arrays are read back lazily and cached.
    """

    def __init__(self, handle: C.c_void_p):
        self._h = handle
        self.prepared = False
        self._cache: dict = {}

    @classmethod
    def from_mtx(cls, path: str) -> "Problem":
        h = C.c_void_p()
        check_host(host_lib().mcbh_problem_from_mtx(path.encode(), C.byref(h)), "mcbh_problem_from_mtx")
        return cls(h)

    @classmethod
    def from_graph(cls, g: Graph) -> "Problem":
        h = C.c_void_p()
        u = np.ascontiguousarray(g.u, np.int32)
        v = np.ascontiguousarray(g.v, np.int32)
        w = np.ascontiguousarray(g.w, np.int32)
        check_host(host_lib().mcbh_problem_from_edges(g.nodes, g.m, ptr(u), ptr(v), ptr(w), C.byref(h)),
                   "mcbh_problem_from_edges")
        return cls(h)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            host_lib().mcbh_problem_free(h)
            self._h = None

    def prepare(self, threads: int = 0, contract_chains: bool = True, keep_trees: bool = False,
                ref_layout: bool = False, cycle_lists: bool = True, structure_only: bool = False) -> "Problem":
        """The driver's steps before its main loop (mcbh_prepare).  With
        `structure_only`, only up to the spanning tree: the candidates then come from a
        device generation (search_trees for the roots it leaves to the host, then
        rank_candidates)."""
        opt = MCBHOptions(threads, int(contract_chains), int(keep_trees), int(ref_layout), int(cycle_lists),
                          int(structure_only))
        check_host(host_lib().mcbh_prepare(self._h, C.byref(opt)), "mcbh_prepare")
        self.prepared = True
        self._opts = opt
        return self

    def search_trees(self, trees, threads: int = 0):
        """The reference's heap-ordered tree searches for FVS indices `trees`:
        (dist int32[count, n], parent_slot int32[count, n]) (mcbh_search_trees)."""
        t = np.ascontiguousarray(trees, np.int32)
        n = self.n
        dist = np.empty((max(len(t), 1), n), np.int32)
        ps = np.empty((max(len(t), 1), n), np.int32)
        check_host(host_lib().mcbh_search_trees(self._h, ptr(t), len(t), threads, ptr(dist), ptr(ps)),
                   "mcbh_search_trees")
        return dist[:len(t)], ps[:len(t)]

    def pairs(self) -> np.ndarray:
        """The lower slot of every reverse-slot pair, ascending (mcbh_get_pairs)."""
        def f():
            out = np.empty(self.info.reduced_edges2 // 2, np.uint32)
            check_host(host_lib().mcbh_get_pairs(self._h, ptr(out)), "mcbh_get_pairs")
            return out
        return self._get("pairs", f)

    def rank_candidates(self, tree_offsets, pair_index, weight, threads: int = 0) -> "Problem":
        """The rank order of externally found candidates (mcbh_rank_candidates): per
        FVS index t, its accepted pairs pair_index[tree_offsets[t]:tree_offsets[t+1]]
        (ascending) and their weights.  Afterwards candidates() is what prepare()
        gives for the same candidates."""
        to = np.ascontiguousarray(tree_offsets, np.int64)
        pi = np.ascontiguousarray(pair_index, np.uint32)
        w = np.ascontiguousarray(weight, np.int32)
        check_host(host_lib().mcbh_rank_candidates(self._h, ptr(to), ptr(pi), ptr(w), threads),
                   "mcbh_rank_candidates")
        self._cache.pop("cands", None)
        return self

    def prepare_with_trees(self, trees, chunk: int = 0, threads: int = 0, keep_trees: bool = False,
                           ref_layout: bool = False, cycle_lists: bool = True, begin=None,
                           trust: bool = False) -> "Problem":
        """prepare() with the per-root shortest-path trees taken from `trees(roots)` ->
        (dist int32[count, n], parent_slot int32[count, n], skip uint8[count]) where it
        offers one (mcbh_prepare_with_trees); every offered tree is checked, and a root
        whose tree fails or is skipped is searched on the host, so the result is
        prepare()'s.  `begin(nodes, row_offsets, cols, weights, rev)` (optional) sees
        the reduced graph first.  info.trees_supplied counts the adopted trees.  With
        `trust`, each tree is checked to be a tree of shortest paths but not that its
        parents are the reference's among equally near ones (for a supplier validated
        against the host's trees)."""
        from ._native import TREE_BEGIN, TREE_TREES, MCBHTreeSource
        state = {}

        def c_begin(ctx, nodes, slots, ro, cols, w, rev):
            try:
                state["n"] = int(nodes)
                if begin is not None:
                    arr = lambda p_, t, k: np.ctypeslib.as_array(C.cast(p_, C.POINTER(t)), shape=(k,)).copy()
                    begin(int(nodes), arr(ro, C.c_uint32, nodes + 1), arr(cols, C.c_uint32, slots),
                          arr(w, C.c_int32, slots), arr(rev, C.c_uint32, slots))
                return 0
            except Exception:
                return 1

        def c_trees(ctx, roots, count, dist, pslot, skip):
            try:
                n = state["n"]
                r = np.ctypeslib.as_array(C.cast(roots, C.POINTER(C.c_uint32)), shape=(count,)).copy()
                d, ps, sk = trees(r)
                np.ctypeslib.as_array(C.cast(dist, C.POINTER(C.c_int32)), shape=(count * n,))[:] = \
                    np.asarray(d, np.int32).reshape(-1)
                np.ctypeslib.as_array(C.cast(pslot, C.POINTER(C.c_int32)), shape=(count * n,))[:] = \
                    np.asarray(ps, np.int32).reshape(-1)
                np.ctypeslib.as_array(C.cast(skip, C.POINTER(C.c_uint8)), shape=(count,))[:] = \
                    np.asarray(sk, np.uint8).reshape(-1)
                return 0
            except Exception:
                return 1

        cb_begin, cb_trees = TREE_BEGIN(c_begin), TREE_TREES(c_trees)
        src = MCBHTreeSource(None, cb_begin, cb_trees, chunk, int(trust))
        opt = MCBHOptions(threads, 1, int(keep_trees), int(ref_layout), int(cycle_lists))
        check_host(host_lib().mcbh_prepare_with_trees(self._h, C.byref(opt), C.byref(src)), "mcbh_prepare_with_trees")
        self.prepared = True
        self._opts = opt
        return self

    def gf2_rank(self, ranks, threads: int = 0) -> int:
        """GF(2) rank of the cycle vectors of the candidates at `ranks` (mcbh_gf2_rank):
        a basis re-verified by elimination has rank == len(ranks) == N."""
        r = np.ascontiguousarray(ranks, np.int64)
        out = C.c_int64()
        check_host(host_lib().mcbh_gf2_rank(self._h, ptr(r), len(r), threads, C.byref(out)), "mcbh_gf2_rank")
        return int(out.value)

    @property
    def info(self) -> MCBHInfo:
        i = MCBHInfo()
        check_host(host_lib().mcbh_get_info(self._h, C.byref(i)), "mcbh_get_info")
        return i

    # sizes
    @property
    def n(self) -> int:
        return self.info.reduced_nodes

    @property
    def N(self) -> int:
        return self.info.num_coords

    @property
    def K(self) -> int:
        return self.info.num_candidates

    @property
    def F(self) -> int:
        return self.info.fvs_size

    def _get(self, key, fn):
        if key not in self._cache:
            self._cache[key] = fn()
        return self._cache[key]

    def reduced_graph(self):
        def f():
            i = self.info
            m2, n = i.reduced_edges2, i.reduced_nodes
            rows = np.empty(m2, np.uint32)
            cols = np.empty(m2, np.uint32)
            w = np.empty(m2, np.int32)
            rev = np.empty(m2, np.uint32)
            ro = np.empty(n + 1, np.uint32)
            check_host(host_lib().mcbh_get_reduced_graph(self._h, ptr(rows), ptr(cols), ptr(w), ptr(rev), ptr(ro)),
                       "mcbh_get_reduced_graph")
            return rows, cols, w, rev, ro
        return self._get("graph", f)

    def fvs(self):
        def f():
            i = self.info
            fa = np.empty(i.reduced_nodes, np.int32)
            fv = np.empty(i.fvs_size, np.uint32)
            check_host(host_lib().mcbh_get_fvs(self._h, ptr(fa), ptr(fv)), "mcbh_get_fvs")
            return fa, fv
        return self._get("fvs", f)

    def vertex_map(self) -> np.ndarray:
        """Input vertex (0-based) of every reduced vertex."""
        def f():
            vm = np.empty(self.info.reduced_nodes, np.int32)
            check_host(host_lib().mcbh_get_vertex_map(self._h, ptr(vm)), "mcbh_get_vertex_map")
            return vm
        return self._get("vertex_map", f)

    def coords(self):
        def f():
            i = self.info
            ce = np.empty(i.num_coords, np.uint32)
            ec = np.empty(i.reduced_edges2, np.int32)
            check_host(host_lib().mcbh_get_coords(self._h, ptr(ce), ptr(ec)), "mcbh_get_coords")
            return ce, ec
        return self._get("coords", f)

    def candidates(self):
        """(root, edge_offset, weight, tree) in rank order."""
        def f():
            K = self.info.num_candidates
            a = [np.empty(K, np.int32) for _ in range(4)]
            check_host(host_lib().mcbh_get_candidates(self._h, *[ptr(x) for x in a]), "mcbh_get_candidates")
            return tuple(a)
        return self._get("cands", f)

    def cycle_lists(self):
        """(offsets[K+1] int64, coords[nnz] int32)."""
        def f():
            i = self.info
            off = np.empty(i.num_candidates + 1, np.int64)
            co = np.empty(i.cycle_nnz, np.int32)
            check_host(host_lib().mcbh_get_cycle_lists(self._h, ptr(off), ptr(co)), "mcbh_get_cycle_lists")
            return off, co
        return self._get("lists", f)

    def tree_parents(self):
        def f():
            i = self.info
            tp = np.empty(i.fvs_size * i.reduced_nodes, np.int32)
            check_host(host_lib().mcbh_get_tree_parents(self._h, ptr(tp)), "mcbh_get_tree_parents")
            return tp
        return self._get("parents", f)

    def ref_layout(self):
        """(level_offsets F x (n+1), parent_pos F x n, edge_offset F x n, nodes_index F x n)."""
        def f():
            i = self.info
            F, n = i.fvs_size, i.reduced_nodes
            lv = np.empty(F * (n + 1), np.uint32)
            pp = np.empty(F * n, np.uint32)
            eo = np.empty(F * n, np.int32)
            ni = np.empty(F * n, np.uint32)
            check_host(host_lib().mcbh_get_ref_layout(self._h, ptr(lv), ptr(pp), ptr(eo), ptr(ni)),
                       "mcbh_get_ref_layout")
            return lv, pp, eo, ni
        return self._get("layout", f)

    def total_weight(self, selected: np.ndarray) -> int:
        """64-bit total weight of the selected candidate ranks."""
        _, _, w, _ = self.candidates()
        return int(w[np.asarray(selected, np.int64)].astype(np.int64).sum())
