/*
 * mcbhost.h — C ABI of the host-side preprocessing library (libmcbhost.so).
 *
 * This is the host half of the minimum-cycle-basis driver: everything the
 * reference's mcb driver does before its de Pina main loop, re-implemented in C++
 * so that its outputs are identical to the reference's:
 *   - symmetric Matrix-Market input          (include/FileReader.h:27-67)
 *   - CSR with both directions, (row,col)-sorted (include/CsrGraph.h:113-174)
 *   - degree-two chain contraction + relabel  (include/CsrGraphDegreeTwoRemoval.cpp:12-126,
 *                                              include/CsrGraphMulti.h:229-300)
 *   - MGA feedback vertex set                 (include/FVS.cpp:166-214)
 *   - DFS spanning tree -> coordinate order   (include/CsrGraphMultiSpanningTree.cpp:11-135,
 *                                              mcb/mcb_cycle_deg_two_remove.cpp:175-187)
 *   - one Dijkstra tree per FVS root and the candidate cycles
 *                                             (include/Dijkstra.h:78-254,
 *                                              include/work_per_thread.h:92-147)
 *   - candidate collection and sort = the tie-break order
 *                                             (mcb/mcb_cycle_deg_two_remove.cpp:244-265)
 * It also builds, per candidate, the sorted list of cycle coordinates that
 * cycle::get_cycle_vector would set (include/cycles.h:144-195), and, on request,
 * the reference's level-ordered per-tree GPU layout (include/Dijkstra.h:151-203).
 *
 * All functions return 0 on success and a negative MCBH_E* code on failure; no
 * function calls exit().  Vertex ids are 0-based.
 */
#ifndef MCBHOST_H
#define MCBHOST_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    MCBH_OK = 0,
    MCBH_E_ARG = -1,       /* bad argument */
    MCBH_E_IO = -2,        /* cannot open / parse the input file */
    MCBH_E_FORMAT = -3,    /* unsupported Matrix-Market banner */
    MCBH_E_GRAPH = -4,     /* graph the reference cannot process (e.g. disconnected) */
    MCBH_E_STATE = -5,     /* call out of order (e.g. accessor before prepare) */
    MCBH_E_NOMEM = -6,     /* allocation failed */
    MCBH_E_SUPPLIER = -7   /* a tree supplier's callback returned an error */
};

typedef struct mcbh_problem mcbh_problem;

typedef struct mcbh_options {
    int threads;          /* OpenMP threads for the per-root tree loop (<=0: all) */
    int contract_chains;  /* 1: degree-two contraction (mcb_cpu / mcb_cuda);
                             0: none, spanning-tree root 0 (mcb_cpu_baseline, mcb/mcb_cycle.cpp:110-113) */
    int keep_trees;       /* keep per-tree vertex-indexed parent edge offsets (F x n int32) */
    int ref_layout;       /* build the reference's level-ordered GPU layout (4 arrays of F x n) */
    int cycle_lists;      /* build per-candidate sorted coordinate lists */
    int structure_only;   /* 1: stop after the spanning tree (chain contraction, FVS, coordinates):
                             no per-root trees and no candidates here; they come from a device
                             candidate generation through mcbh_search_trees (for the roots it
                             leaves to the host) and mcbh_rank_candidates */
} mcbh_options;

typedef struct mcbh_info {
    int32_t nodes;           /* input vertices */
    int64_t edges2;          /* input directed edge slots (2m) */
    int32_t single_cycle;    /* every vertex has degree two: the basis is the graph itself */
    int32_t nodes_removed;   /* vertices removed by chain contraction */
    int32_t reduced_nodes;   /* n' */
    int64_t reduced_edges2;  /* 2m' */
    int32_t source_vertex;   /* root of the initial DFS spanning tree */
    int32_t fvs_size;        /* F */
    int32_t num_coords;      /* N = m' - n' + 1 (non-tree edges = bit-vector coordinates) */
    int64_t num_candidates;  /* K */
    int64_t cycle_nnz;       /* total length of the per-candidate coordinate lists */
    int64_t total_weight_input; /* sum of input edge weights (64-bit) */
    double t_read, t_reduce, t_fvs, t_spanning, t_trees, t_collect; /* seconds */
    int32_t trees_supplied;  /* roots whose tree came from mcbh_prepare_with_trees's supplier */
} mcbh_info;

/* ---- construction ---------------------------------------------------------- */
int mcbh_problem_from_mtx(const char *path, mcbh_problem **out);
/* m undirected edges (u[i], v[i], w[i]), 0-based, inserted in that order. */
int mcbh_problem_from_edges(int32_t nodes, int64_t m, const int32_t *u, const int32_t *v,
                            const int32_t *w, mcbh_problem **out);
/* One preparation per problem: a second call, after success or failure, returns
 * MCBH_E_STATE. */
int mcbh_prepare(mcbh_problem *p, const mcbh_options *opt);
/* A supplier of per-root shortest-path trees for mcbh_prepare_with_trees (e.g. the
 * GPU's, mcbgpu_trees_*).  begin (optional) receives the reduced graph once, before
 * the first trees call: `nodes`, the slot count, row offsets (nodes + 1), and per slot
 * its column, weight and reverse slot.  trees fills, for the `count` roots at `roots`,
 * every vertex's distance (count x nodes), its parent slot (the slot of the parent's
 * row that enters it; -1 at the root) and a per-root flag, nonzero where the supplier
 * leaves the root to the host.  Both return 0 on success. */
typedef struct mcbh_tree_source {
    void *ctx;
    int (*begin)(void *ctx, int32_t nodes, int64_t slots, const uint32_t *row_offsets, const uint32_t *cols,
                 const int32_t *weights, const uint32_t *rev);
    int (*trees)(void *ctx, const uint32_t *roots, int32_t count, int32_t *dist, int32_t *parent_slot,
                 uint8_t *skip);
    int32_t chunk; /* roots per trees call (<= 0: all at once) */
    int32_t trust; /* nonzero: check that each tree is a tree of shortest paths (every
                      parent slot enters its vertex, distances add up along it, no slot
                      gives a shorter path), not that every parent is the one the
                      reference's search keeps among equally near ones; for a supplier
                      already validated against the host's trees.  0: the full check, and
                      a result identical to mcbh_prepare's whatever the supplier returns. */
} mcbh_tree_source;
/* mcbh_prepare with the per-root tree searches taken from `source` where it offers a
 * tree.  Each tree is checked before use (a shortest-path tree whose every parent is
 * the one the reference's heap search keeps, i.e. no two equally near shortest-path
 * parents); a root whose tree fails a check, or that the supplier skips, is searched
 * on the host.  The result is identical to mcbh_prepare's.  Without effect (all roots
 * searched on the host) when some weight is below 1 or opt->ref_layout is set (the
 * layout follows the heap's settle order).  info.trees_supplied counts the adopted
 * trees. */
int mcbh_prepare_with_trees(mcbh_problem *p, const mcbh_options *opt, const mcbh_tree_source *source);
/* ---- the host half of a device candidate generation ------------------------ */
/* After mcbh_prepare with structure_only = 1.  The reference's per-root tree
 * searches (include/Dijkstra.h:78-124, the heap order deciding ties) for the FVS
 * indices trees[0..count): every vertex's distance and parent slot (count x n', -1
 * at the root), OpenMP over roots.  For the roots a device search leaves to the host
 * (two equally near shortest-path parents somewhere in the tree). */
int mcbh_search_trees(const mcbh_problem *p, const int32_t *trees, int32_t count, int threads, int32_t *dist,
                      int32_t *parent_slot);
/* The lower slot of every reverse-slot pair of the reduced graph in ascending order
 * (m' entries): pair k joins rows[pair_slot[k]] and cols[pair_slot[k]].  The order in
 * which the reference's non-tree-edge scan meets the pairs (include/Dijkstra.h:129-149),
 * which is each root's candidate insertion order. */
int mcbh_get_pairs(const mcbh_problem *p, uint32_t *pair_slot);
/* The rank order of candidates found elsewhere (a device candidate test): for FVS
 * index t, its accepted pairs pair_index[tree_offsets[t] .. tree_offsets[t+1]) in
 * ascending pair order, with their cycle weights.  Builds each root's group map with
 * the reference's key and insertion sequence (include/cycle_searcher.h:23-61), walks
 * the roots in vertex-id order and sorts on weight alone with std::sort's permutation
 * (mcb/mcb_cycle_deg_two_remove.cpp:244-258): mcbh_get_candidates then returns the
 * list mcbh_prepare gives for the same candidates.  No coordinate lists (cycle_nnz = 0;
 * the device builds them).  Once per problem, after a structure_only preparation. */
int mcbh_rank_candidates(mcbh_problem *p, const int64_t *tree_offsets, const uint32_t *pair_index,
                         const int32_t *weight, int threads);
/* mcbh_prepare on `count` independent problems (the components of a biconnected
 * split, the graphs of a batch), in parallel over problems with one thread each,
 * largest first; opt->threads is the number of problems prepared at once (<=0:
 * all cores).  Every problem's result is the one mcbh_prepare gives it.  status[i]
 * (optional) receives each problem's return code; the return value is the code of
 * the first problem, in index order, that failed (MCBH_OK if none). */
int mcbh_prepare_many(mcbh_problem **ps, int64_t count, const mcbh_options *opt, int32_t *status);
/* Re-verification of a basis: the GF(2) rank of the cycle vectors of the candidates
 * at `ranks` (rank-ordered candidate indices, e.g. a solver's selected ranks), by
 * Gaussian elimination over their N-bit coordinate vectors (count x N bits held on
 * the host; O(count x N^2 / 64) word operations, OpenMP over rows).  A basis is
 * independent iff *rank_out == count == N.  Needs the cycle lists (cycle_lists = 1). */
int mcbh_gf2_rank(const mcbh_problem *p, const int64_t *ranks, int64_t count, int threads, int64_t *rank_out);
/* The edges of a Matrix-Market file as mcbh_problem_from_mtx reads them (0-based,
 * file order).  Returns the edge count and sets *nodes; with u != NULL also fills
 * u, v, w (cap entries available). */
int64_t mcbh_read_mtx(const char *path, int32_t *nodes, int64_t cap, int32_t *u, int32_t *v, int32_t *w);
void mcbh_problem_free(mcbh_problem *p);

/* ---- accessors (caller-allocated outputs) --------------------------------- */
int mcbh_get_info(const mcbh_problem *p, mcbh_info *info);
/* reduced multigraph CSR, each of length 2m' (row_offsets: n'+1) */
int mcbh_get_reduced_graph(const mcbh_problem *p, uint32_t *rows, uint32_t *cols, int32_t *weights,
                           uint32_t *reverse_edge, uint32_t *row_offsets);
int mcbh_get_fvs(const mcbh_problem *p, int32_t *fvs_array /* n' */, uint32_t *fvs_vertices /* F */);
/* input_vertex[v] = the input vertex (0-based) of reduced vertex v (n'); chain
 * contraction keeps every vertex of degree > 2 and relabels it in order of first
 * appearance (include/CsrGraphMulti.h:229-300).  No reference counterpart: the
 * reference prints reduced ids only. */
int mcbh_get_vertex_map(const mcbh_problem *p, int32_t *input_vertex);
/* coord_edges[c] = edge offset of coordinate c (N); edge_coord[o] = coordinate of offset o or -1 (2m') */
int mcbh_get_coords(const mcbh_problem *p, uint32_t *coord_edges, int32_t *edge_coord);
/* candidates in rank order (K each); tree = FVS index of the root */
int mcbh_get_candidates(const mcbh_problem *p, int32_t *root, int32_t *edge_offset, int32_t *weight,
                        int32_t *tree);
/* offsets (K+1) into coords (cycle_nnz); each list sorted ascending */
int mcbh_get_cycle_lists(const mcbh_problem *p, int64_t *offsets, int32_t *coords);
/* parent_edge[t*n' + v] = edge offset (parent -> v) in tree t, -1 at the root */
int mcbh_get_tree_parents(const mcbh_problem *p, int32_t *parent_edge);
/* reference GPU layout (include/Dijkstra.h:151-203), tree-major:
 *   level_offsets F x (n'+1), parent_pos F x n', edge_offset F x n', nodes_index F x n' */
int mcbh_get_ref_layout(const mcbh_problem *p, uint32_t *level_offsets, uint32_t *parent_pos,
                        int32_t *edge_offset, uint32_t *nodes_index);

/* ---- seeded synthetic inputs (splitmix64) ---------------------------------- */
/* r x c grid, row-major ids, right then down edge per vertex; weights U[wlo,whi].
 * Returns the number of edges written (call with u == NULL to size). */
int64_t mcbh_gen_grid(int32_t r, int32_t c, int32_t wlo, int32_t whi, uint64_t seed,
                      int32_t *u, int32_t *v, int32_t *w);
/* connected random sparse graph: random spanning tree (random-permutation attach)
 * plus uniform extra edges (no loops, no duplicates) up to m edges. */
int64_t mcbh_gen_random(int32_t n, int64_t m, int32_t wlo, int32_t whi, uint64_t seed,
                        int32_t *u, int32_t *v, int32_t *w);
/* random geometric graph: n points in the unit square, k nearest neighbours,
 * symmetrised, weight round(1000*length) (>= 1), plus the shortest bridging edges
 * needed to connect the components (in order of component discovery). */
int64_t mcbh_gen_rgg(int32_t n, int32_t k, uint64_t seed, int32_t *u, int32_t *v, int32_t *w);
/* planar-like graph with degree-two chains: a triangulated grid of about `points`
 * vertices (right and down edges, one diagonal per cell in a random direction),
 * delete_pct% of its edges deleted while a random spanning tree is kept (the graph
 * stays connected), then every kept edge subdivided with probability chain_pct% into
 * a chain of 1..chain_max extra vertices; weights uniform in [wlo, whi] per final
 * edge.  Returns the edge count; *nodes gets the vertex count.  Call with u = NULL
 * first to size the arrays. */
int64_t mcbh_gen_planar_chains(int32_t points, int32_t delete_pct, int32_t chain_pct, int32_t chain_max,
                               int32_t wlo, int32_t whi, uint64_t seed, int32_t *u, int32_t *v, int32_t *w,
                               int32_t *nodes);
/* tree of blocks: `blocks` 2-connected random blocks (a Hamiltonian cycle plus
 * uniform extra edges; size log-uniform in [nmin, nmax], average degree uniform in
 * [deg_lo_x10, deg_hi_x10] / 10), block i > 0 sharing one random earlier vertex (an
 * articulation point).  Returns the edge count; *nodes gets the vertex count. */
int64_t mcbh_gen_block_tree(int32_t blocks, int32_t nmin, int32_t nmax, int32_t deg_lo_x10, int32_t deg_hi_x10,
                            int32_t wlo, int32_t whi, uint64_t seed, int32_t *u, int32_t *v, int32_t *w,
                            int32_t *nodes);
int mcbh_write_mtx(const char *path, int32_t nodes, int64_t m, const int32_t *u, const int32_t *v,
                   const int32_t *w);

/* ---- biconnected components ------------------------------------------------ */
/* Splits the edges of an undirected graph into biconnected components (Hopcroft-
 * Tarjan; a bridge is a component of one edge, a self-loop one of its own).
 * comp_of_edge[i] = component of edge i, components numbered in order of their
 * first edge.  Returns the number of components.  The minimum cycle basis of a graph
 * is the union of its components' bases, so every component can be solved on its
 * own; this replaces the reference's bicc tool + per-component loop (bicc/,
 * main.sh:19-32) inside one process. */
int64_t mcbh_bcc_split(int32_t nodes, int64_t m, const int32_t *u, const int32_t *v, int32_t *comp_of_edge);
/* The order in which the reference's bicc tool writes a component's edges
 * (bicc/include/bicc.h:220-314, print_to_a_file): the slots of the input graph's CSR
 * (include/CsrGraph.h:113-174, the 2m directed slots sorted by (row, col)) whose row
 * exceeds their column, in slot order, each written as (row, column).  order[k] =
 * the input edge of the k-th such slot (m entries at most; self-loops have none).
 * Returns the number written.  A component's edges in this order, with its vertices
 * numbered in order of first appearance (row before column, bicc/Relabeller.cpp:72-126),
 * are the graph the reference's per-component run reads. */
int64_t mcbh_edge_slot_order(int32_t nodes, int64_t m, const int32_t *u, const int32_t *v, int64_t *order);

#ifdef __cplusplus
}
#endif
#endif
