/*
 * mcbgpu.h — C ABI of the GB300 (sm_103a) de Pina hot path (libmcbgpu.so).
 *
 * Three groups of entry points:
 *
 * 1. The reference's own GPU-layer free functions (gpu/common.cuh:18-27), under
 *    their original names, with the reference's behaviour (print + exit on a CUDA
 *    error, utils.h:36-47), plus status-returning mcbgpu_* forms of the same calls.
 *
 * 2. The gpu_struct object (gpu/gpu_struct.cuh:44-84) as a handle: create /
 *    initialize_memory / copy_support_vector / process_shortest_path / clear_memory.
 *    process_shortest_path computes, for every FVS tree and every position of the
 *    reference's level-ordered layout, the parity of the support vector over the
 *    non-tree edges on the root path (gpu/kernel_init_edges.cu:33-75 followed by
 *    gpu/kernel_multi_search.cu:63-108) and copies the labels to the caller's
 *    per-chunk host rows, as the reference does (gpu/gpu_struct.cu:158-193).
 *
 * 3. The device-resident main loop (mcb/mcb_cycle_deg_two_remove.cpp:317-398):
 *    candidates in rank order, each with its sorted list of cycle coordinates,
 *    are uploaded once; the support vectors S_j live in HBM; the search for the
 *    first odd candidate, the cycle vector and the independence update run on the
 *    device.  Two forms give identical results:
 *      - per iteration: mcbgpu_select / mcbgpu_cycle_vector / mcbgpu_update, one
 *        call each per iteration e, as the reference loop calls them;
 *      - blocked: mcbgpu_solver_run, which runs 64 iterations per pass (the search
 *        finds the 64 rank-ordered independent candidates for S_e..S_{e+63} in
 *        one sweep and the update applies the 64 iterations' changes to every later
 *        S_j in one sweep; GF(2) arithmetic is exact, so the selected sequence is
 *        the reference's).
 *
 * All mcbgpu_* functions return MCBGPU_OK (0) or a negative MCBGPU_E* code and
 * never exit; mcbgpu_last_error() describes the last failure of the calling
 * thread.  Streams are passed as `void *` (a cudaStream_t; NULL = legacy default).
 * One handle must not be used from two threads at once.
 */
#ifndef MCBGPU_H
#define MCBGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    MCBGPU_OK = 0,
    MCBGPU_E_ARG = -1,        /* invalid argument / size */
    MCBGPU_E_CUDA = -2,       /* a CUDA runtime call failed */
    MCBGPU_E_NOMEM = -3,      /* device or host allocation failed */
    MCBGPU_E_STATE = -4,      /* call out of order */
    MCBGPU_E_DEVICE = -5,     /* a kernel reported an error status (see mcbgpu_last_error) */
    MCBGPU_E_NO_CANDIDATE = -6 /* no odd candidate for some S_e (input has no cycle basis in its candidate set) */
};

const char *mcbgpu_last_error(void);
int mcbgpu_version(void); /* ABI version, currently 1 */

/* ---- 1. reference free functions (gpu/common.cuh:18-27) ------------------- */
/* gpu/common.cu:9-12 */
void init_cuda(void);
/* gpu/common.cu:14-30: grid = #SMs, block = max threads; returns min(end-start, #SMs) */
size_t configure_grid(int start, int end);
/* gpu/common.cu:32-41: pinned host buffer of chunk*nodes uint32 */
unsigned *allocate_pinned_memory(int chunk, int nodes);
/* gpu/common.cu:43-46 */
void free_pinned_memory(unsigned *ptr);
/* gpu/common.cu:48-67: how many trees of `num_nodes` fit next to the map and S */
size_t calculate_chunk_size(size_t num_nodes, size_t num_edges, size_t size_vector, size_t nstream);

int mcbgpu_init_cuda(int *device, int *sm_count, size_t *total_global_mem);
int mcbgpu_allocate_pinned(size_t bytes, void **out);
int mcbgpu_free_pinned(void *ptr);

/* ---- 2. gpu_struct (gpu/gpu_struct.cuh:44-84) ----------------------------- */
typedef struct mcbgpu_struct mcbgpu_struct;

/* gpu_struct::gpu_struct (gpu/gpu_struct.cuh:44-60, gpu_struct.cu:3-17).
 * num_edges = 2m' (size of the non-tree-edge map), size_vector = ceil(N/64).
 * All fvs_size trees are kept resident in HBM (the reference's chunk streaming,
 * gpu_struct.cu:132-156, is not needed on a 288 GB device); chunk_size only fixes
 * the host row layout of compressed_trees (ceil(F/chunk) rows of chunk trees). */
int mcbgpu_struct_create(mcbgpu_struct **out, int num_edges, int num_non_tree_edges, int size_vector,
                         int original_nodes, int fvs_size, int chunk_size, int nstreams);
/* gpu_struct::initialize_memory (gpu_struct.cu:76-101): the map (num_edges int32)
 * and, per host row i, edge_offset[i] (chunk*n int32), tree_rows[i]
 * (chunk*(n+1) uint32) and tree_cols[i] (chunk*n uint32) as compressed_trees holds
 * them (include/compressed_trees.h:112-128). */
int mcbgpu_struct_initialize_memory(mcbgpu_struct *s, const int32_t *non_tree_edges_map,
                                    const int32_t *const *edge_offset_rows,
                                    const uint32_t *const *tree_rows_rows,
                                    const uint32_t *const *tree_cols_rows);
/* gpu_struct::copy_support_vector (gpu_struct.cu:104-114): upload S (size_vector
 * words); *ms = elapsed milliseconds (may be NULL). */
int mcbgpu_struct_copy_support_vector(mcbgpu_struct *s, const uint64_t *support_vector, float *ms);
/* gpu_struct::process_shortest_path (gpu_struct.cu:169-193): labels of every
 * position of every tree for the current S, written as uint32 0/1 into
 * precompute_rows[i] (chunk*n per host row, the layout of
 * compressed_trees::precompute_value).  precompute_rows may be NULL to keep the
 * labels on the device only.  multiple_transfer is accepted for signature parity;
 * trees are always resident.  A tree whose levels end before position n gives
 * MCBGPU_E_DEVICE, with 0 at the unreached positions. */
int mcbgpu_struct_process_shortest_path(mcbgpu_struct *s, uint32_t *const *precompute_rows,
                                        int multiple_transfer, float *ms);
/* gpu_struct::clear_memory (gpu_struct.cu:19-28); also frees the handle. */
int mcbgpu_struct_clear_memory(mcbgpu_struct *s);

/* No counterpart in the reference.  The labels of process_shortest_path, computed
 * without allocating: for callers that cannot call cudaMalloc (a host framework
 * that owns all device memory through its own pool, or a latency-critical loop
 * that must not take the synchronisation cudaMalloc / cudaFree can imply).  All
 * pointers are device memory owned by the caller, tree-major as in
 * initialize_memory (level_offsets F x (nodes+1), parent_pos and edge_offset
 * F x nodes), the map (num_edges), S (ceil(N/64) words); labels receives F x nodes
 * uint32 0/1.  Working memory is a static device array inside the library
 * (16 MiB of per-CTA label slabs + a status word) that every GPU loading the
 * library keeps until exit; trees of more than 16 Mi vertices are rejected.  The
 * first call on a device looks up the array's device address (cudaGetSymbolAddress)
 * and should come before any stream capture.  Calls share the array: calls that
 * overlap on the GPU (other streams, other threads) race.  The call synchronises
 * `stream` to read the kernel's status.  Every position of a tree must lie on one
 * of its levels (true of every tree of a connected graph): a tree whose levels end
 * before position `nodes` gives MCBGPU_E_DEVICE, with 0 at the unreached positions. */
int mcbgpu_label_forest_noalloc(const uint32_t *level_offsets, const uint32_t *parent_pos,
                                const int32_t *edge_offset, const int32_t *non_tree_edges_map, int num_edges,
                                const uint64_t *support_vector, int num_coords, int fvs_size, int nodes,
                                uint32_t *labels, void *stream);

/* ---- 3. device-resident main loop ------------------------------------------ */
typedef struct mcbgpu_solver mcbgpu_solver;

/* num_coords = N, num_candidates = K (rank order), nnz = total coordinates. */
int mcbgpu_solver_create(mcbgpu_solver **out, int32_t num_coords, int64_t num_candidates, int64_t nnz);
/* Upload the rank-ordered candidates: weight[K], offsets[K+1] (int64, offsets[0]
 * = 0, offsets[K] = nnz) and coords[nnz] (each candidate's list sorted ascending,
 * values in [0, N)).  Resets every S_j to the unit vector e_j (the reference's
 * initial support vectors, mcb/mcb_cycle_deg_two_remove.cpp:274-278).  Asynchronous
 * on `stream` with respect to the device; host buffers must stay valid until the
 * stream has passed this point. */
int mcbgpu_solver_upload(mcbgpu_solver *s, const int32_t *weight, const int64_t *offsets,
                         const int32_t *coords, void *stream);
/* mcbgpu_solver_upload with the three arrays in device memory (e.g. the lists a
 * device candidate generation built, mcbgpu_gen_get_lists): copied on the device. */
int mcbgpu_solver_upload_device(mcbgpu_solver *s, const int32_t *weight, const int64_t *offsets,
                                const int32_t *coords, void *stream);
/* No counterpart in the reference.  Re-verification of a complete run's basis on
 * the device: the product M[i][j] = <C_i, S_j> of the selected cycles' vectors and
 * the final support vectors, over every pair i <= j (O(N^3 / 64) word operations,
 * an N x ceil(N/64) word scratch matrix).  A de Pina run leaves M unit lower
 * triangular, which proves the N cycles GF(2)-independent (rank N of N); any
 * other entry is counted in *violations, the first (row-major) at (*first_bad_i,
 * *first_bad_j) (-1 if none; either may be NULL).  MCBGPU_E_STATE before the run
 * is complete. */
int mcbgpu_solver_verify(mcbgpu_solver *s, int64_t *violations, int64_t *first_bad_i, int64_t *first_bad_j,
                         void *stream);
/* Reset S to the unit vectors without re-uploading the candidates. */
int mcbgpu_solver_reset(mcbgpu_solver *s, void *stream);

/* Per-iteration form.  The caller runs e = 0, 1, ... in order.
 * select: rank of the first candidate with <C, S_e> = 1 (the scan of
 *   mcb/mcb_cycle_deg_two_remove.cpp:329-358); written to *rank (host, after a
 *   stream sync) if rank != NULL, and kept on the device for the next two calls.
 * cycle_vector: C_e of the selected candidate as ceil(N/64) words
 *   (include/cycles.h:144-195) into `words` (host, may be NULL: device only).
 * update: for every j > e with <C_e, S_j> odd, S_j ^= S_e (mcb/mcb_cycle_deg_two_remove.cpp:371-390). */
int mcbgpu_select(mcbgpu_solver *s, int32_t e, int64_t *rank, void *stream);
int mcbgpu_cycle_vector(mcbgpu_solver *s, int32_t e, uint64_t *words, void *stream);
int mcbgpu_update(mcbgpu_solver *s, int32_t e, void *stream);

/* Blocked form: iterations [0, min(max_iterations, N)) (max_iterations < 0: all),
 * enqueued on `stream` without host synchronisation.  Results via
 * mcbgpu_solver_results. */
int mcbgpu_solver_run(mcbgpu_solver *s, int64_t max_iterations, void *stream);
/* A complete solve (reset of S to the unit vectors, then the blocked run over
 * iterations [0, min(max_iterations, N))) as one CUDA graph, launched on `stream`.
 * The first call (and the first after a tuning run, a shape change or another
 * max_iterations) captures the solve on a stream of the handle and instantiates it;
 * later calls replay it.  The graph reads the handle's buffers, so a new upload
 * (same sizes) is solved by the same graph.  Results via mcbgpu_solver_results, as
 * after mcbgpu_solver_run.  Not with profiling on.  No counterpart in the reference
 * (its loop is host code). */
int mcbgpu_solver_run_graph(mcbgpu_solver *s, int64_t max_iterations, void *stream);
/* Per-iteration form over all iterations, enqueued without host synchronisation
 * (select + update per iteration). */
int mcbgpu_solver_run_plain(mcbgpu_solver *s, int64_t max_iterations, void *stream);
/* Synchronises `stream`; copies selected[e] (rank chosen at iteration e) for the
 * iterations run, the 64-bit total weight, and checks the device status word. */
int mcbgpu_solver_results(mcbgpu_solver *s, int64_t *selected, int64_t count, int64_t *total_weight,
                          void *stream);
/* Copy S_j (ceil(N/64) words) to the host (synchronous). */
int mcbgpu_solver_get_support(mcbgpu_solver *s, int32_t j, uint64_t *words, void *stream);
/* Optional live profile.  set_profiling(1) clears the records; from then on every
 * kernel launch of the handle is bracketed by CUDA events on its stream, and the
 * kernels add their algorithmic HBM bytes to per-class counters.  kernel_stats
 * synchronises the device, fills one entry per kernel class launched since, and
 * clears the records. */
typedef struct mcbgpu_kernel_stat {
    const char *name;
    int64_t launches;
    double ms;     /* summed event time of the launches */
    double bytes;  /* summed algorithmic bytes (0 where a kernel does not count) */
} mcbgpu_kernel_stat;
int mcbgpu_solver_set_profiling(mcbgpu_solver *s, int enable);
int mcbgpu_solver_kernel_stats(mcbgpu_solver *s, mcbgpu_kernel_stat *out, int max_entries, int *count);
/* Counters of the blocked search, summed over the blocks run since the last reset:
 * [0] pivot steps (grid barriers), [1] local pivots reported, [2] merge candidates,
 * [3] W tiles loaded, [4] W tiles computed inside the pivot kernel, [5] blocks,
 * [6] / [7] / [8] SM clock cycles of CTA 0 in the scan / barrier / merge parts,
 * [9]-[13] where a bounded barrier wait gave up (CTA+1, step, rank, generation,
 * arrivals), [14]/[15] most/fewest barriers of a CTA in one launch, [16]-[19] first
 * step at which two CTAs disagreed on the merged result (flag, step, CTA, block),
 * [20] / [21] / [22] SM clock cycles of CTA 0 in the block tail: resolve, the tail's
 * grid barrier, final rows; far update: [23] dense non-unit rows gathered,
 * [29] update bits of the changed rows, [30] rows changed, [31] pair words gathered,
 * [32] unit rows reached by the scatter, [38] sparse non-unit rows tested, [39]
 * their listed words, [40] their pair tests; [24]-[28] and [33]-[37] per-phase clock
 * counters of profiling builds.  At most 48 counters; synchronises the device. */
int mcbgpu_solver_diagnostics(mcbgpu_solver *s, int64_t *out, int n, int reset);
/* Search shapes of the blocked run (no counterpart in the reference, whose host scan
 * has no shape).  A shape sets the pivot search's window (W tiles a CTA scans per
 * step, by how many of the block's 64 pivots are known), the local pivots after
 * which a CTA ends its step, and how far past the previous block's last pivot the
 * streaming pass reaches.  Every shape gives the same result; only the time
 * differs.  A solve is cut into MCBGPU_SHAPE_SEGMENTS segments of 64-iteration
 * blocks, each with its own shape (candidate 0, the built-in default, until tuned).
 *
 * tune: one complete blocked run from a reset, the candidate shapes taking turns
 *   group by group (the blocks that share one streaming pass); each segment then
 *   keeps the shape with the least mean search time per block (event-timed on the
 *   device, from a group's first transpose to the end of its last pivot search).
 *   The run's results are valid like those of mcbgpu_solver_run.  Synchronises
 *   `stream`.  ms_per_block (may be NULL): MCBGPU_SHAPE_SEGMENTS x n_shapes means;
 *   chosen (may be NULL): the shape of each segment.  With fewer than 4 groups per
 *   segment and shape the default stays.
 * set_shape: force one candidate for every block (-1: back to the per-segment choice).
 * shapes: the candidates' parameters, MCBGPU_SHAPE_INTS each (window early, rank it
 *   ends at, window middle, rank the tail window starts at, window tail, local-pivot
 *   limit, streaming reach in percent), their number, and each segment's shape. */
#define MCBGPU_SHAPE_SEGMENTS 4
#define MCBGPU_SHAPE_INTS 7
int mcbgpu_solver_tune(mcbgpu_solver *s, double *ms_per_block, int32_t *chosen, void *stream);
int mcbgpu_solver_set_shape(mcbgpu_solver *s, int32_t shape);
int mcbgpu_solver_shapes(const mcbgpu_solver *s, int32_t *params, int32_t max_shapes, int32_t *n_shapes,
                         int32_t *segment_shape);
/* Kernel launches issued by this handle so far (for accounting). */
int64_t mcbgpu_solver_launches(const mcbgpu_solver *s);
/* Device bytes held by the handle. */
int64_t mcbgpu_solver_device_bytes(const mcbgpu_solver *s);
int mcbgpu_solver_destroy(mcbgpu_solver *s);

/* One-shot call with host buffers: create, upload, blocked run, results, destroy.
 * selected[N] receives the rank chosen at each iteration. */
int mcbgpu_solve(int32_t num_coords, int64_t num_candidates, const int32_t *weight, const int64_t *offsets,
                 const int32_t *coords, int64_t *selected, int64_t *total_weight);

/* ---- 4. batched main loop ---------------------------------------------------
 * Many independent problems (the biconnected components of one graph, or many
 * graphs) in one persistent launch, one CTA per problem at a time.
 * Replaces the reference's one-process-per-component loop (main.sh:19-32 runs the
 * whole mcb driver once per bicc component file); every problem's result equals
 * mcbgpu_solver_run's on the same inputs.
 *
 * create: count problems, problem i with num_coords[i] = N_i (at most
 *   mcbgpu_batch_max_coords()) and num_candidates[i] = K_i; nnz = total coordinates.
 * upload: the problems' candidates back to back in problem order: weight[sum K],
 *   offsets[sum K + 1] (int64, one running sequence from 0 to nnz), coords[nnz]
 *   (each list ascending in [0, N_i) of its problem).  Synchronises `stream`: the
 *   offsets are checked on the device (MCBGPU_E_ARG if they are not non-decreasing
 *   from 0 to nnz).
 * run: enqueued on `stream` without host synchronisation.
 * results: selected[sum N] (problem i's iterations at offset N_0 + ... + N_{i-1},
 *   each the candidate's rank within problem i), total_weight[count] (-1 for a
 *   problem that failed), problem_status[count] (0 = solved; may be NULL); returns
 *   MCBGPU_E_ARG if some problem's lists were malformed, MCBGPU_E_NO_CANDIDATE if
 *   some problem's candidates do not span its cycle space. */
typedef struct mcbgpu_batch mcbgpu_batch;
int mcbgpu_batch_max_coords(void);
int mcbgpu_batch_create(mcbgpu_batch **out, int32_t count, const int32_t *num_coords,
                        const int64_t *num_candidates, int64_t nnz);
int mcbgpu_batch_upload(mcbgpu_batch *b, const int32_t *weight, const int64_t *offsets, const int32_t *coords,
                        void *stream);
int mcbgpu_batch_run(mcbgpu_batch *b, void *stream);
int mcbgpu_batch_results(mcbgpu_batch *b, int64_t *selected, int64_t *total_weight, uint32_t *problem_status,
                         void *stream);
/* S_j of problem `problem` after the run (ceil(N/64) words, synchronous). */
int mcbgpu_batch_get_support(mcbgpu_batch *b, int32_t problem, int32_t j, uint64_t *words, void *stream);
/* Optional per-problem profile of the following runs: set_profiling(1) makes the
 * kernel record, for problem i, out[13i..13i+12] = wall ns from its start to its
 * end, SM clock cycles of its CTA in the transposes, the pivot scans, the resolves,
 * the final rows + pairs and the updates of later rows, the candidates scanned, the
 * SM it ran on, the cycles of the scans' list walks (part of the pivot scans), the
 * pivot rounds (CTA-wide searches for the next pivot), the cycles warp 0 spent in
 * the update forming D and beta, and writing rows, and the bytes the scans' list
 * walks read (offsets and coordinates).  profile synchronises the device. */
int mcbgpu_batch_set_profiling(mcbgpu_batch *b, int enable);
int mcbgpu_batch_profile(mcbgpu_batch *b, int64_t *out);
int64_t mcbgpu_batch_launches(const mcbgpu_batch *b);
int64_t mcbgpu_batch_device_bytes(const mcbgpu_batch *b);
int mcbgpu_batch_destroy(mcbgpu_batch *b);
/* One-shot: create, upload, run, results, destroy. */
int mcbgpu_batch_solve(int32_t count, const int32_t *num_coords, const int64_t *num_candidates,
                       const int32_t *weight, const int64_t *offsets, const int32_t *coords, int64_t *selected,
                       int64_t *total_weight);

/* ---- 5. shortest-path trees of many roots (the host's per-root tree searches,
 * include/Dijkstra.h:78-124, on the device) -------------------------------------
 * The graph is the reduced multigraph's CSR: row offsets (nodes + 1), and per slot
 * its column, weight and reverse slot; every weight at least 1 and every distance
 * below 2^31 (MCBGPU_E_ARG otherwise).  mcbgpu_trees_run computes, for `count` <=
 * max_roots roots, every vertex's distance (count x nodes) and parent slot (the slot
 * of the parent's row that enters the vertex, -1 at the root), and per root a tie
 * flag: where it is 0 the parents equal those of the reference's heap search; where
 * it is 1 some vertex has two equally near shortest-path parents, which only the
 * heap's order decides, and the caller must search that root itself.
 * Synchronises `stream`. */
typedef struct mcbgpu_trees mcbgpu_trees;
int mcbgpu_trees_create(mcbgpu_trees **out, int32_t nodes, int64_t slots, const uint32_t *row_offsets,
                        const uint32_t *cols, const int32_t *weights, const uint32_t *rev, int32_t max_roots);
int mcbgpu_trees_run(mcbgpu_trees *t, const uint32_t *roots, int32_t count, int32_t *dist, int32_t *parent_slot,
                     uint8_t *tied, void *stream);
int64_t mcbgpu_trees_device_bytes(const mcbgpu_trees *t);
int mcbgpu_trees_destroy(mcbgpu_trees *t);

/* ---- 6. candidate generation on the device (the host preparation's per-root
 * trees, candidate test and coordinate lists: include/Dijkstra.h:78-254,
 * include/work_per_thread.h:92-147, include/cycles.h:144-195) -------------------
 * For a problem prepared on the host up to its spanning tree (mcbhost.h,
 * mcbh_options.structure_only): the reduced graph (row offsets, and per slot its
 * row, column, weight >= 1, reverse slot and coordinate or -1), the FVS array
 * (n', -1 off the FVS) and vertices (F), the pair list (mcbh_get_pairs), all checked
 * at creation.  `chunk` roots are processed per call; the parent slots of all F
 * trees stay on the device (4 F n' bytes) until mcbgpu_gen_release_trees.
 * Per chunk, in order:
 *   mcbgpu_gen_trees       the trees of FVS indices [t0, t0 + count); tied[i] = 1
 *                          where the host must search root t0 + i itself
 *                          (mcbh_search_trees), then hand its tree over with
 *   mcbgpu_gen_put_trees   (distances and parent slots, count x n', host memory);
 *   mcbgpu_gen_candidates  the candidate test of the chunk: counts[i] candidates of
 *                          root t0 + i, *total for the chunk; then
 *   mcbgpu_gen_fetch       their pair indices (ascending per root, roots in order)
 *                          and weights into host memory (total entries each).
 * After ranking (mcbh_rank_candidates on the host):
 *   mcbgpu_gen_rank        takes the K ranked candidates (tree = FVS index,
 *                          edge_offset = the candidate's slot, weight; rank order,
 *                          host memory) and walks their cycles once: list lengths
 *                          and, with `features` (device, K x 16 bf16, may be NULL),
 *                          each candidate's features for the learned proposal;
 *   mcbgpu_gen_build_lists the sorted coordinate lists of the first K_keep ranked
 *                          candidates on the device; *nnz their total (a proposal
 *                          may keep a prefix; K_keep = K builds them all);
 *   mcbgpu_gen_lists       mcbgpu_gen_rank without features + build of all K;
 *   mcbgpu_gen_get_lists   the device weights (K), offsets (K + 1) and coordinates
 *                          (nnz), valid until the next mcbgpu_gen_lists or destroy:
 *                          pass them to mcbgpu_solver_upload_device.
 * Synchronising calls (each reads the device status); an index out of range in a
 * caller's array gives MCBGPU_E_DEVICE. */
typedef struct mcbgpu_gen mcbgpu_gen;
int mcbgpu_gen_create(mcbgpu_gen **out, int32_t nodes, int64_t slots, const uint32_t *row_offsets,
                      const uint32_t *rows, const uint32_t *cols, const int32_t *weights, const uint32_t *rev,
                      const int32_t *edge_coord, int32_t num_coords, const int32_t *fvs_array,
                      const uint32_t *fvs_vertices, int32_t fvs_size, const uint32_t *pair_slot, int32_t chunk);
int mcbgpu_gen_trees(mcbgpu_gen *g, int32_t t0, int32_t count, uint8_t *tied, void *stream);
/* mcbgpu_gen_trees in two halves, so that the trees of the next chunk run while the
 * host searches the current chunk's tied roots: submit enqueues a chunk's trees into
 * one of two slots and returns; collect waits for the chunk submitted at t0, gives
 * its tie flags and makes it the current chunk (for mcbgpu_gen_put_trees and
 * mcbgpu_gen_candidates).  At most two chunks are submitted and not collected. */
int mcbgpu_gen_trees_submit(mcbgpu_gen *g, int32_t t0, int32_t count, void *stream);
int mcbgpu_gen_trees_collect(mcbgpu_gen *g, int32_t t0, uint8_t *tied, void *stream);
/* 1 while the tree kernel's launch shapes are still being timed (mcbgpu_gen_tree_shapes). */
int mcbgpu_gen_tuning(const mcbgpu_gen *g);
int mcbgpu_gen_put_trees(mcbgpu_gen *g, const int32_t *trees, int32_t count, const int32_t *dist,
                         const int32_t *parent_slot, void *stream);
int mcbgpu_gen_candidates(mcbgpu_gen *g, int64_t *counts, int64_t *total, void *stream);
int mcbgpu_gen_fetch(mcbgpu_gen *g, int64_t total, uint32_t *pair_index, int32_t *weight, void *stream);
int mcbgpu_gen_rank(mcbgpu_gen *g, int64_t K, const int32_t *tree, const int32_t *edge_offset,
                    const int32_t *weight, uint16_t *features, void *stream);
int mcbgpu_gen_build_lists(mcbgpu_gen *g, int64_t K_keep, int64_t *nnz, void *stream);
int mcbgpu_gen_lists(mcbgpu_gen *g, int64_t K, const int32_t *tree, const int32_t *edge_offset,
                     const int32_t *weight, int64_t *nnz, void *stream);
int mcbgpu_gen_get_lists(const mcbgpu_gen *g, const int32_t **weight, const int64_t **offsets,
                         const int32_t **coords);
/* The tree kernel's launch shapes (threads per CTA, CTAs per SM, bucket width in
 * quarters of the mean edge weight; 3 int32 each, up to cap), their measured
 * microseconds per root (-1: not tried) and the index of the one in use (-1: still
 * tuning).  While tuning, the first calls of mcbgpu_gen_trees each try one shape
 * on their chunk (every shape gives the same trees); then the fastest is kept. */
int mcbgpu_gen_tree_shapes(const mcbgpu_gen *g, int32_t *shapes, double *us_per_root, int32_t cap, int32_t *count,
                           int32_t *chosen);
/* The lists copied into host memory: offsets (K + 1) and coordinates (nnz). */
int mcbgpu_gen_copy_lists(const mcbgpu_gen *g, int64_t *offsets, int32_t *coords, void *stream);
/* Frees the resident parent slots (after the lists are built). */
int mcbgpu_gen_release_trees(mcbgpu_gen *g);
int64_t mcbgpu_gen_device_bytes(const mcbgpu_gen *g);
int mcbgpu_gen_destroy(mcbgpu_gen *g);

/* ---- 7. the learned proposal's network -----------------------------------------
 * A two-layer perceptron over the 16 per-candidate features of mcbgpu_gen_rank
 * (16 -> 64 ReLU -> 1): bf16 weights in the forward pass, fp32 accumulation (the
 * first layer on the tensor cores), fp32 master parameters trained with Adam on the
 * mean binary cross-entropy of (candidate, selected?) labels, positives weighted by
 * pos_weight.  Parameters, in order: W1 (64 x 16, row = hidden unit), b1 (64), w2
 * (64), b2 (1): mcbgpu_mlp_param_count() floats.  x (count x 16 bf16), labels
 * (count bytes, nonzero = selected) and logits (count floats) are device memory;
 * params and grads host memory.  Its scores order candidates for a proposal and
 * never decide a result by themselves. */
typedef struct mcbgpu_mlp mcbgpu_mlp;
int mcbgpu_mlp_param_count(void);
int mcbgpu_mlp_create(mcbgpu_mlp **out, const float *params);
int mcbgpu_mlp_get_params(const mcbgpu_mlp *m, float *params);
int mcbgpu_mlp_forward(mcbgpu_mlp *m, const uint16_t *x, int64_t count, float *logits, void *stream);
/* The loss (*loss, mean) and its gradient (grads, mcbgpu_mlp_param_count() floats)
 * at the current parameters. */
int mcbgpu_mlp_gradients(mcbgpu_mlp *m, const uint16_t *x, const uint8_t *labels, int64_t count, float pos_weight,
                         float *grads, float *loss, void *stream);
/* One Adam step (beta 0.9 / 0.999, eps 1e-8) on the batch; *loss (may be NULL) the
 * batch loss before the step. */
int mcbgpu_mlp_train_step(mcbgpu_mlp *m, const uint16_t *x, const uint8_t *labels, int64_t count, float pos_weight,
                          float lr, float *loss, void *stream);
int mcbgpu_mlp_destroy(mcbgpu_mlp *m);

#ifdef __cplusplus
}
#endif
#endif
