// The per-root shortest-path tree kernel shared by the tree handle (mcbgpu_trees.cu)
// and the device candidate generation (mcbgpu_gen.cu).
//
// Shortest-path trees of many roots of one graph (the host's per-root tree searches,
// include/Dijkstra.h:78-124, as one persistent launch): for each root, the distances
// to every vertex and every vertex's parent slot, chosen by the rule that makes any
// exact search agree with the reference's heap search, plus a flag for the roots
// where that rule cannot decide.
//
// Graph: the reduced multigraph's CSR (row offsets, columns, weights, reverse slots),
// every weight at least 1 and every distance below 2^31 (checked at creation).
//
// One CTA per root, persistent over a root counter:
//   1. distances, label-correcting by buckets: each round takes lo = (a lower
//      bound of) the smallest distance among dirty vertices and relaxes (atomicMin)
//      the arcs of every dirty vertex nearer than lo + delta, marking improved heads
//      dirty.  The dirty vertex at lo is final after its round (weights >= 1), so a
//      root needs at most 2 (n + 1) rounds; the loop stops there and flags the root
//      if it has not converged.  Distances and dirty bits live in shared memory up
//      to kTreeSharedMaxN vertices, in a per-CTA global slice beyond.  delta (the
//      bucket width) trades rounds (each a pass over the dirty bits and a barrier)
//      against relaxations repeated inside a bucket; the callers time a few widths
//      and CTA shapes on their first roots and keep the fastest.
//   2. parents: for each vertex c, among its neighbours x on a shortest path
//      (d[x] + w = d[c]) the nearest one, entered through its first slot to c (the
//      smallest slot index of x's row among those arcs); the reference keeps exactly
//      that parent (only a strictly shorter path replaces one, and parents at
//      different distances settle in distance order) unless two different
//      neighbours tie at that nearest distance, which sets the root's flag so that
//      the host searches that root itself.  The same pass checks that the distances
//      are exact: every vertex but the root has a parent with d[x] + w = d[c] (so
//      d[c] is a path length) and no slot offers a shorter one (so it is the
//      shortest); a root that fails is flagged too.  So every tree handed out with
//      its flag clear is the reference's, whatever the rounds before did.
// CTA barriers are cta_sync / cta_sync_and (the non-aligned barrier): the loops
// before them diverge within warps.
#pragma once

#include <climits>
#include <vector>

#include "mcbgpu_internal.cuh"

namespace mcbgpu {
namespace sssp {
// internal linkage: every file that includes this header gets its own copy of the
// kernel, registered with its own module
namespace {

constexpr int kTreeThreads = 1024;      // the shared-memory form's CTA
constexpr int kTreeSharedMaxN = 53248;  // 208 KB of distances + 6.5 KB of dirty bits (of 227 KB)
constexpr int kTreeMaxCtasPerSm = 16;   // the global form's per-CTA slices are sized for this many

struct TreeArgs {
    const uint32_t *ro;
    const uint32_t *cols;
    const int32_t *w;
    const uint32_t *rev;
    int32_t n;
    int32_t delta;
    const uint32_t *roots;
    int32_t count;
    int32_t *dist_out;   // count x n
    int32_t *pedge_out;  // count x n
    uint8_t *tied_out;   // count
    int32_t *gdist;      // gridDim.x x n (global form only)
    uint32_t *gdirty;    // gridDim.x x words (global form only)
    uint32_t *gsumm;     // gridDim.x x summary words (global form only)
    int32_t *next_root;
    unsigned *status;
};

// Threads per CTA: the shared-memory form runs one 1024-thread CTA per SM (its
// distances fill the shared memory); the global form runs kThreads-thread CTAs,
// several per SM, so that the bucket rounds of different roots overlap.
template <bool kShared, int kThreads>
__global__ void __launch_bounds__(kThreads) trees_kernel(TreeArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int s_next[3];
    __shared__ int s_root;
    __shared__ int s_cnt[2];
    const int n = a.n;
    const int words = (n + 31) >> 5;
    const int swords = (words + 31) >> 5;  // summary: one bit per dirty word
    int32_t *dist;
    uint32_t *dirty, *summ;
    if (kShared) {
        dist = reinterpret_cast<int32_t *>(smem);
        dirty = reinterpret_cast<uint32_t *>(smem + (((size_t)n * 4 + 15) & ~(size_t)15));
        summ = dirty + words;
    } else {
        dist = a.gdist + (size_t)blockIdx.x * n;
        dirty = a.gdirty + (size_t)blockIdx.x * words;
        summ = a.gsumm + (size_t)blockIdx.x * swords;
    }
    // global form: the dirty words of a round (words < 65536 entries, 16-bit)
    uint16_t *s_list = reinterpret_cast<uint16_t *>(smem);
    volatile int32_t *vdist = dist;
    volatile uint32_t *vdirty = dirty;
    volatile uint32_t *vsumm = summ;
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31;
    for (;;) {
        if (tid == 0) s_root = atomicAdd(a.next_root, 1);
        cta_sync();
        const int r = s_root;
        cta_sync();  // every thread has read s_root before thread 0 writes it again
        if (r >= a.count) return;
        const uint32_t src = a.roots[r];  // < n, checked by the host
        for (int v = tid; v < n; v += nt) dist[v] = INT_MAX;
        for (int k = tid; k < words; k += nt) dirty[k] = 0;
        for (int k = tid; k < swords; k += nt) summ[k] = 0;
        if (tid == 0) {
            s_next[0] = INT_MAX;
            s_next[1] = INT_MAX;
            s_cnt[0] = 0;
            s_cnt[1] = 0;
        }
        cta_sync();
        if (tid == 0) {
            dist[src] = 0;
            dirty[src >> 5] = 1u << (src & 31);
            summ[src >> 10] = 1u << ((src >> 5) & 31);
        }
        cta_sync();
        // 1. distances.  One pass per round over the dirty bits: vertices nearer than
        // hi = lo + delta are relaxed, the others skipped; the next round's lo is the
        // smallest distance of a skipped vertex or of an improvement made in this
        // round (at most the smallest distance left dirty, so no vertex is missed;
        // an underestimate only costs a round).  The dirty vertex at the true lo is
        // final once relaxed (weights >= 1), so at most 2 (n + 1) rounds; the loop
        // stops there and flags the root if it has not converged.  The round's
        // minimum goes to s_next[round % 3]: the slot read after this round's
        // barrier, reset two rounds later, when every thread has read it.
        bool converged = false;
        int lo = 0;
        for (int round = 0; round <= 2 * n + 1; round++) {
            if (lo == INT_MAX) {
                converged = true;
                break;
            }
            const int hi = lo > INT_MAX - a.delta ? INT_MAX : lo + a.delta;
            const int slot = round % 3;
            if (tid == 0) s_next[(round + 1) % 3] = INT_MAX;
            int mynext = INT_MAX;
            // One dirty word: relax its vertices nearer than hi, keep the others (and
            // their smallest distance for the next round).  Returns whether some
            // vertex was left dirty.
            auto scan_word = [&](int k) {
                uint32_t bits = vdirty[k];
                bool left = false;
                while (bits) {
                    const int b = __ffs(bits) - 1;
                    bits &= bits - 1;
                    const int v = (k << 5) + b;
                    const int d0 = vdist[v];
                    if (d0 >= hi) {
                        mynext = d0 < mynext ? d0 : mynext;
                        left = true;
                        continue;
                    }
                    atomicAnd(&dirty[k], ~(1u << b));
                    // pairs with the fence between a writer's atomicMin and atomicOr:
                    // a bit this atomicAnd cleared was set after its distance was
                    // lowered, so the read below sees that distance; a later
                    // improvement sets the bit again
                    __threadfence_block();
                    const int dv = vdist[v];
                    for (uint32_t o = a.ro[v]; o < a.ro[v + 1]; o++) {
                        const uint32_t x = a.cols[o];
                        const int nd = dv + a.w[o];
                        if (nd < vdist[x]) {
                            const int old = atomicMin(&dist[x], nd);
                            if (nd < old) {
                                __threadfence_block();  // the new distance before the dirty bit
                                atomicOr(&dirty[x >> 5], 1u << (x & 31));
                                if (!kShared) {
                                    __threadfence_block();  // the dirty bit before the summary bit
                                    atomicOr(&summ[x >> 10], 1u << ((x >> 5) & 31));
                                }
                                mynext = nd < mynext ? nd : mynext;
                            }
                        }
                    }
                }
                return left;
            };
            if (kShared) {
                for (int k = tid; k < words; k += nt) scan_word(k);
            } else {
                // the summary words: a set bit marks a dirty word as possibly non-zero.
                // A writer sets the dirty bit, then the summary bit (fence between).
                // Phase 1 clears the summary bits and lists their words; the barrier
                // orders the clears before phase 2's reads of the words, so a bit set
                // before a clear is seen in its word and one set after it leaves the
                // summary bit set for the next round; a word left with skipped
                // vertices gets its summary bit back.  The list spreads the words of
                // one summary word (neighbouring vertices, often all of the frontier)
                // over the CTA.
                int *cnt = &s_cnt[round & 1];
                if (tid == 0) s_cnt[(round + 1) & 1] = 0;  // read last in round - 1, before its barrier
                for (int q = tid; q < swords; q += nt) {
                    uint32_t sb = vsumm[q];
                    if (!sb) continue;
                    atomicAnd(&summ[q], ~sb);
                    while (sb) {
                        const int kb = __ffs(sb) - 1;
                        sb &= sb - 1;
                        s_list[atomicAdd(cnt, 1)] = (uint16_t)((q << 5) + kb);
                    }
                }
                cta_sync();
                const int m = *(volatile int *)cnt;
                for (int i = tid; i < m; i += nt) {
                    const int k = s_list[i];
                    if (scan_word(k)) atomicOr(&summ[k >> 5], 1u << (k & 31));
                }
            }
            mynext = __reduce_min_sync(0xffffffffu, mynext);
            if (lane == 0 && mynext != INT_MAX) atomicMin(&s_next[slot], mynext);
            cta_sync();
            lo = s_next[slot];
        }
        // 2. parents by the rule, and the root's tie flag
        int tie = converged ? 0 : 1;
        for (int c = tid; c < n; c += nt) {
            const int dc = vdist[c];
            int32_t slot = -1;
            if ((uint32_t)c != src && dc != INT_MAX) {
                int bestd = INT_MAX, rival = 0;  // rival: another neighbour as near as the best
                int shorter = 0;                 // some slot offers c a shorter path
                uint32_t bestx = 0xffffffffu, bests = 0xffffffffu;
                for (uint32_t o = a.ro[c]; o < a.ro[c + 1]; o++) {
                    const uint32_t x = a.cols[o];
                    const int dx = vdist[x];
                    if (dx == INT_MAX) continue;
                    // the certificate of exact distances: no slot gives c a shorter
                    // path (with every vertex's distance that of a real path through
                    // its parent, below, the distances are the shortest); a root
                    // that fails it is left to the host
                    if ((long long)dx + a.w[o] < (long long)dc) shorter = 1;
                    if ((long long)dx + a.w[o] != (long long)dc) continue;
                    if (dx < bestd) {
                        bestd = dx;
                        bestx = x;
                        bests = a.rev[o];
                        rival = 0;
                    } else if (dx == bestd) {
                        if (x == bestx)
                            bests = a.rev[o] < bests ? a.rev[o] : bests;
                        else
                            rival = 1;
                    }
                }
                slot = bests == 0xffffffffu ? -1 : (int32_t)bests;
                if (rival || shorter || slot < 0) tie = 1;  // (no shortest-path neighbour cannot happen; left to the host)
            } else if ((uint32_t)c != src) {
                tie = 1;  // unreachable vertex (the graph is not connected): left to the host
            }
            a.dist_out[(size_t)r * n + c] = dc;
            a.pedge_out[(size_t)r * n + c] = slot;
        }
        tie = cta_sync_and(tie == 0) ? 0 : 1;
        if (tid == 0) a.tied_out[r] = tie ? 1 : 0;
        if (!converged && tid == 0) atomicOr(a.status, ST_DIVERGED);
    }
}

// Dynamic shared memory for n vertices: the shared form's distances, dirty bits and
// summary bits; the global form's list of a round's dirty words.
inline size_t trees_smem_bytes(int n) {
    const size_t words = ((size_t)n + 31) / 32;
    return (((size_t)n * 4 + 15) & ~(size_t)15) + words * 4 + ((words + 31) / 32) * 4;
}
inline size_t trees_global_smem_bytes(int n) { return 2 * ((((size_t)n + 31) / 32 + 7) & ~(size_t)7); }
constexpr int kTreeGlobalMaxN = 65536 * 32;  // the global form's 16-bit word list: at most 128 KB

// A launch shape of trees_kernel: CTA size, CTAs per SM (global form) and the
// bucket width as a multiple of the mean edge weight, in quarters.
struct TreeShape {
    int threads, ctas_per_sm, delta_quarters;
};

// The bucket width of a shape on a graph whose mean slot weight is mean_w.
inline int32_t shape_delta(const TreeShape &sh, int32_t mean_w) {
    const long long d = ((long long)mean_w * sh.delta_quarters + 3) / 4;
    return (int32_t)(d < 1 ? 1 : d > (1ll << 30) ? (1ll << 30) : d);
}

// Launches trees_kernel in `shape` over grid CTAs (the shared form: 1024 threads,
// smem bytes of dynamic shared memory).
inline cudaError_t launch_trees(bool shared, const TreeShape &shape, int grid, size_t smem, cudaStream_t st,
                                const TreeArgs &a) {
    if (shared) {
        trees_kernel<true, kTreeThreads><<<grid, kTreeThreads, smem, st>>>(a);
    } else {
        const size_t lb = trees_global_smem_bytes(a.n);
        switch (shape.threads) {
        case 128: trees_kernel<false, 128><<<grid, 128, lb, st>>>(a); break;
        case 256: trees_kernel<false, 256><<<grid, 256, lb, st>>>(a); break;
        case 512: trees_kernel<false, 512><<<grid, 512, lb, st>>>(a); break;
        default: trees_kernel<false, 1024><<<grid, 1024, lb, st>>>(a); break;
        }
    }
    return cudaGetLastError();
}

inline cudaError_t set_trees_smem_limit() {
    cudaError_t e = cudaFuncSetAttribute(trees_kernel<true, kTreeThreads>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)trees_smem_bytes(kTreeSharedMaxN));
    const int lb = (int)trees_global_smem_bytes(kTreeGlobalMaxN);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(trees_kernel<false, 128>, cudaFuncAttributeMaxDynamicSharedMemorySize, lb);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(trees_kernel<false, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize, lb);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(trees_kernel<false, 512>, cudaFuncAttributeMaxDynamicSharedMemorySize, lb);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(trees_kernel<false, 1024>, cudaFuncAttributeMaxDynamicSharedMemorySize, lb);
    return e;
}

}  // namespace
}  // namespace sssp
}  // namespace mcbgpu

