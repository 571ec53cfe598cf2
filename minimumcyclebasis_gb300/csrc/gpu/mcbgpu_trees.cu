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
//   1. distances, label-correcting by buckets: each round takes lo = the smallest
//      distance among dirty vertices and relaxes (atomicMin) the arcs of every dirty
//      vertex nearer than lo + delta, marking improved heads dirty.  The dirty vertex
//      at lo is final after its round (weights >= 1), so a root needs at most n
//      rounds; the loop stops there and flags the root if it has not converged.
//      Distances and dirty bits live in shared memory up to kTreeSharedMaxN vertices,
//      in a per-CTA global slice beyond.
//   2. parents: for each vertex c, among its neighbours x on a shortest path
//      (d[x] + w = d[c]) the nearest one, entered through its first slot to c (the
//      smallest slot index of x's row among those arcs); the reference keeps exactly
//      that parent (only a strictly shorter path replaces one, and parents at
//      different distances settle in distance order) unless two different
//      neighbours tie at that nearest distance, which sets the root's flag so that
//      the host searches that root itself.
// CTA barriers are cta_sync / cta_sync_and (the non-aligned barrier): the loops
// before them diverge within warps.
#include <climits>
#include <vector>

#include "mcbgpu_internal.cuh"

namespace mcbgpu {
namespace {

constexpr int kTreeThreads = 1024;
constexpr int kTreeSharedMaxN = 53248;  // 208 KB of distances + 6.5 KB of dirty bits (of 227 KB)

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
    int32_t *next_root;
    unsigned *status;
};

__device__ __forceinline__ int block_min(int v, int *red) {
    v = __reduce_min_sync(0xffffffffu, v);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) red[warp] = v;
    cta_sync();
    if (warp == 0) {
        int x = lane < (int)(blockDim.x >> 5) ? red[lane] : INT_MAX;
        x = __reduce_min_sync(0xffffffffu, x);
        if (lane == 0) red[32] = x;
    }
    cta_sync();
    return red[32];
}

template <bool kShared>
__global__ void __launch_bounds__(kTreeThreads, 1) trees_kernel(TreeArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int s_red[33];
    __shared__ int s_root;
    const int n = a.n;
    const int words = (n + 31) >> 5;
    int32_t *dist;
    uint32_t *dirty;
    if (kShared) {
        dist = reinterpret_cast<int32_t *>(smem);
        dirty = reinterpret_cast<uint32_t *>(smem + (((size_t)n * 4 + 15) & ~(size_t)15));
    } else {
        dist = a.gdist + (size_t)blockIdx.x * n;
        dirty = a.gdirty + (size_t)blockIdx.x * words;
    }
    volatile int32_t *vdist = dist;
    volatile uint32_t *vdirty = dirty;
    const int tid = threadIdx.x, nt = blockDim.x;
    for (;;) {
        if (tid == 0) s_root = atomicAdd(a.next_root, 1);
        cta_sync();
        const int r = s_root;
        cta_sync();  // every thread has read s_root before thread 0 writes it again
        if (r >= a.count) return;
        const uint32_t src = a.roots[r];  // < n, checked by the host
        for (int v = tid; v < n; v += nt) dist[v] = INT_MAX;
        for (int k = tid; k < words; k += nt) dirty[k] = 0;
        cta_sync();
        if (tid == 0) {
            dist[src] = 0;
            dirty[src >> 5] = 1u << (src & 31);
        }
        cta_sync();
        // 1. distances
        bool converged = false;
        for (int round = 0; round <= n; round++) {
            int m = INT_MAX;
            for (int k = tid; k < words; k += nt) {
                uint32_t bits = vdirty[k];
                while (bits) {
                    const int b = __ffs(bits) - 1;
                    bits &= bits - 1;
                    const int d = vdist[(k << 5) + b];
                    m = d < m ? d : m;
                }
            }
            const int lo = block_min(m, s_red);
            if (lo == INT_MAX) {
                converged = true;
                break;
            }
            const int hi = lo > INT_MAX - a.delta ? INT_MAX : lo + a.delta;
            for (int k = tid; k < words; k += nt) {
                uint32_t bits = vdirty[k];
                while (bits) {
                    const int b = __ffs(bits) - 1;
                    bits &= bits - 1;
                    const int v = (k << 5) + b;
                    if (vdist[v] >= hi) continue;
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
                            }
                        }
                    }
                }
            }
            cta_sync();
        }
        // 2. parents by the rule, and the root's tie flag
        int tie = converged ? 0 : 1;
        for (int c = tid; c < n; c += nt) {
            const int dc = vdist[c];
            int32_t slot = -1;
            if ((uint32_t)c != src && dc != INT_MAX) {
                int bestd = INT_MAX, rival = 0;  // rival: another neighbour as near as the best
                uint32_t bestx = 0xffffffffu, bests = 0xffffffffu;
                for (uint32_t o = a.ro[c]; o < a.ro[c + 1]; o++) {
                    const uint32_t x = a.cols[o];
                    const int dx = vdist[x];
                    if (dx == INT_MAX || (long long)dx + a.w[o] != (long long)dc) continue;
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
                if (rival || slot < 0) tie = 1;  // (no shortest-path neighbour cannot happen; left to the host)
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

}  // namespace
}  // namespace mcbgpu

using namespace mcbgpu;

struct mcbgpu_trees {
    int32_t n = 0;
    int64_t slots = 0;
    int32_t max_roots = 0;
    int32_t delta = 1;
    int sm_count = 0;
    bool shared_form = true;
    size_t smem = 0;
    uint32_t *d_ro = nullptr, *d_cols = nullptr, *d_rev = nullptr, *d_roots = nullptr;
    int32_t *d_w = nullptr, *d_dist = nullptr, *d_pedge = nullptr, *d_gdist = nullptr, *d_next = nullptr;
    uint32_t *d_gdirty = nullptr;
    uint8_t *d_tied = nullptr;
    unsigned *d_status = nullptr;
    long long bytes = 0;
    long long diverged_runs = 0;  // runs in which some root did not converge within n + 1 rounds
};

static void trees_free(mcbgpu_trees *t) {
    cudaFree(t->d_ro);
    cudaFree(t->d_cols);
    cudaFree(t->d_rev);
    cudaFree(t->d_roots);
    cudaFree(t->d_w);
    cudaFree(t->d_dist);
    cudaFree(t->d_pedge);
    cudaFree(t->d_gdist);
    cudaFree(t->d_next);
    cudaFree(t->d_gdirty);
    cudaFree(t->d_tied);
    cudaFree(t->d_status);
    delete t;
}

extern "C" {

int mcbgpu_trees_create(mcbgpu_trees **out, int32_t nodes, int64_t slots, const uint32_t *row_offsets,
                        const uint32_t *cols, const int32_t *weights, const uint32_t *rev, int32_t max_roots) {
    if (!out || nodes <= 0 || slots < 0 || slots >= (1ll << 31) || max_roots <= 0 || !row_offsets ||
        (slots > 0 && (!cols || !weights || !rev))) {
        set_error("mcbgpu_trees_create: invalid arguments");
        return MCBGPU_E_ARG;
    }
    *out = nullptr;
    if (row_offsets[0] != 0 || (int64_t)row_offsets[nodes] != slots) {
        set_error("mcbgpu_trees_create: row offsets must run from 0 to the slot count");
        return MCBGPU_E_ARG;
    }
    for (int32_t v = 0; v < nodes; v++)
        if (row_offsets[v + 1] < row_offsets[v]) {
            set_error("mcbgpu_trees_create: row offsets decrease at vertex %d", (int)v);
            return MCBGPU_E_ARG;
        }
    long long wsum = 0, wmax = 0;
    for (int64_t o = 0; o < slots; o++) {
        if (cols[o] >= (uint32_t)nodes || rev[o] >= (uint64_t)slots || weights[o] < 1) {
            set_error("mcbgpu_trees_create: slot %lld has column %u, reverse %u, weight %d (columns and reverses "
                      "must be in range, weights at least 1)",
                      (long long)o, cols[o], rev[o], (int)weights[o]);
            return MCBGPU_E_ARG;
        }
        wsum += weights[o];
        wmax = weights[o] > wmax ? weights[o] : wmax;
    }
    if (wmax * ((long long)nodes + 1) >= (long long)INT_MAX) {
        set_error("mcbgpu_trees_create: distances could reach 2^31 (largest weight %lld, %d vertices)", wmax,
                  (int)nodes);
        return MCBGPU_E_ARG;
    }
    mcbgpu_trees *t = new mcbgpu_trees();
    t->n = nodes;
    t->slots = slots;
    t->max_roots = max_roots;
    t->delta = slots > 0 ? (int32_t)((wsum + slots - 1) / slots) : 1;  // the mean weight
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&t->sm_count, cudaDevAttrMultiProcessorCount, dev);
    const int words = (nodes + 31) / 32;
    t->shared_form = nodes <= kTreeSharedMaxN;
    t->smem = t->shared_form ? ((((size_t)nodes * 4 + 15) & ~(size_t)15) + (size_t)words * 4) : 0;
    const size_t per_root = (size_t)nodes;
#define TALLOC(ptr, sz)                                            \
    do {                                                           \
        size_t _b = (size_t)(sz);                                  \
        if (_b < 16) _b = 16;                                      \
        if (e == cudaSuccess) e = cudaMalloc((void **)&(ptr), _b); \
        t->bytes += (long long)_b;                                 \
    } while (0)
    TALLOC(t->d_ro, 4 * ((size_t)nodes + 1));
    TALLOC(t->d_cols, 4 * (size_t)slots);
    TALLOC(t->d_rev, 4 * (size_t)slots);
    TALLOC(t->d_w, 4 * (size_t)slots);
    TALLOC(t->d_roots, 4 * (size_t)max_roots);
    TALLOC(t->d_dist, 4 * per_root * (size_t)max_roots);
    TALLOC(t->d_pedge, 4 * per_root * (size_t)max_roots);
    TALLOC(t->d_tied, (size_t)max_roots);
    TALLOC(t->d_next, 4);
    TALLOC(t->d_status, 4);
    if (!t->shared_form) {
        TALLOC(t->d_gdist, 4 * per_root * (size_t)t->sm_count);
        TALLOC(t->d_gdirty, 4 * (size_t)words * (size_t)t->sm_count);
    }
#undef TALLOC
    if (e == cudaSuccess) e = cudaMemcpy(t->d_ro, row_offsets, 4 * ((size_t)nodes + 1), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && slots > 0) {
        e = cudaMemcpy(t->d_cols, cols, 4 * (size_t)slots, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(t->d_rev, rev, 4 * (size_t)slots, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(t->d_w, weights, 4 * (size_t)slots, cudaMemcpyHostToDevice);
    }
    // the kernel's attribute is process-wide: set to the largest shared form, so that
    // handles of different sizes can be used in any order
    if (e == cudaSuccess && t->shared_form)
        e = cudaFuncSetAttribute(trees_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)((size_t)kTreeSharedMaxN * 4 + (size_t)(kTreeSharedMaxN / 32) * 4));
    if (e != cudaSuccess) {
        const int rc = cuda_fail(e, "mcbgpu_trees_create");
        trees_free(t);
        return rc;
    }
    *out = t;
    return MCBGPU_OK;
}

int mcbgpu_trees_run(mcbgpu_trees *t, const uint32_t *roots, int32_t count, int32_t *dist, int32_t *parent_slot,
                     uint8_t *tied, void *stream) {
    if (!t || count < 0 || count > t->max_roots || (count > 0 && (!roots || !dist || !parent_slot || !tied))) {
        set_error("mcbgpu_trees_run: invalid arguments");
        return MCBGPU_E_ARG;
    }
    if (count == 0) return MCBGPU_OK;
    for (int32_t i = 0; i < count; i++)
        if (roots[i] >= (uint32_t)t->n) {
            set_error("mcbgpu_trees_run: root %d is vertex %u of %d", (int)i, roots[i], (int)t->n);
            return MCBGPU_E_ARG;
        }
    cudaStream_t st = (cudaStream_t)stream;
    MCB_CUDA(cudaMemcpyAsync(t->d_roots, roots, 4 * (size_t)count, cudaMemcpyHostToDevice, st));
    MCB_CUDA(cudaMemsetAsync(t->d_next, 0, 4, st));
    MCB_CUDA(cudaMemsetAsync(t->d_status, 0, 4, st));
    TreeArgs a;
    a.ro = t->d_ro;
    a.cols = t->d_cols;
    a.w = t->d_w;
    a.rev = t->d_rev;
    a.n = t->n;
    a.delta = t->delta;
    a.roots = t->d_roots;
    a.count = count;
    a.dist_out = t->d_dist;
    a.pedge_out = t->d_pedge;
    a.tied_out = t->d_tied;
    a.gdist = t->d_gdist;
    a.gdirty = t->d_gdirty;
    a.next_root = t->d_next;
    a.status = t->d_status;
    const int grid = count < t->sm_count ? count : t->sm_count;
    if (t->shared_form)
        trees_kernel<true><<<grid, kTreeThreads, t->smem, st>>>(a);
    else
        trees_kernel<false><<<grid, kTreeThreads, 0, st>>>(a);
    MCB_CUDA(cudaGetLastError());
    const size_t cells = (size_t)count * (size_t)t->n;
    MCB_CUDA(cudaMemcpyAsync(dist, t->d_dist, 4 * cells, cudaMemcpyDeviceToHost, st));
    MCB_CUDA(cudaMemcpyAsync(parent_slot, t->d_pedge, 4 * cells, cudaMemcpyDeviceToHost, st));
    MCB_CUDA(cudaMemcpyAsync(tied, t->d_tied, (size_t)count, cudaMemcpyDeviceToHost, st));
    unsigned status = 0;
    MCB_CUDA(cudaMemcpyAsync(&status, t->d_status, 4, cudaMemcpyDeviceToHost, st));
    MCB_CUDA(cudaStreamSynchronize(st));
    // a root that did not converge carries its tie flag (the host searches it itself)
    // and is counted; any other bit is an error
    if (status & ST_DIVERGED) t->diverged_runs++;
    if (status & ~(unsigned)ST_DIVERGED) {
        set_error("mcbgpu_trees_run: kernel status 0x%x", status);
        return MCBGPU_E_DEVICE;
    }
    return MCBGPU_OK;
}

int64_t mcbgpu_trees_device_bytes(const mcbgpu_trees *t) { return t ? t->bytes : 0; }

int mcbgpu_trees_destroy(mcbgpu_trees *t) {
    if (t) trees_free(t);
    return MCBGPU_OK;
}

}  // extern "C"
