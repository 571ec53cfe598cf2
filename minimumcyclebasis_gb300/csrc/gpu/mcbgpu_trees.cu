// Shortest-path trees of many roots of one graph (the host's per-root tree searches,
// include/Dijkstra.h:78-124, as one persistent launch), for a host tree supplier:
// the kernel (mcbgpu_sssp.cuh) runs on a chunk of roots and the distances, parent
// slots and tie flags are copied back to the host.
#include <climits>
#include <vector>

#include "mcbgpu_sssp.cuh"

using namespace mcbgpu;
using namespace mcbgpu::sssp;

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
    uint32_t *d_gdirty = nullptr, *d_gsumm = nullptr;
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
    cudaFree(t->d_gsumm);
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
    if (nodes > kTreeGlobalMaxN) {
        set_error("mcbgpu_trees_create: %d vertices after chain contraction (at most %d)", (int)nodes, kTreeGlobalMaxN);
        return MCBGPU_E_ARG;
    }
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
    if (path_length_bound(nodes, slots, weights, rev) + wmax >= (long long)INT_MAX) {
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
    t->smem = t->shared_form ? trees_smem_bytes(nodes) : 0;
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
        TALLOC(t->d_gdist, 4 * per_root * (size_t)t->sm_count * kTreeMaxCtasPerSm);
        TALLOC(t->d_gdirty, 4 * (size_t)words * (size_t)t->sm_count * kTreeMaxCtasPerSm);
        TALLOC(t->d_gsumm, 4 * (size_t)((words + 31) / 32) * (size_t)t->sm_count * kTreeMaxCtasPerSm);
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
    if (e == cudaSuccess) e = set_trees_smem_limit();
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
    const TreeShape shape = t->shared_form ? TreeShape{kTreeThreads, 1, 4} : TreeShape{256, 8, 16};
    a.delta = shape_delta(shape, t->delta);
    a.roots = t->d_roots;
    a.count = count;
    a.dist_out = t->d_dist;
    a.pedge_out = t->d_pedge;
    a.tied_out = t->d_tied;
    a.gdist = t->d_gdist;
    a.gdirty = t->d_gdirty;
    a.gsumm = t->d_gsumm;
    a.next_root = t->d_next;
    a.status = t->d_status;
    const int slots_ = t->sm_count * shape.ctas_per_sm;
    const int grid = count < slots_ ? count : slots_;
    MCB_CUDA(launch_trees(t->shared_form, shape, grid, t->smem, st, a));
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
