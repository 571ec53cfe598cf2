// gpu_struct drop-in: the per-tree label pass of the reference GPU path.
//
// The reference computes labels in two kernels per chunk of 720 trees:
//   __kernel_init_edge (gpu/kernel_init_edges.cu:33-75): label[i] = bit of S at the
//     coordinate of the tree edge into position i (0 for initial-spanning-tree edges
//     and for the root), one CTA per tree;
//   __kernel_multi_search_shuffle_based (gpu/kernel_multi_search.cu:63-108): level by
//     level, label[i] ^= label[parent(i)], one warp per tree;
// and copies every label back to the host per iteration (gpu_struct.cu:158-193).
//
// Here both passes are one kernel, one CTA per tree: S is staged once into shared
// memory by a TMA bulk copy, the tree's labels live in shared memory as bytes while
// the levels are swept (positions of a level are contiguous, so the edge-offset and
// parent-position reads are coalesced), and the finished labels are written out as
// the reference's uint32 0/1 array.  All trees stay resident in HBM.
#include <cstdio>
#include <mutex>
#include <vector>

#include "mcbgpu_internal.cuh"

using namespace mcbgpu;

namespace {

constexpr int kLabelThreads = 512;
constexpr size_t kMaxSmem = 200 * 1024;

// Labels of one tree (blockIdx.x = tree index).
//   level_off: F x (n+1) level offsets; parent_pos: F x n; edge_off: F x n
//   map: num_edges coordinates (-1 for spanning-tree edges)
//   S: support vector (words, even-padded); labels_out: F x n uint32
// If lab_global != nullptr the byte labels live there (trees too large for smem).
__global__ void __launch_bounds__(kLabelThreads) label_forest_kernel(
    const uint32_t *__restrict__ level_off, const uint32_t *__restrict__ parent_pos,
    const int32_t *__restrict__ edge_off, const int32_t *__restrict__ map, int num_edges,
    const uint64_t *__restrict__ S, int words_even, int num_coords, int n, uint32_t *__restrict__ labels_out,
    uint8_t *lab_global, int s_in_smem, unsigned *status) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ uint64_t bar;
    const int t = blockIdx.x;
    uint64_t *s_S = reinterpret_cast<uint64_t *>(smem);
    uint8_t *lab = lab_global ? lab_global + (size_t)t * n
                              : smem + (s_in_smem ? (size_t)words_even * 8 : 0);
    const uint64_t *Sv = S;
    if (s_in_smem) {
        if (!stage_words_tma(s_S, S, (uint32_t)words_even, &bar)) {
            if (threadIdx.x == 0) atomicOr(status, ST_WAIT_TIMEOUT);
            return;
        }
        Sv = s_S;
    }
    const uint32_t *R = level_off + (size_t)t * (n + 1);
    const uint32_t *Cp = parent_pos + (size_t)t * n;
    const int32_t *E = edge_off + (size_t)t * n;
    // level 0: the root (edge offset -1 -> label 0)
    if (threadIdx.x == 0) lab[0] = 0;
    cta_sync();
    uint32_t covered = 1;  // positions [0, covered) have their labels
    for (int k = 1; k < n; k++) {
        uint32_t beg = R[k], end = R[k + 1];
        if (beg >= end || end > (uint32_t)n) break;
        covered = end;
        for (uint32_t i = beg + threadIdx.x; i < end; i += blockDim.x) {
            int eo = E[i];
            uint32_t bit = 0;
            if (eo >= 0 && eo < num_edges) {
                int c = map[eo];
                if (c >= 0 && c < num_coords) bit = (uint32_t)(Sv[c >> 6] >> (c & 63)) & 1u;
            }
            uint32_t p = Cp[i];
            uint8_t pl = 0;
            if (p < i)
                pl = lab[p];
            else
                atomicOr(status, ST_BAD_INPUT);  // parent positions precede children
            lab[i] = (uint8_t)(bit ^ pl);
        }
        cta_sync();
    }
    // every position of a tree of a connected graph is on some level; a layout whose
    // levels end early is flagged, and its unreached positions read 0
    if (covered < (uint32_t)n && threadIdx.x == 0) atomicOr(status, ST_BAD_INPUT);
    uint32_t *out = labels_out + (size_t)t * n;
    for (int i = threadIdx.x; i < n; i += blockDim.x) out[i] = (uint32_t)i < covered ? lab[i] : 0u;
}

}  // namespace

struct mcbgpu_struct {
    int num_edges = 0, num_coords = 0, size_vector = 0, n = 0, F = 0, chunk = 0, rows = 0;
    int words_even = 0;
    int32_t *d_map = nullptr, *d_edge = nullptr;
    uint32_t *d_levels = nullptr, *d_parent = nullptr, *d_labels = nullptr;
    uint8_t *d_lab_bytes = nullptr;
    uint64_t *d_S = nullptr;
    unsigned *d_status = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    bool initialized = false;
};

static void free_struct(mcbgpu_struct *s) {
    if (!s) return;
    cudaFree(s->d_map);
    cudaFree(s->d_edge);
    cudaFree(s->d_levels);
    cudaFree(s->d_parent);
    cudaFree(s->d_labels);
    cudaFree(s->d_lab_bytes);
    cudaFree(s->d_S);
    cudaFree(s->d_status);
    if (s->stream) cudaStreamDestroy(s->stream);
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
    delete s;
}

extern "C" {

int mcbgpu_struct_create(mcbgpu_struct **out, int num_edges, int num_non_tree_edges, int size_vector,
                         int original_nodes, int fvs_size, int chunk_size, int nstreams) {
    (void)nstreams;
    if (!out || num_edges <= 0 || num_non_tree_edges < 0 || original_nodes <= 0 || fvs_size < 0 ||
        chunk_size <= 0 || size_vector != (num_non_tree_edges + 63) / 64) {
        set_error("mcbgpu_struct_create: invalid sizes");
        return MCBGPU_E_ARG;
    }
    *out = nullptr;
    mcbgpu_struct *s = new mcbgpu_struct();
    s->num_edges = num_edges;
    s->num_coords = num_non_tree_edges;
    s->size_vector = size_vector;
    s->n = original_nodes;
    s->F = fvs_size;
    s->chunk = chunk_size;
    s->rows = (fvs_size + chunk_size - 1) / chunk_size;
    s->words_even = (size_vector + 1) & ~1;
    if (s->words_even == 0) s->words_even = 2;
    const size_t Fn = (size_t)fvs_size * original_nodes;
    cudaError_t e = cudaSuccess;
#define ALLOC(ptr, bytes)                                              \
    do {                                                               \
        size_t _b = (size_t)(bytes);                                   \
        if (_b == 0) _b = 16;                                          \
        if (e == cudaSuccess) e = cudaMalloc((void **)&(ptr), _b);     \
    } while (0)
    ALLOC(s->d_map, sizeof(int32_t) * (size_t)num_edges);
    ALLOC(s->d_edge, sizeof(int32_t) * Fn);
    ALLOC(s->d_parent, sizeof(uint32_t) * Fn);
    ALLOC(s->d_levels, sizeof(uint32_t) * (size_t)fvs_size * (original_nodes + 1));
    ALLOC(s->d_labels, sizeof(uint32_t) * Fn);
    ALLOC(s->d_S, sizeof(uint64_t) * (size_t)s->words_even);
    ALLOC(s->d_status, sizeof(unsigned));
#undef ALLOC
    if (e == cudaSuccess) e = cudaMemset(s->d_S, 0, sizeof(uint64_t) * (size_t)s->words_even);
    if (e == cudaSuccess) e = cudaMemset(s->d_status, 0, sizeof(unsigned));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&s->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&s->ev1);
    if (e != cudaSuccess) {
        free_struct(s);
        return cuda_fail(e, "mcbgpu_struct_create");
    }
    *out = s;
    return MCBGPU_OK;
}

int mcbgpu_struct_initialize_memory(mcbgpu_struct *s, const int32_t *map, const int32_t *const *edge_offset_rows,
                                    const uint32_t *const *tree_rows_rows, const uint32_t *const *tree_cols_rows) {
    if (!s || !map || !edge_offset_rows || !tree_rows_rows || !tree_cols_rows) {
        set_error("mcbgpu_struct_initialize_memory: NULL argument");
        return MCBGPU_E_ARG;
    }
    const size_t n = (size_t)s->n;
    MCB_CUDA(cudaMemcpyAsync(s->d_map, map, sizeof(int32_t) * (size_t)s->num_edges, cudaMemcpyHostToDevice,
                             s->stream));
    for (int r = 0; r < s->rows; r++) {
        size_t t0 = (size_t)r * s->chunk;
        size_t cnt = (size_t)s->F - t0 < (size_t)s->chunk ? (size_t)s->F - t0 : (size_t)s->chunk;
        if (!edge_offset_rows[r] || !tree_rows_rows[r] || !tree_cols_rows[r]) {
            set_error("mcbgpu_struct_initialize_memory: NULL row %d", r);
            return MCBGPU_E_ARG;
        }
        MCB_CUDA(cudaMemcpyAsync(s->d_edge + t0 * n, edge_offset_rows[r], sizeof(int32_t) * cnt * n,
                                 cudaMemcpyHostToDevice, s->stream));
        MCB_CUDA(cudaMemcpyAsync(s->d_parent + t0 * n, tree_cols_rows[r], sizeof(uint32_t) * cnt * n,
                                 cudaMemcpyHostToDevice, s->stream));
        MCB_CUDA(cudaMemcpyAsync(s->d_levels + t0 * (n + 1), tree_rows_rows[r], sizeof(uint32_t) * cnt * (n + 1),
                                 cudaMemcpyHostToDevice, s->stream));
    }
    MCB_CUDA(cudaStreamSynchronize(s->stream));
    s->initialized = true;
    return MCBGPU_OK;
}

int mcbgpu_struct_copy_support_vector(mcbgpu_struct *s, const uint64_t *S, float *ms) {
    if (!s || !S) {
        set_error("mcbgpu_struct_copy_support_vector: NULL argument");
        return MCBGPU_E_ARG;
    }
    MCB_CUDA(cudaEventRecord(s->ev0, s->stream));
    MCB_CUDA(cudaMemcpyAsync(s->d_S, S, sizeof(uint64_t) * (size_t)s->size_vector, cudaMemcpyHostToDevice,
                             s->stream));
    MCB_CUDA(cudaEventRecord(s->ev1, s->stream));
    MCB_CUDA(cudaEventSynchronize(s->ev1));
    if (ms) MCB_CUDA(cudaEventElapsedTime(ms, s->ev0, s->ev1));
    return MCBGPU_OK;
}

int mcbgpu_struct_process_shortest_path(mcbgpu_struct *s, uint32_t *const *precompute_rows, int multiple_transfer,
                                        float *ms) {
    (void)multiple_transfer;
    if (!s) {
        set_error("mcbgpu_struct_process_shortest_path: NULL handle");
        return MCBGPU_E_ARG;
    }
    if (!s->initialized) {
        set_error("mcbgpu_struct_process_shortest_path: initialize_memory not called");
        return MCBGPU_E_STATE;
    }
    const size_t n = (size_t)s->n;
    MCB_CUDA(cudaEventRecord(s->ev0, s->stream));
    if (s->F > 0) {
        size_t s_bytes = (size_t)s->words_even * 8;
        int s_in_smem = s_bytes <= 96 * 1024;
        size_t smem = (s_in_smem ? s_bytes : 0) + ((n + 15) & ~(size_t)15);
        uint8_t *lab_global = nullptr;
        if (smem > kMaxSmem) {
            smem = s_in_smem ? s_bytes : 0;
            if (!s->d_lab_bytes) MCB_CUDA(cudaMalloc((void **)&s->d_lab_bytes, (size_t)s->F * n));
            lab_global = s->d_lab_bytes;
        }
        MCB_CUDA(cudaFuncSetAttribute(label_forest_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)(smem < 48 * 1024 ? 48 * 1024 : smem)));
        label_forest_kernel<<<s->F, kLabelThreads, smem, s->stream>>>(
            s->d_levels, s->d_parent, s->d_edge, s->d_map, s->num_edges, s->d_S, s->words_even, s->num_coords,
            s->n, s->d_labels, lab_global, s_in_smem, s->d_status);
        MCB_CUDA(cudaGetLastError());
    }
    if (precompute_rows) {
        for (int r = 0; r < s->rows; r++) {
            size_t t0 = (size_t)r * s->chunk;
            size_t cnt = (size_t)s->F - t0 < (size_t)s->chunk ? (size_t)s->F - t0 : (size_t)s->chunk;
            if (!precompute_rows[r]) continue;
            MCB_CUDA(cudaMemcpyAsync(precompute_rows[r], s->d_labels + t0 * n, sizeof(uint32_t) * cnt * n,
                                     cudaMemcpyDeviceToHost, s->stream));
        }
    }
    MCB_CUDA(cudaEventRecord(s->ev1, s->stream));
    MCB_CUDA(cudaEventSynchronize(s->ev1));
    if (ms) MCB_CUDA(cudaEventElapsedTime(ms, s->ev0, s->ev1));
    unsigned st = 0;
    MCB_CUDA(cudaMemcpy(&st, s->d_status, sizeof st, cudaMemcpyDeviceToHost));
    if (st) {
        set_error("label kernel status 0x%x", st);
        cudaMemset(s->d_status, 0, sizeof(unsigned));
        return MCBGPU_E_DEVICE;
    }
    return MCBGPU_OK;
}

int mcbgpu_struct_clear_memory(mcbgpu_struct *s) {
    if (!s) return MCBGPU_OK;
    cudaError_t e = cudaStreamSynchronize(s->stream);
    free_struct(s);
    if (e != cudaSuccess) return cuda_fail(e, "mcbgpu_struct_clear_memory");
    return MCBGPU_OK;
}

}  // extern "C"

// ===========================================================================
// Allocation-free label pass.
//
// Some callers cannot allocate device memory: code that runs inside a host
// framework which owns every byte of device memory through its own pool and does
// not let plugins call cudaMalloc, and latency-critical loops that must not take the
// device-wide synchronisation that cudaMalloc / cudaFree can imply.  For them,
// mcbgpu_label_forest_noalloc computes the same labels as
// mcbgpu_struct_process_shortest_path from buffers the caller already owns, and
// keeps its working memory in the file-scope array below, which is part of the
// library image: every GPU that loads libmcbgpu.so holds it until the process exits.
//
// Layout of the array: a 256-byte header whose first word is the kernel's status,
// then kNoAllocSlabBytes of label slabs, one slab of `nodes` bytes per CTA.
namespace {

constexpr size_t kNoAllocHeaderBytes = 256;
constexpr size_t kNoAllocSlabBytes = (size_t)16 << 20;  // 16 MiB
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocHeaderBytes + kNoAllocSlabBytes];

std::mutex g_noalloc_mutex;
unsigned char *g_noalloc_addr[kNoAllocMaxDevices] = {nullptr};

// Same level sweep as label_forest_kernel; the byte labels of the tree being swept
// live in this CTA's slab of the static scratch, S is read from global memory, and
// each CTA walks trees blockIdx.x, blockIdx.x + gridDim.x, ...
__global__ void __launch_bounds__(kLabelThreads) label_forest_noalloc_kernel(
    const uint32_t *__restrict__ level_off, const uint32_t *__restrict__ parent_pos,
    const int32_t *__restrict__ edge_off, const int32_t *__restrict__ map, int num_edges,
    const uint64_t *__restrict__ S, int num_coords, int n, int F, uint32_t *__restrict__ labels_out,
    uint8_t *slabs, unsigned *status) {
    uint8_t *lab = slabs + (size_t)blockIdx.x * n;
    for (int t = blockIdx.x; t < F; t += gridDim.x) {
        const uint32_t *R = level_off + (size_t)t * (n + 1);
        const uint32_t *Cp = parent_pos + (size_t)t * n;
        const int32_t *E = edge_off + (size_t)t * n;
        if (threadIdx.x == 0) lab[0] = 0;
        cta_sync();
        uint32_t covered = 1;  // positions [0, covered) have this tree's labels
        for (int k = 1; k < n; k++) {
            const uint32_t beg = R[k], end = R[k + 1];
            if (beg >= end || end > (uint32_t)n) break;
            covered = end;
            for (uint32_t i = beg + threadIdx.x; i < end; i += blockDim.x) {
                const int eo = E[i];
                uint32_t bit = 0;
                if (eo >= 0 && eo < num_edges) {
                    const int c = map[eo];
                    if (c >= 0 && c < num_coords) bit = (uint32_t)(S[c >> 6] >> (c & 63)) & 1u;
                }
                const uint32_t p = Cp[i];
                uint8_t pl = 0;
                if (p < i)
                    pl = lab[p];
                else
                    atomicOr(status, ST_BAD_INPUT);
                lab[i] = (uint8_t)(bit ^ pl);
            }
            cta_sync();
        }
        // the slab keeps the previous tree's labels beyond `covered`: a layout whose
        // levels end before position n is flagged, and those positions read 0
        if (covered < (uint32_t)n && threadIdx.x == 0) atomicOr(status, ST_BAD_INPUT);
        uint32_t *out = labels_out + (size_t)t * n;
        for (int i = threadIdx.x; i < n; i += blockDim.x) out[i] = (uint32_t)i < covered ? lab[i] : 0u;
        cta_sync();
    }
}

}  // namespace

extern "C" int mcbgpu_label_forest_noalloc(const uint32_t *level_offsets, const uint32_t *parent_pos,
                                           const int32_t *edge_offset, const int32_t *non_tree_edges_map,
                                           int num_edges, const uint64_t *support_vector, int num_coords,
                                           int fvs_size, int nodes, uint32_t *labels, void *stream) {
    if (!level_offsets || !parent_pos || !edge_offset || !non_tree_edges_map || !support_vector || !labels ||
        num_edges <= 0 || num_coords < 0 || fvs_size < 0 || nodes <= 0) {
        set_error("mcbgpu_label_forest_noalloc: invalid argument");
        return MCBGPU_E_ARG;
    }
    if ((size_t)nodes > kNoAllocSlabBytes) {
        set_error("mcbgpu_label_forest_noalloc: a tree of %d vertices needs more than the %zu-byte static scratch",
                  nodes, kNoAllocSlabBytes);
        return MCBGPU_E_ARG;
    }
    int dev = 0;
    MCB_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoAllocMaxDevices) {
        set_error("mcbgpu_label_forest_noalloc: device %d out of range", dev);
        return MCBGPU_E_ARG;
    }
    unsigned char *base = nullptr;
    {
        // once per device, with that device current: the device address of the array
        std::lock_guard<std::mutex> lock(g_noalloc_mutex);
        if (!g_noalloc_addr[dev]) {
            void *p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
            g_noalloc_addr[dev] = (unsigned char *)p;
        }
        base = g_noalloc_addr[dev];
    }
    cudaStream_t st = (cudaStream_t)stream;
    unsigned *status = reinterpret_cast<unsigned *>(base);
    uint8_t *slabs = base + kNoAllocHeaderBytes;
    MCB_CUDA(cudaMemsetAsync(status, 0, sizeof(unsigned), st));
    if (fvs_size > 0) {
        int sms = 0;
        MCB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        size_t grid = (size_t)(sms > 0 ? sms : 1) * 2;
        const size_t fit = kNoAllocSlabBytes / (size_t)nodes;
        if (grid > fit) grid = fit;
        if (grid > (size_t)fvs_size) grid = (size_t)fvs_size;
        label_forest_noalloc_kernel<<<(unsigned)grid, kLabelThreads, 0, st>>>(
            level_offsets, parent_pos, edge_offset, non_tree_edges_map, num_edges, support_vector, num_coords,
            nodes, fvs_size, labels, slabs, status);
        MCB_CUDA(cudaGetLastError());
    }
    unsigned h = 0;
    MCB_CUDA(cudaMemcpyAsync(&h, status, sizeof h, cudaMemcpyDeviceToHost, st));
    MCB_CUDA(cudaStreamSynchronize(st));
    if (h) {
        set_error("mcbgpu_label_forest_noalloc: kernel status 0x%x", h);
        return MCBGPU_E_DEVICE;
    }
    return MCBGPU_OK;
}
