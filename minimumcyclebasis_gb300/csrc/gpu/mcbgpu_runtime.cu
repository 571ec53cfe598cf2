// Runtime helpers of libmcbgpu.so: error strings and the reference's GPU-layer
// free functions (gpu/common.cu:1-67, declared in gpu/common.cuh:18-27).
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <vector>

#include "mcbgpu_internal.cuh"

namespace mcbgpu {

static thread_local char g_msg[512] = "";

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_msg, sizeof g_msg, fmt, ap);
    va_end(ap);
}

int cuda_fail(cudaError_t e, const char *what) {
    set_error("%s: %s", what, cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? MCBGPU_E_NOMEM : MCBGPU_E_CUDA;
}

long long path_length_bound(int32_t nodes, int64_t slots, const int32_t *weights, const uint32_t *rev) {
    std::vector<long long> w;
    w.reserve((size_t)(slots / 2));
    for (int64_t o = 0; o < slots; o++)
        if ((uint64_t)o < rev[o]) w.push_back(weights[o]);
    const size_t keep = std::min(w.size(), (size_t)(nodes > 1 ? nodes - 1 : 0));
    std::nth_element(w.begin(), w.begin() + keep, w.end(), std::greater<long long>());
    long long s = 0;
    for (size_t i = 0; i < keep; i++) s += w[i];
    return s;
}

// State kept by the reference's globals prop / device_id / dimGrid / dimBlock
// (gpu/common.cu:4-7).
static cudaDeviceProp g_prop;
static int g_device = -1;

// The reference's CudaError macro: print, reset the device, exit (include/utils.h:36-47).
static void die_on(cudaError_t e, const char *what, int line) {
    if (e != cudaSuccess) {
        fprintf(stderr, "Error :%s : %s : line No = %d\n", cudaGetErrorString(e), what, line);
        cudaDeviceReset();
        exit((int)e);
    }
}

}  // namespace mcbgpu

using namespace mcbgpu;

extern "C" {

const char *mcbgpu_last_error(void) { return g_msg; }
int mcbgpu_version(void) { return 1; }

int mcbgpu_init_cuda(int *device, int *sm_count, size_t *total_global_mem) {
    int d = 0;
    MCB_CUDA(cudaGetDevice(&d));
    MCB_CUDA(cudaGetDeviceProperties(&g_prop, d));
    g_device = d;
    if (device) *device = d;
    if (sm_count) *sm_count = g_prop.multiProcessorCount;
    if (total_global_mem) *total_global_mem = g_prop.totalGlobalMem;
    return MCBGPU_OK;
}

void init_cuda(void) {
    die_on(cudaGetDevice(&g_device), "cudaGetDevice", __LINE__);
    die_on(cudaGetDeviceProperties(&g_prop, g_device), "cudaGetDeviceProperties", __LINE__);
}

size_t configure_grid(int start, int end) {
    // grid = number of SMs, block = max threads per block; the reference keeps
    // these in globals that its kernels never read (gpu/common.cu:14-30).
    size_t grid = (size_t)g_prop.multiProcessorCount;
    size_t span = (size_t)(end - start);
    return span < grid ? span : grid;
}

unsigned *allocate_pinned_memory(int chunk, int nodes) {
    unsigned *p = nullptr;
    die_on(cudaMallocHost((void **)&p, sizeof(unsigned) * (size_t)chunk * (size_t)nodes), "cudaMallocHost",
           __LINE__);
    return p;
}

void free_pinned_memory(unsigned *p) { die_on(cudaFreeHost(p), "cudaFreeHost", __LINE__); }

size_t calculate_chunk_size(size_t num_nodes, size_t num_edges, size_t size_vector, size_t nstream) {
    // gpu/common.cu:48-67: bytes left after the map (4 B per edge slot) and S
    // (8 B per word), in 4-byte elements, divided over nstream chunks of
    // (4 arrays x n + 1) elements per tree.
    size_t global_bytes = g_prop.totalGlobalMem;
    size_t static_bytes = 4 * num_edges + 8 * size_vector;
    size_t remaining = global_bytes > static_bytes ? global_bytes - static_bytes : 0;
    size_t elems = remaining / 4;
    size_t denom = nstream * (num_nodes * 4 + 1);
    return denom ? elems / denom : 0;
}

int mcbgpu_allocate_pinned(size_t bytes, void **out) {
    if (!out) {
        set_error("mcbgpu_allocate_pinned: out is NULL");
        return MCBGPU_E_ARG;
    }
    *out = nullptr;
    MCB_CUDA(cudaMallocHost(out, bytes ? bytes : 1));
    return MCBGPU_OK;
}

int mcbgpu_free_pinned(void *ptr) {
    if (ptr) MCB_CUDA(cudaFreeHost(ptr));
    return MCBGPU_OK;
}

}  // extern "C"
