// Shared helpers of libmcbgpu.so: error plumbing, the 1-D TMA bulk copy into
// shared memory with a bounded mbarrier wait, and device status bits.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>

#include "mcbgpu.h"

namespace mcbgpu {

// Device status word bits (written by kernels, read by the host after a run).
enum : unsigned {
    ST_WAIT_TIMEOUT = 1u << 0,     // a bounded spin on a flag or mbarrier gave up
    ST_NO_CANDIDATE = 1u << 1,     // the search found no odd candidate
    ST_RANK_DEFICIT = 1u << 2,     // blocked search ran out of candidates before b pivots
    ST_BAD_INPUT = 1u << 3,        // an index outside its array was seen and skipped
    ST_DIVERGED = 1u << 4,         // CTAs of a cooperative kernel disagreed on a shared result
};

void set_error(const char *fmt, ...);

// An upper bound on every shortest-path distance of a graph with positive weights
// (slot o < rev[o] is one undirected edge): a shortest path is simple, so at most
// nodes - 1 edges; the sum of the nodes - 1 heaviest edges.
long long path_length_bound(int32_t nodes, int64_t slots, const int32_t *weights, const uint32_t *rev);
int cuda_fail(cudaError_t e, const char *what);

#define MCB_CUDA(call)                                              \
    do {                                                            \
        cudaError_t _e = (call);                                    \
        if (_e != cudaSuccess) return ::mcbgpu::cuda_fail(_e, #call); \
    } while (0)

// ---- PTX wrappers -----------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Orders this thread's generic global writes before later bulk copies (async
// proxy) that read the same global memory.
__device__ __forceinline__ void fence_proxy_async_global() {
    asm volatile("fence.proxy.async.global;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

// 1-D bulk copy global -> shared (TMA engine), completion counted on `bar`.
// dst, src and bytes must be multiples of 16.
__device__ __forceinline__ void tma_load_1d(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t phase) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(phase)
        : "memory");
    return ok != 0;
}

// Bounded wait: returns false (and the caller must flag an error) after `limit`
// polls.  try_wait itself suspends for a hardware-chosen interval per poll.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t phase, uint32_t limit) {
    for (uint32_t i = 0; i < limit; i++)
        if (mbar_try_wait(bar, phase)) return true;
    return false;
}

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release_u32(unsigned *p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ int parity64(uint64_t x) { return __popcll(x) & 1; }

// Bulk prefetch of [p, p + bytes) into L2, shrunk to the 16-byte aligned span inside
// it (nothing outside the range is touched).
__device__ __forceinline__ void prefetch_l2(const void *p, unsigned long long bytes) {
    const unsigned long long a = ((unsigned long long)p + 15ull) & ~15ull;
    const unsigned long long e = ((unsigned long long)p + bytes) & ~15ull;
    if (e <= a) return;
    unsigned long long n = e - a;
    if (n > (1ull << 20)) n = 1ull << 20;
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(a), "r"((unsigned)n) : "memory");
}

// XOR of a 64-bit value over the full warp (two warp-reduce instructions).
__device__ __forceinline__ uint64_t warp_xor64(uint64_t v) {
    const unsigned lo = __reduce_xor_sync(0xffffffffu, (unsigned)v);
    const unsigned hi = __reduce_xor_sync(0xffffffffu, (unsigned)(v >> 32));
    return ((uint64_t)hi << 32) | lo;
}

// CTA barriers in the non-aligned form (`barrier.sync`, not the `.aligned` form
// that __syncthreads() emits).  The aligned form lets the hardware assume that
// every warp arrives converged; after lane-divergent loops (per-candidate
// coordinate walks with early exits, per-thread mbarrier polls) a warp can arrive
// in pieces, and on sm_103a an aligned barrier was observed to release while one
// warp of the CTA was still short of it.  The non-aligned form counts threads, so
// a barrier completes only when every thread of the CTA has reached it.  Every
// kernel of this library uses these instead of __syncthreads().
__device__ __forceinline__ void cta_sync() { asm volatile("barrier.sync 0;" ::: "memory"); }

// Programmatic dependent launch.  A kernel launched with the programmatic
// stream-serialisation attribute may be scheduled while its predecessor in the stream
// is still running: griddep_wait() blocks until that predecessor has completed and its
// memory operations are visible (it returns at once for a kernel launched without the
// attribute), and griddep_launch() lets the successor be scheduled once every CTA of
// this kernel has issued it.  A kernel that waits first thing reads nothing of its
// predecessor early, so only the launch latency overlaps.
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void griddep_launch() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// 64 x 64 bit transpose across a warp: lane l holds rows l (r0) and l + 32 (r1), bit j
// of a row being column j; afterwards r0 = column l and r1 = column l + 32 (bit i =
// row i).  The 32 x 32 blocks off the diagonal are swapped in each lane, then both
// halves of the words are transposed as two 32 x 32 matrices at once by the
// recursive block swap (blocks of 16, 8, 4, 2, 1: rows r and r + j exchange with one
// shuffle), five shuffles per word instead of 64 ballots.
__device__ __forceinline__ void warp_transpose64(uint64_t &r0, uint64_t &r1) {
    const int lane = threadIdx.x & 31;
    uint64_t u0 = (r0 & 0x00000000FFFFFFFFull) | (r1 << 32);
    uint64_t u1 = (r0 >> 32) | (r1 & 0xFFFFFFFF00000000ull);
    const uint64_t masks[5] = {0x0000FFFF0000FFFFull, 0x00FF00FF00FF00FFull, 0x0F0F0F0F0F0F0F0Full,
                               0x3333333333333333ull, 0x5555555555555555ull};
#pragma unroll
    for (int s = 0; s < 5; s++) {
        const int j = 16 >> s;
        const uint64_t m = masks[s];
        const uint64_t p0 = __shfl_xor_sync(0xffffffffu, u0, j);
        const uint64_t p1 = __shfl_xor_sync(0xffffffffu, u1, j);
        if ((lane & j) == 0) {
            u0 ^= (((u0 >> j) ^ p0) & m) << j;
            u1 ^= (((u1 >> j) ^ p1) & m) << j;
        } else {
            u0 ^= ((p0 >> j) ^ u0) & m;
            u1 ^= ((p1 >> j) ^ u1) & m;
        }
    }
    r0 = u0;
    r1 = u1;
}

// cta_sync that also returns whether `v` holds in every thread of the CTA.
__device__ __forceinline__ bool cta_sync_and(bool v) {
    unsigned r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "barrier.red.and.pred q, 0, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"(v ? 1u : 0u)
        : "memory");
    return r != 0;
}

// Stage `words_even` u64 words of global memory (16-byte aligned, an even count)
// into shared memory with TMA bulk copies of at most 32 KB each.  Called once per
// kernel by the whole CTA (mbarrier phase 0); every thread waits on the mbarrier
// with a bounded poll.  Returns false in every thread if the wait timed out; in that
// case thread 0 has waited a second bounded interval for the copies in flight.
__device__ __forceinline__ bool stage_words_tma(uint64_t *dst_smem, const uint64_t *src, uint32_t words_even,
                                               uint64_t *bar) {
    const uint32_t bytes = words_even * 8u;
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
        fence_proxy_async_smem();
    }
    cta_sync();
    if (threadIdx.x == 0) {
        mbar_arrive_expect_tx(bar, bytes);
        const uint32_t CH = 32768;
        for (uint32_t off = 0; off < bytes; off += CH) {
            uint32_t n = bytes - off < CH ? bytes - off : CH;
            tma_load_1d((char *)dst_smem + off, (const char *)src + off, n, bar);
        }
    }
    bool ok = mbar_wait_bounded(bar, 0, 1u << 22);
    if (!ok && threadIdx.x == 0) mbar_wait_bounded(bar, 0, 1u << 22);
    return cta_sync_and(ok);
}

}  // namespace mcbgpu
