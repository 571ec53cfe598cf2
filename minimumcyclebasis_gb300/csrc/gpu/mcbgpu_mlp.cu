// The learned proposal's network: a two-layer perceptron over per-candidate
// features, with its inference and training on the device.
//
//   h     = relu(W1 x + b1)        x: 16 features (bf16), W1: 64 x 16 (bf16), b1: 64
//   logit = w2 . h + b2            w2: 64 (bf16-rounded), b2: scalar
//
// Master parameters are fp32 (kept with their Adam moments); the forward pass uses
// bf16 copies of W1 and w2 and accumulates in fp32.  The first layer of the forward
// pass is a tensor-core matrix product: per tile of 128 candidates, one
// tcgen05.mma (kind::f16, M = 128, N = 64, K = 16) with the feature tile and W1 in
// shared memory (no-swizzle K-major core-matrix layout) and the 128 x 64 fp32
// accumulator in tensor memory, read back with tcgen05.ld for the bias, the ReLU
// and the second layer.  The backward pass (binary cross-entropy with a positive
// weight, mean over the batch) and the Adam step run on the CUDA cores.
//
// The network orders candidates for the proposal (minimumcyclebasis_gb300.learned);
// it never decides a result: the solve that uses its proposal checks itself and
// falls back to the full candidate list.
#include <algorithm>
#include <cmath>

#include "mcbgpu_internal.cuh"

namespace mcbgpu {
namespace mlp {

constexpr int kIn = 16, kHid = 64;
constexpr int kParams = kHid * kIn + kHid + kHid + 1;  // W1, b1, w2, b2
constexpr int kTileRows = 128;
constexpr int kFwdThreads = 128;
constexpr int kBwdThreads = 256;
constexpr uint32_t kTmemCols = 64;

__device__ __forceinline__ uint16_t f32_to_bf16(float f) {
    // round to nearest even (finite inputs)
    uint32_t u = __float_as_uint(f);
    u += 0x7fffu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}
__device__ __forceinline__ float bf16_to_f32(uint16_t h) { return __uint_as_float((uint32_t)h << 16); }

// ---- tcgen05 / TMEM wrappers --------------------------------------------------
__device__ __forceinline__ void tmem_alloc(uint32_t *dst_smem, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(dst_smem)),
                 "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// D[tmem] (+)= A[smem] x B[smem]^T, bf16 inputs, fp32 accumulator; one thread issues.
__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
// Arrives on `bar` once every tcgen05.mma this thread issued has completed.
__device__ __forceinline__ void umma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
                 : "memory");
}
// 16 consecutive fp32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// Shared-memory matrix descriptor, no swizzle: start address, the byte distance
// between core matrices (8 rows x 16 bytes) adjacent along K (leading) and along
// M/N (stride), and the descriptor version bit.
__device__ __forceinline__ uint64_t smem_desc(const void *p, uint32_t lead_bytes, uint32_t stride_bytes) {
    uint64_t d = (uint64_t)((smem_addr(p) >> 4) & 0x3fffu);
    d |= (uint64_t)((lead_bytes >> 4) & 0x3fffu) << 16;
    d |= (uint64_t)((stride_bytes >> 4) & 0x3fffu) << 32;
    d |= 1ull << 46;
    return d;
}
// Instruction descriptor of kind::f16: fp32 accumulator, bf16 A and B, both K-major,
// N = 64, M = 128.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kHid >> 3) << 17) |
                            ((uint32_t)(kTileRows >> 4) << 24);

// Byte offset of element (row, k) of a rows x 16 bf16 matrix in the core-matrix
// layout: 8-row groups 256 bytes apart, the two 8-element K halves 128 bytes apart.
__device__ __forceinline__ uint32_t core_off(int row, int k) {
    return (uint32_t)((row >> 3) * 256 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}
constexpr uint32_t kLead = 128, kStride = 256;

// Forward pass over `count` candidates: logits[i], and with `hidden` the post-ReLU
// hidden layer (count x 64 fp32, for the backward pass).
__global__ void __launch_bounds__(kFwdThreads) mlp_forward_kernel(const uint16_t *__restrict__ x, int64_t count,
                                                                  const uint16_t *__restrict__ w1, const float *b1,
                                                                  const float *w2, const float *__restrict__ b2p,
                                                                  float *logits, float *hidden, unsigned *status) {
    __shared__ __align__(1024) unsigned char sA[kTileRows * kIn * 2];
    __shared__ __align__(1024) unsigned char sB[kHid * kIn * 2];
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t s_tmem;
    __shared__ float s_b1[kHid], s_w2[kHid];
    const int tid = threadIdx.x, warp = tid >> 5;
    if (warp == 0) tmem_alloc(&s_tmem, kTmemCols);
    if (tid == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    // W1 (64 x 16, row n = hidden unit) into the core-matrix layout, once
    for (int e = tid; e < kHid * kIn; e += blockDim.x) {
        const int n = e / kIn, k = e % kIn;
        *reinterpret_cast<uint16_t *>(sB + core_off(n, k)) = w1[e];
    }
    for (int j = tid; j < kHid; j += blockDim.x) {
        s_b1[j] = b1[j];
        s_w2[j] = w2[j];
    }
    tc_fence_before();
    cta_sync();
    tc_fence_after();
    if (warp == 0) tmem_relinquish();
    const uint32_t tmem = s_tmem;
    const float b2 = *b2p;
    const uint64_t bdesc = smem_desc(sB, kLead, kStride);
    const uint64_t adesc = smem_desc(sA, kLead, kStride);
    const int64_t ntiles = (count + kTileRows - 1) / kTileRows;
    uint32_t phase = 0;
    bool ok = true;
    // this thread's row of a tile: 16 bf16 = two 16-byte halves; the next tile's row
    // is loaded while the current tile is multiplied and its epilogue runs
    auto load_row = [&](int64_t t, uint4 &lo, uint4 &hi) {
        const int64_t r = t * kTileRows + tid;
        lo = make_uint4(0, 0, 0, 0);
        hi = lo;
        if (t < ntiles && r < count) {
            const uint4 *src = reinterpret_cast<const uint4 *>(x + r * kIn);
            lo = __ldg(src);
            hi = __ldg(src + 1);
        }
    };
    uint4 nlo, nhi;
    load_row(blockIdx.x, nlo, nhi);
    for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const int64_t row = tile * kTileRows + tid;
        *reinterpret_cast<uint4 *>(sA + core_off(tid, 0)) = nlo;
        *reinterpret_cast<uint4 *>(sA + core_off(tid, 8)) = nhi;
        load_row(tile + gridDim.x, nlo, nhi);
        fence_proxy_async_smem();  // generic-proxy writes -> visible to the tensor core
        tc_fence_before();
        cta_sync();
        tc_fence_after();
        if (tid == 0) {
            umma_bf16(tmem, adesc, bdesc, kIdesc, 0);
            umma_commit(&bar);
        }
        ok = mbar_wait_bounded(&bar, phase, 1u << 22);
        phase ^= 1u;
        ok = cta_sync_and(ok);
        if (!ok) break;
        tc_fence_after();
        // lane i of warp w holds row 32 w + i of the 128 x 64 accumulator
        float acc[16];
        float logit = b2;
        float *hrow = hidden && row < count ? hidden + row * kHid : nullptr;
#pragma unroll
        for (int c = 0; c < kHid / 16; c++) {
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(c * 16), acc);
#pragma unroll
            for (int i = 0; i < 16; i++) {
                const float h = fmaxf(acc[i] + s_b1[c * 16 + i], 0.0f);
                logit = fmaf(s_w2[c * 16 + i], h, logit);
                acc[i] = h;
            }
            if (hrow) {
#pragma unroll
                for (int i = 0; i < 16; i += 4)
                    *reinterpret_cast<float4 *>(hrow + c * 16 + i) = make_float4(acc[i], acc[i + 1], acc[i + 2],
                                                                                  acc[i + 3]);
            }
        }
        if (row < count) logits[row] = logit;
        tc_fence_before();
        cta_sync();  // the tile's smem and TMEM are reused by the next tile
    }
    if (!ok) {
        if (tid == 0) {
            atomicOr(status, ST_WAIT_TIMEOUT);
            mbar_wait_bounded(&bar, phase ^ 1u, 1u << 22);  // the MMA in flight, if any
        }
        cta_sync();
    }
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tmem, kTmemCols);
}

__device__ __forceinline__ float softplus(float z) { return fmaxf(z, 0.0f) + log1pf(expf(-fabsf(z))); }

// Gradients of the mean weighted binary cross-entropy over `count` candidates into
// grads (kParams floats, accumulated with atomics) and the loss sum into *loss.
// Thread (s, j) of a block: hidden unit j = tid % 64 of every 4th candidate.
__global__ void __launch_bounds__(kBwdThreads) mlp_backward_kernel(const uint16_t *__restrict__ x,
                                                                   const uint8_t *__restrict__ labels,
                                                                   const float *__restrict__ logits,
                                                                   const float *__restrict__ hidden, int64_t count,
                                                                   float pos_weight, const float *w2, float *grads,
                                                                   float *loss) {
    __shared__ float s_red[kBwdThreads / kHid][kHid][kIn + 2];
    __shared__ float s_misc[kBwdThreads / kHid][2];
    const int j = threadIdx.x % kHid, s = threadIdx.x / kHid, ns = blockDim.x / kHid;
    const float w2j = w2[j];
    const float inv = 1.0f / (float)count;
    float gw1[kIn];
#pragma unroll
    for (int i = 0; i < kIn; i++) gw1[i] = 0.0f;
    float gb1 = 0.0f, gw2 = 0.0f, gb2 = 0.0f, lsum = 0.0f;
    for (int64_t b = (int64_t)blockIdx.x * ns + s; b < count; b += (int64_t)gridDim.x * ns) {
        const float z = logits[b];
        const float y = labels[b] ? 1.0f : 0.0f;
        const float wt = labels[b] ? pos_weight : 1.0f;
        const float sg = 1.0f / (1.0f + expf(-z));
        const float dz = (sg - y) * wt * inv;
        const float h = hidden[b * kHid + j];
        gw2 = fmaf(dz, h, gw2);
        const float dh = h > 0.0f ? dz * w2j : 0.0f;
        gb1 += dh;
        const uint16_t *xb = x + b * kIn;
#pragma unroll
        for (int i = 0; i < kIn; i++) gw1[i] = fmaf(dh, bf16_to_f32(xb[i]), gw1[i]);
        if (j == 0) {
            gb2 += dz;
            lsum += wt * (labels[b] ? softplus(-z) : softplus(z));
        }
    }
    // sum over the sample lanes of each hidden unit in shared memory, then one atomic
    // per parameter and block
    for (int i = 0; i < kIn; i++) s_red[s][j][i] = gw1[i];
    s_red[s][j][kIn] = gb1;
    s_red[s][j][kIn + 1] = gw2;
    if (j == 0) {
        s_misc[s][0] = gb2;
        s_misc[s][1] = lsum;
    }
    cta_sync();
    if (s == 0) {
        for (int i = 0; i < kIn + 2; i++) {
            float v = 0.0f;
            for (int k = 0; k < ns; k++) v += s_red[k][j][i];
            const int at = i < kIn ? j * kIn + i : i == kIn ? kHid * kIn + j : kHid * kIn + kHid + j;
            atomicAdd(&grads[at], v);
        }
    }
    if (threadIdx.x == 0) {
        float a = 0, l = 0;
        for (int k = 0; k < ns; k++) {
            a += s_misc[k][0];
            l += s_misc[k][1];
        }
        atomicAdd(&grads[kParams - 1], a);
        atomicAdd(loss, l);
    }
}

// The forward pass's weight copies: bf16 W1 and bf16-rounded w2 from the masters.
__global__ void mlp_weights_kernel(const float *params, uint16_t *w1_bf16, float *w2_round) {
    for (int e = threadIdx.x; e < kHid * kIn; e += blockDim.x) w1_bf16[e] = f32_to_bf16(params[e]);
    for (int j = threadIdx.x; j < kHid; j += blockDim.x)
        w2_round[j] = bf16_to_f32(f32_to_bf16(params[kHid * kIn + kHid + j]));
}

// One Adam step on every parameter, then the gradients cleared and the bf16 copies
// refreshed.
__global__ void mlp_adam_kernel(float *params, float *grads, float *m1, float *m2, float lr, float beta1,
                                float beta2, float eps, float c1, float c2, uint16_t *w1_bf16, float *w2_round) {
    for (int e = threadIdx.x; e < kParams; e += blockDim.x) {
        const float g = grads[e];
        const float a = beta1 * m1[e] + (1.0f - beta1) * g;
        const float b = beta2 * m2[e] + (1.0f - beta2) * g * g;
        m1[e] = a;
        m2[e] = b;
        params[e] -= lr * (a / c1) / (sqrtf(b / c2) + eps);
        grads[e] = 0.0f;
    }
    cta_sync();
    for (int e = threadIdx.x; e < kHid * kIn; e += blockDim.x) w1_bf16[e] = f32_to_bf16(params[e]);
    for (int j = threadIdx.x; j < kHid; j += blockDim.x)
        w2_round[j] = bf16_to_f32(f32_to_bf16(params[kHid * kIn + kHid + j]));
}

}  // namespace mlp
}  // namespace mcbgpu

using namespace mcbgpu;
using namespace mcbgpu::mlp;

struct mcbgpu_mlp {
    float *d_params = nullptr, *d_grads = nullptr, *d_m1 = nullptr, *d_m2 = nullptr, *d_w2r = nullptr;
    uint16_t *d_w1 = nullptr;
    float *d_loss = nullptr, *d_logits = nullptr, *d_hidden = nullptr;
    unsigned *d_status = nullptr;
    int64_t cap = 0;  // rows of the training buffers
    int64_t steps = 0;
    int sm_count = 0;
};

static void mlp_free(mcbgpu_mlp *m) {
    void *ps[] = {m->d_params, m->d_grads, m->d_m1, m->d_m2, m->d_w2r, m->d_w1, m->d_loss, m->d_logits,
                  m->d_hidden, m->d_status};
    for (void *p : ps) cudaFree(p);
    delete m;
}

static int mlp_status(mcbgpu_mlp *m, cudaStream_t st, const char *what) {
    unsigned h = 0;
    MCB_CUDA(cudaMemcpyAsync(&h, m->d_status, sizeof h, cudaMemcpyDeviceToHost, st));
    MCB_CUDA(cudaStreamSynchronize(st));
    if (h) {
        MCB_CUDA(cudaMemsetAsync(m->d_status, 0, sizeof h, st));
        set_error("%s: device status 0x%x", what, h);
        return MCBGPU_E_DEVICE;
    }
    return MCBGPU_OK;
}

static int mlp_forward(mcbgpu_mlp *m, const uint16_t *x, int64_t count, float *logits, float *hidden,
                       cudaStream_t st) {
    if (count <= 0) return MCBGPU_OK;
    const int64_t tiles = (count + kTileRows - 1) / kTileRows;
    // 8 CTAs per SM: 8 x 64 TMEM columns fill the SM's 512, and with the prefetch of
    // the next tile 16 tiles of features are in flight per SM
    const int grid = (int)std::min<int64_t>(tiles, (int64_t)(m->sm_count > 0 ? m->sm_count : 148) * 8);
    mlp_forward_kernel<<<grid, kFwdThreads, 0, st>>>(x, count, m->d_w1, m->d_params + kHid * kIn,
                                                     m->d_w2r, m->d_params + kParams - 1, logits, hidden,
                                                     m->d_status);
    MCB_CUDA(cudaGetLastError());
    return MCBGPU_OK;
}

static int mlp_buffers(mcbgpu_mlp *m, int64_t count) {
    if (count <= m->cap) return MCBGPU_OK;
    cudaFree(m->d_logits);
    cudaFree(m->d_hidden);
    m->d_logits = nullptr;
    m->d_hidden = nullptr;
    m->cap = 0;
    MCB_CUDA(cudaMalloc((void **)&m->d_logits, sizeof(float) * (size_t)count));
    MCB_CUDA(cudaMalloc((void **)&m->d_hidden, sizeof(float) * kHid * (size_t)count));
    m->cap = count;
    return MCBGPU_OK;
}

// forward with the hidden layer kept, then the gradients (accumulated in d_grads)
static int mlp_grads(mcbgpu_mlp *m, const uint16_t *x, const uint8_t *labels, int64_t count, float pos_weight,
                     cudaStream_t st) {
    int rc = mlp_buffers(m, count);
    if (rc) return rc;
    rc = mlp_forward(m, x, count, m->d_logits, m->d_hidden, st);
    if (rc) return rc;
    MCB_CUDA(cudaMemsetAsync(m->d_loss, 0, sizeof(float), st));
    const int per = kBwdThreads / kHid;
    const int grid = (int)std::min<int64_t>((count + per - 1) / per, (int64_t)(m->sm_count > 0 ? m->sm_count : 148) * 2);
    mlp_backward_kernel<<<grid, kBwdThreads, 0, st>>>(x, labels, m->d_logits, m->d_hidden, count, pos_weight,
                                                      m->d_w2r, m->d_grads, m->d_loss);
    MCB_CUDA(cudaGetLastError());
    return MCBGPU_OK;
}

extern "C" {

int mcbgpu_mlp_param_count(void) { return kParams; }

int mcbgpu_mlp_create(mcbgpu_mlp **out, const float *params) {
    if (!out || !params) {
        set_error("mcbgpu_mlp_create: NULL argument");
        return MCBGPU_E_ARG;
    }
    *out = nullptr;
    mcbgpu_mlp *m = new mcbgpu_mlp();
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&m->sm_count, cudaDevAttrMultiProcessorCount, dev);
    const size_t pb = sizeof(float) * kParams;
    if (e == cudaSuccess) e = cudaMalloc((void **)&m->d_params, pb);
    if (e == cudaSuccess) e = cudaMalloc((void **)&m->d_grads, pb);
    if (e == cudaSuccess) e = cudaMalloc((void **)&m->d_m1, pb);
    if (e == cudaSuccess) e = cudaMalloc((void **)&m->d_m2, pb);
    if (e == cudaSuccess) e = cudaMalloc((void **)&m->d_w2r, sizeof(float) * kHid);
    if (e == cudaSuccess) e = cudaMalloc((void **)&m->d_w1, sizeof(uint16_t) * kHid * kIn);
    if (e == cudaSuccess) e = cudaMalloc((void **)&m->d_loss, sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void **)&m->d_status, sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemcpy(m->d_params, params, pb, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(m->d_grads, 0, pb);
    if (e == cudaSuccess) e = cudaMemset(m->d_m1, 0, pb);
    if (e == cudaSuccess) e = cudaMemset(m->d_m2, 0, pb);
    if (e == cudaSuccess) e = cudaMemset(m->d_status, 0, sizeof(unsigned));
    if (e == cudaSuccess) {
        mlp_weights_kernel<<<1, 256>>>(m->d_params, m->d_w1, m->d_w2r);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        mlp_free(m);
        return cuda_fail(e, "mcbgpu_mlp_create");
    }
    *out = m;
    return MCBGPU_OK;
}

int mcbgpu_mlp_get_params(const mcbgpu_mlp *m, float *params) {
    if (!m || !params) {
        set_error("mcbgpu_mlp_get_params: NULL argument");
        return MCBGPU_E_ARG;
    }
    MCB_CUDA(cudaMemcpy(params, m->d_params, sizeof(float) * kParams, cudaMemcpyDeviceToHost));
    return MCBGPU_OK;
}

int mcbgpu_mlp_forward(mcbgpu_mlp *m, const uint16_t *x, int64_t count, float *logits, void *stream) {
    if (!m || count < 0 || (count > 0 && (!x || !logits))) {
        set_error("mcbgpu_mlp_forward: invalid arguments");
        return MCBGPU_E_ARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    int rc = mlp_forward(m, x, count, logits, nullptr, st);
    if (rc) return rc;
    return mlp_status(m, st, "mcbgpu_mlp_forward");
}

int mcbgpu_mlp_gradients(mcbgpu_mlp *m, const uint16_t *x, const uint8_t *labels, int64_t count, float pos_weight,
                         float *grads, float *loss, void *stream) {
    if (!m || count <= 0 || !x || !labels || !grads || !loss || !(pos_weight > 0.0f)) {
        set_error("mcbgpu_mlp_gradients: invalid arguments");
        return MCBGPU_E_ARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    MCB_CUDA(cudaMemsetAsync(m->d_grads, 0, sizeof(float) * kParams, st));
    int rc = mlp_grads(m, x, labels, count, pos_weight, st);
    if (rc) return rc;
    MCB_CUDA(cudaMemcpyAsync(grads, m->d_grads, sizeof(float) * kParams, cudaMemcpyDeviceToHost, st));
    float l = 0;
    MCB_CUDA(cudaMemcpyAsync(&l, m->d_loss, sizeof(float), cudaMemcpyDeviceToHost, st));
    MCB_CUDA(cudaMemsetAsync(m->d_grads, 0, sizeof(float) * kParams, st));
    rc = mlp_status(m, st, "mcbgpu_mlp_gradients");
    *loss = l / (float)count;
    return rc;
}

int mcbgpu_mlp_train_step(mcbgpu_mlp *m, const uint16_t *x, const uint8_t *labels, int64_t count, float pos_weight,
                          float lr, float *loss, void *stream) {
    if (!m || count <= 0 || !x || !labels || !(pos_weight > 0.0f) || !(lr > 0.0f)) {
        set_error("mcbgpu_mlp_train_step: invalid arguments");
        return MCBGPU_E_ARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    int rc = mlp_grads(m, x, labels, count, pos_weight, st);
    if (rc) return rc;
    m->steps++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - powf(b1, (float)m->steps), c2 = 1.0f - powf(b2, (float)m->steps);
    mlp_adam_kernel<<<1, 256, 0, st>>>(m->d_params, m->d_grads, m->d_m1, m->d_m2, lr, b1, b2, 1e-8f, c1, c2, m->d_w1,
                                       m->d_w2r);
    MCB_CUDA(cudaGetLastError());
    if (loss) {
        float l = 0;
        MCB_CUDA(cudaMemcpyAsync(&l, m->d_loss, sizeof(float), cudaMemcpyDeviceToHost, st));
        rc = mlp_status(m, st, "mcbgpu_mlp_train_step");
        *loss = l / (float)count;
        return rc;
    }
    return MCBGPU_OK;
}

int mcbgpu_mlp_destroy(mcbgpu_mlp *m) {
    if (m) mlp_free(m);
    return MCBGPU_OK;
}

}  // extern "C"
