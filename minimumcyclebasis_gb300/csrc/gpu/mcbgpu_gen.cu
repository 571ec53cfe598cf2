// Candidate generation on the device: the per-root shortest-path trees, the
// candidate test and the cycle coordinate lists of the host preparation
// (include/Dijkstra.h:78-254, include/work_per_thread.h:92-147, include/cycles.h:144-195),
// for a problem whose host preparation stopped after the spanning tree
// (mcbh_options.structure_only).  The host keeps the two steps whose result only
// the standard library's own routines reproduce: the heap-ordered search of the
// roots whose tree has a tie (mcbh_search_trees) and the per-root group maps + the
// sort on weight (mcbh_rank_candidates).
//
// Per chunk of roots (FVS indices t0 .. t0+count):
//   1. trees_kernel (mcbgpu_sssp.cuh): distances into the chunk's distance rows,
//      parent slots into the resident parent array (F x n' int32, kept for the
//      lists), a tie flag per root; the host replaces the tied roots' trees.
//   2. codes_kernel: per vertex, the child of the root its tree path runs through
//      (its branch) or "blocked" if that path holds an FVS vertex with a smaller id
//      than the root, by pointer jumping up the parent chains (O(n' log height)).
//   3. cand_count_kernel: per non-tree pair of slots, the reference's test (both
//      ends unblocked, paths meeting only at the root) as a bitmap, and a count per
//      root; cand_write_kernel: the accepted pairs in pair order with their weights
//      d(a) + d(b) + w, one warp per root, at offsets from a scan of the counts.
// After the host has ranked all candidates:
//   4. walk_kernel (twice): per rank, the coordinates on its two root paths and of
//      its own edge; first the lengths, then (after a scan) the lists;
//      sort_lists_kernel sorts each list ascending (one warp per list, bitonic in
//      shared memory; one CTA per list above 1024 entries).
// Every index read from a caller's array is range-checked; a bad one sets a status
// bit (MCBGPU_E_DEVICE) instead of being followed, and every walk is bounded by n'.
#include <algorithm>
#include <climits>
#include <cstring>
#include <vector>

#include "mcbgpu_sssp.cuh"

using namespace mcbgpu;
using namespace mcbgpu::sssp;

// (a named namespace: an anonymous one here would clash, in the generated launch
// stubs, with the one of mcbgpu_sssp.cuh)
namespace mcbgpu {
namespace gen {

constexpr int kCodeThreads = 1024;
constexpr int kJumpRounds = 40;  // pointer jumping halves every chain per round: heights below 2^39
constexpr int kCandThreads = 512;
constexpr int kWalkThreads = 256;
constexpr int kSortWarpMax = 1024;   // lists up to this length: one warp, 4 KB of shared memory
constexpr int kSortLongMax = 32768;  // longer lists: one CTA, up to 128 KB of shared memory
constexpr int kScanThreads = 1024;

struct GenGraph {
    const uint32_t *ro, *rows, *cols, *rev, *pair_slot, *roots;
    const int32_t *w, *ec, *fvs;
    int32_t n, F;
    int64_t slots, npairs;
};

// pointer-jumping state of a vertex: bits 0-31 the ancestor it points to, 32-62 the
// last vertex below that ancestor on its path, 63 whether the path segment between
// them holds a blocking FVS vertex
__device__ __forceinline__ uint64_t jpack(uint32_t anc, uint32_t top, uint32_t blk) {
    return (uint64_t)anc | ((uint64_t)(top & 0x7fffffffu) << 32) | ((uint64_t)blk << 63);
}
__device__ __forceinline__ uint32_t janc(uint64_t x) { return (uint32_t)x; }
__device__ __forceinline__ uint32_t jtop(uint64_t x) { return (uint32_t)(x >> 32) & 0x7fffffffu; }
__device__ __forceinline__ uint32_t jblk(uint64_t x) { return (uint32_t)(x >> 63); }

constexpr int32_t kCodeRoot = -1, kCodeBlocked = -2;

// Branch codes of the chunk's trees, one CTA per root.  The jump state is updated in
// place: a vertex reads its ancestor's 64-bit state (single-copy atomic), which is at
// least as far along as the synchronous scheme's, so each round at least halves every
// remaining chain; rounds stop when every vertex points at the root.
__global__ void __launch_bounds__(kCodeThreads) codes_kernel(GenGraph g, const int32_t *__restrict__ pedge, int t0,
                                                             int count, uint64_t *jump, int32_t *code,
                                                             unsigned *status) {
    const int n = g.n;
    for (int r = blockIdx.x; r < count; r += gridDim.x) {
        const int t = t0 + r;
        const uint32_t src = g.roots[t];
        const int32_t *pe = pedge + (size_t)t * n;
        volatile unsigned long long *J = reinterpret_cast<volatile unsigned long long *>(jump + (size_t)r * n);
        int bad = 0;
        for (int v = threadIdx.x; v < n; v += blockDim.x) {
            if ((uint32_t)v == src) {
                J[v] = jpack(src, 0, 0);
                continue;
            }
            const int32_t o = pe[v];
            if (o < 0 || (int64_t)o >= g.slots || g.cols[o] != (uint32_t)v) {
                bad = 1;  // not a tree: the vertex is left blocked, so it joins no candidate
                J[v] = jpack(src, v, 1);
                continue;
            }
            J[v] = jpack(g.rows[o], v, (g.fvs[v] >= 0 && (uint32_t)v < src) ? 1u : 0u);
        }
        if (!cta_sync_and(bad == 0) && threadIdx.x == 0) atomicOr(status, ST_BAD_INPUT);
        bool done = false;
        for (int round = 0; round < kJumpRounds && !done; round++) {
            int open = 0;
            for (int v = threadIdx.x; v < n; v += blockDim.x) {
                const uint64_t x = J[v];
                const uint32_t a = janc(x);
                if (a == src) continue;
                if (a >= (uint32_t)n) {  // cannot happen with checked parents; kept finite
                    J[v] = jpack(src, v, 1);
                    continue;
                }
                const uint64_t y = J[a];
                J[v] = jpack(janc(y), jtop(y), jblk(x) | jblk(y));
                open |= janc(y) != src;
            }
            done = cta_sync_and(open == 0);
        }
        if (!done && threadIdx.x == 0) atomicOr(status, ST_BAD_INPUT);  // a parent cycle
        int32_t *cd = code + (size_t)r * n;
        for (int v = threadIdx.x; v < n; v += blockDim.x) {
            const uint64_t x = J[v];
            cd[v] = (uint32_t)v == src ? kCodeRoot : (jblk(x) || janc(x) != src) ? kCodeBlocked : (int32_t)jtop(x);
        }
        cta_sync();
    }
}

// The reference's candidate test per non-tree pair of slots, as one bit per pair
// (32 pairs per warp step), and the number of candidates per root.
__global__ void __launch_bounds__(kCandThreads) cand_count_kernel(GenGraph g, const int32_t *__restrict__ pedge,
                                                                  const int32_t *__restrict__ code, int t0, int count,
                                                                  uint32_t *bits, int64_t words_per_root,
                                                                  int64_t *counts) {
    __shared__ long long s_cnt[kCandThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int n = g.n;
    for (int r = blockIdx.x; r < count; r += gridDim.x) {
        const int t = t0 + r;
        const uint32_t src = g.roots[t];
        const int32_t *pe = pedge + (size_t)t * n;
        const int32_t *cd = code + (size_t)r * n;
        uint32_t *bw = bits + (size_t)r * words_per_root;
        long long cnt = 0;
        for (int64_t wi = warp; wi < words_per_root; wi += nwarps) {
            const int64_t k = wi * 32 + lane;
            int acc = 0;
            if (k < g.npairs) {
                const uint32_t o = g.pair_slot[k];
                const uint32_t a = g.rows[o], b = g.cols[o];
                if (pe[b] != (int32_t)o && pe[a] != (int32_t)g.rev[o]) {
                    const int32_t ca = cd[a], cb = cd[b];
                    acc = ca != kCodeBlocked && cb != kCodeBlocked && (a == src || b == src || ca != cb);
                }
            }
            const uint32_t m = __ballot_sync(0xffffffffu, acc);
            if (lane == 0) {
                bw[wi] = m;
                cnt += __popc(m);
            }
        }
        if (lane == 0) s_cnt[warp] = cnt;
        cta_sync();
        if (threadIdx.x == 0) {
            long long s = 0;
            for (int i = 0; i < nwarps; i++) s += s_cnt[i];
            counts[r] = s;
        }
        cta_sync();
    }
}

// Exclusive prefix sum of `count` int64 values in one CTA; out[count] = the total.
__global__ void __launch_bounds__(kScanThreads) scan_small_kernel(const int64_t *in, int count, int64_t *out) {
    __shared__ long long s_part[kScanThreads / 32];
    __shared__ long long s_carry;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_carry = 0;
    cta_sync();
    for (int base = 0; base < count; base += blockDim.x) {
        const int i = base + threadIdx.x;
        long long v = i < count ? in[i] : 0;
        long long x = v;
        for (int d = 1; d < 32; d <<= 1) {
            const long long y = __shfl_up_sync(0xffffffffu, x, d);
            if (lane >= d) x += y;
        }
        if (lane == 31) s_part[warp] = x;
        cta_sync();
        if (warp == 0) {
            long long p = lane < (int)(blockDim.x >> 5) ? s_part[lane] : 0;
            for (int d = 1; d < 32; d <<= 1) {
                const long long y = __shfl_up_sync(0xffffffffu, p, d);
                if (lane >= d) p += y;
            }
            s_part[lane] = p;  // inclusive prefix of the warp sums
        }
        cta_sync();
        const long long before = s_carry + (warp > 0 ? s_part[warp - 1] : 0);
        if (i < count) out[i] = before + x - v;
        cta_sync();
        if (threadIdx.x == blockDim.x - 1) s_carry = before + x;
        cta_sync();
    }
    if (threadIdx.x == 0) out[count] = s_carry;
}

// The accepted pairs of each root in pair order with their weights, one warp per
// root, written at the root's offset.
__global__ void __launch_bounds__(kCandThreads) cand_write_kernel(GenGraph g, const int32_t *__restrict__ dist,
                                                                  const uint32_t *__restrict__ bits,
                                                                  int64_t words_per_root, int count,
                                                                  const int64_t *__restrict__ offsets, int64_t cap,
                                                                  uint32_t *out_pair, int32_t *out_weight,
                                                                  unsigned *status) {
    const int lane = threadIdx.x & 31;
    const int n = g.n;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (int r = gw; r < count; r += nw) {
        const uint32_t *bw = bits + (size_t)r * words_per_root;
        const int32_t *d = dist + (size_t)r * n;
        int64_t pos = offsets[r];
        const int64_t end = offsets[r + 1];
        for (int64_t wb = 0; wb < words_per_root; wb += 32) {
            const int64_t wi = wb + lane;
            uint32_t m = wi < words_per_root ? bw[wi] : 0u;
            const int c = __popc(m);
            int x = c;
            for (int dd = 1; dd < 32; dd <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, x, dd);
                if (lane >= dd) x += y;
            }
            int64_t p = pos + x - c;
            while (m) {
                const int j = __ffs(m) - 1;
                m &= m - 1;
                const int64_t k = wi * 32 + j;
                const uint32_t o = g.pair_slot[k];
                if (p < end && p < cap) {
                    out_pair[p] = (uint32_t)k;
                    out_weight[p] = d[g.rows[o]] + d[g.cols[o]] + g.w[o];
                } else {
                    atomicOr(status, ST_BAD_INPUT);
                }
                p++;
            }
            pos += __shfl_sync(0xffffffffu, x, 31);
        }
    }
}

__device__ __forceinline__ uint16_t to_bf16(float f) {
    uint32_t u = __float_as_uint(f);
    u += 0x7fffu + ((u >> 16) & 1u);  // round to nearest even (finite inputs)
    return (uint16_t)(u >> 16);
}

// The learned proposal's 16 features of one candidate (bf16), from its walk: its
// weight against the list's median weight, the two root distances and the edge
// weight as shares of the weight, the path hop counts, the list length, its rank
// quantile, the degrees of its root and ends.
__device__ void candidate_features(uint16_t *f, float W, float wmed, float da, float db, float we, int ha, int hb,
                                   int len, float quantile, int deg_root, int deg_ends) {
    const float Wp = W > 0.0f ? W : 1.0f;
    const float v[16] = {W / wmed,
                         fminf(da, db) / Wp,
                         fmaxf(da, db) / Wp,
                         we / Wp,
                         log2f(1.0f + (float)(ha + hb)) * 0.125f,
                         log2f(1.0f + (float)len) * 0.125f,
                         quantile,
                         log2f(1.0f + (float)deg_root) * 0.25f,
                         log2f(1.0f + (float)deg_ends) * 0.25f,
                         fabsf((float)(ha - hb)) / (1.0f + (float)(ha + hb)),
                         1.0f,
                         0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int i = 0; i < 16; i++) f[i] = to_bf16(v[i]);
}

// Per rank: the coordinates of its cycle (its own edge's, then the root paths of its
// two ends).  Without `out`, the count into len[r] (and with `feat`, the candidate's
// features); with it, the coordinates at out[off[r] ...] in walk order.
__global__ void __launch_bounds__(kWalkThreads) walk_kernel(GenGraph g, const int32_t *__restrict__ pedge, int64_t K,
                                                            const int32_t *__restrict__ tree,
                                                            const int32_t *__restrict__ eoff, int32_t *len,
                                                            const int64_t *__restrict__ off, int32_t *out,
                                                            unsigned *status, uint16_t *feat,
                                                            const int32_t *__restrict__ weight, float wmed) {
    const int n = g.n;
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < K; r += (int64_t)gridDim.x * blockDim.x) {
        const int32_t t = tree[r], o = eoff[r];
        if (t < 0 || t >= g.F || o < 0 || (int64_t)o >= g.slots) {
            atomicOr(status, ST_BAD_INPUT);
            if (!out) len[r] = 0;
            if (feat) candidate_features(feat + r * 16, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0);
            continue;
        }
        const uint32_t src = g.roots[t];
        const int32_t *pe = pedge + (size_t)t * n;
        int64_t p = out ? off[r] : 0;
        const int64_t end = out ? off[r + 1] : 0;
        int c = 0;
        auto emit = [&](int32_t coord) {
            if (coord < 0) return;
            if (out) {
                if (p < end)
                    out[p++] = coord;
                else
                    atomicOr(status, ST_BAD_INPUT);
            }
            c++;
        };
        emit(g.ec[o]);
        float dist[2] = {0.0f, 0.0f};
        int hops[2] = {0, 0};
        for (int side = 0; side < 2; side++) {
            uint32_t x = side ? g.cols[o] : g.rows[o];
            for (int steps = 0; x != src; steps++) {
                const int32_t q = pe[x];
                if (steps >= n || q < 0 || (int64_t)q >= g.slots) {
                    atomicOr(status, ST_BAD_INPUT);
                    break;
                }
                emit(g.ec[q]);
                dist[side] += (float)g.w[q];
                hops[side]++;
                x = g.rows[q];
            }
        }
        if (!out) len[r] = c;
        if (feat) {
            const uint32_t a = g.rows[o], b = g.cols[o];
            const int deg_root = (int)(g.ro[src + 1] - g.ro[src]);
            const int deg_ends = (int)(g.ro[a + 1] - g.ro[a] + g.ro[b + 1] - g.ro[b]);
            candidate_features(feat + r * 16, (float)weight[r], wmed, dist[0], dist[1], (float)g.w[o], hops[0],
                               hops[1], c, (float)r / (float)K, deg_root, deg_ends);
        }
    }
}

// Block-level exclusive scan over int32 lengths -> int64 offsets (three passes:
// per-block sums, a scan of the sums in one block, the offsets).
constexpr int kScanItems = 8;  // items per thread in the per-block passes

__global__ void __launch_bounds__(kScanThreads) block_sums_kernel(const int32_t *len, int64_t K, int64_t *sums) {
    __shared__ long long s_part[kScanThreads / 32];
    const int64_t base = (int64_t)blockIdx.x * kScanThreads * kScanItems;
    long long s = 0;
    for (int i = 0; i < kScanItems; i++) {
        const int64_t r = base + (int64_t)i * kScanThreads + threadIdx.x;
        if (r < K) s += len[r];
    }
    for (int d = 16; d > 0; d >>= 1) s += __shfl_down_sync(0xffffffffu, s, d);
    if ((threadIdx.x & 31) == 0) s_part[threadIdx.x >> 5] = s;
    cta_sync();
    if (threadIdx.x == 0) {
        long long tot = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) tot += s_part[i];
        sums[blockIdx.x] = tot;
    }
}

__global__ void __launch_bounds__(kScanThreads) block_offsets_kernel(const int32_t *len, int64_t K,
                                                                     const int64_t *block_base, int64_t *off) {
    __shared__ long long s_part[kScanThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t base = (int64_t)blockIdx.x * kScanThreads * kScanItems;
    // each thread takes kScanItems consecutive items
    const int64_t r0 = base + (int64_t)threadIdx.x * kScanItems;
    long long v[kScanItems];
    long long s = 0;
    for (int i = 0; i < kScanItems; i++) {
        v[i] = r0 + i < K ? len[r0 + i] : 0;
        s += v[i];
    }
    long long x = s;
    for (int d = 1; d < 32; d <<= 1) {
        const long long y = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= d) x += y;
    }
    if (lane == 31) s_part[warp] = x;
    cta_sync();
    if (warp == 0) {
        long long p = lane < (int)(blockDim.x >> 5) ? s_part[lane] : 0;
        for (int d = 1; d < 32; d <<= 1) {
            const long long y = __shfl_up_sync(0xffffffffu, p, d);
            if (lane >= d) p += y;
        }
        s_part[lane] = p;
    }
    cta_sync();
    long long run = block_base[blockIdx.x] + (warp > 0 ? s_part[warp - 1] : 0) + x - s;
    for (int i = 0; i < kScanItems; i++) {
        if (r0 + i < K) off[r0 + i] = run;
        run += v[i];
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) off[K] = run;
}

// Bitonic sort of s[0, P) (P a power of two) by the calling threads: `lane` of
// `width` cooperating threads; sync() between the stages.
template <typename Sync>
__device__ __forceinline__ void bitonic(int32_t *s, int P, int lane, int width, Sync sync) {
    for (int k = 2; k <= P; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = lane; i < P; i += width) {
                const int l = i ^ j;
                if (l > i) {
                    const int32_t a = s[i], b = s[l];
                    if ((a > b) == ((i & k) == 0)) {
                        s[i] = b;
                        s[l] = a;
                    }
                }
            }
            sync();
        }
    }
}

constexpr int kSortWarps = 8;

// Sorts each list ascending: one warp per list of up to kSortWarpMax entries; longer
// lists are appended to `longs` for sort_long_kernel.
__global__ void __launch_bounds__(kSortWarps * 32) sort_lists_kernel(int64_t K, const int64_t *__restrict__ off,
                                                                     int32_t *coords, int64_t *longs,
                                                                     unsigned *nlong, unsigned long long cap_long) {
    __shared__ int32_t s_buf[kSortWarps][kSortWarpMax];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int32_t *s = s_buf[warp];
    const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = gw; r < K; r += nw) {
        const int64_t b = off[r];
        const int L = (int)(off[r + 1] - b);
        if (L <= 1) continue;
        if (L > kSortWarpMax) {
            if (lane == 0) {
                const unsigned q = atomicAdd(nlong, 1u);
                if (q < cap_long) longs[q] = r;
            }
            continue;
        }
        int P = 2;
        while (P < L) P <<= 1;
        for (int i = lane; i < P; i += 32) s[i] = i < L ? coords[b + i] : INT_MAX;
        __syncwarp();
        bitonic(s, P, lane, 32, [] { __syncwarp(); });
        for (int i = lane; i < L; i += 32) coords[b + i] = s[i];
        __syncwarp();
    }
}

__global__ void __launch_bounds__(1024) sort_long_kernel(const int64_t *__restrict__ off, int32_t *coords,
                                                         const int64_t *longs, int count, unsigned *status) {
    extern __shared__ int32_t s_long[];
    for (int q = blockIdx.x; q < count; q += gridDim.x) {
        const int64_t r = longs[q];
        const int64_t b = off[r];
        const int64_t L = off[r + 1] - b;
        if (L > kSortLongMax) {
            if (threadIdx.x == 0) atomicOr(status, ST_BAD_INPUT);
            continue;
        }
        int P = 2;
        while (P < L) P <<= 1;
        for (int i = threadIdx.x; i < P; i += blockDim.x) s_long[i] = i < L ? coords[b + i] : INT_MAX;
        cta_sync();
        bitonic(s_long, P, threadIdx.x, blockDim.x, [] { cta_sync(); });
        for (int i = threadIdx.x; i < L; i += blockDim.x) coords[b + i] = s_long[i];
        cta_sync();
    }
}

}  // namespace gen
}  // namespace mcbgpu

using namespace mcbgpu::gen;

struct mcbgpu_gen {
    int32_t n = 0, F = 0, chunk = 0, N = 0;
    int64_t slots = 0, npairs = 0, words_per_root = 0;
    int sm_count = 0;
    bool shared_form = true;
    size_t smem = 0;
    int delta = 1;  // the mean slot weight
    // launch shapes of the tree kernel: while tuning, call i of mcbgpu_gen_trees
    // runs shapes[i] and records its time per root; then the fastest is kept
    std::vector<TreeShape> shapes;
    std::vector<double> shape_us;  // microseconds per root, per shape tried
    int chosen = -1;
    // two tree slots, so that the trees of the next chunk run while the host searches
    // the current chunk's tied roots: distances, tie flags (device and pinned host),
    // the events around the launch, and what was submitted into each
    int32_t *d_dist_slot[2] = {nullptr, nullptr};
    uint8_t *d_tied_slot[2] = {nullptr, nullptr};
    uint8_t *h_tied[2] = {nullptr, nullptr};
    cudaEvent_t ev_begin[2] = {nullptr, nullptr}, ev_end[2] = {nullptr, nullptr};
    int32_t slot_t0[2] = {-1, -1}, slot_count[2] = {0, 0};
    int slot_shape[2] = {-1, -1};
    int submitted = 0;
    int cur_slot = 0;
    // graph
    uint32_t *d_ro = nullptr, *d_rows = nullptr, *d_cols = nullptr, *d_rev = nullptr, *d_pairs = nullptr,
             *d_roots = nullptr;
    int32_t *d_w = nullptr, *d_ec = nullptr, *d_fvs = nullptr;
    // trees
    int32_t *d_pedge = nullptr;  // F x n, resident
    int32_t *d_dist = nullptr;   // chunk x n
    int32_t *d_code = nullptr;   // chunk x n
    uint64_t *d_jump = nullptr;  // chunk x n
    uint32_t *d_bits = nullptr;  // chunk x words_per_root
    int32_t *d_gdist = nullptr, *d_next = nullptr;
    uint32_t *d_gdirty = nullptr, *d_gsumm = nullptr;
    uint8_t *d_tied = nullptr;
    int64_t *d_counts = nullptr, *d_coff = nullptr;  // chunk, chunk + 1
    uint32_t *d_cpair = nullptr;
    int32_t *d_cweight = nullptr;
    int64_t cand_cap = 0;
    int32_t cur_t0 = -1, cur_count = 0;
    // lists
    int64_t K = 0, K_lists = 0, nnz = 0;
    int32_t *d_tree = nullptr, *d_eoff = nullptr, *d_len = nullptr, *d_coords = nullptr, *d_weight = nullptr;
    int64_t *d_off = nullptr, *d_bsum = nullptr, *d_longs = nullptr;
    unsigned *d_nlong = nullptr;
    unsigned *d_status = nullptr;
    long long bytes = 0;
    long long diverged_runs = 0;
};

static void gen_free_lists(mcbgpu_gen *g) {
    cudaFree(g->d_tree);
    cudaFree(g->d_eoff);
    cudaFree(g->d_len);
    cudaFree(g->d_coords);
    cudaFree(g->d_off);
    cudaFree(g->d_bsum);
    cudaFree(g->d_longs);
    cudaFree(g->d_weight);
    g->d_tree = g->d_eoff = g->d_len = g->d_coords = g->d_weight = nullptr;
    g->d_off = g->d_bsum = g->d_longs = nullptr;
}

static void gen_free(mcbgpu_gen *g) {
    for (int k = 0; k < 2; k++) {
        if (g->ev_begin[k]) cudaEventDestroy(g->ev_begin[k]);
        if (g->ev_end[k]) cudaEventDestroy(g->ev_end[k]);
        if (g->h_tied[k]) cudaFreeHost(g->h_tied[k]);
        cudaFree(g->d_tied_slot[k]);
    }
    cudaFree(g->d_dist_slot[1]);  // slot 0's distances are d_dist
    void *ps[] = {g->d_ro,   g->d_rows,    g->d_cols,   g->d_rev,    g->d_pairs,  g->d_roots,  g->d_w,
                  g->d_ec,   g->d_fvs,     g->d_pedge,  g->d_dist_slot[0], g->d_code, g->d_jump, g->d_bits,
                  g->d_gdist, g->d_next,   g->d_gdirty, g->d_gsumm, g->d_tied,   g->d_counts, g->d_coff,   g->d_cpair,
                  g->d_cweight, g->d_nlong, g->d_status};
    for (void *p : ps) cudaFree(p);
    gen_free_lists(g);
    delete g;
}

static GenGraph graph_of(const mcbgpu_gen *g) {
    GenGraph a;
    a.ro = g->d_ro;
    a.rows = g->d_rows;
    a.cols = g->d_cols;
    a.rev = g->d_rev;
    a.pair_slot = g->d_pairs;
    a.roots = g->d_roots;
    a.w = g->d_w;
    a.ec = g->d_ec;
    a.fvs = g->d_fvs;
    a.n = g->n;
    a.F = g->F;
    a.slots = g->slots;
    a.npairs = g->npairs;
    return a;
}

static int check_status(mcbgpu_gen *g, cudaStream_t st, const char *what) {
    unsigned h = 0;
    MCB_CUDA(cudaMemcpyAsync(&h, g->d_status, sizeof h, cudaMemcpyDeviceToHost, st));
    MCB_CUDA(cudaStreamSynchronize(st));
    if (h & ST_DIVERGED) g->diverged_runs++;
    if (h & ~(unsigned)ST_DIVERGED) {
        MCB_CUDA(cudaMemsetAsync(g->d_status, 0, sizeof(unsigned), st));
        set_error("%s: device status 0x%x (an index out of range was skipped)", what, h);
        return MCBGPU_E_DEVICE;
    }
    MCB_CUDA(cudaMemsetAsync(g->d_status, 0, sizeof(unsigned), st));
    return MCBGPU_OK;
}

extern "C" {

int mcbgpu_gen_create(mcbgpu_gen **out, int32_t nodes, int64_t slots, const uint32_t *row_offsets,
                      const uint32_t *rows, const uint32_t *cols, const int32_t *weights, const uint32_t *rev,
                      const int32_t *edge_coord, int32_t num_coords, const int32_t *fvs_array,
                      const uint32_t *fvs_vertices, int32_t fvs_size, const uint32_t *pair_slot, int32_t chunk) {
    if (!out || nodes <= 0 || slots <= 0 || slots >= (1ll << 31) || (slots & 1) || fvs_size <= 0 || chunk <= 0 ||
        num_coords < 0 || !row_offsets || !rows || !cols || !weights || !rev || !edge_coord || !fvs_array ||
        !fvs_vertices || !pair_slot) {
        set_error("mcbgpu_gen_create: invalid arguments");
        return MCBGPU_E_ARG;
    }
    *out = nullptr;
    if (nodes > kTreeGlobalMaxN) {
        set_error("mcbgpu_gen_create: %d vertices after chain contraction (at most %d)", (int)nodes, kTreeGlobalMaxN);
        return MCBGPU_E_ARG;
    }
    // the graph is checked here once, so the kernels can index with it
    if (row_offsets[0] != 0 || (int64_t)row_offsets[nodes] != slots) {
        set_error("mcbgpu_gen_create: row offsets must run from 0 to the slot count");
        return MCBGPU_E_ARG;
    }
    for (int32_t v = 0; v < nodes; v++)
        if (row_offsets[v + 1] < row_offsets[v]) {
            set_error("mcbgpu_gen_create: row offsets decrease at vertex %d", (int)v);
            return MCBGPU_E_ARG;
        }
    long long wsum = 0, wmax = 0;
    for (int32_t v = 0; v < nodes; v++)
        for (uint32_t o = row_offsets[v]; o < row_offsets[v + 1]; o++)
            if (rows[o] != (uint32_t)v) {
                set_error("mcbgpu_gen_create: slot %u is in row %d but names row %u", o, (int)v, rows[o]);
                return MCBGPU_E_ARG;
            }
    for (int64_t o = 0; o < slots; o++) {
        if (cols[o] >= (uint32_t)nodes || rev[o] >= (uint64_t)slots || rev[rev[o]] != (uint32_t)o ||
            rows[rev[o]] != cols[o] || weights[o] < 1 || weights[rev[o]] != weights[o] || edge_coord[o] < -1 ||
            edge_coord[o] >= num_coords) {
            set_error("mcbgpu_gen_create: slot %lld is not a consistent reverse pair with weight >= 1 and a "
                      "coordinate in [-1, N)",
                      (long long)o);
            return MCBGPU_E_ARG;
        }
        wsum += weights[o];
        wmax = weights[o] > wmax ? weights[o] : wmax;
    }
    if (path_length_bound(nodes, slots, weights, rev) + wmax >= (long long)INT_MAX) {
        set_error("mcbgpu_gen_create: distances could reach 2^31 (the n' - 1 heaviest edges weigh too much)");
        return MCBGPU_E_ARG;
    }
    const int64_t npairs = slots / 2;
    for (int64_t k = 0; k < npairs; k++)
        if ((int64_t)pair_slot[k] >= slots || pair_slot[k] >= rev[pair_slot[k]] ||
            (k > 0 && pair_slot[k] <= pair_slot[k - 1])) {
            set_error("mcbgpu_gen_create: pair %lld is not the lower slot of an ascending pair list", (long long)k);
            return MCBGPU_E_ARG;
        }
    for (int32_t t = 0; t < fvs_size; t++)
        if (fvs_vertices[t] >= (uint32_t)nodes || fvs_array[fvs_vertices[t]] != t) {
            set_error("mcbgpu_gen_create: FVS vertex %d is not consistent with the FVS array", (int)t);
            return MCBGPU_E_ARG;
        }
    mcbgpu_gen *g = new mcbgpu_gen();
    g->n = nodes;
    g->F = fvs_size;
    g->N = num_coords;
    g->slots = slots;
    g->npairs = npairs;
    g->chunk = chunk < fvs_size ? chunk : fvs_size;
    g->words_per_root = (npairs + 31) / 32;
    g->delta = (int32_t)((wsum + slots - 1) / slots);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&g->sm_count, cudaDevAttrMultiProcessorCount, dev);
    const int words = (nodes + 31) / 32;
    g->shared_form = nodes <= kTreeSharedMaxN;
    g->smem = g->shared_form ? trees_smem_bytes(nodes) : 0;
    const size_t n = (size_t)nodes, C = (size_t)g->chunk;
#define GALLOC(ptr, sz)                                            \
    do {                                                           \
        size_t _b = (size_t)(sz);                                  \
        if (_b < 16) _b = 16;                                      \
        if (e == cudaSuccess) e = cudaMalloc((void **)&(ptr), _b); \
        g->bytes += (long long)_b;                                 \
    } while (0)
    GALLOC(g->d_ro, 4 * (n + 1));
    GALLOC(g->d_rows, 4 * (size_t)slots);
    GALLOC(g->d_cols, 4 * (size_t)slots);
    GALLOC(g->d_rev, 4 * (size_t)slots);
    GALLOC(g->d_w, 4 * (size_t)slots);
    GALLOC(g->d_ec, 4 * (size_t)slots);
    GALLOC(g->d_fvs, 4 * n);
    GALLOC(g->d_pairs, 4 * (size_t)npairs);
    GALLOC(g->d_roots, 4 * (size_t)fvs_size);
    GALLOC(g->d_pedge, 4 * n * (size_t)fvs_size);
    GALLOC(g->d_dist, 4 * n * C);
    g->d_dist_slot[0] = g->d_dist;
    GALLOC(g->d_code, 4 * n * C);
    GALLOC(g->d_jump, 8 * n * C);
    GALLOC(g->d_bits, 4 * (size_t)g->words_per_root * C);
    GALLOC(g->d_tied, C);
    GALLOC(g->d_counts, 8 * C);
    GALLOC(g->d_coff, 8 * (C + 1));
    GALLOC(g->d_next, 4);
    GALLOC(g->d_status, 4);
    GALLOC(g->d_nlong, 4);
    if (!g->shared_form) {
        GALLOC(g->d_gdist, 4 * n * (size_t)g->sm_count * kTreeMaxCtasPerSm);
        GALLOC(g->d_gdirty, 4 * (size_t)words * (size_t)g->sm_count * kTreeMaxCtasPerSm);
        GALLOC(g->d_gsumm, 4 * (size_t)((words + 31) / 32) * (size_t)g->sm_count * kTreeMaxCtasPerSm);
    }
    // shapes the tuner tries (the shared form: one 1024-thread CTA per SM, bucket
    // widths only); with fewer chunks than twice the shapes, the first one is kept
    if (g->shared_form)
        g->shapes = {{kTreeThreads, 1, 4}, {kTreeThreads, 1, 8}, {kTreeThreads, 1, 16}, {kTreeThreads, 1, 2}};
    else
        g->shapes = {{256, 8, 8}, {256, 8, 4}, {256, 8, 2}, {256, 8, 16}, {512, 4, 8}, {128, 16, 8}};
    const int nchunks = (fvs_size + g->chunk - 1) / g->chunk;
    if (nchunks < 2 * (int)g->shapes.size()) g->chosen = 0;
    for (int k = 0; k < 2; k++) {
        if (e == cudaSuccess) e = cudaEventCreate(&g->ev_begin[k]);
        if (e == cudaSuccess) e = cudaEventCreate(&g->ev_end[k]);
        if (e == cudaSuccess) e = cudaMallocHost((void **)&g->h_tied[k], C);
        if (e == cudaSuccess) e = cudaMalloc((void **)&g->d_tied_slot[k], C);
    }
    if (e == cudaSuccess) e = cudaMalloc((void **)&g->d_dist_slot[1], 4 * n * C);
    g->bytes += 4ll * (long long)n * (long long)C + 2ll * (long long)C;
#undef GALLOC
    auto up = [&](void *dst, const void *src, size_t b) {
        if (e == cudaSuccess) e = cudaMemcpy(dst, src, b, cudaMemcpyHostToDevice);
    };
    up(g->d_ro, row_offsets, 4 * (n + 1));
    up(g->d_rows, rows, 4 * (size_t)slots);
    up(g->d_cols, cols, 4 * (size_t)slots);
    up(g->d_rev, rev, 4 * (size_t)slots);
    up(g->d_w, weights, 4 * (size_t)slots);
    up(g->d_ec, edge_coord, 4 * (size_t)slots);
    up(g->d_fvs, fvs_array, 4 * n);
    up(g->d_pairs, pair_slot, 4 * (size_t)npairs);
    up(g->d_roots, fvs_vertices, 4 * (size_t)fvs_size);
    if (e == cudaSuccess) e = cudaMemset(g->d_status, 0, 4);
    if (e == cudaSuccess) e = set_trees_smem_limit();
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(sort_long_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(sizeof(int32_t) * kSortLongMax));
    if (e != cudaSuccess) {
        const int rc = cuda_fail(e, "mcbgpu_gen_create");
        gen_free(g);
        return rc;
    }
    *out = g;
    return MCBGPU_OK;
}

int mcbgpu_gen_trees_submit(mcbgpu_gen *g, int32_t t0, int32_t count, void *stream) {
    if (!g || t0 < 0 || count <= 0 || count > g->chunk || t0 + (int64_t)count > g->F) {
        set_error("mcbgpu_gen_trees_submit: invalid arguments");
        return MCBGPU_E_ARG;
    }
    if (!g->d_pedge) {
        set_error("mcbgpu_gen_trees_submit: the trees were released");
        return MCBGPU_E_STATE;
    }
    const int k = g->submitted & 1;
    if (g->slot_t0[k] >= 0) {
        set_error("mcbgpu_gen_trees_submit: both tree slots are taken (collect a chunk first)");
        return MCBGPU_E_STATE;
    }
    cudaStream_t st = (cudaStream_t)stream;
    // the shape: the next untried one while tuning; once every shape has been
    // submitted, the fastest collected so far (the chosen one once all are timed)
    int si;
    if (g->chosen >= 0)
        si = g->chosen;
    else if (g->submitted < (int)g->shapes.size())
        si = g->submitted;
    else
        si = g->shape_us.empty() ? 0
                                 : (int)(std::min_element(g->shape_us.begin(), g->shape_us.end()) - g->shape_us.begin());
    const TreeShape shape = g->shapes[(size_t)si];
    MCB_CUDA(cudaMemsetAsync(g->d_next, 0, 4, st));
    TreeArgs a;
    a.ro = g->d_ro;
    a.cols = g->d_cols;
    a.w = g->d_w;
    a.rev = g->d_rev;
    a.n = g->n;
    a.delta = shape_delta(shape, g->delta);
    a.roots = g->d_roots + t0;
    a.count = count;
    a.dist_out = g->d_dist_slot[k];
    a.pedge_out = g->d_pedge + (size_t)t0 * g->n;
    a.tied_out = g->d_tied_slot[k];
    a.gdist = g->d_gdist;
    a.gdirty = g->d_gdirty;
    a.gsumm = g->d_gsumm;
    a.next_root = g->d_next;
    a.status = g->d_status;
    const int cap = g->sm_count * shape.ctas_per_sm;
    const int grid = count < cap ? count : cap;
    MCB_CUDA(cudaEventRecord(g->ev_begin[k], st));
    MCB_CUDA(launch_trees(g->shared_form, shape, grid, g->smem, st, a));
    MCB_CUDA(cudaEventRecord(g->ev_end[k], st));
    MCB_CUDA(cudaMemcpyAsync(g->h_tied[k], g->d_tied_slot[k], (size_t)count, cudaMemcpyDeviceToHost, st));
    g->slot_t0[k] = t0;
    g->slot_count[k] = count;
    g->slot_shape[k] = si;
    g->submitted++;
    return MCBGPU_OK;
}

int mcbgpu_gen_trees_collect(mcbgpu_gen *g, int32_t t0, uint8_t *tied, void *stream) {
    if (!g || !tied) {
        set_error("mcbgpu_gen_trees_collect: invalid arguments");
        return MCBGPU_E_ARG;
    }
    const int k = g->slot_t0[0] == t0 ? 0 : g->slot_t0[1] == t0 ? 1 : -1;
    if (k < 0 || t0 < 0) {
        set_error("mcbgpu_gen_trees_collect: no chunk at tree %d was submitted", (int)t0);
        return MCBGPU_E_STATE;
    }
    cudaStream_t st = (cudaStream_t)stream;
    MCB_CUDA(cudaEventSynchronize(g->ev_end[k]));
    const int count = g->slot_count[k];
    // the tie flags' copy follows ev_end on the same stream
    MCB_CUDA(cudaStreamSynchronize(st));
    std::memcpy(tied, g->h_tied[k], (size_t)count);
    g->cur_t0 = t0;
    g->cur_count = count;
    g->cur_slot = k;
    g->d_dist = g->d_dist_slot[k];
    const int rc = check_status(g, st, "mcbgpu_gen_trees");
    if (rc) return rc;
    const int si = g->slot_shape[k];
    if (g->chosen < 0 && si == (int)g->shape_us.size() && si < (int)g->shapes.size()) {
        float ms = 0;
        MCB_CUDA(cudaEventElapsedTime(&ms, g->ev_begin[k], g->ev_end[k]));
        g->shape_us.push_back(1e3 * (double)ms / count);
        if (g->shape_us.size() == g->shapes.size())
            g->chosen = (int)(std::min_element(g->shape_us.begin(), g->shape_us.end()) - g->shape_us.begin());
    }
    g->slot_t0[k] = -1;  // free for the next submission (its distances stay until then)
    return MCBGPU_OK;
}

int mcbgpu_gen_trees(mcbgpu_gen *g, int32_t t0, int32_t count, uint8_t *tied, void *stream) {
    if (!tied) {
        set_error("mcbgpu_gen_trees: invalid arguments");
        return MCBGPU_E_ARG;
    }
    int rc = mcbgpu_gen_trees_submit(g, t0, count, stream);
    if (rc) return rc;
    return mcbgpu_gen_trees_collect(g, t0, tied, stream);
}

int mcbgpu_gen_tuning(const mcbgpu_gen *g) { return g && g->chosen < 0 ? 1 : 0; }

int mcbgpu_gen_put_trees(mcbgpu_gen *g, const int32_t *trees, int32_t count, const int32_t *dist,
                         const int32_t *parent_slot, void *stream) {
    if (!g || count < 0 || (count > 0 && (!trees || !dist || !parent_slot))) {
        set_error("mcbgpu_gen_put_trees: invalid arguments");
        return MCBGPU_E_ARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    const size_t n = (size_t)g->n;
    for (int32_t i = 0; i < count; i++) {
        const int32_t t = trees[i];
        if (t < g->cur_t0 || t >= g->cur_t0 + g->cur_count) {
            set_error("mcbgpu_gen_put_trees: tree %d is not in the current chunk", (int)t);
            return MCBGPU_E_ARG;
        }
        MCB_CUDA(cudaMemcpyAsync(g->d_dist + (size_t)(t - g->cur_t0) * n, dist + (size_t)i * n, 4 * n,
                                 cudaMemcpyHostToDevice, st));
        MCB_CUDA(cudaMemcpyAsync(g->d_pedge + (size_t)t * n, parent_slot + (size_t)i * n, 4 * n,
                                 cudaMemcpyHostToDevice, st));
    }
    MCB_CUDA(cudaStreamSynchronize(st));
    return MCBGPU_OK;
}

int mcbgpu_gen_candidates(mcbgpu_gen *g, int64_t *counts, int64_t *total, void *stream) {
    if (!g || !counts || !total || g->cur_t0 < 0) {
        set_error("mcbgpu_gen_candidates: invalid arguments (mcbgpu_gen_trees first)");
        return MCBGPU_E_ARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    const GenGraph gg = graph_of(g);
    const int count = g->cur_count;
    const int grid = count < g->sm_count * 2 ? count : g->sm_count * 2;
    codes_kernel<<<grid, kCodeThreads, 0, st>>>(gg, g->d_pedge, g->cur_t0, count, g->d_jump, g->d_code,
                                                g->d_status);
    MCB_CUDA(cudaGetLastError());
    cand_count_kernel<<<count < g->sm_count * 4 ? count : g->sm_count * 4, kCandThreads, 0, st>>>(
        gg, g->d_pedge, g->d_code, g->cur_t0, count, g->d_bits, g->words_per_root, g->d_counts);
    MCB_CUDA(cudaGetLastError());
    scan_small_kernel<<<1, kScanThreads, 0, st>>>(g->d_counts, count, g->d_coff);
    MCB_CUDA(cudaGetLastError());
    MCB_CUDA(cudaMemcpyAsync(counts, g->d_counts, 8 * (size_t)count, cudaMemcpyDeviceToHost, st));
    MCB_CUDA(cudaMemcpyAsync(total, g->d_coff + count, 8, cudaMemcpyDeviceToHost, st));
    int rc = check_status(g, st, "mcbgpu_gen_candidates");
    if (rc) return rc;
    if (*total > g->cand_cap) {
        cudaFree(g->d_cpair);
        cudaFree(g->d_cweight);
        g->d_cpair = nullptr;
        g->d_cweight = nullptr;
        const int64_t cap = *total + *total / 4 + 1024;
        MCB_CUDA(cudaMalloc((void **)&g->d_cpair, 4 * (size_t)cap));
        MCB_CUDA(cudaMalloc((void **)&g->d_cweight, 4 * (size_t)cap));
        g->cand_cap = cap;
    }
    const int wgrid = (int)std::min<long long>((count + (kCandThreads / 32) - 1) / (kCandThreads / 32),
                                               (long long)g->sm_count * 8);
    cand_write_kernel<<<wgrid, kCandThreads, 0, st>>>(gg, g->d_dist, g->d_bits, g->words_per_root, count, g->d_coff,
                                                      g->cand_cap, g->d_cpair, g->d_cweight, g->d_status);
    MCB_CUDA(cudaGetLastError());
    return MCBGPU_OK;
}

int mcbgpu_gen_fetch(mcbgpu_gen *g, int64_t total, uint32_t *pair_index, int32_t *weight, void *stream) {
    if (!g || total < 0 || total > g->cand_cap || (total > 0 && (!pair_index || !weight))) {
        set_error("mcbgpu_gen_fetch: invalid arguments");
        return MCBGPU_E_ARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    if (total > 0) {
        MCB_CUDA(cudaMemcpyAsync(pair_index, g->d_cpair, 4 * (size_t)total, cudaMemcpyDeviceToHost, st));
        MCB_CUDA(cudaMemcpyAsync(weight, g->d_cweight, 4 * (size_t)total, cudaMemcpyDeviceToHost, st));
    }
    return check_status(g, st, "mcbgpu_gen_fetch");
}

int mcbgpu_gen_rank(mcbgpu_gen *g, int64_t K, const int32_t *tree, const int32_t *edge_offset,
                    const int32_t *weight, uint16_t *features, void *stream) {
    if (!g || K < 0 || (K > 0 && (!tree || !edge_offset || !weight))) {
        set_error("mcbgpu_gen_rank: invalid arguments");
        return MCBGPU_E_ARG;
    }
    if (!g->d_pedge) {
        set_error("mcbgpu_gen_rank: the trees were released");
        return MCBGPU_E_STATE;
    }
    cudaStream_t st = (cudaStream_t)stream;
    gen_free_lists(g);
    g->K = K;
    g->K_lists = 0;
    g->nnz = 0;
    const size_t k1 = (size_t)(K > 0 ? K : 1);
    const int64_t nblk = (K + (int64_t)kScanThreads * kScanItems - 1) / ((int64_t)kScanThreads * kScanItems);
    MCB_CUDA(cudaMalloc((void **)&g->d_tree, 4 * k1));
    MCB_CUDA(cudaMalloc((void **)&g->d_eoff, 4 * k1));
    MCB_CUDA(cudaMalloc((void **)&g->d_len, 4 * k1));
    MCB_CUDA(cudaMalloc((void **)&g->d_weight, 4 * k1));
    MCB_CUDA(cudaMalloc((void **)&g->d_off, 8 * (size_t)(K + 1)));
    MCB_CUDA(cudaMalloc((void **)&g->d_bsum, 8 * (size_t)(nblk + 1)));
    if (K == 0) return MCBGPU_OK;
    MCB_CUDA(cudaMemcpyAsync(g->d_tree, tree, 4 * (size_t)K, cudaMemcpyHostToDevice, st));
    MCB_CUDA(cudaMemcpyAsync(g->d_eoff, edge_offset, 4 * (size_t)K, cudaMemcpyHostToDevice, st));
    MCB_CUDA(cudaMemcpyAsync(g->d_weight, weight, 4 * (size_t)K, cudaMemcpyHostToDevice, st));
    const float wmed = (float)(weight[K / 2] > 0 ? weight[K / 2] : 1);  // the list is sorted by weight
    const GenGraph gg = graph_of(g);
    const int wgrid = (int)std::min<long long>((K + kWalkThreads - 1) / kWalkThreads, (long long)g->sm_count * 16);
    walk_kernel<<<wgrid, kWalkThreads, 0, st>>>(gg, g->d_pedge, K, g->d_tree, g->d_eoff, g->d_len, nullptr, nullptr,
                                                g->d_status, features, g->d_weight, wmed);
    MCB_CUDA(cudaGetLastError());
    return check_status(g, st, "mcbgpu_gen_rank");
}

int mcbgpu_gen_build_lists(mcbgpu_gen *g, int64_t K_keep, int64_t *nnz, void *stream) {
    if (!g || !nnz || K_keep < 0 || K_keep > g->K || !g->d_len) {
        set_error("mcbgpu_gen_build_lists: invalid arguments (mcbgpu_gen_rank first)");
        return MCBGPU_E_ARG;
    }
    if (!g->d_pedge) {
        set_error("mcbgpu_gen_build_lists: the trees were released");
        return MCBGPU_E_STATE;
    }
    cudaStream_t st = (cudaStream_t)stream;
    cudaFree(g->d_coords);
    cudaFree(g->d_longs);
    g->d_coords = nullptr;
    g->d_longs = nullptr;
    g->K_lists = K_keep;
    g->nnz = 0;
    if (K_keep == 0) {
        MCB_CUDA(cudaMemsetAsync(g->d_off, 0, 8, st));
        MCB_CUDA(cudaStreamSynchronize(st));
        *nnz = 0;
        return MCBGPU_OK;
    }
    const int64_t K = K_keep;
    const int64_t nblk = (K + (int64_t)kScanThreads * kScanItems - 1) / ((int64_t)kScanThreads * kScanItems);
    block_sums_kernel<<<(unsigned)nblk, kScanThreads, 0, st>>>(g->d_len, K, g->d_bsum);
    MCB_CUDA(cudaGetLastError());
    scan_small_kernel<<<1, kScanThreads, 0, st>>>(g->d_bsum, (int)nblk, g->d_bsum);
    MCB_CUDA(cudaGetLastError());
    block_offsets_kernel<<<(unsigned)nblk, kScanThreads, 0, st>>>(g->d_len, K, g->d_bsum, g->d_off);
    MCB_CUDA(cudaGetLastError());
    int64_t total = 0;
    MCB_CUDA(cudaMemcpyAsync(&total, g->d_off + K, 8, cudaMemcpyDeviceToHost, st));
    int rc = check_status(g, st, "mcbgpu_gen_build_lists (offsets)");
    if (rc) return rc;
    MCB_CUDA(cudaMalloc((void **)&g->d_coords, 4 * (size_t)(total > 0 ? total : 1)));
    const GenGraph gg = graph_of(g);
    const int wgrid = (int)std::min<long long>((K + kWalkThreads - 1) / kWalkThreads, (long long)g->sm_count * 16);
    walk_kernel<<<wgrid, kWalkThreads, 0, st>>>(gg, g->d_pedge, K, g->d_tree, g->d_eoff, g->d_len, g->d_off,
                                                g->d_coords, g->d_status, nullptr, nullptr, 1.0f);
    MCB_CUDA(cudaGetLastError());
    const unsigned long long cap_long = (unsigned long long)(K < 65536 ? K : 65536);
    MCB_CUDA(cudaMalloc((void **)&g->d_longs, 8 * (size_t)cap_long));
    MCB_CUDA(cudaMemsetAsync(g->d_nlong, 0, 4, st));
    const int sgrid = (int)std::min<long long>((K + kSortWarps - 1) / kSortWarps, (long long)g->sm_count * 8);
    sort_lists_kernel<<<sgrid, kSortWarps * 32, 0, st>>>(K, g->d_off, g->d_coords, g->d_longs, g->d_nlong, cap_long);
    MCB_CUDA(cudaGetLastError());
    unsigned nlong = 0;
    MCB_CUDA(cudaMemcpyAsync(&nlong, g->d_nlong, 4, cudaMemcpyDeviceToHost, st));
    MCB_CUDA(cudaStreamSynchronize(st));
    if (nlong > cap_long) {
        set_error("mcbgpu_gen_build_lists: %u lists longer than %d entries (at most %llu)", nlong, kSortWarpMax,
                  cap_long);
        return MCBGPU_E_ARG;
    }
    if (nlong > 0) {
        sort_long_kernel<<<std::min<unsigned>(nlong, (unsigned)g->sm_count), 1024, sizeof(int32_t) * kSortLongMax,
                           st>>>(g->d_off, g->d_coords, g->d_longs, (int)nlong, g->d_status);
        MCB_CUDA(cudaGetLastError());
    }
    rc = check_status(g, st, "mcbgpu_gen_build_lists");
    if (rc) return rc;
    g->nnz = total;
    *nnz = total;
    return MCBGPU_OK;
}

int mcbgpu_gen_lists(mcbgpu_gen *g, int64_t K, const int32_t *tree, const int32_t *edge_offset,
                     const int32_t *weight, int64_t *nnz, void *stream) {
    if (!nnz) {
        set_error("mcbgpu_gen_lists: NULL nnz");
        return MCBGPU_E_ARG;
    }
    int rc = mcbgpu_gen_rank(g, K, tree, edge_offset, weight, nullptr, stream);
    if (rc) return rc;
    return mcbgpu_gen_build_lists(g, K, nnz, stream);
}

int mcbgpu_gen_get_lists(const mcbgpu_gen *g, const int32_t **weight, const int64_t **offsets,
                         const int32_t **coords) {
    if (!g || !weight || !offsets || !coords || !g->d_off || (g->K_lists > 0 && !g->d_coords)) {
        set_error("mcbgpu_gen_get_lists: no lists (mcbgpu_gen_build_lists first)");
        return MCBGPU_E_STATE;
    }
    *weight = g->d_weight;
    *offsets = g->d_off;
    *coords = g->d_coords;
    return MCBGPU_OK;
}

int mcbgpu_gen_copy_lists(const mcbgpu_gen *g, int64_t *offsets, int32_t *coords, void *stream) {
    if (!g || !offsets || (g->nnz > 0 && !coords) || !g->d_off || (g->K_lists > 0 && !g->d_coords)) {
        set_error("mcbgpu_gen_copy_lists: invalid arguments or no lists");
        return MCBGPU_E_ARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    MCB_CUDA(cudaMemcpyAsync(offsets, g->d_off, 8 * (size_t)(g->K_lists + 1), cudaMemcpyDeviceToHost, st));
    if (g->nnz > 0)
        MCB_CUDA(cudaMemcpyAsync(coords, g->d_coords, 4 * (size_t)g->nnz, cudaMemcpyDeviceToHost, st));
    MCB_CUDA(cudaStreamSynchronize(st));
    return MCBGPU_OK;
}

int mcbgpu_gen_release_trees(mcbgpu_gen *g) {
    if (!g) return MCBGPU_OK;
    cudaFree(g->d_pedge);
    g->d_pedge = nullptr;
    g->bytes -= 4ll * g->n * g->F;
    return MCBGPU_OK;
}

int mcbgpu_gen_tree_shapes(const mcbgpu_gen *g, int32_t *shapes, double *us_per_root, int32_t cap, int32_t *count,
                           int32_t *chosen) {
    if (!g || !count || !chosen || (cap > 0 && (!shapes || !us_per_root))) {
        set_error("mcbgpu_gen_tree_shapes: invalid arguments");
        return MCBGPU_E_ARG;
    }
    *count = (int32_t)g->shapes.size();
    *chosen = g->chosen;
    for (int32_t i = 0; i < cap && i < *count; i++) {
        shapes[3 * i] = g->shapes[(size_t)i].threads;
        shapes[3 * i + 1] = g->shapes[(size_t)i].ctas_per_sm;
        shapes[3 * i + 2] = g->shapes[(size_t)i].delta_quarters;
        us_per_root[i] = (size_t)i < g->shape_us.size() ? g->shape_us[(size_t)i] : -1.0;
    }
    return MCBGPU_OK;
}

int64_t mcbgpu_gen_device_bytes(const mcbgpu_gen *g) {
    return g ? g->bytes + 4 * (g->K * 3) + 8 * (g->K + 1) + 4 * g->nnz + 8 * g->cand_cap : 0;
}

int mcbgpu_gen_destroy(mcbgpu_gen *g) {
    if (g) gen_free(g);
    return MCBGPU_OK;
}

}  // extern "C"
