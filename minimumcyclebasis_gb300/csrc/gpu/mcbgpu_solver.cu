// Device-resident de Pina main loop (mcb/mcb_cycle_deg_two_remove.cpp:317-398).
//
// Data in HBM:
//   S       N rows x P words (P = ceil(N/64) rounded up to 4 words, 32-byte rows);
//           row j is the support vector S_j, which only ever has bits in [0, j]
//           (it starts as e_j and only earlier S_i are XORed into it).
//   cands   weight[K], off[K+1] (int64), coords[nnz] (int32, sorted ascending per
//           candidate) in the reference's rank order.  <C_r, S> = parity of S over
//           the coordinates of candidate r, which equals the reference's label test
//           S[e(u,v)] ^ P_t[u] ^ P_t[v] (include/cycles.h:144-195 builds the same set).
//
// Per-iteration form (select / cycle_vector / update):
//   search_kernel   S_e's prefix [0, e] is staged into shared memory by a TMA bulk
//                   copy; persistent CTAs take 1024-candidate tiles in rank order,
//                   compute each candidate's parity, and the first odd rank is found
//                   with a ballot per warp and an atomicMin across CTAs.  CTAs stop
//                   once their next tile starts above the best rank found.
//   update_kernel   one warp per row j > e: <C_e, S_j> by gathering S_j at C_e's
//                   coordinates, then S_j ^= S_e over the words of [0, e].
//
// Blocked form (64 iterations per pass; GF(2) arithmetic, so exact):
//   T[c] (64-bit) = bits S^0_{e0+k}[c], k < 64  — transpose of the block's rows
//   W_r = XOR of T over C_r's coordinates = <C_r, S^0_{e0+k}> for all 64 k at once
//   The candidate chosen at iteration e0+k is always one whose W_r is independent
//   of every earlier candidate's W (a "pivot"): if all earlier W's are even for the
//   current mask, so is anything in their span.  So one rank-ordered sweep finds the
//   first 64 pivots, the 64 iterations are then resolved on 64-bit masks, and every
//   later row S_j receives the block's combined update in one pass.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <utility>
#include <vector>

#include "mcbgpu_internal.cuh"

using namespace mcbgpu;

namespace {

constexpr int kTile = 1024;           // candidates per tile
constexpr int kHead = 8;              // coordinates of a list's head (one aligned 32-byte slot per candidate)
constexpr int kScanThreads = 256;     // 4 candidates per thread
constexpr int kPer = kTile / kScanThreads;
constexpr unsigned kSpinLimit = 1u << 24;
constexpr int kDiagWords = 48;  // counters of mcbgpu_solver_diagnostics (the pivot kernel's check area follows)
// Shape parameters of the blocked search; each can be overridden at build time
// (-DMCB_LMAX=... and so on) to sweep them.
#ifndef MCB_LMAX
#define MCB_LMAX 6
#endif
#ifndef MCB_WIN_TILES
#define MCB_WIN_TILES 6
#endif
#ifndef MCB_UPD_ROWS
#define MCB_UPD_ROWS 8
#endif
#ifndef MCB_W_CHUNK
#define MCB_W_CHUNK 8
#endif
#ifndef MCB_OTF_PAIRS
#define MCB_OTF_PAIRS 1  // pivot kernel: walk two candidates per thread together on the fly
#endif
#ifndef MCB_W_PREFETCH
#define MCB_W_PREFETCH 1  // streaming pass: bulk L2 prefetch of the CTA's next tile
#endif
#ifndef MCB_PIVOT_DIV
#define MCB_PIVOT_DIV 1  // pivot kernel grid = SM count / MCB_PIVOT_DIV
#endif
#ifndef MCB_GROUP
#define MCB_GROUP 2  // blocks per streaming pass (1..3); the later blocks' W by blk_wfix_kernel
#endif
#ifndef MCB_PAIR_MARGIN
#define MCB_PAIR_MARGIN 5  // percent more tiles per additional block of a grouped streaming pass
#endif
constexpr int kGroup = MCB_GROUP;
static_assert(kGroup >= 1 && kGroup <= 3, "MCB_GROUP must be 1, 2 or 3");
constexpr int kGStride = kGroup == 3 ? 4 : kGroup;  // words per coordinate in the grouped transpose
#ifndef MCB_UPD_SPLIT
#define MCB_UPD_SPLIT 1  // warps per row group in the block update (1, 2, 4 or 8)
#endif

#ifndef MCB_EARLY_WIN
#define MCB_EARLY_WIN 2  // window while the rank is below MCB_EARLY_RANK
#endif
#ifndef MCB_EARLY_RANK
#define MCB_EARLY_RANK 48
#endif
#ifndef MCB_TAIL_WIN
#define MCB_TAIL_WIN 8  // window once the rank is at least MCB_TAIL_RANK
#endif
#ifndef MCB_TAIL_RANK
#define MCB_TAIL_RANK 60
#endif
#ifndef MCB_PDL
#define MCB_PDL 1  // blocked run: critical-path kernels launched with programmatic stream serialisation
#endif
#ifndef MCB_MERGE_CHUNKED
#define MCB_MERGE_CHUNKED 0  // merge echelon by chunks of 32 with a table rebuild per chunk (1) or serially (0)
#endif
#ifndef MCB_MERGE_FAST
#define MCB_MERGE_FAST 1  // merge: skip the sort and echelon when no report lies below D
#endif
#ifndef MCB_LMAX_CAP
#define MCB_LMAX_CAP 8  // report slots per CTA and step: the largest local-pivot limit a shape may use
#endif
#ifndef MCB_WIN_CAP
#define MCB_WIN_CAP 12  // the largest window (tiles per CTA and step) a shape may use
#endif
constexpr int kLmax = MCB_LMAX_CAP;       // report slots per CTA and pivot step
constexpr int kWinTiles = MCB_WIN_TILES;  // tiles a CTA scans per pivot step (default shape)
static_assert(MCB_LMAX >= 1 && MCB_LMAX <= kLmax, "MCB_LMAX above MCB_LMAX_CAP");
static_assert(MCB_EARLY_WIN <= MCB_WIN_CAP && MCB_WIN_TILES <= MCB_WIN_CAP && MCB_TAIL_WIN <= MCB_WIN_CAP &&
                  MCB_WIN_CAP <= 32, "a window above MCB_WIN_CAP (at most 32)");

// The runtime shape of the blocked search (blk_pivot_kernel and the streaming pass's
// reach).  Every shape gives the same pivots (the search is exact for any window
// and local-pivot limit); only the time differs, by graph and by how far a solve has
// got, so a solver can time several on its own graph (mcbgpu_solver_tune).
struct PivotShape {
    int win_early, rank_early;  // tiles per CTA and step while fewer than rank_early pivots are known
    int win_mid;                // ... from rank_early on
    int rank_tail, win_tail;    // ... once rank_tail pivots are known
    int lmax;                   // local pivots after which a CTA ends its step (<= kLmax)
    int stream_pct;             // the streaming pass reaches this percent past the last block's last pivot
};
constexpr PivotShape kDefaultShape = {MCB_EARLY_WIN, MCB_EARLY_RANK, MCB_WIN_TILES, MCB_TAIL_RANK,
                                      MCB_TAIL_WIN,  MCB_LMAX,       25};
constexpr int kUpdRows = MCB_UPD_ROWS;    // rows per warp group in the block update (<= 32)
constexpr unsigned long long kNone = 0xFFFFFFFFFFFFFFFFull;
constexpr unsigned kNoIndex = 0xFFFFFFFFu;

// Kernel classes for the optional per-launch profile (events + algorithmic bytes).
enum KernelClass {
    KC_INIT, KC_TILE_MINC, KC_TRANSPOSE, KC_WSTREAM, KC_PIVOT,
    KC_BLK_UPDATE, KC_SEARCH, KC_UPDATE, KC_CYCLE, KC_RESET, KC_VALIDATE, KC_WFIX, KC_BLK_UPDATE_NEAR, KC_COUNT
};
const char *const kKernelNames[KC_COUNT] = {
    "init_identity", "tile_minc", "blk_transpose", "blk_w", "blk_pivot", "far_update", "search", "update",
    "cycle_vector", "reset_state", "validate", "blk_wfix", "near_update"};

struct IterSlot {            // state of one per-iteration search
    unsigned long long best; // first odd rank (kNone until found)
    unsigned next_tile;
    unsigned pad;
};

struct BlockState {
    unsigned rank, epoch, b;
    unsigned failed;               // a block ran out of candidates: every later block's kernels return at once
    long long last_pivot;          // rank of the previous block's last pivot
    long long pred_tiles;          // tiles the streaming pass computes for this block
    long long max_tile;            // deepest tile the previous block's pivot search touched
    unsigned long long total;      // running 64-bit total weight of the basis
    unsigned tail_ok, pad_;        // the pivot kernel's CTA 0 resolved the block
    long long pair_tiles;          // tiles the grouped streaming pass computed for the group's later blocks
    long long pivrank[64];
    unsigned long long pivW[64];   // the pivots' W as found (not reduced)
    unsigned long long mask[64];   // final S_{e0+k} as a combination of S^0_{e0+l}
    unsigned long long gcol[2][64];  // by block parity: gcol[k] bit i = <C_sel_k, S_{e0+i}>, i < k
};

// Grid barrier state of the cooperative pivot kernel (see grid_barrier).
struct GridBar {
    unsigned count, gen, abort, pad;
};

// ---------------------------------------------------------------------------
__global__ void init_identity_kernel(uint64_t *S, int N, int P) {
    size_t total = (size_t)N * P;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        int j = (int)(i / P), w = (int)(i % P);
        S[i] = (w == (j >> 6)) ? (1ull << (j & 63)) : 0ull;
    }
}

__global__ void reset_state_kernel(IterSlot *slots, BlockState *bs, unsigned *status) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        slots[0].best = kNone;
        slots[0].next_tile = 0;
        slots[1].best = kNone;
        slots[1].next_tile = 0;
        bs->total = 0;  // epoch keeps counting across runs: old tile marks never match
        bs->failed = 0;
        *status = 0;
    }
}

// Validates the uploaded candidate lists before any kernel indexes with them:
// offsets non-decreasing from 0 to nnz, coordinates strictly ascending inside each
// list and inside [0, N).  Records the longest list.  One thread per candidate.
__global__ void validate_kernel(const int64_t *__restrict__ off, const int32_t *__restrict__ coords, long long K,
                                long long nnz, int N, unsigned *bad, unsigned *max_len) {
    for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < K; r += (long long)gridDim.x * blockDim.x) {
        const int64_t b = off[r], e = off[r + 1];
        if (r == 0 && b != 0) atomicOr(bad, 1u);
        if (r == K - 1 && e != nnz) atomicOr(bad, 1u);
        if (e < b || b < 0 || e > nnz) {
            atomicOr(bad, 1u);
            continue;
        }
        int prev = -1;
        for (int64_t i = b; i < e; i++) {
            const int c = coords[i];
            if (c <= prev || c >= N) {
                atomicOr(bad, 2u);
                break;
            }
            prev = c;
        }
        if (e - b > 0) atomicMax(max_len, (unsigned)(e - b));
    }
}

// Smallest first coordinate per tile of 1024 candidates (lists are ascending, so a
// tile whose value is >= the block's bound has W = 0 for every candidate).
// head[r] = the first kHead coordinates of candidate r's list, INT_MAX past its end:
// one aligned 32-byte slot per candidate, read by the W walks before (and mostly
// instead of) the list itself.
__global__ void head_kernel(const int64_t *__restrict__ off, const int32_t *__restrict__ coords, long long K,
                            int32_t *head) {
    for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < K; r += (long long)gridDim.x * blockDim.x) {
        const int64_t a = off[r], e = off[r + 1];
        int v[kHead];
#pragma unroll
        for (int q = 0; q < kHead; q++) v[q] = a + q < e ? coords[a + q] : 0x7fffffff;
        int4 *h = reinterpret_cast<int4 *>(head + (size_t)r * kHead);
        h[0] = make_int4(v[0], v[1], v[2], v[3]);
        h[1] = make_int4(v[4], v[5], v[6], v[7]);
    }
}

__global__ void tile_minc_kernel(const int64_t *__restrict__ off, const int32_t *__restrict__ coords, long long K,
                                 int32_t *tile_minc, long long ntiles) {
    for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
        int m = 0x7fffffff;
        for (long long r = t * kTile + threadIdx.x; r < K && r < (t + 1) * kTile; r += blockDim.x)
            if (off[r + 1] > off[r]) m = min(m, coords[off[r]]);
        for (int d = 16; d > 0; d >>= 1) m = min(m, __shfl_xor_sync(0xffffffffu, m, d));
        __shared__ int sm[32];
        if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
        cta_sync();
        if (threadIdx.x == 0) {
            int v = sm[0];
            for (int w = 1; w < (int)(blockDim.x >> 5); w++) v = min(v, sm[w]);
            tile_minc[t] = v;
        }
        cta_sync();
    }
}

// ---------------------------------------------------------------------------
// Per-iteration search for the first candidate with <C_r, S_e> = 1.
__global__ void __launch_bounds__(kScanThreads) search_kernel(const uint64_t *__restrict__ Se, int e,
                                                              int words_even, const int64_t *__restrict__ off,
                                                              const int32_t *__restrict__ coords, long long K,
                                                              IterSlot *slot, unsigned *status,
                                                              unsigned long long *bytes) {
    unsigned long long nb = 0;
    extern __shared__ __align__(16) uint64_t s_S[];
    __shared__ uint64_t bar;
    __shared__ unsigned s_tile, s_go;
    __shared__ unsigned long long s_best;
    if (!stage_words_tma(s_S, Se, (uint32_t)words_even, &bar)) {
        if (threadIdx.x == 0) atomicOr(status, ST_WAIT_TIMEOUT);
        return;
    }
    const long long ntiles = (K + kTile - 1) / kTile;
    for (;;) {
        if (threadIdx.x == 0) {
            const unsigned t = atomicAdd(&slot->next_tile, 1u);
            // stop when out of tiles or when an earlier tile already found an odd one
            const unsigned long long gb = *((volatile unsigned long long *)&slot->best);
            s_tile = t;
            s_go = ((long long)t < ntiles && (unsigned long long)((long long)t * kTile) <= gb) ? 1u : 0u;
            s_best = kNone;
        }
        cta_sync();
        if (!s_go) break;
        const long long tile = s_tile;
        const long long r0 = tile * kTile;
        unsigned long long mine = kNone;
        for (int q = 0; q < kPer; q++) {
            long long r = r0 + q * kScanThreads + threadIdx.x;
            if (r >= K) break;
            int64_t b = off[r], en = off[r + 1];
            unsigned par = 0;
            nb += 8;
            for (int64_t i = b; i < en; i++) {
                int c = __ldg(coords + i);
                nb += 4;
                if (c > e) break;
                par ^= (unsigned)(s_S[c >> 6] >> (c & 63)) & 1u;
            }
            if (par) {
                mine = (unsigned long long)r;
                break;  // later q only give larger ranks
            }
        }
        // warp-level min of odd ranks, then CTA-level
        unsigned long long wmin = mine;
        for (int d = 16; d > 0; d >>= 1) {
            unsigned long long o = __shfl_xor_sync(0xffffffffu, wmin, d);
            wmin = o < wmin ? o : wmin;
        }
        if ((threadIdx.x & 31) == 0 && wmin != kNone) atomicMin(&s_best, wmin);
        cta_sync();
        if (threadIdx.x == 0 && s_best != kNone) atomicMin(&slot->best, s_best);
        cta_sync();
    }
    for (int d = 16; d > 0; d >>= 1) nb += __shfl_xor_sync(0xffffffffu, nb, d);
    if ((threadIdx.x & 31) == 0 && nb) atomicAdd(bytes, nb);
}

// One warp per row j in (e, N): if <C_e, S_j> is odd, S_j ^= S_e (words [0, e/64]).
// Block 0 also records the selection and resets the next iteration's slot.
__global__ void update_kernel(uint64_t *S, int N, int P, int e, const int64_t *__restrict__ off,
                              const int32_t *__restrict__ coords, const int32_t *__restrict__ weight,
                              IterSlot *slot, IterSlot *next_slot, long long *selected,
                              BlockState *bs, unsigned *status) {
    const unsigned long long r = *((volatile unsigned long long *)&slot->best);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        next_slot->best = kNone;
        next_slot->next_tile = 0;
        if (r == kNone) {
            atomicOr(status, ST_NO_CANDIDATE);
            selected[e] = -1;
        } else {
            selected[e] = (long long)r;
            bs->total += (unsigned long long)(long long)weight[r];
        }
    }
    if (r == kNone) return;
    const int64_t b = off[r], len = off[r + 1] - b;
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    const int we = (e >> 6) + 1;
    const uint64_t *Se = S + (size_t)e * P;
    for (int j = e + 1 + ((blockIdx.x * blockDim.x + threadIdx.x) >> 5); j < N; j += warps) {
        uint64_t *Sj = S + (size_t)j * P;
        unsigned par = 0;
        for (int64_t i = lane; i < len; i += 32) {
            int c = coords[b + i];
            par ^= (unsigned)(Sj[c >> 6] >> (c & 63)) & 1u;
        }
        par = __reduce_xor_sync(0xffffffffu, par);
        if (par)
            for (int w = lane; w < we; w += 32) Sj[w] ^= Se[w];
    }
}

// C_e of the selected candidate as a bit vector (include/cycles.h:144-195).
__global__ void cycle_vector_kernel(uint64_t *C, int W, const int64_t *__restrict__ off,
                                    const int32_t *__restrict__ coords, const IterSlot *slot) {
    const unsigned long long r = slot->best;
    for (int w = threadIdx.x; w < W; w += blockDim.x) C[w] = 0;
    cta_sync();
    if (r == kNone) return;
    for (int64_t i = off[r] + threadIdx.x; i < off[r + 1]; i += blockDim.x) {
        int c = coords[i];
        atomicOr((unsigned long long *)&C[c >> 6], 1ull << (c & 63));
    }
}

// ---------------------------------------------------------------------------
// Blocked form.
//
// blk_transpose_kernel: T[64w + i] bit k = S[e0+k] bit (64w+i), for w < Wb.
// One warp per word column; also resets the block state (runs first in the block).
// The first block of a group also writes Tg[kGStride c + j] for the grouped streaming
// pass: slot 0 = T[c], slot j = bit k of S[e0+64j+k] bit c (the group's j-th later
// block's bj rows as they are now), for words w < Wbj of that block.
// transpose_rows writes T[64w + i] (T may be NULL) and, with Tg, the same into
// Tg[kGStride (64w + i) + slot].
__device__ __forceinline__ void transpose_rows(const uint64_t *__restrict__ S, int P, int r0, int b, int Wb,
                                               uint64_t *__restrict__ T, uint64_t *__restrict__ Tg, int slot) {
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < Wb; w += warps) {
        uint64_t a = lane < b ? S[(size_t)(r0 + lane) * P + w] : 0ull;
        uint64_t c = (32 + lane) < b ? S[(size_t)(r0 + 32 + lane) * P + w] : 0ull;
        warp_transpose64(a, c);  // a: column 64w + lane, c: column 64w + 32 + lane
        if (T) {
            T[(size_t)w * 64 + lane] = a;
            T[(size_t)w * 64 + 32 + lane] = c;
        }
        if (Tg) {
            Tg[kGStride * ((size_t)w * 64 + lane) + slot] = a;
            Tg[kGStride * ((size_t)w * 64 + 32 + lane) + slot] = c;
        }
    }
}

__global__ void blk_transpose_kernel(const uint64_t *__restrict__ S, int P, int e0, int b, int Wb,
                                     uint64_t *__restrict__ T, BlockState *bs, long long ntiles,
                                     GridBar *gb, long long window_tiles, int stream_pct,
                                     uint64_t *__restrict__ Tg, int b1, int Wb1, int b2, int Wb2) {
    griddep_wait();
    griddep_launch();
    if (*(volatile const unsigned *)&bs->failed) {  // set by an earlier block's pivot kernel (same stream)
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            bs->pred_tiles = 0;  // the streaming pass and its correction then cover no tile
            bs->pair_tiles = 0;
        }
        return;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        gb->count = 0;
        gb->abort = 0;
        bs->rank = 0;
        bs->epoch = bs->epoch + 1;
        bs->b = (unsigned)b;
        // stream stream_pct percent past the previous block's deepest pivot; the
        // pivot kernel computes any further tile it needs
        long long pred = ntiles;
        if (e0 != 0) {
            const long long lp = bs->last_pivot + 1;
            const long long a = (lp + lp * stream_pct / 100) / kTile + 1, m = bs->max_tile + 1;
            pred = (a > m ? a : m) + window_tiles;
        }
        const int later = (b1 > 0 ? 1 : 0) + (b2 > 0 ? 1 : 0);  // the pass serves the group's later blocks too
        if (later > 0 && e0 != 0) pred += pred * MCB_PAIR_MARGIN * later / 100;
        bs->pred_tiles = pred < ntiles ? pred : ntiles;
        if (later > 0) bs->pair_tiles = bs->pred_tiles;  // read by the later blocks' blk_wfix_kernel
        bs->max_tile = 0;
    }
    transpose_rows(S, P, e0, b, Wb, T, b1 > 0 ? Tg : nullptr, 0);
    if (b1 > 0) transpose_rows(S, P, e0 + 64, b1, Wb1, nullptr, Tg, 1);
    if (b2 > 0) transpose_rows(S, P, e0 + 128, b2, Wb2, nullptr, Tg, 2);
}

// Reduce W by the basis held as Four-Russians tables: tab[g][pat] = XOR of the basis
// vectors whose pivot bits form `pat` within byte g (0 for non-pivot bits).
__device__ __forceinline__ uint64_t fr_reduce(uint64_t W, const uint64_t (*tab)[256]) {
    uint64_t r = W;
#pragma unroll
    for (int g = 0; g < 8; g++) r ^= tab[g][(W >> (8 * g)) & 255];
    return r;
}

// Build tab from the basis held in shared memory (rank vectors, pivot bits).
__device__ void fr_build(uint64_t (*tab)[256], const uint64_t *basis, const unsigned *pivbit, unsigned rank) {
    __shared__ uint64_t byBit[64];
    if (threadIdx.x < 64) byBit[threadIdx.x] = 0;
    cta_sync();
    for (unsigned q = threadIdx.x; q < rank; q += blockDim.x) byBit[pivbit[q] & 63] = basis[q];
    cta_sync();
    for (int idx = threadIdx.x; idx < 8 * 256; idx += blockDim.x) {
        int g = idx >> 8, pat = idx & 255;
        uint64_t v = 0;
        for (int i = 0; i < 8; i++)
            if (pat & (1 << i)) v ^= byBit[8 * g + i];
        tab[g][pat] = v;
    }
    cta_sync();
}

// ---- grid-wide barrier for the cooperative pivot kernel ----------------------
// All CTAs of a cooperative launch are co-resident.  The wait is bounded: after
// kSpinLimit polls a CTA raises `abort`, every waiter sees it and the kernel ends
// with ST_WAIT_TIMEOUT instead of hanging.

// Arrive: acq_rel add on the counter (releases this CTA's writes, and the last
// arriver acquires everyone's); the last arriver then releases `gen`, which the
// others acquire.  Lane 0 of warp 0 does the atomics and loads; the whole warp
// runs the wait loop together (values broadcast by shuffle), so it reaches the
// CTA barrier converged.  Lane 0 ends with an acquire fence and the CTA barrier
// carries the ordering to the other threads.
__device__ __forceinline__ unsigned atomic_add_acq_rel(unsigned *p, unsigned v) {
    unsigned old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

__device__ __forceinline__ void fence_acq_rel_gpu() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }

__device__ bool grid_barrier(GridBar *gb, unsigned nctas, unsigned &gen_local) {
    __shared__ unsigned s_ok;
    cta_sync();
    if (threadIdx.x < 32) {
        const unsigned lane = threadIdx.x;
        const unsigned g = gen_local;
        unsigned last = 0;
        if (lane == 0) {
            __threadfence();
            last = atomic_add_acq_rel(&gb->count, 1u) == nctas - 1;
            if (last) {
                atomicExch(&gb->count, 0u);
                __threadfence();
                st_release_u32(&gb->gen, g + 1);
            }
        }
        last = __shfl_sync(0xffffffffu, last, 0);
        unsigned ok = 1;
        if (!last) {
            for (unsigned spins = 0;; spins++) {
                unsigned cur = g, ab = 0;
                if (lane == 0) {
                    cur = ld_acquire_u32(&gb->gen);
                    ab = *((volatile unsigned *)&gb->abort);
                }
                cur = __shfl_sync(0xffffffffu, cur, 0);
                ab = __shfl_sync(0xffffffffu, ab, 0);
                if (cur != g) break;
                if (ab) {
                    ok = 0;
                    break;
                }
                if (spins > kSpinLimit) {
                    if (lane == 0) atomicExch(&gb->abort, 1u);
                    ok = 0;
                    break;
                }
                __nanosleep(20);
            }
        }
        __syncwarp();
        if (lane == 0) {
            fence_acq_rel_gpu();
            s_ok = ok;
        }
        gen_local = g + 1;
    }
    cta_sync();
    return s_ok != 0;
}

// W of one candidate: XOR of T over its coordinates below `bound`.  Coordinates
// are read kWChunk at a time (independent loads), then their T words are gathered
// (independent loads), so a list costs two memory round trips per kWChunk
// coordinates.  The list is ascending: a chunk whose last coordinate is >= bound
// ends the walk, and its coordinates >= bound gather nothing.  `nread` counts the
// coordinates read.
constexpr int kWChunk = MCB_W_CHUNK;
static_assert(kWChunk == kHead, "the first chunk of a W walk is the list's head");

// The first kHead coordinates of candidate r (INT_MAX past the end of its list), from
// the head array: consecutive candidates' heads are consecutive 32-byte slots, so a
// warp's first chunks are one coalesced read, and no offset is needed unless the
// list goes on below the bound.
__device__ __forceinline__ void load_head(const int32_t *__restrict__ head, long long r, int (&cv)[kHead]) {
    const int4 *h = reinterpret_cast<const int4 *>(head + (size_t)r * kHead);
    const int4 a = __ldg(h), b = __ldg(h + 1);
    cv[0] = a.x;
    cv[1] = a.y;
    cv[2] = a.z;
    cv[3] = a.w;
    cv[4] = b.x;
    cv[5] = b.y;
    cv[6] = b.z;
    cv[7] = b.w;
}

__device__ __forceinline__ uint64_t w_chunk(const int (&cv)[kWChunk], const uint64_t *__restrict__ T, int bound) {
    uint64_t tv[kWChunk];
#pragma unroll
    for (int q = 0; q < kWChunk; q++) tv[q] = cv[q] < bound ? __ldg(T + cv[q]) : 0ull;
    uint64_t W = 0;
#pragma unroll
    for (int q = 0; q < kWChunk; q++) W ^= tv[q];
    return W;
}

// W_r = XOR of T[c] over the coordinates c < bound of candidate r's list.  The head
// gives the first kHead coordinates; a list whose head ends below the bound goes on
// from its offset, kWChunk coordinates at a time (independent loads), then their T
// words (independent loads).  The list is ascending: a chunk whose last coordinate
// is >= bound ends the walk, and its coordinates >= bound gather nothing.  `nread`
// counts the 4-byte words read (head, offsets, further coordinates).
__device__ __forceinline__ uint64_t w_of_candidate(long long r, const int64_t *__restrict__ off,
                                                   const int32_t *__restrict__ coords,
                                                   const int32_t *__restrict__ head,
                                                   const uint64_t *__restrict__ T, int bound, unsigned &nread) {
    int cv[kWChunk];
    load_head(head, r, cv);
    uint64_t W = w_chunk(cv, T, bound);
    nread += kHead;
    if (cv[kHead - 1] < bound) {
        int64_t i = __ldg(off + r) + kHead;
        const int64_t e = __ldg(off + r + 1);
        nread += 2;
        while (i < e) {
#pragma unroll
            for (int q = 0; q < kWChunk; q++) cv[q] = i + q < e ? __ldg(coords + i + q) : 0x7fffffff;
            W ^= w_chunk(cv, T, bound);
            nread += (unsigned)(e - i < kWChunk ? e - i : kWChunk);
            if (cv[kWChunk - 1] >= bound) break;
            i += kWChunk;
        }
    }
    return W;
}

// W of two candidates walked in lockstep (their loads overlap); rb < 0: only ra.
__device__ __forceinline__ void w_of_two(long long ra, long long rb, const int64_t *__restrict__ off,
                                         const int32_t *__restrict__ coords, const int32_t *__restrict__ head,
                                         const uint64_t *__restrict__ T, int bound, unsigned &nread, uint64_t &Wa,
                                         uint64_t &Wb) {
    int ca[kWChunk], cb[kWChunk];
    load_head(head, ra, ca);
    if (rb >= 0) {
        load_head(head, rb, cb);
    } else {
#pragma unroll
        for (int q = 0; q < kWChunk; q++) cb[q] = 0x7fffffff;
    }
    Wa = w_chunk(ca, T, bound);
    Wb = w_chunk(cb, T, bound);
    nread += rb >= 0 ? 2 * kHead : kHead;
    int64_t ia = 0, ea = 0, ib = 0, eb = 0;
    if (ca[kHead - 1] < bound) {
        ia = __ldg(off + ra) + kHead;
        ea = __ldg(off + ra + 1);
        nread += 2;
    }
    if (rb >= 0 && cb[kHead - 1] < bound) {
        ib = __ldg(off + rb) + kHead;
        eb = __ldg(off + rb + 1);
        nread += 2;
    }
    while (ia < ea || ib < eb) {
#pragma unroll
        for (int q = 0; q < kWChunk; q++) {
            ca[q] = ia + q < ea ? __ldg(coords + ia + q) : 0x7fffffff;
            cb[q] = ib + q < eb ? __ldg(coords + ib + q) : 0x7fffffff;
        }
        Wa ^= w_chunk(ca, T, bound);
        Wb ^= w_chunk(cb, T, bound);
        if (ia < ea) nread += (unsigned)(ea - ia < kWChunk ? ea - ia : kWChunk);
        if (ib < eb) nread += (unsigned)(eb - ib < kWChunk ? eb - ib : kWChunk);
        ia = ca[kWChunk - 1] >= bound ? ea : ia + kWChunk;
        ib = cb[kWChunk - 1] >= bound ? eb : ib + kWChunk;
    }
}

// W of one candidate for the kG blocks of a group at once: W[0] against this block's
// rows (coordinates below bd[0]), W[j] against the group's j-th later block's rows as
// they are now (below bd[j], ascending), one walk of the list (head first); Tg holds
// kGStride words per coordinate (one 16- or 32-byte gather).
template <int kG>
__device__ __forceinline__ void w_group_chunk(const int (&cv)[kWChunk], const uint64_t *__restrict__ Tg,
                                              const int (&bd)[3], uint64_t (&W)[kG]) {
    const int last = bd[kG - 1];
    uint64_t tv[kWChunk][kG];
#pragma unroll
    for (int q = 0; q < kWChunk; q++) {
        const bool in = cv[q] < last;
        const ulonglong2 t01 = in ? __ldg(reinterpret_cast<const ulonglong2 *>(Tg + (size_t)kGStride * cv[q]))
                                  : make_ulonglong2(0ull, 0ull);
        tv[q][0] = cv[q] < bd[0] ? t01.x : 0ull;
        tv[q][1] = cv[q] < bd[1] ? t01.y : 0ull;
        if (kG == 3) {
            const ulonglong2 t23 = in ? __ldg(reinterpret_cast<const ulonglong2 *>(Tg + (size_t)kGStride * cv[q] + 2))
                                      : make_ulonglong2(0ull, 0ull);
            tv[q][kG - 1] = t23.x;
        }
    }
#pragma unroll
    for (int q = 0; q < kWChunk; q++)
#pragma unroll
        for (int g = 0; g < kG; g++) W[g] ^= tv[q][g];
}

template <int kG>
__device__ __forceinline__ void w_of_group(long long r, const int64_t *__restrict__ off,
                                           const int32_t *__restrict__ coords, const int32_t *__restrict__ head,
                                           const uint64_t *__restrict__ Tg, const int (&bd)[3], unsigned &nread,
                                           uint64_t (&W)[kG]) {
    const int last = bd[kG - 1];
#pragma unroll
    for (int g = 0; g < kG; g++) W[g] = 0;
    int cv[kWChunk];
    load_head(head, r, cv);
    w_group_chunk<kG>(cv, Tg, bd, W);
    nread += kHead;
    if (cv[kHead - 1] < last) {
        int64_t i = __ldg(off + r) + kHead;
        const int64_t e = __ldg(off + r + 1);
        nread += 2;
        while (i < e) {
#pragma unroll
            for (int q = 0; q < kWChunk; q++) cv[q] = i + q < e ? __ldg(coords + i + q) : 0x7fffffff;
            w_group_chunk<kG>(cv, Tg, bd, W);
            nread += (unsigned)(e - i < kWChunk ? e - i : kWChunk);
            if (cv[kWChunk - 1] >= last) break;
            i += kWChunk;
        }
    }
}

// Streaming pass: W for tiles [0, bs->pred_tiles), one candidate per thread (1024
// threads = one tile per CTA pass), written to Warr and tagged with the block's
// epoch.  This is the bandwidth-bound part of the block's search.
#ifndef MCB_W_MINB
#define MCB_W_MINB 1  // resident 1024-thread CTAs per SM the W pass is compiled for
#endif
// kG > 1 (the first block of a group): also W against each later block's rows as
// they are now (Tg, bounds bd[1..]) into Wl[0..kG-2], for blk_wfix_kernel.
template <int kG>
__global__ void __launch_bounds__(kTile, MCB_W_MINB) blk_w_kernel(long long K, const int64_t *__restrict__ off,
                                                    const int32_t *__restrict__ coords,
                                                    const int32_t *__restrict__ head,
                                                    const int32_t *__restrict__ tile_minc,
                                                    const uint64_t *__restrict__ T, int bound, const BlockState *bs,
                                                    uint64_t *Warr, unsigned *tile_epoch, unsigned long long *bytes,
                                                    const uint64_t *__restrict__ Tg, int bound1, int bound2,
                                                    uint64_t *Wl1, uint64_t *Wl2) {
    griddep_wait();
    griddep_launch();
    const unsigned epoch = bs->epoch;
    const long long ntiles = bs->pred_tiles;
    unsigned long long nb = (blockIdx.x == 0 && threadIdx.x == 0) ? 8ull * (unsigned long long)bound : 0ull;
    if (kG > 1) {
        const int bd[3] = {bound, bound1, bound2};
        const int last = bd[kG - 1];
        for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
#if MCB_W_PREFETCH
            if (threadIdx.x == 0 && t + gridDim.x < ntiles) {  // this CTA's next tile's heads into L2
                const long long r0 = (t + gridDim.x) * kTile, r1 = min(r0 + kTile, K);
                if (r0 < r1) prefetch_l2(head + (size_t)r0 * kHead, 4ull * kHead * (unsigned long long)(r1 - r0));
            }
#endif
            if (tile_minc[t] >= last) {  // every W of the tile is 0
                if (threadIdx.x == 0) nb += 8;
                continue;
            }
            const long long r = t * kTile + threadIdx.x;
            uint64_t W[kG];
#pragma unroll
            for (int g = 0; g < kG; g++) W[g] = 0;
            unsigned nread = 0;
            if (r < K) {
                w_of_group<kG>(r, off, coords, head, Tg, bd, nread, W);
                nb += 8ull * kG + 4ull * nread;  // kG W writes, head / offsets / coordinates read
            }
            Warr[r] = W[0];
            Wl1[r] = W[1];
            if (kG == 3) Wl2[r] = W[kG - 1];
        }
        for (long long t = blockIdx.x + (long long)threadIdx.x * gridDim.x; t < ntiles;
             t += (long long)blockDim.x * gridDim.x)
            tile_epoch[t] = (epoch << 1) | (tile_minc[t] >= bound ? 1u : 0u);
        for (int d = 16; d > 0; d >>= 1) nb += __shfl_xor_sync(0xffffffffu, nb, d);
        if ((threadIdx.x & 31) == 0 && nb) atomicAdd(bytes, nb);
        return;
    }
    // no barrier per tile: a thread moves on to its next tile as soon as its own
    // candidate is done; the tags (read only by the next kernel) are written at the end
    for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
        if (tile_minc[t] >= bound) {  // every W of the tile is 0: nothing to write
            if (threadIdx.x == 0) nb += 8;
            continue;
        }
        const long long r = t * kTile + threadIdx.x;
        uint64_t W = 0;
        unsigned nread = 0;
        if (r < K) {
            W = w_of_candidate(r, off, coords, head, T, bound, nread);
            nb += 8 + 4ull * nread;  // W write, head / offsets / coordinates read
        }
        Warr[r] = W;
    }
    for (long long t = blockIdx.x + (long long)threadIdx.x * gridDim.x; t < ntiles; t += (long long)blockDim.x * gridDim.x)
        tile_epoch[t] = (epoch << 1) | (tile_minc[t] >= bound ? 1u : 0u);
    for (int d = 16; d > 0; d >>= 1) nb += __shfl_xor_sync(0xffffffffu, nb, d);
    if ((threadIdx.x & 31) == 0 && nb) atomicAdd(bytes, nb);
}

// A later block of a group (the j-th, j = kJ): W of every candidate the grouped pass
// covered.  Wout holds W against this block's rows as they were before the group's
// first kJ blocks updated them.  Block i of the group (i < kJ) added to this
// block's row r the combination gamma_ir = XOR_{k in beta_ir} m_ik of block i's
// starting rows (beta_ir: row r's update bits in block i, written by block i's near
// update; m_ik: block i's final masks), so bit r of W gains parity(W_i & gamma_ir),
// with W_i = block i's W (Win[i]).  Each of these 64x64 GF(2) products is applied
// through eight 256-entry tables.  Block kJ - 1's masks are read from the block
// state and kept in masks[kJ - 1] for the group's next block.
template <int kJ>
__global__ void __launch_bounds__(kTile) blk_wfix_kernel(const int32_t *__restrict__ tile_minc, int bound,
                                                         BlockState *bs, const uint64_t *__restrict__ beta,
                                                         uint64_t *masks, int b, uint64_t *Win0, uint64_t *Win1,
                                                         uint64_t *Wout, unsigned *tile_epoch,
                                                         unsigned long long *bytes) {
    __shared__ uint64_t s_m[64], s_g[64], s_col[64];
    __shared__ uint64_t s_tab[kJ][8][256];
    griddep_wait();
    griddep_launch();
    const unsigned epoch = bs->epoch;
    const long long ntiles = bs->pair_tiles;
    const int tid = threadIdx.x;
    for (int i = 0; i < kJ; i++) {
        // block i's masks: the block state holds block kJ - 1's; earlier ones were kept
        if (tid < 64) {
            const uint64_t mk = i == kJ - 1 ? bs->mask[tid] : masks[i * 64 + tid];
            s_m[tid] = mk;
            if (i == kJ - 1 && blockIdx.x == 0) masks[i * 64 + tid] = mk;
        }
        cta_sync();
        if (tid < 64) {  // beta of this block's row tid in block i: near rows of block i start
            uint64_t g = 0;  // at block i + 1, so this block's rows sit (kJ - 1 - i) blocks in
            if (tid < b)
                for (uint64_t bb = beta[i * 192 + (kJ - 1 - i) * 64 + tid]; bb; bb &= bb - 1)
                    g ^= s_m[__ffsll((long long)bb) - 1];
            s_g[tid] = g;
        }
        cta_sync();
        if (tid < 32) {  // col_t bit r = bit t of gamma_r: a 64x64 bit transpose (warp 0)
            uint64_t g0 = s_g[tid], g1 = s_g[tid + 32];
            warp_transpose64(g0, g1);
            s_col[tid] = g0;
            s_col[tid + 32] = g1;
        }
        if (tid < 8) s_tab[i][tid][0] = 0;
        cta_sync();
        // tab[g][v] for v in [2^u, 2^(u+1)) = tab[g][v - 2^u] ^ col[8g + u]
        for (int u = 0; u < 8; u++) {
            const int n = 8 << u;  // 8 groups x 2^u entries
            for (int idx = tid; idx < n; idx += blockDim.x) {
                const int grp = idx >> u, v = (1 << u) + (idx & ((1 << u) - 1));
                s_tab[i][grp][v] = s_tab[i][grp][v - (1 << u)] ^ s_col[grp * 8 + u];
            }
            cta_sync();
        }
    }
    unsigned long long nb = 0;
    // four tiles per pass: their loads are in flight together
    constexpr int kU = 4;
    for (long long t0 = blockIdx.x; t0 < ntiles; t0 += (long long)kU * gridDim.x) {
        uint64_t w0[kU], w1[kU], x[kU];
        bool live[kU];
#pragma unroll
        for (int u = 0; u < kU; u++) {
            const long long t = t0 + (long long)u * gridDim.x;
            live[u] = t < ntiles && tile_minc[t] < bound;  // else W = 0 for the whole tile: tagged below
            const long long r = t * kTile + tid;
            w0[u] = live[u] ? Win0[r] : 0ull;
            w1[u] = live[u] && kJ > 1 ? Win1[r] : 0ull;
            x[u] = live[u] ? Wout[r] : 0ull;
        }
#pragma unroll
        for (int u = 0; u < kU; u++) {
            if (!live[u]) continue;
#pragma unroll
            for (int grp = 0; grp < 8; grp++) x[u] ^= s_tab[0][grp][(w0[u] >> (8 * grp)) & 255];
            if (kJ > 1) {
#pragma unroll
                for (int grp = 0; grp < 8; grp++) x[u] ^= s_tab[kJ - 1][grp][(w1[u] >> (8 * grp)) & 255];
            }
            Wout[(t0 + (long long)u * gridDim.x) * kTile + tid] = x[u];
            nb += 16 + 8ull * kJ;
        }
    }
    for (long long t = blockIdx.x + (long long)tid * gridDim.x; t < ntiles; t += (long long)blockDim.x * gridDim.x)
        tile_epoch[t] = (epoch << 1) | (tile_minc[t] >= bound ? 1u : 0u);
    for (int d = 16; d > 0; d >>= 1) nb += __shfl_xor_sync(0xffffffffu, nb, d);
    if ((tid & 31) == 0 && nb) atomicAdd(bytes, nb);
}

// Cooperative pivot extraction, several pivots per grid barrier.
//
// Definitions: B = the pivots found so far (a reduced row-echelon basis, held by
// every CTA as Four-Russians tables); s = scan start: every candidate before s has
// its W in span(B).  A pivot is a candidate whose W is not in the span of all
// earlier W's.
//
// Step, part 1 (no communication): CTA c scans its own tiles t = c (mod G) from s
// on, up to the shape's window of them.  It keeps a local basis B ∪ L_c and, in rank
// order, turns every candidate whose residual against B ∪ L_c is non-zero into a
// local pivot (appended to L_c).  It stops early after the shape's lmax local
// pivots.  It reports
// its local pivots (rank, W) and `end`: every candidate of its tiles below `end`
// has been processed.
// Part 2, after one grid barrier, in every CTA identically: D = min over CTAs of
// `end`.  Every candidate z below D is in span(B ∪ L_c' before z) for its CTA c',
// so span(W's below r) = span(B ∪ reported local pivots below r) for any r <= D.
// Hence the global pivots below D are exactly the reported local pivots below D
// that, taken in rank order, are not in the span of B and the ones accepted
// before them.  Accept them that way (first non-zero residual against the global
// tables, add, repeat), then s = D.
// The reductions below leave one value per warp in a shared slot array (plain
// stores by lane 0, no shared atomics) and every thread combines the slots after
// the barrier.  A caller must pass a barrier between reading one call's slots and
// the next call that writes the same slots.
constexpr int kPivotThreads = 512;        // threads of a pivot-kernel CTA
constexpr int kWarps = kPivotThreads / 32;
constexpr int kWinMax = MCB_WIN_CAP;  // largest window
constexpr int kWinW = kWinMax * kTile;  // W's the window buffer holds

__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long v) {
    for (int d = 16; d > 0; d >>= 1) {
        const unsigned long long o = __shfl_xor_sync(0xffffffffu, v, d);
        v = o < v ? o : v;
    }
    return v;
}

// Minimum over the CTA (every thread gets it).
__device__ __forceinline__ unsigned long long block_min_u64(unsigned long long v, unsigned long long *slots) {
    v = warp_min_u64(v);
    if ((threadIdx.x & 31) == 0) slots[threadIdx.x >> 5] = v;
    cta_sync();
    unsigned long long m = slots[0];
#pragma unroll
    for (int w = 1; w < kWarps; w++) m = slots[w] < m ? slots[w] : m;
    return m;
}

// Adds v (already reduced against the basis, v != 0) to an RREF basis held as
// vectors + pivot bits + Four-Russians tables.  Called by the whole CTA; `slots`
// holds kWarps words.
__device__ void basis_add(uint64_t (*tab)[256], uint64_t *basis, unsigned *piv, int &rank, uint64_t v,
                          unsigned long long *slots) {
    const unsigned qb = (unsigned)(__ffsll((long long)v) - 1) & 63u;
    const bool mine = threadIdx.x < (unsigned)rank && ((basis[threadIdx.x] >> qb) & 1ull);
    unsigned long long m = mine ? (1ull << (piv[threadIdx.x] & 63u)) : 0ull;
    for (int d = 16; d > 0; d >>= 1) m |= __shfl_xor_sync(0xffffffffu, m, d);
    if ((threadIdx.x & 31) == 0) slots[threadIdx.x >> 5] = m;
    cta_sync();
    unsigned long long chg = 1ull << qb;
#pragma unroll
    for (int w = 0; w < kWarps; w++) chg |= slots[w];
    for (int idx = threadIdx.x; idx < 8 * 256; idx += blockDim.x) {
        const int g = idx >> 8, pat = idx & 255;
        if (__popc(pat & (unsigned)((chg >> (8 * g)) & 255)) & 1) (&tab[0][0])[idx] ^= v;
    }
    if (mine) basis[threadIdx.x] ^= v;
    if (threadIdx.x == 0 && rank < 64) {
        basis[rank] = v;
        piv[rank] = qb;
    }
    rank++;
    cta_sync();
}

// First window position p in [from, valid) whose W has a non-zero residual against
// tab, or kNoIndex.  Window positions are in rank order.  `slots` holds kWarps words.
__device__ unsigned window_first_nonzero(const uint64_t *win, const uint64_t (*tab)[256], unsigned from,
                                         unsigned valid, unsigned *slots) {
    unsigned best = kNoIndex;
    for (unsigned base = from & ~(unsigned)(kPivotThreads - 1); base < valid; base += kPivotThreads) {
        const unsigned p = base + threadIdx.x;
        const bool nz = p >= from && p < valid && fr_reduce(win[p], tab) != 0;
        const unsigned bal = __ballot_sync(0xffffffffu, nz);
        if (bal) {  // warp-uniform: this warp's first hit
            best = base + (threadIdx.x & ~31u) + (unsigned)(__ffs(bal) - 1);
            break;
        }
    }
    if ((threadIdx.x & 31) == 0) slots[threadIdx.x >> 5] = best;
    cta_sync();
    unsigned r = slots[0];
#pragma unroll
    for (int w = 1; w < kWarps; w++) r = slots[w] < r ? slots[w] : r;
    return r;
}

// Index of the j-th set bit of a window mask.
__device__ __forceinline__ int nth_bit(unsigned mask, unsigned j) {
    for (unsigned q = 0; q < j; q++) mask &= mask - 1;
    return __ffs(mask) - 1;
}

// ---- block tail, run inside the pivot kernel after its last step -------------
struct TailArgs {
    uint64_t *S;
    long long *selected;
    const int32_t *weight;
    unsigned *pairs, *sorted, *word_end;
    unsigned pair_cap;
    int P, e0, Wb;
    int par;  // block parity: which gcol / sorted pairs to write
};

// Named CTA barrier 1 over the warps 1.. of the CTA (warp 0 is busy elsewhere);
// non-aligned form, like cta_sync.
__device__ __forceinline__ void helpers_sync(unsigned nthreads) {
    asm volatile("barrier.sync 1, %0;" ::"r"(nthreads) : "memory");
}

// Resolve the block's b iterations on masks (one CTA of at least 64 + 32 threads).
// Pivot index = rank order.  m_k starts as e_k; iteration k takes the first pivot p
// with <W_p, m_k> odd; every later m_j with <W_p, m_j> odd gets m_j ^= m_k (the
// reference's update restricted to the block, mcb/mcb_cycle_deg_two_remove.cpp:371-390).
// Warp 0 runs the b sequential steps.  The selected cycles are the b pivots in some
// order, so meanwhile the other warps gather the pivots' coordinates into (coordinate,
// pivot) pairs and sort them by S word (counting sort; word_end[w] = number of pairs
// whose word is below w).  At the end the pivot index of every pair is replaced by
// the iteration that selected it.  `hist` is shared scratch of P + 1 words.  Returns
// false (and sets a status bit) if the block cannot be resolved.
#ifdef MCB_TAIL_PROFILE
__device__ unsigned long long g_tail_prof[8];
#define TAIL_STAMP(i) \
    do { \
        if (threadIdx.x == 0 || threadIdx.x == 32) atomicAdd(&g_tail_prof[i], (unsigned long long)(clock64() - t_start)); \
    } while (0)
#else
#define TAIL_STAMP(i) \
    do { \
    } while (0)
#endif

__device__ bool resolve_block(BlockState *bs, int rank, const int64_t *__restrict__ off,
                              const int32_t *__restrict__ coords, const TailArgs &ta, unsigned *hist,
                              unsigned *status) {
#ifdef MCB_TAIL_PROFILE
    const long long t_start = clock64();
#endif
    const int e0 = ta.e0, P = ta.P;
    const int32_t *__restrict__ weight = ta.weight;
    unsigned *pairs = ta.pairs, *sorted = ta.sorted, *word_end = ta.word_end;
    const unsigned pair_cap = ta.pair_cap;
    __shared__ uint64_t s_w[64];
    __shared__ long long s_r[64];
    __shared__ int s_sel[64], s_kof[64];
    __shared__ int64_t s_beg[64];
    __shared__ unsigned s_pre[65];
    __shared__ unsigned s_part[32];
    __shared__ unsigned s_fail;
    const int tid = threadIdx.x, lane = tid & 31;
    const int b = (int)bs->b;
    if (rank < b) {
        if (tid == 0) atomicOr(status, ST_RANK_DEFICIT);
        return false;
    }
    if (tid < 64) {
        s_w[tid] = tid < b ? bs->pivW[tid] : 0ull;
        s_r[tid] = tid < b ? bs->pivrank[tid] : -1;
        s_kof[tid] = 0;
    }
    if (tid == 0) s_fail = 0;
    cta_sync();
    TAIL_STAMP(0);
    if (tid < 32) {
        // A[j][p] = <m_j, W_p> as 64 rows of 64 bits, lane l holding rows l and l + 32;
        // m_j = e_j at the start, so A is the bit transpose of the W's.  Iteration k:
        // p_k = the first unused p with A[k][p] = 1; every later row j with
        // A[j][p_k] = 1 takes row k (m_j ^= m_k, and A[j] ^= A[k] with it).  Rows
        // i < k are final, so gcol[k] bit i = A[i][p_k].
        uint64_t a0 = s_w[lane], a1 = s_w[32 + lane];
        warp_transpose64(a0, a1);  // row j of A = bit j of every W
        // The loop carries only what the next iteration needs (row k + 1 after this
        // iteration's XORs); the selections stay in the lane of their iteration and
        // gcol is read off the final rows afterwards.
        uint64_t m0 = 1ull << lane, m1 = 1ull << (32 + lane);
        uint64_t used = 0;
        int psel0 = 0, psel1 = 0;  // lane l: the pivots of iterations l and l + 32
        bool fail = false;
        for (int k = 0; k < b; k++) {
            const uint64_t ak = __shfl_sync(0xffffffffu, k < 32 ? a0 : a1, k & 31);
            const uint64_t mk = __shfl_sync(0xffffffffu, k < 32 ? m0 : m1, k & 31);
            const uint64_t cand = ak & ~used;
            if (!cand) {  // warp-uniform
                fail = true;
                break;
            }
            const int p = __ffsll((long long)cand) - 1;
            used |= 1ull << p;
            if (lane == (k & 31)) {
                if (k < 32)
                    psel0 = p;
                else
                    psel1 = p;
            }
            const bool h0 = (a0 >> p) & 1ull, h1 = (a1 >> p) & 1ull;
            if (lane > k && h0) {
                a0 ^= ak;
                m0 ^= mk;
            }
            if (32 + lane > k && h1) {
                a1 ^= ak;
                m1 ^= mk;
            }
        }
        if (fail) {
            if (lane == 0) s_fail = 1;
        } else {
            // rows i < k do not change after iteration i, so gcol[k] bit i = A[i][p_k] of
            // the final rows: column c of A (lane c & 31 keeps columns c and c + 32),
            // then iteration k (lane k & 31) fetches column p_k
            uint64_t col0 = a0, col1 = a1;
            warp_transpose64(col0, col1);
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int k = lane + 32 * h;
                const int p = h ? psel1 : psel0;
                const uint64_t c0 = __shfl_sync(0xffffffffu, col0, p & 31);
                const uint64_t c1 = __shfl_sync(0xffffffffu, col1, p & 31);
                if (k < b) {
                    s_sel[k] = p;
                    s_kof[p] = k;
                    bs->gcol[ta.par][k] = (p < 32 ? c0 : c1) & ((1ull << k) - 1ull);
                }
            }
        }
        bs->mask[lane] = m0;
        bs->mask[32 + lane] = m1;
        TAIL_STAMP(1);
    } else {
        // warps 1..: the pivots' (coordinate, pivot) pairs, sorted by S word
        const unsigned nh = blockDim.x - 32, t = tid - 32;
        const unsigned nw = (unsigned)P + 1;
        for (unsigned w = t; w < nw; w += nh) hist[w] = 0;
        unsigned long long wsum = 0;
        if (t < 64) {
            unsigned len = 0;
            if ((int)t < b) {
                const long long r = s_r[t];
                s_beg[t] = off[r];
                len = (unsigned)(off[r + 1] - off[r]);
                wsum = (unsigned long long)(long long)weight[r];
            }
            unsigned incl = len;
            for (int d = 1; d < 32; d <<= 1) {
                const unsigned v = __shfl_up_sync(0xffffffffu, incl, d);
                if (lane >= d) incl += v;
            }
            s_pre[t + 1] = incl;  // per-warp inclusive; fixed up below
            for (int d = 16; d > 0; d >>= 1) wsum += __shfl_xor_sync(0xffffffffu, wsum, d);
            if (lane == 0) atomicAdd(&bs->total, wsum);
        }
        helpers_sync(nh);
        if (t == 0) {
            s_pre[0] = 0;
            const unsigned carry = s_pre[32];
            for (int i = 33; i <= 64; i++) s_pre[i] += carry;
            const unsigned total = s_pre[64];
            if (total > pair_cap) atomicOr(status, ST_BAD_INPUT);
        }
        helpers_sync(nh);
        const unsigned total = s_pre[64] < pair_cap ? s_pre[64] : pair_cap;
        for (unsigned i = t; i < total; i += nh) {
            int lo = 0, hi = b - 1;  // last pivot with s_pre[p] <= i
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (s_pre[mid] <= i)
                    lo = mid;
                else
                    hi = mid - 1;
            }
            const unsigned c = (unsigned)coords[s_beg[lo] + (i - s_pre[lo])];
            pairs[i] = (c << 6) | (unsigned)lo;
            atomicAdd(&hist[c >> 6], 1u);
        }
        helpers_sync(nh);
        TAIL_STAMP(2);
        {
            const unsigned per = (nw + nh - 1) / nh;
            const unsigned a = t * per < nw ? t * per : nw, z = a + per < nw ? a + per : nw;
            unsigned sum = 0;
            for (unsigned w = a; w < z; w++) sum += hist[w];
            unsigned incl = sum;
            for (int d = 1; d < 32; d <<= 1) {
                const unsigned v = __shfl_up_sync(0xffffffffu, incl, d);
                if (lane >= d) incl += v;
            }
            if (lane == 31) s_part[t >> 5] = incl;
            helpers_sync(nh);
            unsigned run = incl - sum;
            for (int x = 0; x < (int)(t >> 5); x++) run += s_part[x];
            for (unsigned w = a; w < z; w++) {
                const unsigned h = hist[w];
                hist[w] = run;
                word_end[w] = run;
                run += h;
            }
        }
        helpers_sync(nh);
        for (unsigned i = t; i < total; i += nh) {
            const unsigned pr = pairs[i];
            sorted[atomicAdd(&hist[pr >> 12], 1u)] = pr;
        }
        TAIL_STAMP(3);
    }
    cta_sync();
    TAIL_STAMP(4);
    if (s_fail) {
        if (tid == 0) atomicOr(status, ST_NO_CANDIDATE);
        return false;
    }
    // selections, and the iteration of every sorted pair in place of its pivot
    if (tid < b) {
        ta.selected[e0 + tid] = s_r[s_sel[tid]];
    }
    const unsigned total = s_pre[64] < pair_cap ? s_pre[64] : pair_cap;
    for (unsigned i = tid; i < total; i += blockDim.x) {
        const unsigned pr = sorted[i];
        sorted[i] = (pr & ~63u) | (unsigned)s_kof[pr & 63u];
    }
    TAIL_STAMP(5);
    return true;
}

// S_{e0+k} := XOR of S^0_{e0+l} over l in mask[k], in place, words [0, Wb): the
// block's final rows, which every later row update XORs in directly.  Column groups
// of kMatCols words, group cg handled by CTA cg mod G; `buf` is shared scratch of
// 64 x (kMatCols + 1) words.
#ifndef MCB_MAT_COLS
#define MCB_MAT_COLS 8
#endif
constexpr int kMatCols = MCB_MAT_COLS;

__device__ void materialize_rows(const TailArgs &ta, const BlockState *bs, int b, uint64_t *buf) {
    uint64_t(*s0)[kMatCols + 1] = reinterpret_cast<uint64_t(*)[kMatCols + 1]>(buf);
    __shared__ uint64_t sm[64];
    if (threadIdx.x < 64) sm[threadIdx.x] = (int)threadIdx.x < b ? bs->mask[threadIdx.x] : 0ull;
    const int Wb = ta.Wb, P = ta.P, e0 = ta.e0;
    const int ng = (Wb + kMatCols - 1) / kMatCols;
    for (int cg = blockIdx.x; cg < ng; cg += gridDim.x) {
        const int w0 = cg * kMatCols;
        cta_sync();  // the masks are in place; the previous group's rows are read
        for (int idx = threadIdx.x; idx < 64 * kMatCols; idx += blockDim.x) {
            const int l = idx / kMatCols, w = idx % kMatCols;
            s0[l][w] = (l < b && w0 + w < Wb) ? ta.S[(size_t)(e0 + l) * P + w0 + w] : 0ull;
        }
        cta_sync();
        for (int idx = threadIdx.x; idx < 64 * kMatCols; idx += blockDim.x) {
            const int k = idx / kMatCols, w = idx % kMatCols;
            if (k < b && w0 + w < Wb) {
                uint64_t acc = 0;
                for (uint64_t m = sm[k]; m; m &= m - 1) acc ^= s0[__ffsll((long long)m) - 1][w];
                ta.S[(size_t)(e0 + k) * P + w0 + w] = acc;
            }
        }
    }
}

#ifdef MCB_MERGE_PROFILE
__device__ long long g_merge_prof[5];
#define MERGE_STAMP(i)                                                  \
    do {                                                                \
        const long long mp1 = clock64();                                \
        if (threadIdx.x == 0 && c == 0) g_merge_prof[i] += mp1 - mp0;  \
        mp0 = mp1;                                                      \
    } while (0)
#else
#define MERGE_STAMP(i) \
    do {               \
    } while (0)
#endif
#ifdef MCB_SCAN_PROFILE
__device__ long long g_scan_prof[4];
#endif
#ifndef MCB_PIVOT_MINB
#define MCB_PIVOT_MINB 1  // pivot-kernel CTAs the register budget is sized for per SM
#endif
__global__ void __launch_bounds__(kPivotThreads, MCB_PIVOT_MINB) blk_pivot_kernel(
    long long K, const int64_t *__restrict__ off, const int32_t *__restrict__ coords,
    const int32_t *__restrict__ head, const int32_t *__restrict__ tile_minc, const uint64_t *__restrict__ T,
    int bound, BlockState *bs,
    uint64_t *Warr, unsigned *tile_epoch, unsigned long long *reports, GridBar *gb, unsigned *status,
    unsigned long long *bytes, unsigned long long *diag, unsigned long long *dbg, TailArgs ta, PivotShape sh) {
    // dynamic shared memory: global tables | local tables | window W's | merge buffers | report staging
    extern __shared__ __align__(128) unsigned char dsm[];
    const unsigned G = gridDim.x;
    uint64_t(*gtab)[256] = reinterpret_cast<uint64_t(*)[256]>(dsm);
    uint64_t(*ltab)[256] = reinterpret_cast<uint64_t(*)[256]>(dsm + 16384);
    uint64_t *win = reinterpret_cast<uint64_t *>(dsm + 32768);                                      // kWinW
    unsigned long long *mr = reinterpret_cast<unsigned long long *>(dsm + 32768 + 8 * (size_t)kWinW);  // 2 G kLmax
    uint64_t *mw = reinterpret_cast<uint64_t *>(mr + 2 * (size_t)G * kLmax);                          // 3 G kLmax
    unsigned long long *lr = mr + 5 * (size_t)G * kLmax;  // G (2 kLmax + 2)
    __shared__ uint64_t gbasis[64], lbasis[64];
    __shared__ unsigned gpiv[64], lpiv[64];
    __shared__ unsigned s_first[kWarps], s_wcnt[kWarps];
    __shared__ unsigned long long s_chg[kWarps], s_dmin[kWarps];
    __shared__ unsigned s_tag[kWinMax];
    __shared__ __align__(8) uint64_t s_bar;  // completion of the window's bulk copies
    __shared__ uint64_t s_newv[64];
    __shared__ unsigned s_newq[64];
    __shared__ int s_nnew;
    __shared__ unsigned long long sr_rank[kLmax], sr_w[kLmax];

    griddep_wait();
    griddep_launch();
    // an earlier block ran out of candidates (flag written by an earlier launch, so
    // every CTA reads the same value and none waits at a grid barrier)
    if (*(volatile const unsigned *)&bs->failed) return;
    unsigned long long n_loaded = 0, n_computed = 0, n_local = 0, n_cand = 0;
    long long cyc_scan = 0, cyc_bar = 0, cyc_merge = 0;
    unsigned long long nbar = 0;
    unsigned long long nb = 0;
    const unsigned epoch = bs->epoch;
    const int b = (int)bs->b;
    const long long ntiles = (K + kTile - 1) / kTile;
    const long long c = blockIdx.x;
    unsigned gen = ld_acquire_u32(&gb->gen);
    for (int i = threadIdx.x; i < 8 * 256; i += blockDim.x) (&gtab[0][0])[i] = 0;
    if (threadIdx.x == 0) {
        mbar_init(&s_bar, 1);
        fence_mbar_init();
    }
    unsigned mphase = 0;  // uses of s_bar so far
    long long maxt = 0;   // deepest tile this CTA touched
    long long s = 0;
    int grank = 0;
    bool ok = true;
    unsigned k = 0;
    cta_sync();
    while (grank < b) {
        unsigned long long *rep_rank =
            reports + (size_t)(k & 1) * G * (2 * kLmax + 2);
        unsigned long long *rep_w = rep_rank + (size_t)G * kLmax;
        unsigned long long *rep_end = rep_w + (size_t)G * kLmax;
        unsigned long long *rep_n = rep_end + G;
        // ---- part 1: local pivots over this CTA's window ----
        const long long c0 = clock64();
        for (int i = threadIdx.x; i < 8 * 256; i += blockDim.x) (&ltab[0][0])[i] = (&gtab[0][0])[i];
        if (threadIdx.x < 64) {
            lbasis[threadIdx.x] = gbasis[threadIdx.x];
            lpiv[threadIdx.x] = gpiv[threadIdx.x];
        }
        int lrank = grank;
        // window: this CTA's tiles tf, tf + G, ... (t = c mod G) from the scan start on
        const long long t0 = s / kTile;
        const long long tf = t0 + (((long long)c - t0 % G) + G) % G;
#ifdef MCB_SCAN_PROFILE
        long long sp0 = clock64();
#define SCAN_STAMP(i)                                                 \
    do {                                                              \
        const long long sp1 = clock64();                              \
        if (threadIdx.x == 0 && c == 0) g_scan_prof[i] += sp1 - sp0; \
        sp0 = sp1;                                                    \
    } while (0)
#else
#define SCAN_STAMP(i) \
    do {              \
    } while (0)
#endif
        const int wsz = grank < sh.rank_early ? sh.win_early
                        : grank >= sh.rank_tail ? sh.win_tail
                                                : sh.win_mid;  // same in every CTA
        const int nwin = tf >= ntiles ? 0 : (int)min((long long)wsz, (ntiles - 1 - tf) / G + 1);
        if (threadIdx.x < (unsigned)nwin) s_tag[threadIdx.x] = ld_acquire_u32(&tile_epoch[tf + (long long)threadIdx.x * G]);
        cta_sync();
        unsigned copymask = 0, zeromask = 0, missmask = 0;
        for (int m = 0; m < nwin; m++) {
            const unsigned tag = s_tag[m];
            if ((tag >> 1) != epoch) missmask |= 1u << m;
            else if (tag & 1u) zeromask |= 1u << m;
            else copymask |= 1u << m;
        }
        maxt = nwin > 0 && tf + (long long)(nwin - 1) * G > maxt ? tf + (long long)(nwin - 1) * G : maxt;
        // tiles the streaming pass computed: one bulk copy each into the window
        if (copymask && threadIdx.x == 0) {
            fence_proxy_async_smem();  // the previous step's reads of the window come first
            mbar_arrive_expect_tx(&s_bar, (unsigned)__popc(copymask) * 8u * kTile);
            for (unsigned mm = copymask; mm; mm &= mm - 1) {
                const int m = __ffs(mm) - 1;
                tma_load_1d(win + (size_t)m * kTile, Warr + (size_t)(tf + (long long)m * G) * kTile, 8u * kTile, &s_bar);
            }
            nb += 8ull * kTile * (unsigned)__popc(copymask);
        }
        for (unsigned mm = zeromask; mm; mm &= mm - 1) {
            const int m = __ffs(mm) - 1;
            for (int i = threadIdx.x; i < kTile; i += blockDim.x) win[(size_t)m * kTile + i] = 0;
        }
        n_loaded += (unsigned)__popc(copymask | zeromask);
        SCAN_STAMP(0);
        if (missmask) {  // tiles beyond the streaming pass: W's computed here by the whole CTA
            const unsigned nm = (unsigned)__popc(missmask);
            unsigned nread = 0;
#if MCB_OTF_PAIRS
            // two candidates per thread walked together (positions idx and idx + half)
            const unsigned tot = nm * kTile, half = (tot + 1) / 2;
            for (unsigned idx = threadIdx.x; idx < half; idx += blockDim.x) {
                const unsigned jdx = idx + half;
                const int ma = nth_bit(missmask, idx / kTile);
                const long long ta_ = tf + (long long)ma * G, ra = ta_ * kTile + idx % kTile;
                const bool va = ra < K && tile_minc[ta_] < bound;
                long long rb = -1;
                int mb = 0;
                if (jdx < tot) {
                    mb = nth_bit(missmask, jdx / kTile);
                    const long long tb_ = tf + (long long)mb * G;
                    rb = tb_ * kTile + jdx % kTile;
                    if (!(rb < K && tile_minc[tb_] < bound)) rb = -2;
                }
                uint64_t Wa = 0, Wb = 0;
                if (va || rb >= 0) w_of_two(va ? ra : rb, va ? (rb >= 0 ? rb : -1) : -1, off, coords, head, T, bound, nread, Wa, Wb);
                if (!va) {  // the walk ran on rb alone
                    Wb = Wa;
                    Wa = 0;
                }
                win[(size_t)ma * kTile + idx % kTile] = Wa;
                Warr[ra] = Wa;
                if (jdx < tot) {
                    win[(size_t)mb * kTile + jdx % kTile] = rb >= 0 ? Wb : 0ull;
                    Warr[(tf + (long long)mb * G) * kTile + jdx % kTile] = rb >= 0 ? Wb : 0ull;
                }
            }
#else
            for (unsigned idx = threadIdx.x; idx < nm * kTile; idx += blockDim.x) {
                const int m = nth_bit(missmask, idx / kTile);
                const unsigned i = idx % kTile;
                const long long t = tf + (long long)m * G;
                const long long r = t * kTile + i;
                uint64_t W = 0;
                if (r < K && tile_minc[t] < bound) W = w_of_candidate(r, off, coords, head, T, bound, nread);
                win[(size_t)m * kTile + i] = W;
                Warr[r] = W;
            }
#endif
            fence_proxy_async_global();  // a later step may bulk-copy these tiles
            nb += 4ull * nread + (threadIdx.x == 0 ? 16ull * kTile * nm : 0ull);
            n_computed += nm;
        }
        SCAN_STAMP(1);
        if (copymask) {
            bool done = mbar_wait_bounded(&s_bar, mphase & 1u, 1u << 22);
            mphase++;
            if (!cta_sync_and(done)) {
                if (threadIdx.x == 0) {
                    mbar_wait_bounded(&s_bar, (mphase - 1) & 1u, 1u << 22);  // copies still in flight
                    atomicOr(status, ST_WAIT_TIMEOUT);
                    atomicExch(&gb->abort, 1u);
                }
                ok = false;
                break;
            }
        }
        cta_sync();
        if (missmask && threadIdx.x == 0) {
            __threadfence();
            for (unsigned mm = missmask; mm; mm &= mm - 1)
                tile_epoch[tf + (long long)(__ffs(mm) - 1) * G] = epoch << 1;
        }
        SCAN_STAMP(2);
        // local echelon over the window in rank order
        const unsigned valid = (unsigned)nwin * kTile;
        unsigned from = (nwin > 0 && tf == t0) ? (unsigned)(s - t0 * kTile) : 0u;
        int nloc = 0;
        long long end = K;
        bool trunc = false;
        for (;;) {
            const unsigned p = window_first_nonzero(win, ltab, from, valid, s_first);
            if (p >= valid) break;
            const uint64_t w = win[p];
            const uint64_t x = fr_reduce(w, ltab);
            const long long rank = (tf + (long long)(p / kTile) * G) * kTile + (p % kTile);
            if (threadIdx.x == 0) {
                sr_rank[nloc] = (unsigned long long)rank;
                sr_w[nloc] = w;
            }
            cta_sync();
            basis_add(ltab, lbasis, lpiv, lrank, x, s_chg);
            nloc++;
            from = p + 1;
            if (nloc == sh.lmax) {
                end = rank + 1;
                trunc = true;
                break;
            }
        }
        SCAN_STAMP(3);
        if (!trunc && nwin == wsz) {  // a shorter window reached the last tile: end = K
            const long long tl = tf + (long long)(wsz - 1) * G;
            end = (tl + 1) * kTile < K ? (tl + 1) * kTile : K;
        }
        n_local += nloc;
        if (threadIdx.x == 0) {
            for (int j = 0; j < nloc; j++) {
                rep_rank[c * kLmax + j] = sr_rank[j];
                rep_w[c * kLmax + j] = sr_w[j];
            }
            rep_end[c] = (unsigned long long)end;
            rep_n[c] = (unsigned long long)nloc;
        }
        const long long c1 = clock64();
        nbar++;
        if (!grid_barrier(gb, G, gen)) {
            if (threadIdx.x == 0) {  // where the wait gave up
                atomicExch(&diag[9], (unsigned long long)c + 1);
                atomicExch(&diag[10], (unsigned long long)k);
                atomicExch(&diag[11], (unsigned long long)grank);
                atomicExch(&diag[12], (unsigned long long)gen);
                atomicExch(&diag[13], (unsigned long long)*((volatile unsigned *)&gb->count));
            }
            ok = false;
            break;
        }
        const long long c2 = clock64();
        cyc_scan += c1 - c0;
        cyc_bar += c2 - c1;
        if (k > 0 && c == 0 && threadIdx.x < G) {  // compare the previous step's merge results
            const unsigned long long *prev = dbg + (size_t)((k - 1) & 1) * G;
            if (__ldcg(prev + threadIdx.x) != __ldcg(prev)) {
                atomicOr(status, ST_DIVERGED);
                if (atomicCAS(&diag[16], 0ull, 1ull) == 0ull) {
                    diag[17] = (unsigned long long)(k - 1);
                    diag[18] = (unsigned long long)threadIdx.x;
                    diag[19] = epoch;
                }
            }
        }
        // ---- part 2: merge (identical in every CTA) ----
#ifdef MCB_MERGE_PROFILE
        long long mp0 = clock64();
#endif
        // all reports into shared memory with independent loads (one round trip)
        const unsigned words = G * (2 * kLmax + 2);
        for (unsigned i = threadIdx.x; i < words; i += blockDim.x) lr[i] = __ldcg(rep_rank + i);
        cta_sync();
        const unsigned long long *l_rank = lr, *l_w = lr + (size_t)G * kLmax, *l_end = l_w + (size_t)G * kLmax,
                                 *l_n = l_end + G;
        unsigned long long dmin = kNone;
        for (unsigned i = threadIdx.x; i < G; i += blockDim.x) dmin = l_end[i] < dmin ? l_end[i] : dmin;
        const unsigned long long D = block_min_u64(dmin, s_dmin);
        MERGE_STAMP(0);
        // the reports below D, CTA by CTA (a CTA's ranks ascend): per-CTA counts,
        // block prefix sum, copy
        unsigned cnt = 0;
        const unsigned lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        for (unsigned cb = 0; cb < G; cb += blockDim.x) {
            const unsigned cc = cb + threadIdx.x;
            unsigned n = 0;
            if (cc < G) {
                const unsigned ln = l_n[cc] < (unsigned long long)kLmax ? (unsigned)l_n[cc] : (unsigned)kLmax;
                while (n < ln && l_rank[(size_t)cc * kLmax + n] < D) n++;
            }
            unsigned incl = n;
            for (int d = 1; d < 32; d <<= 1) {
                const unsigned v = __shfl_up_sync(0xffffffffu, incl, d);
                if (lane >= (unsigned)d) incl += v;
            }
            if (lane == 31) s_wcnt[wid] = incl;
            cta_sync();
            unsigned before = 0, all = 0;
#pragma unroll
            for (int x = 0; x < kWarps; x++) {
                const unsigned v = s_wcnt[x];
                before += (unsigned)x < wid ? v : 0u;
                all += v;
            }
            const unsigned o = cnt + before + incl - n;
            for (unsigned j = 0; j < n && o + j < G * kLmax; j++) {
                mr[o + j] = l_rank[(size_t)cc * kLmax + j];
                mw[o + j] = l_w[(size_t)cc * kLmax + j];
            }
            cnt += all;
            cta_sync();
        }
        if (cnt > G * kLmax) cnt = G * kLmax;
        n_cand += cnt;
        MERGE_STAMP(1);
        int nnew = 0;
#if MCB_MERGE_CHUNKED
        if (!MCB_MERGE_FAST || cnt > 0) {  // no report below D: no new pivot (uniform)
            // rank order: each candidate's position = number of smaller ranks (ranks are distinct)
            unsigned long long *sr = mr + cnt;  // sorted ranks
            uint64_t *sw = mw + cnt;            // sorted W
            for (unsigned i = threadIdx.x; i < cnt; i += blockDim.x) {
                const unsigned long long r = mr[i];
                unsigned pos = 0;
                for (unsigned j = 0; j < cnt; j++) pos += mr[j] < r;
                sr[pos] = r;
                sw[pos] = mw[i];
            }
            cta_sync();
            MERGE_STAMP(2);
            // greedy echelon in rank order, 32 candidates at a time.  Warp 0 reduces the
            // chunk against the basis (its Four-Russians tables hold every pivot
            // accepted so far, this step's included), accepts in order the candidates
            // whose residual is not in the span of the basis and of the chunk's accepted
            // ones before them, and brings those to reduced form among themselves
            // (latest first); then the whole CTA clears their pivot bits from the basis,
            // appends them and rebuilds the tables for the next chunk.
            for (unsigned base = 0; base < cnt && grank < b; base += 32) {
                if (threadIdx.x < 32) {
                    int nn = 0;
                    uint64_t z = base + lane < cnt ? fr_reduce(sw[base + lane], gtab) : 0ull;
                    for (;;) {
                        const unsigned bal = __ballot_sync(0xffffffffu, z != 0);
                        if (!bal || grank + nn >= b) break;
                        const int pl = __ffs(bal) - 1;
                        const uint64_t v = __shfl_sync(0xffffffffu, z, pl);
                        const unsigned qb = (unsigned)(__ffsll((long long)v) - 1);
                        if (lane == 0) {
                            s_newv[nn] = v;
                            s_newq[nn] = qb;
                            if (c == 0) {
                                bs->pivrank[grank + nn] = (long long)sr[base + pl];
                                bs->pivW[grank + nn] = sw[base + pl];
                            }
                        }
                        nn++;
                        if ((z >> qb) & 1ull) z ^= v;
                    }
                    __syncwarp();
                    uint64_t va = lane < (unsigned)nn ? s_newv[lane] : 0ull;  // nn <= 32
                    for (int j = nn - 1; j >= 1; j--) {
                        const uint64_t vj = __shfl_sync(0xffffffffu, va, j);
                        const unsigned qj = s_newq[j];
                        if ((int)lane < j && ((va >> qj) & 1ull)) va ^= vj;
                    }
                    __syncwarp();
                    if (lane < (unsigned)nn) s_newv[lane] = va;
                    if (lane == 0) s_nnew = nn;
                }
                cta_sync();
                const int nc = s_nnew;
                if (nc > 0) {
                    if (threadIdx.x < (unsigned)grank) {
                        uint64_t v = gbasis[threadIdx.x];
                        for (int j = 0; j < nc; j++)
                            if ((v >> s_newq[j]) & 1ull) v ^= s_newv[j];
                        gbasis[threadIdx.x] = v;
                    }
                    if (threadIdx.x < (unsigned)nc && grank + threadIdx.x < 64) {
                        gbasis[grank + threadIdx.x] = s_newv[threadIdx.x];
                        gpiv[grank + threadIdx.x] = s_newq[threadIdx.x];
                    }
                    grank += nc;
                    nnew += nc;
                    cta_sync();
                    fr_build(gtab, gbasis, gpiv, (unsigned)grank);  // ends with a barrier: s_new* are free
                } else {
                    cta_sync();  // s_nnew is read by every thread before warp 0 writes it again
                }
            }
            MERGE_STAMP(3);
        }
#else
        if (!MCB_MERGE_FAST || cnt > 0) {  // no report below D: no new pivot (uniform)
            // rank order: each candidate's position = number of smaller ranks (ranks are distinct)
            unsigned long long *sr = mr + cnt;  // sorted ranks
            uint64_t *sz = mw + cnt;            // sorted residuals against the global basis
            uint64_t *sw = sz + cnt;            // sorted W
            for (unsigned i = threadIdx.x; i < cnt; i += blockDim.x) {
                const unsigned long long r = mr[i];
                unsigned pos = 0;
                for (unsigned j = 0; j < cnt; j++) pos += mr[j] < r;
                sr[pos] = r;
                sw[pos] = mw[i];
                sz[pos] = fr_reduce(mw[i], gtab);
            }
            cta_sync();
            MERGE_STAMP(2);
            // greedy echelon in rank order (warp 0): a candidate is a new global pivot iff
            // its residual is not in the span of the new pivots before it; then the new
            // vectors are brought to reduced form among themselves, latest first (lane l
            // holds vectors l and l + 32)
            if (threadIdx.x < 32) {
                int nn = 0;
                for (unsigned base = 0; base < cnt && grank + nn < b; base += 32) {
                    uint64_t z = base + lane < cnt ? sz[base + lane] : 0ull;
                    for (int j = 0; j < nn; j++)
                        if ((z >> s_newq[j]) & 1ull) z ^= s_newv[j];
                    for (;;) {
                        const unsigned bal = __ballot_sync(0xffffffffu, z != 0);
                        if (!bal || grank + nn >= b) break;
                        const int pl = __ffs(bal) - 1;
                        const uint64_t v = __shfl_sync(0xffffffffu, z, pl);
                        const unsigned qb = (unsigned)(__ffsll((long long)v) - 1);
                        if (lane == 0) {
                            s_newv[nn] = v;
                            s_newq[nn] = qb;
                            if (c == 0) {
                                bs->pivrank[grank + nn] = (long long)sr[base + pl];
                                bs->pivW[grank + nn] = sw[base + pl];
                            }
                        }
                        nn++;
                        if ((z >> qb) & 1ull) z ^= v;
                    }
                    __syncwarp();
                }
                uint64_t va = lane < (unsigned)nn ? s_newv[lane] : 0ull;
                uint64_t vb = lane + 32 < (unsigned)nn ? s_newv[lane + 32] : 0ull;
                for (int j = nn - 1; j >= 1; j--) {
                    const uint64_t vj = __shfl_sync(0xffffffffu, j < 32 ? va : vb, j & 31);
                    const unsigned qj = s_newq[j];
                    if ((int)lane < j && ((va >> qj) & 1ull)) va ^= vj;
                    if ((int)lane + 32 < j && ((vb >> qj) & 1ull)) vb ^= vj;
                }
                __syncwarp();
                if (lane < (unsigned)nn) s_newv[lane] = va;
                if (lane + 32 < (unsigned)nn) s_newv[lane + 32] = vb;
                if (lane == 0) s_nnew = nn;
            }
            cta_sync();
            nnew = s_nnew;
            MERGE_STAMP(3);
        }
        if (nnew > 0) {
            // clear the new pivot bits from the old basis vectors, append, rebuild tables
            if (threadIdx.x < (unsigned)grank) {
                uint64_t v = gbasis[threadIdx.x];
                for (int j = 0; j < nnew; j++)
                    if ((v >> s_newq[j]) & 1ull) v ^= s_newv[j];
                gbasis[threadIdx.x] = v;
            }
            if (threadIdx.x < (unsigned)nnew && grank + threadIdx.x < 64) {
                gbasis[grank + threadIdx.x] = s_newv[threadIdx.x];
                gpiv[grank + threadIdx.x] = s_newq[threadIdx.x];
            }
            grank += nnew;
            cta_sync();
            fr_build(gtab, gbasis, gpiv, (unsigned)grank);
            MERGE_STAMP(4);
        }
#endif
        if (nnew == 0 && D >= (unsigned long long)K) {
            if (c == 0 && threadIdx.x == 0) {
                atomicOr(status, ST_RANK_DEFICIT);
                bs->failed = 1;
            }
            ok = false;
            break;
        }
        s = (long long)D;
        if (threadIdx.x == 0) {  // self-check: every CTA must reach the same merge result
            unsigned long long h = 1469598103934665603ull;
            h = (h ^ (unsigned long long)grank) * 1099511628211ull;
            h = (h ^ D) * 1099511628211ull;
            h = (h ^ (unsigned long long)cnt) * 1099511628211ull;
            dbg[(size_t)(k & 1) * G + c] = h;
        }
        k++;
        cyc_merge += clock64() - c2;
    }
    // ---- block tail: CTA 0 resolves the block; then every CTA materialises its
    // column groups of the final rows and their tables ----
    long long cyc_resolve = 0, cyc_tailbar = 0, cyc_mat = 0;
    if (ok) {
        const long long c3 = clock64();
        if (c == 0) {
            const bool done = resolve_block(bs, grank, off, coords, ta, reinterpret_cast<unsigned *>(win), status);
            if (threadIdx.x == 0) bs->tail_ok = done ? 1u : 0u;
        }
        const long long c4 = clock64();
        nbar++;
        if (!grid_barrier(gb, G, gen)) {
            ok = false;
        } else {
            const long long c5 = clock64();
            if (*((volatile unsigned *)&bs->tail_ok)) materialize_rows(ta, bs, b, win);
            cta_sync();
            cyc_tailbar = c5 - c4;
            cyc_mat = clock64() - c5;
        }
        cyc_resolve = c4 - c3;
    }
    if (!ok && threadIdx.x == 0 && (*((volatile unsigned *)&gb->abort))) atomicOr(status, ST_WAIT_TIMEOUT);
    for (int d = 16; d > 0; d >>= 1) nb += __shfl_xor_sync(0xffffffffu, nb, d);
    if ((threadIdx.x & 31) == 0 && nb) atomicAdd(bytes, nb);
    if (threadIdx.x == 0) {
        atomicMax(&diag[14], nbar);
        atomicMin(&diag[15], nbar);
        atomicMax((unsigned long long *)&bs->max_tile, (unsigned long long)maxt);
        atomicAdd(&diag[1], n_local);
        atomicAdd(&diag[3], n_loaded);
        atomicAdd(&diag[4], n_computed);
    }
    if (c == 0 && threadIdx.x == 0) {
        bs->rank = (unsigned)grank;
        bs->last_pivot = grank > 0 ? bs->pivrank[grank - 1] : 0;
        atomicAdd(&diag[0], (unsigned long long)k);
        atomicAdd(&diag[2], n_cand);
        atomicAdd(&diag[5], 1ull);
        atomicAdd(&diag[6], (unsigned long long)cyc_scan);
        atomicAdd(&diag[7], (unsigned long long)cyc_bar);
        atomicAdd(&diag[8], (unsigned long long)cyc_merge);
        atomicAdd(&diag[20], (unsigned long long)cyc_resolve);
        atomicAdd(&diag[21], (unsigned long long)cyc_tailbar);
        atomicAdd(&diag[22], (unsigned long long)cyc_mat);
#ifdef MCB_MERGE_PROFILE
        for (int i = 0; i < 5; i++) diag[33 + i] = (unsigned long long)g_merge_prof[i];
#endif
#ifdef MCB_SCAN_PROFILE
        for (int i = 0; i < 4; i++) diag[24 + i] = (unsigned long long)g_scan_prof[i];
#endif
#ifdef MCB_TAIL_PROFILE
        for (int i = 0; i < 6; i++) diag[24 + i] = g_tail_prof[i];
#endif
    }
}

// Dynamic shared memory of blk_pivot_kernel for a grid of G CTAs: two sets of
// Four-Russians tables, the window of kWinMax tiles of W's, the merge buffers
// (5 x G x kLmax words) and the report staging (G x (2 kLmax + 2) words).
size_t pivot_smem_bytes(int G) {
    return 32768 + 8 * (size_t)kWinW + 8 * 5 * (size_t)G * kLmax + 8 * (size_t)G * (2 * kLmax + 2);
}

// Rows j >= e0+b in groups of kUpdRows consecutive rows, kUpdSplit warps per group.
// D_j (64 bits) = <C_sel_k, S_j>: the group's warps split the chosen cycles'
// (coordinate, k) pairs, sorted by S word, and each pair is applied to all rows of
// the group (independent gathers of neighbouring words); pairs whose word lies above
// the group's last row are skipped (S_j has support [0, j]).  The warps' partial D's
// meet in shared memory (two buffers by iteration parity, one named barrier per
// group and iteration).  Then lane i computes, for row i of the group, beta_k =
// D_k ^ <beta_{<k}, gcol_k> (the sequential effect of the block's 64 updates); then
// S_j ^= XOR_k beta_k S_{e0+k} through the tables, the group's warps split the
// row's words.
#ifndef MCB_UPD_CTAS
#define MCB_UPD_CTAS 8  // block update: CTAs per SM at most (each loops over row groups)
#endif
constexpr int kUpdThreads = 256;
constexpr int kUpdSplit = MCB_UPD_SPLIT;
constexpr int kUpdGroups = kUpdThreads / 32 / kUpdSplit;  // row groups per CTA

// beta of one row from its D: beta_k = D_k ^ <beta_{<k}, gcol_k> (the sequential
// effect of the block's updates; beta = D (I + G)^-1, G[i][k] = bit i of gcol_k, an
// invertible map, so beta = 0 exactly when D = 0).  Far rows rarely change (a few
// dozen per block against thousands tested on the planar-chain family), so the rows
// that do run the b-step recurrence in one lane.
__device__ __forceinline__ uint64_t beta_of(uint64_t D, const uint64_t *__restrict__ gcol, int b) {
    uint64_t beta = 0;
    for (int k = 0; k < b; k++)
        beta |= (((D >> k) & 1ull) ^ (uint64_t)parity64(beta & __ldg(gcol + k))) << k;
    return beta;
}

// Appends v to list (counter *count) for the lanes with pred: one atomic per warp.
// All 32 lanes call it.
__device__ __forceinline__ unsigned warp_append(bool pred, int32_t v, int32_t *list, unsigned *count) {
    const unsigned m = __ballot_sync(0xffffffffu, pred);
    if (!m) return 0xFFFFFFFFu;
    const int lane = threadIdx.x & 31, lead = __ffs(m) - 1;
    unsigned base = 0;
    if (lane == lead) base = atomicAdd(count, (unsigned)__popc(m));
    base = __shfl_sync(0xffffffffu, base, lead);
    const unsigned pos = base + (unsigned)__popc(m & ((1u << lane) - 1u));
    if (pred) list[pos] = v;
    return pos;
}

// Far rows that are no longer unit vectors are kept as lists of their nonzero
// 64-bit words.  A far row j (j >= the far start, so j / 64 >= Wb) has support in
// [0, Wb) (the XORs of earlier blocks' final rows) and in its own word j / 64 (bit j
// alone): its list is its nonzero words below Wb plus j / 64, in any order.  D_j
// then only needs the chosen cycles' pairs that fall into those words (the pairs
// are sorted by S word, word_end[w] .. word_end[w + 1] being word w's), instead of
// every pair up to the row.  On the planar-chain family the support vectors stay
// local: a non-unit far row has 3 nonzero words at the median and rarely more than
// a few dozen of its thousands.  A row with more than kNzCap words is dense and goes
// through the gather of every pair (dense list).
#ifndef MCB_NZ_CAP
#define MCB_NZ_CAP 32  // words listed per sparse far row; beyond that the row is dense
#endif
constexpr int kNzCap = MCB_NZ_CAP;
constexpr uint16_t kDenseRow = 0xFFFFu;
static_assert(kNzCap >= 2 && kNzCap < 0xFFFF, "MCB_NZ_CAP out of range");

// D of a sparse far row from its word list: for each listed word that holds pairs
// of this block, the row's word is read once and tested against them.  List entries
// in batches of four (independent loads).
__device__ __forceinline__ uint64_t sparse_D(const uint64_t *S, long long j, int P, unsigned cnt, const uint32_t *nzw,
                                             const unsigned *__restrict__ word_end, const unsigned *__restrict__ pairs,
                                             unsigned long long &tests, unsigned long long &words) {
    const uint32_t *L = nzw + (size_t)j * kNzCap;
    const uint64_t *Sj = S + (size_t)j * P;
    uint64_t D = 0;
    for (unsigned i = 0; i < cnt; i += 4) {
        uint32_t w[4];
        unsigned lo[4], hi[4];
#pragma unroll
        for (int q = 0; q < 4; q++) w[q] = i + q < cnt ? L[i + q] : 0xFFFFFFFFu;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            lo[q] = w[q] != 0xFFFFFFFFu ? __ldg(word_end + w[q]) : 0u;
            hi[q] = w[q] != 0xFFFFFFFFu ? __ldg(word_end + w[q] + 1) : 0u;
        }
#pragma unroll
        for (int q = 0; q < 4; q++) {
            if (lo[q] >= hi[q]) continue;
            const uint64_t x = Sj[w[q]];
            words++;
            for (unsigned p = lo[q]; p < hi[q]; p++) {
                const unsigned pr = __ldg(pairs + p);
                D ^= ((x >> ((pr >> 6) & 63u)) & 1ull) << (pr & 63u);
            }
            tests += hi[q] - lo[q];
        }
    }
    return D;
}

// The far update of a block: every row j >= row_begin (the rows past the near
// update's) takes D_j = <C_sel_k, S_j> (k < b), beta_j = D_j (I + G)^-1 and
// S_j ^= XOR_k beta_jk S_{e0+k} over the first Wb words.  Most far rows are still
// their unit vector (S_j = e_j: no update has reached them yet), and for those
// D_j bit k is simply whether coordinate j lies on the selected cycle C_sel_k.  Few
// rows change, so finding them and changing them are separate launches, all on the
// far stream:
//   far_scatter_kernel: every (coordinate c, k) pair of the block's selected cycles
//     with c a unit far row sets bit k of Dfar[c] (first touch lists c);
//   far_rows_kernel:    D and beta of the non-unit far rows (lists carried from update
//     to update; sparse rows test the pairs of their listed words, one row per lane;
//     dense rows gather every pair up to their own word, as the reference's update
//     does) and of the touched unit rows; unchanged rows are carried over, changed
//     rows go to a (row, beta) list;
//   far_apply_kernel:   one CTA per changed row: S_j ^= XOR_k beta_k S_{e0+k} spread
//     over the CTA's threads, then the row is relisted (sparse or dense).
// Far-row starts never decrease from block to block (the near rows of a block are
// below every later far range), so a listed row below the current start is dropped
// for good.
// Dense rows in groups of kUpdRows list entries, kUpdSplit warps per group.  D_j (64
// bits): the group's warps split the chosen cycles' (coordinate, k) pairs, sorted by
// S word, and each pair is applied to all rows of the group (independent gathers);
// pairs whose word lies above the group's last row are skipped (S_j has support [0,
// j]).  The warps' partial D's meet in shared memory (two buffers by iteration
// parity, one named barrier per group and iteration).  gcol, pairs and word_end are
// the block's (double-buffered by block parity, so the next block's tail can run
// while these rows are updated).
struct FarLists {
    const int32_t *sp_in, *dn_in;
    const unsigned *n_in;     // [sparse, dense]
    int32_t *sp_out, *dn_out;
    unsigned *n_out;          // [sparse, dense, touched, changed]
    const int32_t *touch;     // touched unit rows (count n_out[2])
    int32_t *chg_row;         // changed rows (count n_out[3])
    unsigned long long *chg_beta;
    uint16_t *nzc;            // per row: listed words, or kDenseRow
    uint32_t *nzw;            // per row: kNzCap word indices
};

__global__ void __launch_bounds__(kUpdThreads) far_rows_kernel(const uint64_t *__restrict__ S, long long row_begin,
                                                               int P, int b, const uint64_t *__restrict__ gcol,
                                                               const unsigned *__restrict__ pairs,
                                                               const unsigned *__restrict__ word_end, FarLists fl,
                                                               unsigned long long *Dfar, uint8_t *unit,
                                                               unsigned long long *bytes, unsigned long long *diag) {
    const unsigned nsparse = fl.n_in[0], ndense = fl.n_in[1], ntouch = fl.n_out[2];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long groups = (long long)gridDim.x * kUpdGroups;
    const bool dense_work = (long long)blockIdx.x * kUpdGroups * kUpdRows < (long long)ndense;
    const bool sparse_work = (long long)blockIdx.x * kUpdThreads < (long long)nsparse + ntouch;
    if (!dense_work && !sparse_work) return;  // CTA-uniform
    unsigned long long nb = 0, n_rows = 0, n_changed = 0, n_gather = 0, n_betabits = 0;
    unsigned long long n_sparse = 0, n_words = 0, n_tests = 0, n_swords = 0, n_touched = 0;
    __shared__ uint64_t sD[2][kUpdGroups][kUpdSplit][kUpdRows];
    const int gi = warp / kUpdSplit, h = warp % kUpdSplit;
    int par = 0;
    for (long long base = kUpdRows * ((long long)blockIdx.x * kUpdGroups + gi); base < (long long)ndense;
         base += kUpdRows * groups, par ^= 1) {
        const int rows = (int)(((long long)ndense - base) < kUpdRows ? ((long long)ndense - base) : kUpdRows);
        // lane r < rows: its listed row, kept if still a far row
        const long long jr = lane < rows ? (long long)__ldg(fl.dn_in + base + lane) : -1;
        const bool keep = jr >= row_begin;
        const unsigned kmask = __ballot_sync(0xffffffffu, keep);
        if (!kmask) continue;  // warp-uniform
        long long jmax = keep ? jr : -1;
        for (int d = 16; d > 0; d >>= 1) {
            const long long o = __shfl_xor_sync(0xffffffffu, jmax, d);
            jmax = o > jmax ? o : jmax;
        }
        const int wl = (int)(jmax >> 6) + 1 < P ? (int)(jmax >> 6) + 1 : P;
        const unsigned np = __ldg(word_end + wl);
        // the group's rows as 32-bit words: bit c of a row is bit c & 31 of word c >> 5
        const uint32_t *Sr[kUpdRows];
#pragma unroll
        for (int r = 0; r < kUpdRows; r++) {
            const long long j = __shfl_sync(0xffffffffu, jr, r);
            Sr[r] = ((kmask >> r) & 1u) ? reinterpret_cast<const uint32_t *>(S + (size_t)j * P) : nullptr;
        }
        uint64_t D[kUpdRows];
#pragma unroll
        for (int r = 0; r < kUpdRows; r++) D[r] = 0;
        for (unsigned i = h * 32 + lane; i < np; i += 32 * kUpdSplit) {
            const unsigned pr = __ldg(pairs + i);
            const unsigned c = pr >> 6, q = c >> 5, sh = c & 31u;
            const uint64_t m = 1ull << (pr & 63u);
#pragma unroll
            for (int r = 0; r < kUpdRows; r++)
                if (Sr[r] && ((Sr[r][q] >> sh) & 1u)) D[r] ^= m;
        }
        uint64_t Dmine = 0;
#pragma unroll
        for (int r = 0; r < kUpdRows; r++) {
            const uint64_t d = warp_xor64(D[r]);
            if (lane == r) Dmine = d;
        }
        if (kUpdSplit > 1) {
            if (lane < kUpdRows) sD[par][gi][h][lane] = Dmine;
            asm volatile("barrier.sync %0, %1;" ::"r"(1 + gi), "r"(32 * kUpdSplit) : "memory");
            if (lane < kUpdRows) {
                Dmine = 0;
#pragma unroll
                for (int q = 0; q < kUpdSplit; q++) Dmine ^= sD[par][gi][q][lane];
            }
        }
        if (h != 0) continue;  // the group's first warp carries the rows over
        if (!keep) Dmine = 0;
        // an unchanged row stays in the dense list; a changed one goes to the apply
        warp_append(keep && Dmine == 0, (int32_t)jr, fl.dn_out, fl.n_out + 1);
        const uint64_t beta = Dmine ? beta_of(Dmine, gcol, b) : 0ull;
        const unsigned pos = warp_append(beta != 0, (int32_t)jr, fl.chg_row, fl.n_out + 3);
        if (beta) fl.chg_beta[pos] = beta;
        if (keep) {
            nb += 8ull * np;
            n_rows++;
            n_changed += beta ? 1 : 0;
            n_gather += np;
            n_betabits += (unsigned)__popcll(beta);
        }
    }
    // sparse rows, then the touched unit rows, one per lane
    const long long gw = (long long)blockIdx.x * (kUpdThreads / 32) + warp;
    const long long nwarps = (long long)gridDim.x * (kUpdThreads / 32);
    const long long nall = (long long)nsparse + ntouch;
    for (long long base = gw * 32; base < nall; base += nwarps * 32) {
        const long long i = base + lane;
        const bool touched = i >= (long long)nsparse && i < nall;
        long long j = -1;
        if (i < (long long)nsparse)
            j = __ldg(fl.sp_in + i);
        else if (touched)
            j = __ldg(fl.touch + (i - nsparse));
        const bool keep = !touched && j >= row_begin;
        uint64_t D = 0;
        if (keep) {
            const unsigned cnt = fl.nzc[j];
            D = sparse_D(S, j, P, cnt, fl.nzw, word_end, pairs, n_tests, n_swords);
            n_sparse++;
            n_words += cnt;
            nb += 4ull + 2ull + 12ull * cnt;  // list entry, count, listed words + their two word_end entries
        } else if (touched) {  // a unit row the scatter reached: D was scattered (never zero)
            D = Dfar[j];
            Dfar[j] = 0;  // ready for the next block
            unit[j] = 0;
            n_touched++;
            nb += 4ull + 16ull;
        }
        warp_append(keep && D == 0, (int32_t)j, fl.sp_out, fl.n_out);
        const uint64_t beta = D ? beta_of(D, gcol, b) : 0ull;
        const unsigned pos = warp_append(beta != 0, (int32_t)j, fl.chg_row, fl.n_out + 3);
        if (beta) {
            fl.chg_beta[pos] = beta;
            n_changed++;
            n_betabits += (unsigned)__popcll(beta);
        }
    }
    nb += 8ull * n_swords + 4ull * n_tests;
    for (int d = 16; d > 0; d >>= 1) {
        nb += __shfl_xor_sync(0xffffffffu, nb, d);
        n_rows += __shfl_xor_sync(0xffffffffu, n_rows, d);
        n_changed += __shfl_xor_sync(0xffffffffu, n_changed, d);
        n_gather += __shfl_xor_sync(0xffffffffu, n_gather, d);
        n_betabits += __shfl_xor_sync(0xffffffffu, n_betabits, d);
        n_sparse += __shfl_xor_sync(0xffffffffu, n_sparse, d);
        n_words += __shfl_xor_sync(0xffffffffu, n_words, d);
        n_tests += __shfl_xor_sync(0xffffffffu, n_tests, d);
        n_touched += __shfl_xor_sync(0xffffffffu, n_touched, d);
    }
    if (lane == 0 && nb) atomicAdd(bytes, nb);
    if (lane == 0 && diag && (n_rows || n_sparse || n_touched)) {
        // dense rows gathered, changed rows, pair words gathered, beta bits, touched
        // unit rows; sparse rows tested, their listed words, pair tests
        atomicAdd(&diag[23], n_rows);
        atomicAdd(&diag[30], n_changed);
        atomicAdd(&diag[31], n_gather);
        atomicAdd(&diag[29], n_betabits);
        atomicAdd(&diag[32], n_touched);
        atomicAdd(&diag[38], n_sparse);
        atomicAdd(&diag[39], n_words);
        atomicAdd(&diag[40], n_tests);
    }
}

// Every pair (c, k) of the block's sorted pairs with c a unit row in [row_begin,
// row_end): bit k of Dfar[c] (a cycle's coordinates are distinct, so the bits of one
// row come from distinct cycles and OR is XOR); a row's first touch lists it.
__global__ void __launch_bounds__(256) far_scatter_kernel(const unsigned *__restrict__ pairs,
                                                         const unsigned *__restrict__ word_end, int P,
                                                         long long row_begin, long long row_end,
                                                         const uint8_t *__restrict__ unit, unsigned long long *Dfar,
                                                         int32_t *touch, unsigned *n_touch,
                                                         unsigned long long *bytes) {
    const unsigned np = __ldg(word_end + P);
    unsigned long long nb = 0;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
        const unsigned pr = __ldg(pairs + i);
        const long long c = (long long)(pr >> 6);
        nb += 4;
        if (c < row_begin || c >= row_end || !unit[c]) continue;
        const unsigned long long old = atomicOr(Dfar + c, 1ull << (pr & 63u));
        if (!old) touch[atomicAdd(n_touch, 1u)] = (int32_t)c;
        nb += 8;
    }
    for (int d = 16; d > 0; d >>= 1) nb += __shfl_xor_sync(0xffffffffu, nb, d);
    if ((threadIdx.x & 31) == 0 && nb) atomicAdd(bytes, nb);
}

// The changed far rows, one CTA each: S_j ^= XOR_k beta_k S_{e0+k} over words [0, Wb)
// (the final rows are written once by the block tail and never change again), four
// words per thread at a time so their loads overlap; the nonzero words are counted
// and listed as they are written (shared counter, any order), then the row's own
// word j / 64 joins the list and the row goes to the sparse list, or to the dense
// list past kNzCap words.
constexpr int kApplyThreads = 256;

__global__ void __launch_bounds__(kApplyThreads) far_apply_kernel(uint64_t *S, int P, int e0, int Wb, FarLists fl,
                                                                 unsigned long long *bytes) {
    const unsigned nchg = fl.n_out[3];
    if (blockIdx.x >= nchg) return;
    __shared__ int sk[64];
    __shared__ unsigned s_cnt;
    unsigned long long nb = 0;
    for (unsigned item = blockIdx.x; item < nchg; item += gridDim.x) {
        const long long j = fl.chg_row[item];
        const uint64_t bt = fl.chg_beta[item];
        const int nbits = __popcll(bt);
        if (threadIdx.x < 64) sk[threadIdx.x] = (bt >> threadIdx.x) & 1ull ? __popcll(bt & ((1ull << threadIdx.x) - 1ull)) : -1;
        if (threadIdx.x == 0) s_cnt = 0;
        cta_sync();
        __shared__ int skl[64];
        if (threadIdx.x < 64 && sk[threadIdx.x] >= 0) skl[sk[threadIdx.x]] = (int)threadIdx.x;
        cta_sync();
        uint64_t *Sj = S + (size_t)j * P;
        uint32_t *L = fl.nzw + (size_t)j * kNzCap;
        for (int w0 = threadIdx.x; w0 < Wb; w0 += 4 * kApplyThreads) {
            uint64_t acc[4] = {0ull, 0ull, 0ull, 0ull};
#pragma unroll 4
            for (int i = 0; i < nbits; i++) {
                const uint64_t *F = S + (size_t)(e0 + skl[i]) * P;
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int w = w0 + q * kApplyThreads;
                    if (w < Wb) acc[q] ^= F[w];
                }
            }
            uint64_t x[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {  // the row's four words loaded together, then stored
                const int w = w0 + q * kApplyThreads;
                x[q] = w < Wb ? Sj[w] ^ acc[q] : 0ull;
            }
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int w = w0 + q * kApplyThreads;
                if (w < Wb) {
                    Sj[w] = x[q];
                    if (x[q]) {
                        const unsigned pos = atomicAdd(&s_cnt, 1u);
                        if (pos < (unsigned)kNzCap) L[pos] = (uint32_t)w;
                    }
                }
            }
        }
        cta_sync();
        if (threadIdx.x == 0) {
            unsigned cnt = s_cnt;
            if (cnt < (unsigned)kNzCap) L[cnt] = (uint32_t)(j >> 6);
            cnt++;
            const bool dense = cnt > (unsigned)kNzCap;
            fl.nzc[j] = dense ? kDenseRow : (uint16_t)cnt;
            if (dense)
                fl.dn_out[atomicAdd(fl.n_out + 1, 1u)] = (int32_t)j;
            else
                fl.sp_out[atomicAdd(fl.n_out, 1u)] = (int32_t)j;
            nb += (16ull + 8ull * (unsigned)nbits) * (unsigned long long)Wb + 4ull * (cnt < kNzCap ? cnt : kNzCap);
        }
        cta_sync();  // sk, skl and s_cnt are reset for the next row
    }
    if (threadIdx.x == 0 && nb) atomicAdd(bytes, nb);
}

// The update of the next block's rows (at most 3 x 64, on the critical path: the
// next block's transpose reads them), spread over the whole GPU in two launches.
// near_d_kernel: D_j = <C_sel_k, S_j> bits for every near row j, one (row, chunk of
// kNearChunk pairs) item per warp, XOR-accumulated into Dbuf[j - row_begin] (one of
// two buffers by block parity; the next block's near_apply_kernel clears it).
constexpr int kNearPer = 16;               // pairs per lane of an item
constexpr int kNearChunk = 32 * kNearPer;  // pairs per item
constexpr int kNearMaxRows = 192;

__global__ void __launch_bounds__(256) near_d_kernel(const uint64_t *__restrict__ S, long long row_begin, int nrows,
                                                    int P, const unsigned *__restrict__ pairs,
                                                    const unsigned *__restrict__ word_end,
                                                    unsigned long long *Dbuf, unsigned long long *bytes) {
    griddep_wait();
    griddep_launch();
    const int lane = threadIdx.x & 31;
    const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    const unsigned npmax = __ldg(word_end + P);
    const long long chunks = (npmax + kNearChunk - 1) / kNearChunk;
    unsigned long long nb = 0;
    for (long long it = gw; it < (long long)nrows * chunks; it += nw) {
        const int r = (int)(it % nrows);
        const long long ch = it / nrows;
        const long long j = row_begin + r;
        const int wl = (int)(j >> 6) + 1 < P ? (int)(j >> 6) + 1 : P;
        const unsigned np = __ldg(word_end + wl);
        const unsigned i0 = (unsigned)(ch * kNearChunk);
        if (i0 >= np) continue;  // warp-uniform
        const uint64_t *Sj = S + (size_t)j * P;
        uint64_t D = 0;
#pragma unroll
        for (int q = 0; q < kNearPer; q++) {
            const unsigned i = i0 + q * 32 + lane;
            if (i < np) {
                const unsigned pr = __ldg(pairs + i);
                const unsigned c = pr >> 6, k = pr & 63u;
                D ^= ((Sj[c >> 6] >> (c & 63u)) & 1ull) << k;
            }
        }
        D = warp_xor64(D);
        if (lane == 0) {
            if (D) atomicXor(Dbuf + r, (unsigned long long)D);
            const unsigned e = np - i0 < (unsigned)kNearChunk ? np - i0 : (unsigned)kNearChunk;
            nb += 8ull * e;
        }
    }
    if (lane == 0 && nb) atomicAdd(bytes, nb);
}

// near_apply_kernel: every CTA computes beta_k = D_k ^ <beta_{<k}, gcol_k> (the
// sequential effect of the block's updates) of every near row (CTA 0 writes them to
// beta_out for the grouped pass's correction and clears the other parity's D
// buffer for the next block), then takes columns [w0, w0 + kNearCols) of the block's
// final rows into shared memory and applies S_j ^= XOR_k beta_k S_{e0+k} there to
// every near row: one read of the final rows in all, the near rows read and written
// once, column-contiguous.
constexpr int kNearCols = 32;
constexpr int kNearBatch = 8;  // near rows per thread whose words are loaded together

__global__ void __launch_bounds__(256) near_apply_kernel(uint64_t *S, long long row_begin, int nrows, int P, int b,
                                                        int e0, int Wb, const uint64_t *__restrict__ gcol,
                                                        const unsigned long long *__restrict__ Dbuf,
                                                        unsigned long long *Dnext, uint64_t *beta_out,
                                                        unsigned long long *bytes) {
    __shared__ uint64_t sg[64];
    __shared__ uint64_t sbeta[kNearMaxRows];
    __shared__ uint64_t srow[65][kNearCols];  // row 64: zeros, the padding of a short batch of bits
    griddep_wait();
    griddep_launch();
    if (threadIdx.x < 64) sg[threadIdx.x] = (int)threadIdx.x < b ? gcol[threadIdx.x] : 0;
    cta_sync();
    unsigned long long nb = 0;
    for (int r = threadIdx.x; r < nrows; r += blockDim.x) {
        const uint64_t D = Dbuf[r];
        uint64_t beta = 0;
        for (int k = 0; k < b; k++) beta |= ((((D >> k) & 1ull) ^ (uint64_t)parity64(beta & sg[k]))) << k;
        sbeta[r] = beta;
        if (blockIdx.x == 0) {
            if (beta_out) beta_out[r] = beta;
            nb += beta ? 16ull * (unsigned long long)Wb : 0ull;
        }
    }
    if (blockIdx.x == 0)
        for (int r = threadIdx.x; r < kNearMaxRows; r += blockDim.x) Dnext[r] = 0;
    cta_sync();
    const int w = threadIdx.x % kNearCols, rs = threadIdx.x / kNearCols, rstep = blockDim.x / kNearCols;
    for (int w0 = blockIdx.x * kNearCols; w0 < Wb; w0 += gridDim.x * kNearCols) {
        for (int idx = threadIdx.x; idx < 65 * kNearCols; idx += blockDim.x) {
            const int l = idx / kNearCols, x = idx % kNearCols;
            srow[l][x] = (l < b && w0 + x < Wb) ? S[(size_t)(e0 + l) * P + w0 + x] : 0ull;
        }
        if (threadIdx.x == 0) nb += 8ull * (unsigned long long)b * (unsigned long long)min(kNearCols, Wb - w0);
        cta_sync();
        if (w0 + w < Wb) {
            // rows in batches of eight: their XORs from shared memory, then the eight
            // row words loaded together (one memory round trip per batch, not per
            // row), then stored
            for (int r0 = rs; r0 < nrows; r0 += kNearBatch * rstep) {
                uint64_t acc[kNearBatch], old[kNearBatch];
                bool act[kNearBatch];
#pragma unroll
                for (int q = 0; q < kNearBatch; q++) {
                    const int r = r0 + q * rstep;
                    uint64_t bt = r < nrows ? sbeta[r] : 0ull;
                    act[q] = bt != 0;
                    // four independent accumulators: the shared-memory reads of a row's
                    // bits overlap instead of waiting one after the other
                    uint64_t a0 = 0, a1 = 0, a2 = 0, a3 = 0;
                    while (bt) {
                        const int k0 = __ffsll((long long)bt) - 1;
                        bt &= bt - 1;
                        const int k1 = bt ? __ffsll((long long)bt) - 1 : 64;
                        bt &= bt - 1;
                        const int k2 = bt ? __ffsll((long long)bt) - 1 : 64;
                        bt &= bt - 1;
                        const int k3 = bt ? __ffsll((long long)bt) - 1 : 64;
                        bt &= bt - 1;
                        a0 ^= srow[k0][w];
                        a1 ^= srow[k1][w];
                        a2 ^= srow[k2][w];
                        a3 ^= srow[k3][w];
                    }
                    acc[q] = (a0 ^ a1) ^ (a2 ^ a3);
                }
#pragma unroll
                for (int q = 0; q < kNearBatch; q++)
                    old[q] = act[q] ? S[(size_t)(row_begin + r0 + q * rstep) * P + w0 + w] : 0ull;
#pragma unroll
                for (int q = 0; q < kNearBatch; q++)
                    if (act[q]) S[(size_t)(row_begin + r0 + q * rstep) * P + w0 + w] = old[q] ^ acc[q];
            }
        }
        cta_sync();  // srow is refilled for the next column chunk
    }
    for (int d = 16; d > 0; d >>= 1) nb += __shfl_xor_sync(0xffffffffu, nb, d);
    if ((threadIdx.x & 31) == 0 && nb) atomicAdd(bytes, nb);
}

// ---- independence certificate --------------------------------------------------
// After a complete run, the final support vectors certify the basis: S_j was made
// orthogonal to every C_i chosen before it and is never changed after iteration j,
// where <C_j, S_j> = 1.  So the N x N matrix M[i][j] = <C_i, S_j> is unit lower
// triangular (M[i][j] = 0 for i < j, 1 for i = j) and has full rank, and with it the
// N cycle vectors C_i (rank(M) <= rank(C)).  Whatever S holds, finding that
// pattern in the product proves the selected cycles GF(2)-independent.
// cert_rows_kernel: C as an N x P bit matrix from the selected candidates' lists.
__global__ void cert_rows_kernel(const long long *__restrict__ selected, int N, int P, long long K,
                                 const int64_t *__restrict__ off, const int32_t *__restrict__ coords,
                                 unsigned long long *C, unsigned *status) {
    const int lane = threadIdx.x & 31;
    const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long i = gw; i < N; i += nw) {
        const long long r = selected[i];
        if (r < 0 || r >= K) {
            if (lane == 0) atomicOr(status, ST_BAD_INPUT);
            continue;
        }
        for (long long q = off[r] + lane; q < off[r + 1]; q += 32) {
            const int c = coords[q];
            if (c >= 0 && c < N) atomicOr(C + (size_t)i * P + (c >> 6), 1ull << (c & 63));
        }
    }
}

// cert_check_kernel: one CTA per 64 x 64 tile (ti <= tj) of M: row i of C against row
// j of S over the words of S_j's support (bits [0, j]); parity(XOR_w C_i[w] & S_j[w])
// must be 1 on the diagonal and 0 above it.  Counts the pairs where it is not.
constexpr int kCertWords = 32;
__global__ void __launch_bounds__(256) cert_check_kernel(const unsigned long long *__restrict__ C,
                                                        const uint64_t *__restrict__ S, int N, int P,
                                                        unsigned long long *violations,
                                                        unsigned long long *first_bad) {
    const int ti = blockIdx.x, tj = blockIdx.y;
    if (ti > tj) return;
    __shared__ unsigned long long sC[64][kCertWords + 1], sS[64][kCertWords + 1];
    const int t = threadIdx.x, ig = t >> 4, jg = t & 15;
    unsigned long long acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) acc[a][b] = 0;
    const int words = (tj + 1) < P ? tj + 1 : P;  // S_j, j < 64 (tj + 1), has no bit beyond word tj
    for (int w0 = 0; w0 < words; w0 += kCertWords) {
        for (int e = t; e < 64 * kCertWords; e += blockDim.x) {
            const int row = e / kCertWords, w = w0 + e % kCertWords;
            const long long i = 64ll * ti + row, j = 64ll * tj + row;
            sC[row][e % kCertWords] = (i < N && w < words) ? C[(size_t)i * P + w] : 0ull;
            sS[row][e % kCertWords] = (j < N && w < words) ? S[(size_t)j * P + w] : 0ull;
        }
        cta_sync();
#pragma unroll 4
        for (int w = 0; w < kCertWords; w++) {
            unsigned long long ci[4], sj[4];
#pragma unroll
            for (int a = 0; a < 4; a++) ci[a] = sC[ig * 4 + a][w];
#pragma unroll
            for (int b = 0; b < 4; b++) sj[b] = sS[jg * 4 + b][w];
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int b = 0; b < 4; b++) acc[a][b] ^= ci[a] & sj[b];
        }
        cta_sync();
    }
    unsigned long long bad = 0;
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) {
            const long long i = 64ll * ti + ig * 4 + a, j = 64ll * tj + jg * 4 + b;
            if (i >= N || j >= N || i > j) continue;
            const unsigned bit = (unsigned)__popcll(acc[a][b]) & 1u;
            if (bit != (i == j ? 1u : 0u)) {
                bad++;
                atomicMin(first_bad, (unsigned long long)i * (unsigned long long)N + (unsigned long long)j);
            }
        }
    if (bad) atomicAdd(violations, bad);
}

}  // namespace

// ===========================================================================
// The candidate search shapes a solver times (mcbgpu_solver_tune): the compiled-in
// default, more local pivots per step, wider windows, deeper streaming passes.  A
// solve is cut into kShapeSegs segments of blocks, each with its own shape (the
// pivots of later blocks lie deeper in the rank order).  On the 1M-vertex
// planar-chain graph's prefix solve the wider windows with 8 local pivots (candidate
// 2) take 0.113-0.146 ms per block against 0.128-0.164 ms for the default, from the
// first quarter of the solve to the last (a one-tile early window was 10x slower
// there and is not a candidate).
constexpr int kShapeSegs = 4;
constexpr int kShapeInts = 7;  // ints per shape in mcbgpu_solver_shapes
const PivotShape kCandidateShapes[] = {
    kDefaultShape,
    {2, 48, 6, 60, 8, 8, 25},
    {4, 48, 8, 56, 12, 8, 25},
    {3, 40, 8, 56, 12, 8, 60},
    {2, 40, 8, 56, 12, 8, 40},
    {3, 40, 8, 56, 12, 8, 40},
};
constexpr int kNumShapes = (int)(sizeof(kCandidateShapes) / sizeof(kCandidateShapes[0]));

struct mcbgpu_solver {
    int N = 0, W = 0, P = 0, words_cap = 0;
    long long K = 0, nnz = 0;
    int max_len = 0;
    int sm_count = 0;
    int32_t *d_weight = nullptr;
    int64_t *d_off = nullptr;
    int32_t *d_coords = nullptr;
    int32_t *d_head = nullptr;     // K x kHead: each list's first coordinates (INT_MAX past its end)
    uint64_t *d_S = nullptr;
    uint64_t *d_C = nullptr;       // cycle vector buffer (W words)
    uint64_t *d_T = nullptr;       // 64 * P words
    uint64_t *d_Warr = nullptr;    // W per candidate (tiles * 1024)
    uint64_t *d_Warr2 = nullptr;   // W of a group's second block (the grouped pass, then its correction)
    uint64_t *d_Warr3 = nullptr;   // W of a group's third block
    uint64_t *d_Tg = nullptr;      // the group's blocks' rows transposed, kGStride words per coordinate
    uint64_t *d_beta = nullptr;    // 3 x 192: update bits of the near rows of a group's first blocks
    unsigned long long *d_nearD = nullptr;  // 2 x kNearMaxRows: D of the near rows by block parity (zero between uses)
    // far update: rows whose support vector is still the unit vector get D by scatter
    uint8_t *d_unit = nullptr;               // N: 1 while S_j = e_j (far rows only kept exact)
    unsigned long long *d_Dfar = nullptr;    // N: scattered D of unit far rows (zero between uses)
    int32_t *d_rowlist[2] = {};              // N each: the sparse non-unit far rows, read / written by turns
    int32_t *d_denselist[2] = {};            // N each: the dense non-unit far rows, the same way
    uint16_t *d_nzc = nullptr;               // N: listed nonzero words of a sparse far row, or kDenseRow
    uint32_t *d_nzw = nullptr;               // N x kNzCap: those words
    int32_t *d_touch = nullptr;              // N: unit far rows the scatter reached
    int32_t *d_chg_row = nullptr;            // N: far rows that change in this block's update
    unsigned long long *d_chg_beta = nullptr;  // N: their update bits
    unsigned *d_fcnt = nullptr;              // per list set l: [4l] sparse rows, [4l + 1] dense rows, [4l + 2] touched,
                                             // [4l + 3] changed
    int list_cur = 0;                        // the list set the next far update reads
    uint64_t *d_masks = nullptr;   // 2 x 64: final masks of a group's first blocks
    unsigned *d_tile_epoch = nullptr;
    int32_t *d_tile_minc = nullptr;
    unsigned long long *d_reports = nullptr;  // two step parities of G x (2 kLmax + 2) words
    GridBar *d_gbar = nullptr;
    int pivot_grid = 0;
    unsigned *d_pairs = nullptr;     // 3 x pair_cap: resolve scratch, sorted pairs of the two block parities
    unsigned pair_cap = 0;
    unsigned *d_word_end = nullptr;  // 2 x (P + 1): sorted pairs with S word < w, by block parity
    cudaStream_t st1 = nullptr;      // the blocked run's critical path (highest priority)
    cudaStream_t st2 = nullptr;      // the update of the rows beyond the next block (lowest priority)
    cudaEvent_t ev_join = nullptr;   // the end of a blocked run, for the caller's stream
    cudaEvent_t ev_fork = nullptr, ev_tail = nullptr, ev_upd[4] = {}, ev_par[2] = {};
    IterSlot *d_slots = nullptr;   // 2
    BlockState *d_bs = nullptr;
    long long *d_selected = nullptr;
    unsigned *d_status = nullptr;
    unsigned *d_check = nullptr;   // [bad flags, longest list]
    bool uploaded = false;
    long long iters_run = 0;
    long long launches = 0;
    long long device_bytes = 0;
    // optional per-launch profile: events around every launch, per-class byte counters
    struct ProfRec {
        int cls;
        cudaEvent_t a, b;
    };
    bool profiling = false;
    std::vector<ProfRec> recs;
    std::vector<cudaEvent_t> pool;
    size_t pool_next = 0;
    unsigned long long *d_bytes = nullptr;  // KC_COUNT counters
    unsigned long long *d_diag = nullptr;   // pivot-kernel counters (see mcbgpu_solver_diagnostics)
    // search shapes: the shape of each segment of a solve (0 = the default until a
    // tuning run picks), a shape forced for every block (-1: none), and while a
    // tuning run is on, the blocks' search times (transpose to pivot-kernel end on
    // the critical stream) by segment and shape
    int seg_shape[kShapeSegs] = {};
    int forced_shape = -1;
    bool pdl = MCB_PDL != 0;  // critical-path kernels with programmatic dependent launch
    bool tuning = false;
    struct TuneRec {
        int seg, shape, blocks;  // a group of `blocks` blocks
        cudaEvent_t a, b;
    };
    std::vector<TuneRec> tune_recs;
    std::vector<cudaEvent_t> tpool;
    // a complete solve (reset + blocked run) captured as one CUDA graph
    cudaStream_t cap = nullptr;      // the stream the capture starts on
    cudaGraphExec_t gexec = nullptr;
    int64_t gexec_iters = -1;        // iterations the graph runs
    long long gexec_launches = 0;    // kernel launches per replay
    int gexec_list_end = 0;          // list set the replay leaves current
};

namespace {

// A launch on the critical stream of the blocked run: with programmatic stream
// serialisation when the handle uses it (the kernel is scheduled while its
// predecessor finishes and waits for it in griddep_wait), cooperative when asked.
template <typename... Exp, typename... Act>
cudaError_t launch_k(bool pdl, void (*kern)(Exp...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                     Act &&...args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    if (pdl) {
        at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[0].val.programmaticStreamSerializationAllowed = 1;
    }
    cfg.attrs = at;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kern, std::forward<Act>(args)...);
}

cudaError_t launch_coop(bool pdl, const void *kern, dim3 grid, dim3 block, void **args, size_t smem,
                        cudaStream_t st) {
    if (!pdl) return cudaLaunchCooperativeKernel(kern, grid, block, args, smem, st);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[2];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[1].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 2;
    return cudaLaunchKernelExC(&cfg, kern, args);
}

cudaEvent_t pool_event(mcbgpu_solver *s) {
    if (s->pool_next == s->pool.size()) {
        cudaEvent_t e = nullptr;
        cudaEventCreate(&e);
        s->pool.push_back(e);
    }
    return s->pool[s->pool_next++];
}

// Counts a launch of class `cls`; when profiling, brackets it with events.
struct Launch {
    mcbgpu_solver *s;
    int cls;
    cudaStream_t st;
    cudaEvent_t a = nullptr;
    int kernels;  // kernel launches inside the bracket
    Launch(mcbgpu_solver *s_, int cls_, cudaStream_t st_, int kernels_ = 1)
        : s(s_), cls(cls_), st(st_), kernels(kernels_) {
        if (s->profiling) {
            a = pool_event(s);
            cudaEventRecord(a, st);
        }
    }
    ~Launch() {
        if (s->profiling) {
            cudaEvent_t b = pool_event(s);
            cudaEventRecord(b, st);
            s->recs.push_back({cls, a, b});
        }
        s->launches += kernels;
    }
    unsigned long long *bytes() const { return s->d_bytes + cls; }
};

}  // namespace

namespace {

void drop_graph(mcbgpu_solver *s) {
    if (s->gexec) cudaGraphExecDestroy(s->gexec);
    s->gexec = nullptr;
    s->gexec_iters = -1;
}

void free_solver(mcbgpu_solver *s) {
    if (!s) return;
    drop_graph(s);
    if (s->cap) cudaStreamDestroy(s->cap);
    for (cudaEvent_t e : s->tpool) cudaEventDestroy(e);
    cudaFree(s->d_weight);
    cudaFree(s->d_off);
    cudaFree(s->d_coords);
    cudaFree(s->d_head);
    cudaFree(s->d_S);
    cudaFree(s->d_C);
    cudaFree(s->d_T);
    cudaFree(s->d_Warr);
    cudaFree(s->d_Warr2);
    cudaFree(s->d_Warr3);
    cudaFree(s->d_Tg);
    cudaFree(s->d_beta);
    cudaFree(s->d_nearD);
    cudaFree(s->d_unit);
    cudaFree(s->d_Dfar);
    cudaFree(s->d_rowlist[0]);
    cudaFree(s->d_rowlist[1]);
    cudaFree(s->d_denselist[0]);
    cudaFree(s->d_denselist[1]);
    cudaFree(s->d_nzc);
    cudaFree(s->d_nzw);
    cudaFree(s->d_touch);
    cudaFree(s->d_chg_row);
    cudaFree(s->d_chg_beta);
    cudaFree(s->d_fcnt);
    cudaFree(s->d_masks);
    cudaFree(s->d_tile_epoch);
    cudaFree(s->d_tile_minc);
    cudaFree(s->d_reports);
    cudaFree(s->d_gbar);
    cudaFree(s->d_pairs);
    cudaFree(s->d_word_end);
    if (s->st2) cudaStreamDestroy(s->st2);
    if (s->st1) cudaStreamDestroy(s->st1);
    if (s->ev_join) cudaEventDestroy(s->ev_join);
    if (s->ev_fork) cudaEventDestroy(s->ev_fork);
    if (s->ev_tail) cudaEventDestroy(s->ev_tail);
    for (cudaEvent_t e : s->ev_par)
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : s->ev_upd)
        if (e) cudaEventDestroy(e);
    cudaFree(s->d_slots);
    cudaFree(s->d_bs);
    cudaFree(s->d_selected);
    cudaFree(s->d_status);
    cudaFree(s->d_check);
    cudaFree(s->d_bytes);
    cudaFree(s->d_diag);
    for (cudaEvent_t e : s->pool) cudaEventDestroy(e);
    delete s;
}

int check_status(mcbgpu_solver *s, cudaStream_t st) {
    unsigned v = 0;
    MCB_CUDA(cudaMemcpyAsync(&v, s->d_status, sizeof v, cudaMemcpyDeviceToHost, st));
    MCB_CUDA(cudaStreamSynchronize(st));
    if (v & (ST_NO_CANDIDATE | ST_RANK_DEFICIT)) {
        set_error("no odd candidate for some support vector (status 0x%x)", v);
        return MCBGPU_E_NO_CANDIDATE;
    }
    if (v) {
        set_error("device status 0x%x", v);
        return MCBGPU_E_DEVICE;
    }
    return MCBGPU_OK;
}

int search_smem_words(const mcbgpu_solver *s, int e) {
    int we = (e >> 6) + 1;
    return (we + 1) & ~1;
}

}  // namespace

extern "C" {

int mcbgpu_solver_create(mcbgpu_solver **out, int32_t N, int64_t K, int64_t nnz) {
    if (!out || N < 0 || K < 0 || nnz < 0 || N >= (1 << 26)) {
        set_error("mcbgpu_solver_create: invalid sizes (N must be < 2^26)");
        return MCBGPU_E_ARG;
    }
    *out = nullptr;
    mcbgpu_solver *s = new mcbgpu_solver();
    s->N = N;
    s->K = K;
    s->nnz = nnz;
    s->W = (N + 63) / 64;
    s->P = ((s->W + 3) / 4) * 4;
    if (s->P == 0) s->P = 4;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&s->sm_count, cudaDevAttrMultiProcessorCount, dev);
    const size_t ntiles = (size_t)((K + kTile - 1) / kTile) + 2;
    long long bytes = 0;
#define ALLOC(ptr, sz)                                                         \
    do {                                                                       \
        size_t _b = (size_t)(sz);                                              \
        if (_b < 16) _b = 16;                                                  \
        if (e == cudaSuccess) e = cudaMalloc((void **)&(ptr), _b);             \
        bytes += (long long)_b;                                                \
    } while (0)
    ALLOC(s->d_weight, sizeof(int32_t) * (size_t)K);
    ALLOC(s->d_off, sizeof(int64_t) * (size_t)(K + 1));
    ALLOC(s->d_coords, sizeof(int32_t) * (size_t)(nnz + 16));  // aligned 16-byte loads read up to 11 past the end
    ALLOC(s->d_head, sizeof(int32_t) * kHead * (size_t)K);
    ALLOC(s->d_S, sizeof(uint64_t) * (size_t)N * s->P);
    ALLOC(s->d_C, sizeof(uint64_t) * (size_t)s->P);
    ALLOC(s->d_T, sizeof(uint64_t) * 64 * (size_t)s->P);
    ALLOC(s->d_Warr, sizeof(uint64_t) * (size_t)kTile * ntiles);
    if (kGroup > 1) {
        ALLOC(s->d_Warr2, sizeof(uint64_t) * (size_t)kTile * ntiles);
        if (kGroup > 2) ALLOC(s->d_Warr3, sizeof(uint64_t) * (size_t)kTile * ntiles);
        ALLOC(s->d_Tg, sizeof(uint64_t) * kGStride * 64 * (size_t)s->P);
        ALLOC(s->d_beta, sizeof(uint64_t) * 3 * 192);
        ALLOC(s->d_masks, sizeof(uint64_t) * 2 * 64);
    }
    ALLOC(s->d_nearD, sizeof(unsigned long long) * 2 * kNearMaxRows);
    ALLOC(s->d_unit, (size_t)N);
    ALLOC(s->d_Dfar, sizeof(unsigned long long) * (size_t)N);
    ALLOC(s->d_rowlist[0], sizeof(int32_t) * (size_t)N);
    ALLOC(s->d_rowlist[1], sizeof(int32_t) * (size_t)N);
    ALLOC(s->d_denselist[0], sizeof(int32_t) * (size_t)N);
    ALLOC(s->d_denselist[1], sizeof(int32_t) * (size_t)N);
    ALLOC(s->d_nzc, sizeof(uint16_t) * (size_t)N);
    ALLOC(s->d_nzw, sizeof(uint32_t) * kNzCap * (size_t)N);
    ALLOC(s->d_touch, sizeof(int32_t) * (size_t)N);
    ALLOC(s->d_chg_row, sizeof(int32_t) * (size_t)N);
    ALLOC(s->d_chg_beta, sizeof(unsigned long long) * (size_t)N);
    ALLOC(s->d_fcnt, sizeof(unsigned) * 8);
    ALLOC(s->d_tile_epoch, sizeof(unsigned) * ntiles);
    ALLOC(s->d_tile_minc, sizeof(int32_t) * ntiles);
    ALLOC(s->d_gbar, sizeof(GridBar));
    ALLOC(s->d_word_end, sizeof(unsigned) * 2 * ((size_t)s->P + 1));
    ALLOC(s->d_slots, sizeof(IterSlot) * 2);
    ALLOC(s->d_bs, sizeof(BlockState));
    ALLOC(s->d_selected, sizeof(long long) * (size_t)(N > 0 ? N : 1));
    ALLOC(s->d_status, sizeof(unsigned));
    ALLOC(s->d_bytes, sizeof(unsigned long long) * KC_COUNT);
    ALLOC(s->d_check, sizeof(unsigned) * 2);
    ALLOC(s->d_diag, sizeof(unsigned long long) * (kDiagWords + 8 * 1024));
#undef ALLOC
    if (e == cudaSuccess) e = cudaMemset(s->d_diag, 0, sizeof(unsigned long long) * kDiagWords);
    if (e == cudaSuccess) e = cudaMemset(s->d_bytes, 0, sizeof(unsigned long long) * KC_COUNT);
    if (e == cudaSuccess) e = cudaMemset(s->d_tile_epoch, 0, sizeof(unsigned) * ntiles);
    if (e == cudaSuccess) e = cudaMemset(s->d_gbar, 0, sizeof(GridBar));
    if (e == cudaSuccess) e = cudaMemset(s->d_nearD, 0, sizeof(unsigned long long) * 2 * kNearMaxRows);
    if (e == cudaSuccess) e = cudaMemset(s->d_Dfar, 0, sizeof(unsigned long long) * ((size_t)N > 0 ? (size_t)N : 2));
    if (e == cudaSuccess) e = cudaMemset(s->d_unit, 1, (size_t)N > 0 ? (size_t)N : 16);
    if (e == cudaSuccess) e = cudaMemset(s->d_fcnt, 0, sizeof(unsigned) * 8);
    if (e == cudaSuccess) e = cudaMemset(s->d_word_end, 0, sizeof(unsigned) * 2 * ((size_t)s->P + 1));
    // the far update fills every SM when it runs; with the critical path (transpose,
    // streaming pass, pivot search, near update) on a higher-priority stream, the
    // block scheduler gives that path's CTAs the SMs as they free up
    int prio_low = 0, prio_high = 0;
    if (e == cudaSuccess) e = cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&s->st2, cudaStreamNonBlocking, prio_low);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&s->st1, cudaStreamNonBlocking, prio_high);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_join, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_tail, cudaEventDisableTiming);
    for (int i = 0; i < 4 && e == cudaSuccess; i++) e = cudaEventCreateWithFlags(&s->ev_upd[i], cudaEventDisableTiming);
    for (int i = 0; i < 2 && e == cudaSuccess; i++) e = cudaEventCreateWithFlags(&s->ev_par[i], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMemset(s->d_coords, 0, sizeof(int32_t) * (size_t)(nnz + 16));
    if (e == cudaSuccess) {
        const int G = s->sm_count > 0 ? std::max(1, s->sm_count / MCB_PIVOT_DIV) : 1;  // one CTA per SM
        const size_t smem = pivot_smem_bytes(G);
        e = cudaFuncSetAttribute(blk_pivot_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        // the block tail sorts the pairs in shared memory past the tables (P + 1 counters)
        // and materialises 2 x 64 x (kMatCols + 1) words there
        if (e == cudaSuccess && sizeof(unsigned) * ((size_t)s->P + 1) > smem - 32768) e = cudaErrorInvalidValue;
        int per_sm = 0;
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, blk_pivot_kernel, kPivotThreads, smem);
        if (e == cudaSuccess && per_sm < 1) e = cudaErrorInvalidConfiguration;
        s->pivot_grid = G;
        // two step-parity halves of: ranks + W's (G x kLmax each), ends, counts (G each)
        const size_t rb = sizeof(unsigned long long) * 2 * (size_t)G * (2 * kLmax + 2);
        if (e == cudaSuccess) e = cudaMalloc((void **)&s->d_reports, rb);
        bytes += (long long)rb;
    }
    if (e == cudaSuccess) e = cudaMemset(s->d_bs, 0, sizeof(BlockState));
    if (e == cudaSuccess) e = cudaMemset(s->d_status, 0, sizeof(unsigned));
    if (e != cudaSuccess) {
        free_solver(s);
        return cuda_fail(e, "mcbgpu_solver_create");
    }
    s->device_bytes = bytes;
    *out = s;
    return MCBGPU_OK;
}

int mcbgpu_solver_reset(mcbgpu_solver *s, void *stream) {
    if (!s) {
        set_error("mcbgpu_solver_reset: NULL handle");
        return MCBGPU_E_ARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    if (s->N > 0) {
        int grid = s->sm_count > 0 ? s->sm_count * 4 : 256;
        {
            Launch L(s, KC_INIT, st);
            init_identity_kernel<<<grid, 256, 0, st>>>(s->d_S, s->N, s->P);
        }
        MCB_CUDA(cudaGetLastError());
    }
    {
        Launch L(s, KC_RESET, st);
        reset_state_kernel<<<1, 32, 0, st>>>(s->d_slots, s->d_bs, s->d_status);
    }
    MCB_CUDA(cudaMemsetAsync(s->d_nearD, 0, sizeof(unsigned long long) * 2 * kNearMaxRows, st));
    if (s->N > 0) {  // every row is a unit vector again; no non-unit rows, no scattered D left over
        MCB_CUDA(cudaMemsetAsync(s->d_unit, 1, (size_t)s->N, st));
        MCB_CUDA(cudaMemsetAsync(s->d_Dfar, 0, sizeof(unsigned long long) * (size_t)s->N, st));
    }
    MCB_CUDA(cudaMemsetAsync(s->d_fcnt, 0, sizeof(unsigned) * 8, st));
    s->list_cur = 0;
    MCB_CUDA(cudaGetLastError());
    s->iters_run = 0;
    return MCBGPU_OK;
}

// The upload of both entry points: `kind` says where the three arrays live.
static int solver_upload(mcbgpu_solver *s, const int32_t *weight, const int64_t *offsets, const int32_t *coords,
                         void *stream, cudaMemcpyKind kind) {
    if (!s || (s->K > 0 && (!weight || !offsets)) || (s->nnz > 0 && !coords)) {
        set_error("mcbgpu_solver_upload: NULL argument");
        return MCBGPU_E_ARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    s->uploaded = false;
    if (s->K > 0) {
        MCB_CUDA(cudaMemcpyAsync(s->d_weight, weight, sizeof(int32_t) * (size_t)s->K, kind, st));
        MCB_CUDA(cudaMemcpyAsync(s->d_off, offsets, sizeof(int64_t) * (size_t)(s->K + 1), kind, st));
    }
    if (s->nnz > 0) MCB_CUDA(cudaMemcpyAsync(s->d_coords, coords, sizeof(int32_t) * (size_t)s->nnz, kind, st));
    // the lists are checked on the device before any other kernel reads them
    unsigned chk[2] = {0, 0};
    MCB_CUDA(cudaMemsetAsync(s->d_check, 0, sizeof chk, st));
    if (s->K > 0) {
        Launch L(s, KC_VALIDATE, st);
        int grid = (int)std::min<long long>((s->K + 255) / 256, (long long)(s->sm_count > 0 ? s->sm_count : 148) * 16);
        validate_kernel<<<grid, 256, 0, st>>>(s->d_off, s->d_coords, s->K, s->nnz, s->N, s->d_check, s->d_check + 1);
    }
    MCB_CUDA(cudaGetLastError());
    MCB_CUDA(cudaMemcpyAsync(chk, s->d_check, sizeof chk, cudaMemcpyDeviceToHost, st));
    MCB_CUDA(cudaStreamSynchronize(st));
    if (chk[0]) {
        set_error("mcbgpu_solver_upload: %s", (chk[0] & 1u) ? "offsets must be non-decreasing from 0 to nnz"
                                                             : "coordinates must be ascending in [0, N)");
        return MCBGPU_E_ARG;
    }
    s->max_len = (int)chk[1];
    unsigned cap = (unsigned)(64 * (size_t)(s->max_len > 0 ? s->max_len : 1));
    if (cap > s->pair_cap) {  // resolve scratch + sorted pairs of the two block parities
        cudaFree(s->d_pairs);
        s->d_pairs = nullptr;
        MCB_CUDA(cudaMalloc((void **)&s->d_pairs, sizeof(unsigned) * 3 * (size_t)cap));
        s->device_bytes += (long long)sizeof(unsigned) * 3 * cap;
        s->pair_cap = cap;
    }
    const long long ntiles = (s->K + kTile - 1) / kTile;
    if (ntiles > 0) {
        {
            Launch L(s, KC_VALIDATE, st);
            const int hgrid = (int)std::min<long long>((s->K + 255) / 256, (long long)(s->sm_count > 0 ? s->sm_count : 148) * 16);
            head_kernel<<<hgrid, 256, 0, st>>>(s->d_off, s->d_coords, s->K, s->d_head);
        }
        int grid = (int)std::min<long long>(ntiles, (long long)(s->sm_count > 0 ? s->sm_count : 148) * 8);
        {
            Launch L(s, KC_TILE_MINC, st);
            tile_minc_kernel<<<grid, 256, 0, st>>>(s->d_off, s->d_coords, s->K, s->d_tile_minc, ntiles);
        }
        MCB_CUDA(cudaGetLastError());
    }
    s->uploaded = true;
    return mcbgpu_solver_reset(s, stream);
}

int mcbgpu_solver_upload(mcbgpu_solver *s, const int32_t *weight, const int64_t *offsets, const int32_t *coords,
                         void *stream) {
    return solver_upload(s, weight, offsets, coords, stream, cudaMemcpyHostToDevice);
}

int mcbgpu_solver_upload_device(mcbgpu_solver *s, const int32_t *weight, const int64_t *offsets,
                                const int32_t *coords, void *stream) {
    return solver_upload(s, weight, offsets, coords, stream, cudaMemcpyDeviceToDevice);
}

int mcbgpu_select(mcbgpu_solver *s, int32_t e, int64_t *rank, void *stream) {
    if (!s || e < 0 || e >= s->N) {
        set_error("mcbgpu_select: invalid iteration");
        return MCBGPU_E_ARG;
    }
    if (!s->uploaded) {
        set_error("mcbgpu_select: candidates not uploaded");
        return MCBGPU_E_STATE;
    }
    cudaStream_t st = (cudaStream_t)stream;
    const int we = search_smem_words(s, e);
    const size_t smem = (size_t)we * 8;
    if (smem > 200 * 1024) {
        set_error("mcbgpu_select: support vector prefix too large for shared memory");
        return MCBGPU_E_ARG;
    }
    if (smem > 48 * 1024) MCB_CUDA(cudaFuncSetAttribute(search_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    // the S row pitch is a multiple of 4 words, so reading `we` (even) words is in bounds
    int grid = s->sm_count > 0 ? s->sm_count * 4 : 256;
    long long ntiles = (s->K + kTile - 1) / kTile;
    if (ntiles < grid) grid = (int)(ntiles > 0 ? ntiles : 1);
    IterSlot *slot = s->d_slots + (e & 1);
    {
        Launch L(s, KC_SEARCH, st);
        search_kernel<<<grid, kScanThreads, smem, st>>>(s->d_S + (size_t)e * s->P, e, we, s->d_off, s->d_coords,
                                                         s->K, slot, s->d_status, L.bytes());
    }
    MCB_CUDA(cudaGetLastError());
    if (rank) {
        unsigned long long r = 0;
        MCB_CUDA(cudaMemcpyAsync(&r, &slot->best, sizeof r, cudaMemcpyDeviceToHost, st));
        MCB_CUDA(cudaStreamSynchronize(st));
        *rank = r == kNone ? -1 : (int64_t)r;
        if (r == kNone) {
            set_error("mcbgpu_select: no odd candidate at iteration %d", e);
            return MCBGPU_E_NO_CANDIDATE;
        }
    }
    return MCBGPU_OK;
}

int mcbgpu_cycle_vector(mcbgpu_solver *s, int32_t e, uint64_t *words, void *stream) {
    if (!s || e < 0 || e >= s->N) {
        set_error("mcbgpu_cycle_vector: invalid iteration");
        return MCBGPU_E_ARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    {
        Launch L(s, KC_CYCLE, st);
        cycle_vector_kernel<<<1, 256, 0, st>>>(s->d_C, s->W, s->d_off, s->d_coords, s->d_slots + (e & 1));
    }
    MCB_CUDA(cudaGetLastError());
    if (words) {
        MCB_CUDA(cudaMemcpyAsync(words, s->d_C, sizeof(uint64_t) * (size_t)s->W, cudaMemcpyDeviceToHost, st));
        MCB_CUDA(cudaStreamSynchronize(st));
    }
    return MCBGPU_OK;
}

int mcbgpu_update(mcbgpu_solver *s, int32_t e, void *stream) {
    if (!s || e < 0 || e >= s->N) {
        set_error("mcbgpu_update: invalid iteration");
        return MCBGPU_E_ARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    int rows = s->N - e - 1;
    int grid = (rows + 7) / 8;
    int cap = s->sm_count > 0 ? s->sm_count * 8 : 1024;
    if (grid > cap) grid = cap;
    if (grid < 1) grid = 1;
    {
        Launch L(s, KC_UPDATE, st);
        update_kernel<<<grid, 256, 0, st>>>(s->d_S, s->N, s->P, e, s->d_off, s->d_coords, s->d_weight,
                                            s->d_slots + (e & 1), s->d_slots + ((e + 1) & 1), s->d_selected,
                                            s->d_bs, s->d_status);
    }
    MCB_CUDA(cudaGetLastError());
    if (e + 1 > s->iters_run) s->iters_run = e + 1;
    return MCBGPU_OK;
}

int mcbgpu_solver_run_plain(mcbgpu_solver *s, int64_t max_iterations, void *stream) {
    if (!s) {
        set_error("mcbgpu_solver_run_plain: NULL handle");
        return MCBGPU_E_ARG;
    }
    int64_t iters = (max_iterations >= 0 && max_iterations < s->N) ? max_iterations : s->N;
    for (int64_t e = 0; e < iters; e++) {
        int rc = mcbgpu_select(s, (int32_t)e, nullptr, stream);
        if (rc) return rc;
        rc = mcbgpu_update(s, (int32_t)e, stream);
        if (rc) return rc;
    }
    return MCBGPU_OK;
}

int mcbgpu_solver_run(mcbgpu_solver *s, int64_t max_iterations, void *stream) {
    if (!s) {
        set_error("mcbgpu_solver_run: NULL handle");
        return MCBGPU_E_ARG;
    }
    if (!s->uploaded) {
        set_error("mcbgpu_solver_run: candidates not uploaded");
        return MCBGPU_E_STATE;
    }
    cudaStream_t caller = (cudaStream_t)stream;
    cudaStream_t st = s->st1;  // the critical path; joined back into the caller's stream at the end
    const int64_t iters = (max_iterations >= 0 && max_iterations < s->N) ? max_iterations : s->N;
    const int64_t nblocks = (iters + 63) / 64;
    const bool pdl = s->pdl;
    size_t tnext = 0;             // tuning events used
    cudaEvent_t tev_a = nullptr;  // start of the group being timed
    const int sms = s->sm_count > 0 ? s->sm_count : 148;
    long long ntiles = (s->K + kTile - 1) / kTile;
    // The update of a block is split: the next rows on `st` (the next block's
    // transpose needs them), every later row on st2, where it overlaps the next
    // block's transpose, streaming pass and pivot search.  Dependencies across the
    // two streams:
    //  - a block's near rows wait for the last far update that reaches them (far
    //    updates run in order on st2, so the last one suffices);
    //  - the buffers the far update reads (gcol, tables, sorted pairs, word_end)
    //    alternate by block parity, so a block's pivot kernel (whose tail rewrites
    //    them) waits for the far update two blocks back.
    // Blocks in groups of kGroup (MCB_GROUP): the first block's streaming pass also
    // computes W against each later block's rows as they are then; each later block
    // corrects those W's (blk_wfix_kernel) instead of streaming the lists again.  So
    // the later blocks' rows must be final up to the block before the group when the
    // group starts: the last block of a group updates the next kGroup x 64 rows on
    // `st`, and block i < kGroup - 1 of a group the rows of the group's later blocks
    // (their update bits go to beta slab i for the corrections).
    MCB_CUDA(cudaEventRecord(s->ev_fork, caller));
    MCB_CUDA(cudaStreamWaitEvent(st, s->ev_fork, 0));
    MCB_CUDA(cudaStreamWaitEvent(s->st2, s->ev_fork, 0));
    struct FarRec {
        long long start;  // first row of the far update
        int slot;         // its event in ev_upd
    };
    FarRec fars[4];
    int nfar = 0, ring = 0;
    bool par_far[2] = {false, false};  // a far update of this parity was recorded in ev_par
    uint64_t *Wpos[3] = {s->d_Warr, s->d_Warr2, s->d_Warr3};
    for (int64_t e0 = 0; e0 < iters; e0 += 64) {
        const int b = (int)std::min<int64_t>(64, iters - e0);
        const int par = (int)((e0 / 64) & 1);
        const int pos = (int)((e0 / 64) % kGroup);  // position in its group
        const int Wb = (int)((e0 + b + 63) / 64);
        const int bound = (int)(e0 + b);
        int bl[2] = {0, 0};  // a group's first block: b of the later blocks
        if (pos == 0)
            for (int jj = 1; jj < kGroup; jj++) bl[jj - 1] = (int)std::max<int64_t>(0, std::min<int64_t>(64, iters - e0 - 64 * jj));
        const int nl = (bl[0] > 0 ? 1 : 0) + (bl[1] > 0 ? 1 : 0);
        const int bd1 = (int)(e0 + 64 + bl[0]), bd2 = (int)(e0 + 128 + bl[1]);
        const int Wb1 = bl[0] > 0 ? (bd1 + 63) / 64 : 0, Wb2 = bl[1] > 0 ? (bd2 + 63) / 64 : 0;
        // this block's search shape: by segment (tuned or default), forced, or while
        // tuning every candidate in turn, group by group (a group's blocks share one
        // streaming pass, so a group is the unit that is timed: from its first
        // transpose to its last pivot search)
        const int64_t blk = e0 / 64;
        const int seg = (int)(blk * kShapeSegs / nblocks);
        const int shp = s->tuning ? (int)((blk / kGroup) % kNumShapes)
                        : s->forced_shape >= 0 ? s->forced_shape
                                               : s->seg_shape[seg];
        const PivotShape sh = kCandidateShapes[shp];
        if (s->tuning && pos == 0) {
            while (s->tpool.size() < tnext + 2) {
                cudaEvent_t ev = nullptr;
                MCB_CUDA(cudaEventCreate(&ev));
                s->tpool.push_back(ev);
            }
            tev_a = s->tpool[tnext++];
            MCB_CUDA(cudaEventRecord(tev_a, st));
        }
        {
            Launch L(s, KC_TRANSPOSE, st);
            MCB_CUDA(launch_k(pdl, blk_transpose_kernel, dim3((std::max(Wb, std::max(Wb1, Wb2)) + 7) / 8), dim3(256), 0,
                              st, (const uint64_t *)s->d_S, s->P, (int)e0, b, Wb, s->d_T, s->d_bs, ntiles, s->d_gbar,
                              (long long)s->pivot_grid * sh.win_mid, sh.stream_pct, s->d_Tg, bl[0], Wb1, bl[1],
                              Wb2));
        }
        if (ntiles > 0 && pos > 0) {
            Launch L(s, KC_WFIX, st);
            if (pos == 1)
                MCB_CUDA(launch_k(pdl, blk_wfix_kernel<1>, dim3(sms), dim3(kTile), 0, st, (const int32_t *)s->d_tile_minc,
                                  bound, s->d_bs, (const uint64_t *)s->d_beta, s->d_masks, b, Wpos[0], Wpos[1], Wpos[1],
                                  s->d_tile_epoch, L.bytes()));
            else
                MCB_CUDA(launch_k(pdl, blk_wfix_kernel<2>, dim3(sms), dim3(kTile), 0, st, (const int32_t *)s->d_tile_minc,
                                  bound, s->d_bs, (const uint64_t *)s->d_beta, s->d_masks, b, Wpos[0], Wpos[1], Wpos[2],
                                  s->d_tile_epoch, L.bytes()));
        } else if (ntiles > 0) {
            Launch L(s, KC_WSTREAM, st);
            const int64_t *woff = s->d_off;
            const int32_t *wco = s->d_coords, *whd = s->d_head, *wtm = s->d_tile_minc;
            const uint64_t *wT = s->d_T, *wTg = s->d_Tg;
            const BlockState *wbs = s->d_bs;
            uint64_t *nul = nullptr;
            if (nl == 2)
                MCB_CUDA(launch_k(pdl, blk_w_kernel<3>, dim3(sms * 2), dim3(kTile), 0, st, s->K, woff, wco, whd, wtm, wT,
                                  bound, wbs, Wpos[0], s->d_tile_epoch, L.bytes(), wTg, bd1, bd2, Wpos[1], Wpos[2]));
            else if (nl == 1)
                MCB_CUDA(launch_k(pdl, blk_w_kernel<2>, dim3(sms * 2), dim3(kTile), 0, st, s->K, woff, wco, whd, wtm, wT,
                                  bound, wbs, Wpos[0], s->d_tile_epoch, L.bytes(), wTg, bd1, bd1, Wpos[1], nul));
            else
                MCB_CUDA(launch_k(pdl, blk_w_kernel<1>, dim3(sms * 2), dim3(kTile), 0, st, s->K, woff, wco, whd, wtm, wT,
                                  bound, wbs, Wpos[0], s->d_tile_epoch, L.bytes(), (const uint64_t *)nullptr, 0, 0, nul,
                                  nul));
        }
        // this block's tail rewrites the parity buffers the far update two blocks back reads
        if (par_far[par]) MCB_CUDA(cudaStreamWaitEvent(st, s->ev_par[par], 0));
        {
            Launch L(s, KC_PIVOT, st);
            long long K = s->K;
            const int64_t *off = s->d_off;
            const int32_t *co = s->d_coords;
            const int32_t *hd = s->d_head;
            const int32_t *tm = s->d_tile_minc;
            const uint64_t *T = s->d_T;
            BlockState *bs = s->d_bs;
            uint64_t *Wa = Wpos[pos];
            unsigned *te = s->d_tile_epoch;
            GridBar *gb = s->d_gbar;
            unsigned *stt = s->d_status;
            unsigned long long *rp = s->d_reports;
            unsigned long long *nb = L.bytes();
            unsigned long long *dg = s->d_diag;
            unsigned long long *db = s->d_diag + kDiagWords;
            TailArgs ta;
            ta.S = s->d_S;
            ta.selected = s->d_selected;
            ta.weight = s->d_weight;
            ta.pairs = s->d_pairs;
            ta.sorted = s->d_pairs + (size_t)(1 + par) * s->pair_cap;
            ta.word_end = s->d_word_end + (size_t)par * (s->P + 1);
            ta.pair_cap = s->pair_cap;
            ta.P = s->P;
            ta.e0 = (int)e0;
            ta.Wb = Wb;
            ta.par = par;
            PivotShape shv = sh;
            void *args[] = {&K, &off, &co, &hd, &tm, &T, (void *)&bound, &bs, &Wa, &te, &rp, &gb, &stt, &nb, &dg, &db, &ta,
                            &shv};
            MCB_CUDA(launch_coop(pdl, (const void *)blk_pivot_kernel, dim3(s->pivot_grid), dim3(kPivotThreads), args,
                                 pivot_smem_bytes(s->pivot_grid), st));
        }
        if (s->tuning && (pos == kGroup - 1 || e0 + b >= iters)) {  // the group's last block
            cudaEvent_t tev_b = s->tpool[tnext++];
            MCB_CUDA(cudaEventRecord(tev_b, st));
            s->tune_recs.push_back({seg, shp, (int)(blk % kGroup) + 1, tev_a, tev_b});
        }
        if (e0 + b < s->N) {
            const int near_rows = kGroup == 1 ? 64 : pos == kGroup - 1 ? 64 * kGroup : 64 * (kGroup - 1 - pos);
            const long long near_end = std::min<long long>(e0 + b + near_rows, s->N), far_end = s->N;
            const uint64_t *gcol = reinterpret_cast<const uint64_t *>(&s->d_bs->gcol[par][0]);
            const unsigned *pairs = s->d_pairs + (size_t)(1 + par) * s->pair_cap;
            const unsigned *wend = s->d_word_end + (size_t)par * (s->P + 1);
            auto grid_for = [&](long long rows) {
                long long g = (rows + kUpdGroups * kUpdRows - 1) / (kUpdGroups * kUpdRows);
                return (int)std::max<long long>(1, std::min<long long>(g, (long long)sms * MCB_UPD_CTAS));
            };
            // the last earlier far update that reaches the near rows [e0 + b, near_end)
            int wait_slot = -1;
            for (int q = 0; q < nfar; q++)
                if (fars[q].start < near_end) wait_slot = fars[q].slot;  // fars[] in launch order
            if (near_end < far_end) {  // far rows: on st2 once this block's tail is done
                MCB_CUDA(cudaEventRecord(s->ev_tail, st));
                MCB_CUDA(cudaStreamWaitEvent(s->st2, s->ev_tail, 0));
                // scatter into the unit rows, gather the listed non-unit rows, apply the
                // touched unit rows; the lists swap for the next far update
                const int lin = s->list_cur, lout = 1 - lin;
                MCB_CUDA(cudaMemsetAsync(s->d_fcnt + 4 * lout, 0, sizeof(unsigned) * 4, s->st2));
                FarLists fl;
                fl.sp_in = s->d_rowlist[lin];
                fl.dn_in = s->d_denselist[lin];
                fl.n_in = s->d_fcnt + 4 * lin;
                fl.sp_out = s->d_rowlist[lout];
                fl.dn_out = s->d_denselist[lout];
                fl.n_out = s->d_fcnt + 4 * lout;
                fl.touch = s->d_touch;
                fl.chg_row = s->d_chg_row;
                fl.chg_beta = s->d_chg_beta;
                fl.nzc = s->d_nzc;
                fl.nzw = s->d_nzw;
                Launch L(s, KC_BLK_UPDATE, s->st2, 3);
                far_scatter_kernel<<<sms * 2, 256, 0, s->st2>>>(pairs, wend, s->P, near_end, far_end, s->d_unit,
                                                                 s->d_Dfar, s->d_touch, s->d_fcnt + 4 * lout + 2,
                                                                 L.bytes());
                // grid-stride over the listed rows: two CTAs per SM cover ~78k sparse rows per
                // pass (a block lists ~12k at the 1M-vertex graph); more CTAs would mostly exit
                far_rows_kernel<<<std::min(grid_for(far_end - near_end), sms * 2), kUpdThreads, 0, s->st2>>>(
                    s->d_S, near_end, s->P, b, gcol, pairs, wend, fl, s->d_Dfar, s->d_unit, L.bytes(), s->d_diag);
                far_apply_kernel<<<sms * 2, kApplyThreads, 0, s->st2>>>(s->d_S, s->P, (int)e0, Wb, fl, L.bytes());
                s->list_cur = lout;
            }
            if (wait_slot >= 0) MCB_CUDA(cudaStreamWaitEvent(st, s->ev_upd[wait_slot], 0));
            {
                Launch L(s, KC_BLK_UPDATE_NEAR, st, 2);
                const int nrows = (int)(near_end - (e0 + b));
                uint64_t *bo = kGroup > 1 && pos < kGroup - 1 ? s->d_beta + (size_t)pos * 192 : nullptr;
                unsigned long long *Dn = s->d_nearD + (size_t)par * kNearMaxRows;
                unsigned long long *Dn_next = s->d_nearD + (size_t)(par ^ 1) * kNearMaxRows;
                const int agrid = (int)std::min<long long>((Wb + kNearCols - 1) / kNearCols, (long long)sms * 2);
                MCB_CUDA(launch_k(pdl, near_d_kernel, dim3(sms), dim3(256), 0, st, (const uint64_t *)s->d_S,
                                  (long long)(e0 + b), nrows, s->P, pairs, wend, Dn, L.bytes()));
                MCB_CUDA(launch_k(pdl, near_apply_kernel, dim3(agrid), dim3(256), 0, st, s->d_S, (long long)(e0 + b), nrows,
                                  s->P, b, (int)e0, Wb, gcol, (const unsigned long long *)Dn, Dn_next, bo, L.bytes()));
            }
            if (near_end < far_end) {
                const int slot = ring;
                ring = (ring + 1) & 3;
                MCB_CUDA(cudaEventRecord(s->ev_upd[slot], s->st2));
                MCB_CUDA(cudaEventRecord(s->ev_par[par], s->st2));
                par_far[par] = true;
                if (nfar == 4) {  // keep the last three
                    for (int q = 1; q < 4; q++) fars[q - 1] = fars[q];
                    nfar = 3;
                }
                fars[nfar++] = {near_end, slot};
            }
        }
        MCB_CUDA(cudaGetLastError());
    }
    if (nfar > 0) MCB_CUDA(cudaStreamWaitEvent(st, s->ev_upd[fars[nfar - 1].slot], 0));
    MCB_CUDA(cudaEventRecord(s->ev_join, st));
    MCB_CUDA(cudaStreamWaitEvent(caller, s->ev_join, 0));

    s->iters_run = iters;
    return MCBGPU_OK;
}

int mcbgpu_solver_results(mcbgpu_solver *s, int64_t *selected, int64_t count, int64_t *total_weight, void *stream) {
    if (!s) {
        set_error("mcbgpu_solver_results: NULL handle");
        return MCBGPU_E_ARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    if (count > s->iters_run) count = s->iters_run;
    if (selected && count > 0)
        MCB_CUDA(cudaMemcpyAsync(selected, s->d_selected, sizeof(int64_t) * (size_t)count, cudaMemcpyDeviceToHost, st));
    unsigned long long tot = 0;
    MCB_CUDA(cudaMemcpyAsync(&tot, &s->d_bs->total, sizeof tot, cudaMemcpyDeviceToHost, st));
    int rc = check_status(s, st);
    if (total_weight) *total_weight = (int64_t)tot;
    return rc;
}

int mcbgpu_solver_get_support(mcbgpu_solver *s, int32_t j, uint64_t *words, void *stream) {
    if (!s || !words || j < 0 || j >= s->N) {
        set_error("mcbgpu_solver_get_support: invalid argument");
        return MCBGPU_E_ARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    MCB_CUDA(cudaMemcpyAsync(words, s->d_S + (size_t)j * s->P, sizeof(uint64_t) * (size_t)s->W,
                             cudaMemcpyDeviceToHost, st));
    MCB_CUDA(cudaStreamSynchronize(st));
    return MCBGPU_OK;
}

int mcbgpu_solver_verify(mcbgpu_solver *s, int64_t *violations, int64_t *first_bad_i, int64_t *first_bad_j,
                         void *stream) {
    if (!s || !violations) {
        set_error("mcbgpu_solver_verify: invalid argument");
        return MCBGPU_E_ARG;
    }
    if (s->iters_run != s->N) {
        set_error("mcbgpu_solver_verify: the basis is not complete (%lld of %d iterations run)",
                  (long long)s->iters_run, s->N);
        return MCBGPU_E_STATE;
    }
    int rc = check_status(s, (cudaStream_t)stream);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    *violations = 0;
    if (s->N == 0) return MCBGPU_OK;
    unsigned long long *C = nullptr, *cnt = nullptr;
    const size_t cbytes = sizeof(unsigned long long) * (size_t)s->N * s->P;
    cudaError_t e = cudaMalloc((void **)&C, cbytes);
    if (e == cudaSuccess) e = cudaMalloc((void **)&cnt, 2 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemsetAsync(C, 0, cbytes, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(cnt + 1, 0xff, sizeof(unsigned long long), st);
    if (e == cudaSuccess) {
        const int sms = s->sm_count > 0 ? s->sm_count : 148;
        cert_rows_kernel<<<sms * 8, 256, 0, st>>>(s->d_selected, s->N, s->P, s->K, s->d_off, s->d_coords, C,
                                                  s->d_status);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        const unsigned tiles = (unsigned)((s->N + 63) / 64);
        cert_check_kernel<<<dim3(tiles, tiles), 256, 0, st>>>(C, s->d_S, s->N, s->P, cnt, cnt + 1);
        e = cudaGetLastError();
    }
    unsigned long long h[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, cnt, sizeof h, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(C);
    cudaFree(cnt);
    if (e != cudaSuccess) return cuda_fail(e, "mcbgpu_solver_verify");
    rc = check_status(s, st);
    if (rc) return rc;
    *violations = (int64_t)h[0];
    if (first_bad_i) *first_bad_i = h[0] ? (int64_t)(h[1] / (unsigned long long)s->N) : -1;
    if (first_bad_j) *first_bad_j = h[0] ? (int64_t)(h[1] % (unsigned long long)s->N) : -1;
    return MCBGPU_OK;
}

int mcbgpu_solver_set_profiling(mcbgpu_solver *s, int enable) {
    if (!s) {
        set_error("mcbgpu_solver_set_profiling: NULL handle");
        return MCBGPU_E_ARG;
    }
    MCB_CUDA(cudaDeviceSynchronize());
    s->recs.clear();
    s->pool_next = 0;
    MCB_CUDA(cudaMemset(s->d_bytes, 0, sizeof(unsigned long long) * KC_COUNT));
    s->profiling = enable != 0;
    return MCBGPU_OK;
}

int mcbgpu_solver_kernel_stats(mcbgpu_solver *s, mcbgpu_kernel_stat *out, int max_entries, int *count) {
    if (!s || (!out && max_entries > 0)) {
        set_error("mcbgpu_solver_kernel_stats: invalid argument");
        return MCBGPU_E_ARG;
    }
    MCB_CUDA(cudaDeviceSynchronize());
    double ms[KC_COUNT] = {0};
    long long n[KC_COUNT] = {0};
    for (const auto &r : s->recs) {
        float t = 0;
        MCB_CUDA(cudaEventElapsedTime(&t, r.a, r.b));
        ms[r.cls] += t;
        n[r.cls]++;
    }
    unsigned long long bytes[KC_COUNT];
    MCB_CUDA(cudaMemcpy(bytes, s->d_bytes, sizeof bytes, cudaMemcpyDeviceToHost));
    int c = 0;
    for (int k = 0; k < KC_COUNT; k++) {
        if (!n[k]) continue;
        if (c < max_entries) {
            out[c].name = kKernelNames[k];
            out[c].launches = n[k];
            out[c].ms = ms[k];
            out[c].bytes = (double)bytes[k];
        }
        c++;
    }
    if (count) *count = c;
    s->recs.clear();
    s->pool_next = 0;
    MCB_CUDA(cudaMemset(s->d_bytes, 0, sizeof(unsigned long long) * KC_COUNT));
    return MCBGPU_OK;
}

int mcbgpu_solver_diagnostics(mcbgpu_solver *s, int64_t *out, int n, int reset) {
    if (!s || (!out && n > 0) || n > kDiagWords) {
        set_error("mcbgpu_solver_diagnostics: invalid argument");
        return MCBGPU_E_ARG;
    }
    unsigned long long v[kDiagWords];
    MCB_CUDA(cudaDeviceSynchronize());
    MCB_CUDA(cudaMemcpy(v, s->d_diag, sizeof v, cudaMemcpyDeviceToHost));
    for (int i = 0; i < n; i++) out[i] = (int64_t)v[i];
    if (reset) {
        MCB_CUDA(cudaMemset(s->d_diag, 0, sizeof v));
        MCB_CUDA(cudaMemset(s->d_diag + 15, 0xff, sizeof(unsigned long long)));
    }
    return MCBGPU_OK;
}

int mcbgpu_solver_tune(mcbgpu_solver *s, double *ms_per_block, int32_t *chosen, void *stream) {
    if (!s) {
        set_error("mcbgpu_solver_tune: NULL handle");
        return MCBGPU_E_ARG;
    }
    if (!s->uploaded) {
        set_error("mcbgpu_solver_tune: candidates not uploaded");
        return MCBGPU_E_STATE;
    }
    const int64_t nblocks = ((int64_t)s->N + 63) / 64;
    // a few groups of every shape in every segment, else the default shape stays
    const bool enough = nblocks >= 4LL * kGroup * kNumShapes * kShapeSegs;
    drop_graph(s);  // the shapes change
    int rc = mcbgpu_solver_reset(s, stream);
    if (rc) return rc;
    s->tune_recs.clear();
    s->tuning = enough;
    rc = mcbgpu_solver_run(s, -1, stream);
    s->tuning = false;
    if (rc) return rc;
    MCB_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    double sum[kShapeSegs][kNumShapes] = {};
    long long cnt[kShapeSegs][kNumShapes] = {};
    for (const auto &r : s->tune_recs) {
        float t = 0;
        MCB_CUDA(cudaEventElapsedTime(&t, r.a, r.b));
        sum[r.seg][r.shape] += t;
        cnt[r.seg][r.shape] += r.blocks;
    }
    s->tune_recs.clear();
    for (int g = 0; g < kShapeSegs; g++) {
        int best = -1;
        double bt = 0;
        for (int k = 0; k < kNumShapes; k++) {
            const double m = cnt[g][k] ? sum[g][k] / (double)cnt[g][k] : 0.0;
            if (ms_per_block) ms_per_block[g * kNumShapes + k] = m;
            if (cnt[g][k] && (best < 0 || m < bt)) {
                best = k;
                bt = m;
            }
        }
        if (enough && best >= 0) s->seg_shape[g] = best;
        if (chosen) chosen[g] = s->seg_shape[g];
    }
    return MCBGPU_OK;
}

int mcbgpu_solver_set_shape(mcbgpu_solver *s, int32_t shape) {
    if (!s || shape < -1 || shape >= kNumShapes) {
        set_error("mcbgpu_solver_set_shape: invalid argument");
        return MCBGPU_E_ARG;
    }
    if (s->forced_shape != shape) drop_graph(s);
    s->forced_shape = shape;
    return MCBGPU_OK;
}

int mcbgpu_solver_run_graph(mcbgpu_solver *s, int64_t max_iterations, void *stream) {
    if (!s) {
        set_error("mcbgpu_solver_run_graph: NULL handle");
        return MCBGPU_E_ARG;
    }
    if (!s->uploaded || s->profiling || s->tuning) {
        set_error("mcbgpu_solver_run_graph: candidates not uploaded, or profiling on");
        return MCBGPU_E_STATE;
    }
    const int64_t iters = (max_iterations >= 0 && max_iterations < s->N) ? max_iterations : s->N;
    if (!s->gexec || s->gexec_iters != iters) {
        drop_graph(s);
        if (!s->cap) MCB_CUDA(cudaStreamCreateWithFlags(&s->cap, cudaStreamNonBlocking));
        // the solver's streams must be idle: their work joins the capture through events
        MCB_CUDA(cudaStreamSynchronize(s->st1));
        MCB_CUDA(cudaStreamSynchronize(s->st2));
        const long long l0 = s->launches;
        MCB_CUDA(cudaStreamBeginCapture(s->cap, cudaStreamCaptureModeThreadLocal));
        int rc = mcbgpu_solver_reset(s, s->cap);
        if (rc == MCBGPU_OK) rc = mcbgpu_solver_run(s, iters, s->cap);
        cudaGraph_t g = nullptr;
        const cudaError_t ec = cudaStreamEndCapture(s->cap, &g);
        const long long per = s->launches - l0;
        s->launches = l0;
        if (rc != MCBGPU_OK || ec != cudaSuccess || !g) {
            if (g) cudaGraphDestroy(g);
            (void)cudaGetLastError();
            if (rc == MCBGPU_OK) return ::mcbgpu::cuda_fail(ec != cudaSuccess ? ec : cudaErrorStreamCaptureInvalidated,
                                                            "cudaStreamEndCapture (solve graph)");
            return rc;
        }
        const cudaError_t ei = cudaGraphInstantiate(&s->gexec, g, 0);
        cudaGraphDestroy(g);
        if (ei != cudaSuccess) {
            s->gexec = nullptr;
            return ::mcbgpu::cuda_fail(ei, "cudaGraphInstantiate (solve graph)");
        }
        s->gexec_iters = iters;
        s->gexec_launches = per;
        s->gexec_list_end = s->list_cur;  // the host state a replay ends in (the capture ran the loop once)
    }
    MCB_CUDA(cudaGraphLaunch(s->gexec, (cudaStream_t)stream));
    s->launches += s->gexec_launches;
    s->list_cur = s->gexec_list_end;
    s->iters_run = iters;
    return MCBGPU_OK;
}

int mcbgpu_solver_shapes(const mcbgpu_solver *s, int32_t *params, int32_t max_shapes, int32_t *n_shapes,
                         int32_t *segment_shape) {
    if (!s || (!params && max_shapes > 0)) {
        set_error("mcbgpu_solver_shapes: invalid argument");
        return MCBGPU_E_ARG;
    }
    for (int k = 0; k < kNumShapes && k < max_shapes; k++) {
        const PivotShape &h = kCandidateShapes[k];
        const int32_t v[kShapeInts] = {h.win_early, h.rank_early, h.win_mid, h.rank_tail, h.win_tail, h.lmax,
                                       h.stream_pct};
        for (int i = 0; i < kShapeInts; i++) params[k * kShapeInts + i] = v[i];
    }
    if (n_shapes) *n_shapes = kNumShapes;
    if (segment_shape)
        for (int g = 0; g < kShapeSegs; g++) segment_shape[g] = s->forced_shape >= 0 ? s->forced_shape : s->seg_shape[g];
    return MCBGPU_OK;
}

int64_t mcbgpu_solver_launches(const mcbgpu_solver *s) { return s ? s->launches : 0; }
int64_t mcbgpu_solver_device_bytes(const mcbgpu_solver *s) { return s ? s->device_bytes : 0; }

int mcbgpu_solver_destroy(mcbgpu_solver *s) {
    if (!s) return MCBGPU_OK;
    cudaError_t e = cudaDeviceSynchronize();
    free_solver(s);
    if (e != cudaSuccess) return cuda_fail(e, "mcbgpu_solver_destroy");
    return MCBGPU_OK;
}

int mcbgpu_solve(int32_t N, int64_t K, const int32_t *weight, const int64_t *offsets, const int32_t *coords,
                 int64_t *selected, int64_t *total_weight) {
    if (K < 0 || !offsets) {
        set_error("mcbgpu_solve: invalid argument");
        return MCBGPU_E_ARG;
    }
    mcbgpu_solver *s = nullptr;
    int rc = mcbgpu_solver_create(&s, N, K, offsets[K]);
    if (rc) return rc;
    rc = mcbgpu_solver_upload(s, weight, offsets, coords, nullptr);
    if (!rc) rc = mcbgpu_solver_run(s, -1, nullptr);
    if (!rc) rc = mcbgpu_solver_results(s, selected, N, total_weight, nullptr);
    int rc2 = mcbgpu_solver_destroy(s);
    return rc ? rc : rc2;
}

}  // extern "C"
