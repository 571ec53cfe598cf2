// Batched de Pina solver: many independent problems (the biconnected components of
// one graph, or many graphs) solved in one persistent launch.
//
// The reference solves one graph per process and, for a graph split into
// biconnected components, runs the whole driver once per component file
// (main.sh:19-32 loops `run.sh` over bicc's output).  Here every problem is a
// (N, candidates, coordinate lists) triple as mcbgpu_solver takes it; one CTA owns
// one problem at a time and pulls the next from a device work counter (problems
// in order of decreasing N, so the longest start first).
//
// Per problem the CTA runs the blocked loop of mcbgpu_solver_run (64 iterations per
// block) with everything block-local in shared memory:
//   1. T[c] = bits i of S_{e0+i}[c] for the block's rows (64x64 bit transposes of
//      the rows' words by warp ballots; unit bits for c in [e0, bound));
//   2. the rank-ordered scan: W_r = XOR of T over C_r's coordinates below the
//      bound; the first b candidates whose W is independent of the earlier ones'
//      (a reduced row echelon basis keyed by lead bit) are the pivots;
//   3. resolve: the reference's loop restricted to the block on 64-bit masks
//      (iteration k takes the first pivot with parity(W_p & m_k) = 1, later masks
//      with odd parity absorb m_k), which selects the reference's candidate for
//      every iteration (mcb/mcb_cycle_deg_two_remove.cpp:329-358);
//   4. the block's final rows S_{e0+k} = XOR_{l in m_k} S^0_{e0+l}, computed from T;
//   5. every later row j: D_j[k] = <C_sel_k, S_j>, beta = the sequential effect of
//      the 64 updates (a 64x64 GF(2) matrix applied to D), S_j ^= XOR_{k in beta}
//      S_{e0+k} (mcb/mcb_cycle_deg_two_remove.cpp:371-390 for 64 iterations).
// There is no inter-CTA synchronisation: the only shared word is the work counter.
#include <algorithm>
#include <vector>

#include "mcbgpu_internal.cuh"

using namespace mcbgpu;

namespace {

constexpr int kBThreads = 512;
constexpr int kBWarps = kBThreads / 32;
#ifndef MCB_BATCH_Q0
#define MCB_BATCH_Q0 2  // candidates per thread per scan round, problems with N <= 1024
#endif
#ifndef MCB_BATCH_Q
#define MCB_BATCH_Q 4   // the same for the larger classes
#endif
#ifndef MCB_BATCH_SINGLE
#define MCB_BATCH_SINGLE 1  // one launch for the whole batch (0: one launch per size class)
#endif
#ifndef MCB_BATCH_PREFETCH
#define MCB_BATCH_PREFETCH 1  // bulk L2 prefetch of the next scan chunk's offsets and lists
#endif
#ifndef MCB_BATCH_CHUNK
#define MCB_BATCH_CHUNK 4
#endif
constexpr int kBChunk = MCB_BATCH_CHUNK;  // coordinates of each candidate loaded together in a W walk
constexpr int kBatchMaxN = 12288;        // largest N a CTA holds (T and the final rows in shared memory)
constexpr unsigned kPairSmemMax = 8192;  // pairs kept in shared memory (more go to the CTA's global scratch)
constexpr size_t kSmemBudget = 220 * 1024;  // dynamic shared memory per CTA at most (static adds 3.4 KB)
constexpr int kClasses = 3;
constexpr int kClassMaxN[kClasses] = {1024, 4096, kBatchMaxN};

constexpr int kBProf = 13;  // profile words per problem (mcbgpu_batch_profile)

struct BatchGraph {
    long long cand;  // first candidate (index into weight / offsets)
    long long K;     // candidates
    long long srow;  // first word of the problem's support vectors (N rows of P words)
    long long sel;   // first entry of the problem in `selected`
    int N, P;
};

__device__ __forceinline__ int ffs64(uint64_t x) { return __ffsll((long long)x) - 1; }

// W of the kBQ consecutive candidates r0 .. r0 + kBQ - 1 (0 past K) from the block's
// T in shared memory.  The lists are walked in lockstep, kBChunk coordinates of each
// per step, so kBQ x kBChunk independent loads are in flight per thread.  `walked`
// counts the offsets and coordinates read (for the profile's byte count).
template <int kBQ>
__device__ __forceinline__ void w_smem_q(long long r0, long long K, long long cand,
                                         const int64_t *__restrict__ off, const int32_t *__restrict__ coords,
                                         const uint64_t *T, int bound, uint64_t (&W)[kBQ],
                                         unsigned long long &walked) {
    long long ia[kBQ], ea[kBQ];
#pragma unroll
    for (int q = 0; q < kBQ; q++) {
        W[q] = 0;
        ia[q] = ea[q] = 0;
        if (r0 + q < K) {
            ia[q] = __ldg(off + cand + r0 + q);
            ea[q] = __ldg(off + cand + r0 + q + 1);
            walked += 16;
        }
    }
    for (;;) {
        bool any = false;
#pragma unroll
        for (int q = 0; q < kBQ; q++) any |= ia[q] < ea[q];
        if (!any) break;
        int cv[kBQ][kBChunk];
#pragma unroll
        for (int q = 0; q < kBQ; q++)
#pragma unroll
            for (int t = 0; t < kBChunk; t++) cv[q][t] = ia[q] + t < ea[q] ? __ldg(coords + ia[q] + t) : 0x7fffffff;
#pragma unroll
        for (int q = 0; q < kBQ; q++) {
            walked += 4ull * (unsigned long long)min((long long)kBChunk, ea[q] - ia[q] > 0 ? ea[q] - ia[q] : 0);
#pragma unroll
            for (int t = 0; t < kBChunk; t++)
                if (cv[q][t] < bound) W[q] ^= T[cv[q][t]];
            ia[q] = cv[q][kBChunk - 1] >= bound ? ea[q] : ia[q] + kBChunk;
        }
    }
}

// kBQ: candidates per thread in one scan round; kRowRegs: row words per lane in the
// update (ceil(largest N of the class / 2048)).
template <int kBQ, int kRowRegs, int kMinBlocks>
__global__ void __launch_bounds__(kBThreads, kMinBlocks) batch_solve_kernel(
    const BatchGraph *__restrict__ graphs, const int *__restrict__ order, int count, unsigned *next,
    const int32_t *__restrict__ weight, const int64_t *__restrict__ off, const int32_t *__restrict__ coords,
    uint64_t *S, long long *selected, long long *total, unsigned *gstatus, unsigned *status, unsigned *pair_scratch,
    unsigned pair_cap, int ncap, unsigned pcap, long long *prof) {
    extern __shared__ __align__(16) uint64_t smem[];
    const int wcap = ncap >> 6;                       // ncap is a multiple of 64
    uint64_t *T = smem;                               // ncap words (the row buffers of the update alias it)
    uint64_t *F = smem + ncap;                        // 64 x wcap words: the block's final rows
    unsigned *sPairs = (unsigned *)(F + 64 * wcap);   // pcap pairs
    unsigned *gPairs = pair_scratch + (size_t)blockIdx.x * pair_cap;

    __shared__ uint64_t sB[64];     // reduced echelon basis, by lead bit
    __shared__ uint64_t sPivW[64];  // W of the pivots, in rank order
    __shared__ int sPivR[64];       // their ranks
    __shared__ uint64_t sMask[64];  // final masks m_k
    __shared__ uint64_t sGcol[64];  // bit i of gcol[k] = <C_sel_k, S_{e0+i}> (i < k)
    __shared__ uint64_t sMrow[64];  // beta of a row = XOR of sMrow[k] over the k with D bit k
    __shared__ int sSel[64];        // rank selected at iteration e0 + k
    __shared__ unsigned sPre[65];   // pair offsets of the selected lists
    __shared__ int sWmin[kBWarps];
    __shared__ uint64_t sNewRes, sNewW;
    __shared__ int sGi;
    __shared__ unsigned sFail;
    // profile (thread 0): cycles in T, scan, resolve, final rows, update; candidates
    // scanned; cycles of the scan's list walks; pivot rounds; cycles of warp 0 in the
    // update's D + beta and in its row writes
    __shared__ long long pc[10];
    __shared__ unsigned long long s_walked;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned full = 0xffffffffu;

    for (;;) {
        if (tid == 0) sGi = (int)atomicAdd(next, 1u);
        cta_sync();
        const int gi = sGi;
        if (gi >= count) break;
        const int gx = order[gi];
        const BatchGraph g = graphs[gx];
        const int N = g.N, P = g.P;
        const long long K = g.K, cand = g.cand;
        uint64_t *Sg = S + g.srow;

        // the problem's coordinate lists: ascending, in [0, N); lengths fit the pair scratch
        bool ok = N <= ncap;
        for (long long r = tid; ok && r < K; r += kBThreads) {
            const long long a = off[cand + r], e = off[cand + r + 1];
            if (e - a > (long long)(pair_cap / 64)) ok = false;
            int prev = -1;
            for (long long i = a; ok && i < e; i++) {
                const int c = coords[i];
                if (c <= prev || c >= N) ok = false;
                prev = c;
            }
        }
        if (!cta_sync_and(ok)) {
            if (tid == 0) {
                gstatus[gx] |= ST_BAD_INPUT;
                atomicOr(status, ST_BAD_INPUT);
            }
            continue;  // the loop head's barrier separates the problems
        }
        // S_j = e_j; only words [0, j/64] of row j are ever read or written
        for (int j = warp; j < N; j += kBWarps) {
            uint64_t *row = Sg + (size_t)j * P;
            for (int w = lane; w <= (j >> 6); w += 32) row[w] = w == (j >> 6) ? 1ull << (j & 63) : 0ull;
        }
        long long tot = 0;
        unsigned long long t_start = 0;
        unsigned long long walked = 0;  // this thread's list-walk bytes (offsets + coordinates)
        if (prof && tid == 0) s_walked = 0;
        if (prof && tid == 0) asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t_start));
        if (tid == 0) {
            sFail = 0;
            for (int q = 0; q < 10; q++) pc[q] = 0;
        }
        cta_sync();

        for (int e0 = 0; e0 < N; e0 += 64) {
            const int b = min(64, N - e0), bound = e0 + b, wl = e0 >> 6, Wb = wl + 1;
            long long c0 = prof ? clock64() : 0;
            // ---- 1. T
            for (int c = e0 + tid; c < bound; c += kBThreads) T[c] = 1ull << (c - e0);
            for (int w = warp; w < wl; w += kBWarps) {
                const uint64_t *r0 = Sg + (size_t)(e0 + lane) * P + w;
                const uint64_t x0 = lane < b ? r0[0] : 0ull;
                const uint64_t x1 = lane + 32 < b ? r0[(size_t)32 * P] : 0ull;
                uint64_t v0 = 0, v1 = 0;
#pragma unroll 8
                for (int t = 0; t < 32; t++) {
                    const unsigned lo = __ballot_sync(full, (x0 >> t) & 1), hi = __ballot_sync(full, (x1 >> t) & 1);
                    if (lane == t) v0 = ((uint64_t)hi << 32) | lo;
                }
#pragma unroll 8
                for (int t = 0; t < 32; t++) {
                    const unsigned lo = __ballot_sync(full, (x0 >> (t + 32)) & 1),
                                   hi = __ballot_sync(full, (x1 >> (t + 32)) & 1);
                    if (lane == t) v1 = ((uint64_t)hi << 32) | lo;
                }
                T[(w << 6) + lane] = v0;
                T[(w << 6) + 32 + lane] = v1;
            }
            cta_sync();
            if (prof && tid == 0) {
                const long long c = clock64();
                pc[0] += c - c0;
                c0 = c;
            }

            // ---- 2. pivots: the first b rank-ordered candidates with independent W
            int npiv = 0;
            uint64_t lead = 0;
            for (long long base = 0; npiv < b; base += (long long)kBThreads * kBQ) {
                if (base >= K) {  // fewer than b independent candidates
                    if (tid == 0) sFail = 1;
                    break;
                }
#if MCB_BATCH_PREFETCH
                if (tid == 0) {  // the next chunk's offsets and lists into L2 while this one is walked
                    const long long nb = base + (long long)kBThreads * kBQ;
                    if (nb < K) {
                        const long long ne = min(nb + (long long)kBThreads * kBQ, K);
                        prefetch_l2(off + cand + nb, 8ull * (unsigned long long)(ne - nb + 1));
                        const long long c0 = off[cand + nb], c1 = off[cand + ne];
                        prefetch_l2(coords + c0, 4ull * (unsigned long long)(c1 - c0));
                    }
                }
#endif
                // thread tid holds ranks base + tid * kBQ + q: key tid * kBQ + q is rank order
                const long long cw = prof ? clock64() : 0;
                bool first_round = true;
                uint64_t W[kBQ], res[kBQ];
                w_smem_q<kBQ>(base + (long long)tid * kBQ, K, cand, off, coords, T, bound, W, walked);
#pragma unroll
                for (int q = 0; q < kBQ; q++) {
                    res[q] = W[q];
                    for (uint64_t m = W[q] & lead; m; m &= m - 1) res[q] ^= sB[ffs64(m)];
                }
                for (;;) {
                    int myq = kBQ;
#pragma unroll
                    for (int q = kBQ - 1; q >= 0; q--)
                        if (res[q]) myq = q;
                    const unsigned bal = __ballot_sync(full, myq < kBQ);
                    if (bal) {
                        const int fl = __ffs(bal) - 1;
                        const int fq = __shfl_sync(full, myq, fl);
                        if (lane == 0) sWmin[warp] = (warp * 32 + fl) * kBQ + fq;
                    } else if (lane == 0) {
                        sWmin[warp] = 0x7fffffff;
                    }
                    cta_sync();
                    if (prof && tid == 0) {
                        if (first_round) pc[6] += clock64() - cw;
                        pc[7]++;
                    }
                    first_round = false;
                    int best = 0x7fffffff;
#pragma unroll
                    for (int q = 0; q < kBWarps; q++) best = min(best, sWmin[q]);
                    if (best == 0x7fffffff) break;
                    {
                        uint64_t sr = 0, sw = 0;  // selects, not an indexed access (keeps res / W in registers)
#pragma unroll
                        for (int q = 0; q < kBQ; q++) {
                            const bool h = tid * kBQ + q == best;
                            sr = h ? res[q] : sr;
                            sw = h ? W[q] : sw;
                        }
                        if (tid == best / kBQ) {
                            sNewRes = sr;
                            sNewW = sw;
                        }
                    }
                    cta_sync();
                    const uint64_t nr = sNewRes;
                    const int L = ffs64(nr);
                    if (warp == 0) {  // keep the basis reduced: clear bit L from the older vectors
                        if (((lead >> lane) & 1) && ((sB[lane] >> L) & 1)) sB[lane] ^= nr;
                        if (((lead >> (lane + 32)) & 1) && ((sB[lane + 32] >> L) & 1)) sB[lane + 32] ^= nr;
                        if (lane == 0) {
                            sB[L] = nr;
                            sPivW[npiv] = sNewW;
                            sPivR[npiv] = (int)(base + best);
                        }
                    }
                    lead |= 1ull << L;
                    npiv++;
#pragma unroll
                    for (int q = 0; q < kBQ; q++) {
                        if (tid * kBQ + q == best)
                            res[q] = 0;
                        else if ((res[q] >> L) & 1)
                            res[q] ^= nr;
                    }
                    if (npiv == b) break;
                }
                cta_sync();
                if (tid == 0) pc[5] += kBThreads * kBQ;
            }
            cta_sync();
            if (prof && tid == 0) {
                const long long c = clock64();
                pc[1] += c - c0;
                c0 = c;
            }
            if (sFail) break;

            // ---- 3. resolve (warp 0), gcol, the beta matrix, selected ranks, pair offsets
            if (warp == 0) {
                const uint64_t W0 = lane < b ? sPivW[lane] : 0ull, W1 = lane + 32 < b ? sPivW[lane + 32] : 0ull;
                uint64_t m0 = lane < b ? 1ull << lane : 0ull, m1 = lane + 32 < b ? 1ull << (lane + 32) : 0ull;
                int p0 = 0, p1 = 0;  // pivot of iteration lane / lane + 32
                bool bad = false;
                for (int k = 0; k < b; k++) {
                    const uint64_t mk = __shfl_sync(full, k < 32 ? m0 : m1, k & 31);
                    const unsigned o0 = __ballot_sync(full, parity64(W0 & mk));
                    const unsigned o1 = __ballot_sync(full, parity64(W1 & mk));
                    const int p = o0 ? __ffs(o0) - 1 : (o1 ? 31 + __ffs(o1) : -1);
                    if (p < 0) {  // cannot happen for independent pivots; guards the indexing
                        bad = true;
                        break;
                    }
                    const uint64_t Wp = __shfl_sync(full, p < 32 ? W0 : W1, p & 31);
                    if (lane == (k & 31)) {
                        if (k < 32)
                            p0 = p;
                        else
                            p1 = p;
                    }
                    if (lane > k && parity64(Wp & m0)) m0 ^= mk;
                    if (lane + 32 > k && parity64(Wp & m1)) m1 ^= mk;
                }
                sMask[lane] = m0;
                sMask[lane + 32] = m1;
                if (bad) {
                    if (lane == 0) sFail = 1;
                } else {
                    __syncwarp();
                    // gcol[k] bit i = parity(W_{p_k} & m_i), i < k
                    for (int h = 0; h < 2; h++) {
                        const int k = lane + 32 * h;
                        uint64_t gc = 0;
                        if (k < b) {
                            const uint64_t Wk = sPivW[h ? p1 : p0];
                            for (int i = 0; i < k; i++) gc |= (uint64_t)parity64(Wk & sMask[i]) << i;
                            sSel[k] = sPivR[h ? p1 : p0];
                        }
                        sGcol[k] = gc;
                    }
                    __syncwarp();
                    // beta for D = e_k: beta_i = 0 (i < k), 1 (i = k), parity(beta & gcol[i]) (i > k)
                    for (int h = 0; h < 2; h++) {
                        const int k = lane + 32 * h;
                        uint64_t bt = 0;
                        if (k < b) {
                            bt = 1ull << k;
                            for (int i = k + 1; i < b; i++) bt |= (uint64_t)parity64(bt & sGcol[i]) << i;
                        }
                        sMrow[k] = bt;
                    }
                    // pair offsets of the selected lists
                    long long l0 = 0, l1 = 0;
                    if (lane < b) l0 = off[cand + sSel[lane] + 1] - off[cand + sSel[lane]];
                    if (lane + 32 < b) l1 = off[cand + sSel[lane + 32] + 1] - off[cand + sSel[lane + 32]];
                    unsigned s0 = (unsigned)l0, s1 = (unsigned)l1;
                    for (int d = 1; d < 32; d <<= 1) {
                        const unsigned a0 = __shfl_up_sync(full, s0, d), a1 = __shfl_up_sync(full, s1, d);
                        if (lane >= d) {
                            s0 += a0;
                            s1 += a1;
                        }
                    }
                    const unsigned t0 = __shfl_sync(full, s0, 31);
                    sPre[lane + 1] = s0;
                    sPre[lane + 33] = t0 + s1;
                    if (lane == 0) sPre[0] = 0;
                    if (lane == 0)
                        for (int k = 0; k < b; k++) tot += weight[cand + sSel[k]];
                }
            }
            cta_sync();
            if (prof && tid == 0) {
                const long long c = clock64();
                pc[2] += c - c0;
                c0 = c;
            }
            if (sFail) break;
            const unsigned np = sPre[b];
            unsigned *pairs = np <= pcap ? sPairs : gPairs;

            // ---- 4. final rows of the block (shared F and global S), 5. pairs
            for (int item = warp; item < b * wl; item += kBWarps) {
                const int k = item / wl, w = item - k * wl;
                const uint64_t mk = sMask[k];
                const unsigned lo = __ballot_sync(full, parity64(T[(w << 6) + lane] & mk));
                const unsigned hi = __ballot_sync(full, parity64(T[(w << 6) + 32 + lane] & mk));
                if (lane == 0) {
                    const uint64_t v = ((uint64_t)hi << 32) | lo;
                    F[k * Wb + w] = v;
                    Sg[(size_t)(e0 + k) * P + w] = v;
                }
            }
            for (int k = tid; k < b; k += kBThreads) {
                F[k * Wb + wl] = sMask[k];
                Sg[(size_t)(e0 + k) * P + wl] = sMask[k];
            }
            for (int k = warp; k < b; k += kBWarps) {
                const long long a = off[cand + sSel[k]], e = off[cand + sSel[k] + 1];
                const unsigned o = sPre[k];
                for (long long i = a + lane; i < e; i += 32)
                    pairs[o + (unsigned)(i - a)] = ((unsigned)coords[i] << 6) | (unsigned)k;
            }
            cta_sync();
            if (prof && tid == 0) {
                const long long c = clock64();
                pc[3] += c - c0;
                c0 = c;
            }

            // ---- 6. later rows: one warp per row.  The row's words [0, Wb) are loaded
            // once (coalesced) into registers and, below e0, into the warp's row buffer
            // (T's storage, free until the next block); D_j from the pairs against the
            // buffer, beta = D_j x Mrow, then S_j ^= XOR_{k in beta} F_k.
            uint64_t *rowbuf = T + (size_t)warp * wcap;
            for (int j = bound + warp; j < N; j += kBWarps) {
                const long long cu0 = prof ? clock64() : 0;
                uint64_t *Sj = Sg + (size_t)j * P;
                uint64_t v[kRowRegs];
#pragma unroll
                for (int i = 0; i < kRowRegs; i++) {
                    const int w = lane + 32 * i;
                    v[i] = w < Wb ? Sj[w] : 0ull;
                    if (w < wl) rowbuf[w] = v[i];
                }
                __syncwarp();
                uint64_t D = 0;
                for (unsigned i = lane; i < np; i += 32) {
                    const unsigned pr = pairs[i];
                    const int c = (int)(pr >> 6);
                    const uint64_t bit = c < e0 ? (rowbuf[c >> 6] >> (c & 63)) & 1ull : (uint64_t)(c == j);
                    D ^= bit << (pr & 63);
                }
                D = warp_xor64(D);
                uint64_t beta = ((D >> lane) & 1) ? sMrow[lane] : 0ull;
                if ((D >> (lane + 32)) & 1) beta ^= sMrow[lane + 32];
                beta = warp_xor64(beta);
                const long long cu1 = prof ? clock64() : 0;
                if (prof && tid == 0) pc[8] += cu1 - cu0;
                if (beta) {
#pragma unroll
                    for (int i = 0; i < kRowRegs; i++) {
                        const int w = lane + 32 * i;
                        if (w < Wb) {
                            uint64_t x = 0;
                            for (uint64_t bb = beta; bb; bb &= bb - 1) x ^= F[ffs64(bb) * Wb + w];
                            Sj[w] = v[i] ^ x;
                        }
                    }
                }
                if (prof && tid == 0) pc[9] += clock64() - cu1;
                __syncwarp();
            }
            if (tid == 0)
                for (int k = 0; k < b; k++) selected[g.sel + e0 + k] = sSel[k];
            cta_sync();
            if (prof && tid == 0) pc[4] += clock64() - c0;
        }
        if (tid == 0) {
            if (sFail) {
                gstatus[gx] |= ST_RANK_DEFICIT;
                atomicOr(status, ST_RANK_DEFICIT);
            }
        }
        if (warp == 0) {
            // tot lives in lane 0 of warp 0
            if (lane == 0) total[gx] = sFail ? -1 : tot;
        }
        if (prof) {
            atomicAdd(&s_walked, walked);
            cta_sync();
        }
        if (prof && tid == 0) {
            unsigned long long t_end;
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t_end));
            unsigned smid;
            asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
            long long *o = prof + (size_t)gx * kBProf;
            o[0] = (long long)(t_end - t_start);
            for (int q = 0; q < 6; q++) o[1 + q] = pc[q];
            o[7] = smid;
            o[8] = pc[6];
            o[9] = pc[7];
            o[10] = pc[8];
            o[11] = pc[9];
            o[12] = (long long)s_walked;
        }
    }
}

}  // namespace

namespace {

// The uploaded offsets: non-decreasing from 0 to nnz (out[0] = 1 if not); out[1] =
// the longest list (it sizes the pair scratch).
__global__ void batch_validate_kernel(const int64_t *__restrict__ off, long long K, long long nnz, unsigned *out) {
    unsigned long long mx = 0;
    unsigned bad = 0;
    for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < K; r += (long long)gridDim.x * blockDim.x) {
        const long long a = off[r], e = off[r + 1];
        if (e < a || a < 0 || e > nnz)
            bad = 1;
        else if ((unsigned long long)(e - a) > mx)
            mx = (unsigned long long)(e - a);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0 && (off[0] != 0 || off[K] != nnz)) bad = 1;
    if (mx > 0xffffffffull) mx = 0xffffffffull;
    unsigned m32 = (unsigned)mx;
    m32 = __reduce_max_sync(0xffffffffu, m32);
    bad = __reduce_or_sync(0xffffffffu, bad);
    if ((threadIdx.x & 31) == 0) {
        if (m32) atomicMax(out + 1, m32);
        if (bad) atomicOr(out, 1u);
    }
}

}  // namespace

struct mcbgpu_batch {
    int count = 0;
    int sm_count = 0;
    long long total_K = 0, nnz = 0, total_N = 0, s_words = 0;
    unsigned pair_cap = 0;   // pair scratch words per CTA (64 x the longest list)
    int pair_slabs = 0;      // CTA slabs per class
    std::vector<BatchGraph> graphs;
    std::vector<int> order;            // problems grouped by class, by decreasing N within a class
    int class_off[kClasses + 1] = {};  // class c holds order[class_off[c], class_off[c + 1])
    int class_ncap[kClasses] = {};     // largest N of the class (rounded up to 64)
    int class_grid[kClasses] = {};
    BatchGraph *d_graphs = nullptr;
    int *d_order = nullptr;
    unsigned *d_next = nullptr;  // one work counter per class
    int32_t *d_weight = nullptr;
    int64_t *d_off = nullptr;
    int32_t *d_coords = nullptr;
    uint64_t *d_S = nullptr;
    long long *d_selected = nullptr;
    long long *d_total = nullptr;
    unsigned *d_gstatus = nullptr;
    unsigned *d_status = nullptr;
    unsigned *d_check = nullptr;  // [bad offsets, longest list]
    unsigned *d_pairs = nullptr;
    long long *d_prof = nullptr;  // optional per-problem profile (count x 8)
    cudaStream_t st[kClasses] = {};
    cudaEvent_t ev_fork = nullptr, ev_join[kClasses] = {};
    bool uploaded = false;
    long long launches = 0;
    long long device_bytes = 0;
};

namespace {

// Pairs kept in shared memory next to T and F for a class of largest N = ncap.
unsigned batch_pair_smem(int ncap) {
    const size_t tf = 16 * (size_t)ncap;
    const size_t room = kSmemBudget > tf ? (kSmemBudget - tf) / 4 : 0;
    return (unsigned)std::min<size_t>(kPairSmemMax, room & ~(size_t)31);
}

size_t batch_smem_bytes(int ncap) { return 16 * (size_t)ncap + 4 * (size_t)batch_pair_smem(ncap); }

void free_batch(mcbgpu_batch *b) {
    if (!b) return;
    cudaFree(b->d_graphs);
    cudaFree(b->d_order);
    cudaFree(b->d_next);
    cudaFree(b->d_weight);
    cudaFree(b->d_off);
    cudaFree(b->d_coords);
    cudaFree(b->d_S);
    cudaFree(b->d_selected);
    cudaFree(b->d_total);
    cudaFree(b->d_gstatus);
    cudaFree(b->d_status);
    cudaFree(b->d_check);
    cudaFree(b->d_pairs);
    cudaFree(b->d_prof);
    for (int c = 0; c < kClasses; c++) {
        if (b->st[c]) cudaStreamDestroy(b->st[c]);
        if (b->ev_join[c]) cudaEventDestroy(b->ev_join[c]);
    }
    if (b->ev_fork) cudaEventDestroy(b->ev_fork);
    delete b;
}

using BatchKernel = void (*)(const BatchGraph *, const int *, int, unsigned *, const int32_t *, const int64_t *,
                            const int32_t *, uint64_t *, long long *, long long *, unsigned *, unsigned *, unsigned *,
                            unsigned, int, unsigned, long long *);

// Class c's kernel: problems with N <= kClassMaxN[c] (row words per lane in the
// update = kClassMaxN[c] / 2048, rounded up).
BatchKernel class_kernel(int c) {
    switch (c) {
        case 0: return batch_solve_kernel<MCB_BATCH_Q0, 1, 2>;
        case 1: return batch_solve_kernel<MCB_BATCH_Q, 2, 1>;
        default: return batch_solve_kernel<MCB_BATCH_Q, (kBatchMaxN / 64 + 31) / 32, 1>;
    }
}

// The launch a problem goes to.  With MCB_BATCH_SINGLE (the default) a batch is one
// queue in order of decreasing N: on the small-problem kernel (two CTAs per SM) when
// every problem has N <= kClassMaxN[0], else on the largest-class kernel.  One queue
// keeps the longest problems first across the whole batch (4096 graphs of the
// batched configuration: 156 ms against 218 ms with a launch per size class, whose
// large-problem CTAs take every SM first).
int class_of(int N, int maxN) {
    if (MCB_BATCH_SINGLE) return maxN <= kClassMaxN[0] ? 0 : kClasses - 1;
    int c = 0;
    while (c < kClasses - 1 && N > kClassMaxN[c]) c++;
    return c;
}

}  // namespace

extern "C" {

int mcbgpu_batch_max_coords(void) { return kBatchMaxN; }

int mcbgpu_batch_create(mcbgpu_batch **out, int32_t count, const int32_t *num_coords,
                        const int64_t *num_candidates, int64_t nnz) {
    if (!out || count < 0 || nnz < 0 || (count > 0 && (!num_coords || !num_candidates))) {
        set_error("mcbgpu_batch_create: invalid arguments");
        return MCBGPU_E_ARG;
    }
    *out = nullptr;
    for (int i = 0; i < count; i++) {
        if (num_coords[i] < 0 || num_coords[i] > kBatchMaxN || num_candidates[i] < 0 ||
            num_candidates[i] >= (1ll << 31)) {
            set_error("mcbgpu_batch_create: problem %d has N = %d, K = %lld (the batch takes N <= %d and "
                      "K < 2^31; solve larger problems with mcbgpu_solver)",
                      i, (int)num_coords[i], (long long)num_candidates[i], kBatchMaxN);
            return MCBGPU_E_ARG;
        }
    }
    mcbgpu_batch *b = new mcbgpu_batch();
    b->count = count;
    b->nnz = nnz;
    b->graphs.resize(count);
    for (int i = 0; i < count; i++) {
        BatchGraph &g = b->graphs[i];
        g.N = num_coords[i];
        g.P = (g.N + 63) / 64;
        g.K = num_candidates[i];
        g.cand = b->total_K;
        g.sel = b->total_N;
        g.srow = b->s_words;
        b->total_K += g.K;
        b->total_N += g.N;
        b->s_words += (long long)g.N * g.P;
    }
    // problems with no coordinate need no work; the rest by class, each by decreasing N
    std::vector<int> idx;
    for (int i = 0; i < count; i++)
        if (b->graphs[i].N > 0) idx.push_back(i);
    std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) { return b->graphs[x].N > b->graphs[y].N; });
    const int maxN = idx.empty() ? 0 : b->graphs[idx[0]].N;
    for (int c = 0; c < kClasses; c++) {
        b->class_off[c] = (int)b->order.size();
        for (int i : idx)
            if (class_of(b->graphs[i].N, maxN) == c) {
                b->order.push_back(i);
                b->class_ncap[c] = std::max(b->class_ncap[c], (b->graphs[i].N + 63) & ~63);
            }
    }
    b->class_off[kClasses] = (int)b->order.size();
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, dev);
    long long bytes = 0;
#define ALLOC(ptr, sz)                                             \
    do {                                                           \
        size_t _b = (size_t)(sz);                                  \
        if (_b < 16) _b = 16;                                      \
        if (e == cudaSuccess) e = cudaMalloc((void **)&(ptr), _b); \
        bytes += (long long)_b;                                    \
    } while (0)
    ALLOC(b->d_graphs, sizeof(BatchGraph) * (size_t)count);
    ALLOC(b->d_order, sizeof(int) * b->order.size());
    ALLOC(b->d_next, sizeof(unsigned) * kClasses);
    ALLOC(b->d_weight, sizeof(int32_t) * (size_t)b->total_K);
    ALLOC(b->d_off, sizeof(int64_t) * (size_t)(b->total_K + 1));
    ALLOC(b->d_coords, sizeof(int32_t) * (size_t)nnz);
    ALLOC(b->d_S, sizeof(uint64_t) * (size_t)b->s_words);
    ALLOC(b->d_selected, sizeof(long long) * (size_t)b->total_N);
    ALLOC(b->d_total, sizeof(long long) * (size_t)count);
    ALLOC(b->d_gstatus, sizeof(unsigned) * (size_t)count);
    ALLOC(b->d_status, sizeof(unsigned));
    ALLOC(b->d_check, 2 * sizeof(unsigned));
#undef ALLOC
    if (e == cudaSuccess && count > 0)
        e = cudaMemcpy(b->d_graphs, b->graphs.data(), sizeof(BatchGraph) * (size_t)count, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !b->order.empty())
        e = cudaMemcpy(b->d_order, b->order.data(), sizeof(int) * b->order.size(), cudaMemcpyHostToDevice);
    for (int c = 0; c < kClasses && e == cudaSuccess; c++) {
        e = cudaStreamCreateWithFlags(&b->st[c], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_join[c], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming);
    // one persistent grid per class: as many CTAs as are resident at once, at most one per problem
    // the attribute is per kernel, shared by all handles: the class's largest need
    for (int c = 0; c < kClasses && e == cudaSuccess; c++)
        e = cudaFuncSetAttribute(class_kernel(c), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)batch_smem_bytes(kClassMaxN[c]));
    for (int c = 0; c < kClasses && e == cudaSuccess; c++) {
        const int n = b->class_off[c + 1] - b->class_off[c];
        if (n == 0) continue;
        int per_sm = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, class_kernel(c), kBThreads,
                                                          batch_smem_bytes(b->class_ncap[c]));
        if (e == cudaSuccess && per_sm < 1) e = cudaErrorInvalidConfiguration;
        b->class_grid[c] = (int)std::min<long long>(n, (long long)per_sm * std::max(b->sm_count, 1));
    }
    if (e != cudaSuccess) {
        free_batch(b);
        return cuda_fail(e, "mcbgpu_batch_create");
    }
    b->device_bytes = bytes;
    *out = b;
    return MCBGPU_OK;
}

int mcbgpu_batch_upload(mcbgpu_batch *b, const int32_t *weight, const int64_t *offsets, const int32_t *coords,
                        void *stream) {
    if (!b || (b->total_K > 0 && (!weight || !offsets)) || (b->nnz > 0 && !coords)) {
        set_error("mcbgpu_batch_upload: NULL argument");
        return MCBGPU_E_ARG;
    }
    b->uploaded = false;
    cudaStream_t st = (cudaStream_t)stream;
    if (b->total_K > 0) {
        MCB_CUDA(cudaMemcpyAsync(b->d_weight, weight, sizeof(int32_t) * (size_t)b->total_K, cudaMemcpyHostToDevice,
                                 st));
        MCB_CUDA(cudaMemcpyAsync(b->d_off, offsets, sizeof(int64_t) * (size_t)(b->total_K + 1),
                                 cudaMemcpyHostToDevice, st));
    }
    if (b->nnz > 0)
        MCB_CUDA(cudaMemcpyAsync(b->d_coords, coords, sizeof(int32_t) * (size_t)b->nnz, cudaMemcpyHostToDevice, st));
    // offsets checked on the device (non-decreasing from 0 to nnz); the longest list
    // sizes the pair scratch; the coordinate lists are checked by the solve itself
    unsigned chk[2] = {0, 0};
    if (b->total_K > 0) {
        MCB_CUDA(cudaMemsetAsync(b->d_check, 0, sizeof chk, st));
        const int grid = (int)std::min<long long>((b->total_K + 255) / 256, (long long)std::max(b->sm_count, 1) * 8);
        batch_validate_kernel<<<grid, 256, 0, st>>>(b->d_off, b->total_K, b->nnz, b->d_check);
        MCB_CUDA(cudaGetLastError());
        MCB_CUDA(cudaMemcpyAsync(chk, b->d_check, sizeof chk, cudaMemcpyDeviceToHost, st));
    }
    MCB_CUDA(cudaStreamSynchronize(st));
    if (chk[0]) {
        set_error("mcbgpu_batch_upload: offsets must be non-decreasing from 0 to nnz");
        return MCBGPU_E_ARG;
    }
    const long long max_len = chk[1];
    if (max_len > kBatchMaxN) {  // a list has at most N distinct coordinates
        set_error("mcbgpu_batch_upload: a coordinate list is longer than N");
        return MCBGPU_E_ARG;
    }
    const unsigned cap = (unsigned)(64 * std::max<long long>(max_len, 1));
    int slabs = 1;
    for (int c = 0; c < kClasses; c++) slabs = std::max(slabs, b->class_grid[c]);
    if (cap > b->pair_cap) {  // one slab per CTA of the widest class grid, for each class
        cudaFree(b->d_pairs);
        b->d_pairs = nullptr;
        b->pair_cap = 0;
        const size_t n = (size_t)cap * (size_t)slabs * kClasses;
        MCB_CUDA(cudaMalloc((void **)&b->d_pairs, sizeof(unsigned) * n));
        b->device_bytes += (long long)(sizeof(unsigned) * n);
        b->pair_cap = cap;
        b->pair_slabs = slabs;
    }
    b->uploaded = true;
    return MCBGPU_OK;
}

int mcbgpu_batch_run(mcbgpu_batch *b, void *stream) {
    if (!b || !b->uploaded) {
        set_error("mcbgpu_batch_run: %s", b ? "upload first" : "NULL handle");
        return b ? MCBGPU_E_STATE : MCBGPU_E_ARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    MCB_CUDA(cudaMemsetAsync(b->d_next, 0, sizeof(unsigned) * kClasses, st));
    MCB_CUDA(cudaMemsetAsync(b->d_status, 0, sizeof(unsigned), st));
    if (b->count > 0) {
        MCB_CUDA(cudaMemsetAsync(b->d_gstatus, 0, sizeof(unsigned) * (size_t)b->count, st));
        MCB_CUDA(cudaMemsetAsync(b->d_total, 0, sizeof(long long) * (size_t)b->count, st));
    }
    MCB_CUDA(cudaEventRecord(b->ev_fork, st));
    for (int c = 0; c < kClasses; c++) {
        const int n = b->class_off[c + 1] - b->class_off[c];
        if (n == 0) continue;
        MCB_CUDA(cudaStreamWaitEvent(b->st[c], b->ev_fork, 0));
        class_kernel(c)<<<b->class_grid[c], kBThreads, batch_smem_bytes(b->class_ncap[c]), b->st[c]>>>(
            b->d_graphs, b->d_order + b->class_off[c], n, b->d_next + c, b->d_weight, b->d_off, b->d_coords, b->d_S,
            b->d_selected, b->d_total, b->d_gstatus, b->d_status,
            b->d_pairs + (size_t)c * b->pair_cap * (size_t)b->pair_slabs, b->pair_cap, b->class_ncap[c],
            batch_pair_smem(b->class_ncap[c]), b->d_prof);
        MCB_CUDA(cudaGetLastError());
        b->launches++;
        MCB_CUDA(cudaEventRecord(b->ev_join[c], b->st[c]));
        MCB_CUDA(cudaStreamWaitEvent(st, b->ev_join[c], 0));
    }
    return MCBGPU_OK;
}

int mcbgpu_batch_results(mcbgpu_batch *b, int64_t *selected, int64_t *total_weight, uint32_t *problem_status,
                         void *stream) {
    if (!b) {
        set_error("mcbgpu_batch_results: NULL handle");
        return MCBGPU_E_ARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    unsigned v = 0;
    MCB_CUDA(cudaMemcpyAsync(&v, b->d_status, sizeof v, cudaMemcpyDeviceToHost, st));
    if (selected && b->total_N > 0)
        MCB_CUDA(cudaMemcpyAsync(selected, b->d_selected, sizeof(long long) * (size_t)b->total_N,
                                 cudaMemcpyDeviceToHost, st));
    if (total_weight && b->count > 0)
        MCB_CUDA(cudaMemcpyAsync(total_weight, b->d_total, sizeof(long long) * (size_t)b->count,
                                 cudaMemcpyDeviceToHost, st));
    if (problem_status && b->count > 0)
        MCB_CUDA(cudaMemcpyAsync(problem_status, b->d_gstatus, sizeof(unsigned) * (size_t)b->count,
                                 cudaMemcpyDeviceToHost, st));
    MCB_CUDA(cudaStreamSynchronize(st));
    if (v & ST_RANK_DEFICIT) {
        set_error("a problem's candidates do not span its cycle space (status 0x%x)", v);
        return MCBGPU_E_NO_CANDIDATE;
    }
    if (v) {
        set_error("a problem's coordinate lists are not ascending in [0, N) (status 0x%x)", v);
        return MCBGPU_E_ARG;
    }
    return MCBGPU_OK;
}

int mcbgpu_batch_get_support(mcbgpu_batch *b, int32_t problem, int32_t j, uint64_t *words, void *stream) {
    if (!b || problem < 0 || problem >= b->count || !words || j < 0 || j >= b->graphs[problem].N) {
        set_error("mcbgpu_batch_get_support: invalid arguments");
        return MCBGPU_E_ARG;
    }
    const BatchGraph &g = b->graphs[problem];
    cudaStream_t st = (cudaStream_t)stream;
    // words beyond j / 64 are never written: report them as zero
    for (int w = 0; w < g.P; w++) words[w] = 0;
    MCB_CUDA(cudaMemcpyAsync(words, b->d_S + g.srow + (size_t)j * g.P, sizeof(uint64_t) * (size_t)(j / 64 + 1),
                             cudaMemcpyDeviceToHost, st));
    MCB_CUDA(cudaStreamSynchronize(st));
    return MCBGPU_OK;
}

int mcbgpu_batch_set_profiling(mcbgpu_batch *b, int enable) {
    if (!b) {
        set_error("mcbgpu_batch_set_profiling: NULL handle");
        return MCBGPU_E_ARG;
    }
    if (enable && !b->d_prof) {
        MCB_CUDA(cudaMalloc((void **)&b->d_prof, sizeof(long long) * kBProf * (size_t)std::max(b->count, 1)));
        MCB_CUDA(cudaMemset(b->d_prof, 0, sizeof(long long) * kBProf * (size_t)std::max(b->count, 1)));
    } else if (!enable && b->d_prof) {
        MCB_CUDA(cudaFree(b->d_prof));
        b->d_prof = nullptr;
    }
    return MCBGPU_OK;
}

int mcbgpu_batch_profile(mcbgpu_batch *b, int64_t *out) {
    if (!b || !out || !b->d_prof) {
        set_error("mcbgpu_batch_profile: %s", b && b->d_prof ? "NULL output" : "profiling is off");
        return MCBGPU_E_ARG;
    }
    MCB_CUDA(cudaDeviceSynchronize());
    MCB_CUDA(cudaMemcpy(out, b->d_prof, sizeof(long long) * kBProf * (size_t)b->count, cudaMemcpyDeviceToHost));
    return MCBGPU_OK;
}

int64_t mcbgpu_batch_launches(const mcbgpu_batch *b) { return b ? b->launches : 0; }
int64_t mcbgpu_batch_device_bytes(const mcbgpu_batch *b) { return b ? b->device_bytes : 0; }

int mcbgpu_batch_destroy(mcbgpu_batch *b) {
    free_batch(b);
    return MCBGPU_OK;
}

int mcbgpu_batch_solve(int32_t count, const int32_t *num_coords, const int64_t *num_candidates,
                       const int32_t *weight, const int64_t *offsets, const int32_t *coords, int64_t *selected,
                       int64_t *total_weight) {
    long long totK = 0;
    for (int i = 0; i < count; i++) totK += num_candidates ? num_candidates[i] : 0;
    const int64_t nnz = totK > 0 && offsets ? offsets[totK] : 0;
    mcbgpu_batch *b = nullptr;
    int rc = mcbgpu_batch_create(&b, count, num_coords, num_candidates, nnz);
    if (rc) return rc;
    rc = mcbgpu_batch_upload(b, weight, offsets, coords, nullptr);
    if (!rc) rc = mcbgpu_batch_run(b, nullptr);
    if (!rc) rc = mcbgpu_batch_results(b, selected, total_weight, nullptr, nullptr);
    mcbgpu_batch_destroy(b);
    return rc;
}

}  // extern "C"
