// ORACLE — test infrastructure, not part of the product.
//
// A CPU restatement of the reference's de Pina main loop, used by the tests as the
// parity checker and by bench.py as the timed CPU baseline ("port" of the reference
// CPU driver).  Nothing in the product path links or calls this file.
//
// It follows mcb/mcb_non_cpu_rd.cpp:246-342 step by step:
//   S_j := e_j                                    (:246-250)
//   for e in 0..N-1:
//     labels P_t[v] for every FVS tree           (worker_thread::precompute_supportVec,
//                                                  include/work_per_thread.h:154-210)
//     first candidate in list order with
//       S_e[coord(e_uv)] ^ P_t[u] ^ P_t[v] == 1   (:292-322); erase it from the list
//     C_e := cycle vector of that candidate      (cycle::get_cycle_vector,
//                                                  include/cycles.h:144-195)
//     for j > e: if <C_e, S_j> odd: S_j ^= S_e    (:333-338, bit_vector::dot_product /
//                                                  do_xor, include/bit_vector.h:73-84,127-141)
// Inputs are the prepared problem's arrays (reduced graph, coordinate map, per-tree
// parent edges, candidates in rank order).  Built as oracle/libmcboracle.so.
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <chrono>
#include <vector>
#include <omp.h>

namespace {

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

inline uint32_t getbit(const uint64_t *v, int64_t pos) { return (uint32_t)((v[pos >> 6] >> (pos & 63)) & 1ULL); }

struct Forest {
    int n = 0, F = 0;
    const uint32_t *rows = nullptr, *cols = nullptr;
    const int32_t *edge_coord = nullptr;
    const int32_t *parent_edge = nullptr;  // F x n
    std::vector<int32_t> order;            // F x n: BFS order from the root (parents first)

    void build(int threads) {
        order.assign((size_t)F * n, 0);
#pragma omp parallel num_threads(threads)
        {
            std::vector<int32_t> head(n), nxt(n), q;
            q.reserve(n);
#pragma omp for schedule(dynamic, 4)
            for (int t = 0; t < F; t++) {
                const int32_t *pe = parent_edge + (size_t)t * n;
                std::fill(head.begin(), head.end(), -1);
                int root = -1;
                // children lists from parent edges (compressed_trees::copy,
                // include/compressed_trees.cpp:47-88, builds the same tree CSR)
                for (int v = n - 1; v >= 0; v--) {
                    if (pe[v] < 0) {
                        root = v;
                        continue;
                    }
                    int p = (int)rows[pe[v]];
                    nxt[v] = head[p];
                    head[p] = v;
                }
                q.clear();
                if (root >= 0) q.push_back(root);
                for (size_t i = 0; i < q.size(); i++)
                    for (int c = head[q[i]]; c >= 0; c = nxt[c]) q.push_back(c);
                std::memcpy(&order[(size_t)t * n], q.data(), sizeof(int32_t) * q.size());
            }
        }
    }

    // precompute_supportVec: P[root] = 0, P[child] = P[parent] ^ S[coord(edge)]
    void labels(const uint64_t *S, uint8_t *P, int threads) const {
#pragma omp parallel for num_threads(threads) schedule(dynamic, 4)
        for (int t = 0; t < F; t++) {
            const int32_t *pe = parent_edge + (size_t)t * n;
            const int32_t *ord = &order[(size_t)t * n];
            uint8_t *lab = P + (size_t)t * n;
            lab[ord[0]] = 0;
            for (int i = 1; i < n; i++) {
                int v = ord[i];
                int e = pe[v];
                int c = edge_coord[e];
                uint8_t b = c >= 0 ? (uint8_t)getbit(S, c) : 0;
                lab[v] = lab[rows[e]] ^ b;
            }
        }
    }

    // get_cycle_vector: OR of the coordinates on both root paths and of the edge
    void cycle_vector(int tree, int edge, int words, uint64_t *C) const {
        std::memset(C, 0, sizeof(uint64_t) * words);
        const int32_t *pe = parent_edge + (size_t)tree * n;
        if (edge_coord[edge] >= 0) C[edge_coord[edge] >> 6] |= 1ULL << (edge_coord[edge] & 63);
        for (int side = 0; side < 2; side++) {
            uint32_t x = side ? cols[edge] : rows[edge];
            while (pe[x] >= 0) {
                int e = pe[x];
                int c = edge_coord[e];
                if (c >= 0) C[c >> 6] |= 1ULL << (c & 63);
                x = rows[e] != x ? rows[e] : cols[e];
            }
        }
    }
};

}  // namespace

extern "C" {

// Labels of every tree for one support vector: labels[t*n + v] in {0,1}.
int mcbo_labels(int n, int F, const uint32_t *rows, const uint32_t *cols, const int32_t *edge_coord,
                const int32_t *parent_edge, const uint64_t *S, uint8_t *labels, int threads) {
    if (n <= 0 || F < 0 || !rows || !cols || !edge_coord || !parent_edge || !S || !labels) return -1;
    if (threads <= 0) threads = omp_get_max_threads();
    Forest f;
    f.n = n;
    f.F = F;
    f.rows = rows;
    f.cols = cols;
    f.edge_coord = edge_coord;
    f.parent_edge = parent_edge;
    f.build(threads);
    f.labels(S, labels, threads);
    return 0;
}

// The de Pina loop.  Outputs selected[e] = rank of the candidate chosen at
// iteration e (e < iterations run), *total = sum of their weights (64-bit),
// *seconds = wall time of the loop (labels + scan + cycle vector + update).
// max_iter < 0 runs all N iterations.  Returns the number of iterations run, or a
// negative value if some iteration found no odd candidate (-(e+1)) / bad input.
int64_t mcbo_solve(int n, int F, int N, int64_t K, const uint32_t *rows, const uint32_t *cols,
                   const int32_t *edge_coord, const int32_t *parent_edge, const int32_t *cand_edge,
                   const int32_t *cand_weight, const int32_t *cand_tree, int threads, int64_t max_iter,
                   int64_t *selected, int64_t *total, double *seconds) {
    if (n <= 0 || F < 0 || N < 0 || K < 0 || !selected || !total) return -1000000000LL;
    if (threads <= 0) threads = omp_get_max_threads();
    const int words = (N + 63) / 64;
    Forest f;
    f.n = n;
    f.F = F;
    f.rows = rows;
    f.cols = cols;
    f.edge_coord = edge_coord;
    f.parent_edge = parent_edge;
    f.build(threads);
    std::vector<uint64_t> S((size_t)N * words, 0);
    for (int j = 0; j < N; j++) S[(size_t)j * words + (j >> 6)] |= 1ULL << (j & 63);
    std::vector<uint8_t> P((size_t)F * n);
    std::vector<uint8_t> removed((size_t)K, 0);
    std::vector<uint64_t> C(words);
    int64_t iters = (max_iter >= 0 && max_iter < N) ? max_iter : N;
    int64_t tot = 0;
    double t0 = now_s();
    for (int64_t e = 0; e < iters; e++) {
        const uint64_t *Se = &S[(size_t)e * words];
        f.labels(Se, P.data(), threads);
        int64_t chosen = -1;
        for (int64_t r = 0; r < K; r++) {
            if (removed[r]) continue;
            int ed = cand_edge[r];
            uint32_t bit = 0;
            if (edge_coord[ed] >= 0) bit = getbit(Se, edge_coord[ed]);
            const uint8_t *lab = &P[(size_t)cand_tree[r] * n];
            bit = (bit + lab[rows[ed]]) % 2;
            bit = (bit + lab[cols[ed]]) % 2;
            if (bit == 1) {
                chosen = r;
                break;
            }
        }
        if (chosen < 0) {
            if (seconds) *seconds = now_s() - t0;
            *total = tot;
            return -(e + 1);
        }
        removed[chosen] = 1;
        selected[e] = chosen;
        tot += cand_weight[chosen];
        f.cycle_vector(cand_tree[chosen], cand_edge[chosen], words, C.data());
#pragma omp parallel for num_threads(threads) schedule(static)
        for (int64_t j = e + 1; j < N; j++) {
            uint64_t *Sj = &S[(size_t)j * words];
            uint64_t acc = 0;
            for (int w = 0; w < words; w++) acc ^= C[w] & Sj[w];
            if (__builtin_popcountll(acc) & 1)
                for (int w = 0; w < words; w++) Sj[w] ^= Se[w];
        }
    }
    if (seconds) *seconds = now_s() - t0;
    *total = tot;
    return iters;
}

// The support vector S_e in force at iteration `at` of the loop above, for label
// parity tests: runs `at` iterations and copies S_at (words = ceil(N/64)).
int64_t mcbo_support_vector_at(int n, int F, int N, int64_t K, const uint32_t *rows, const uint32_t *cols,
                               const int32_t *edge_coord, const int32_t *parent_edge, const int32_t *cand_edge,
                               const int32_t *cand_tree, int threads, int64_t at, uint64_t *S_out) {
    if (at < 0 || at >= N || !S_out) return -1;
    if (threads <= 0) threads = omp_get_max_threads();
    const int words = (N + 63) / 64;
    Forest f;
    f.n = n;
    f.F = F;
    f.rows = rows;
    f.cols = cols;
    f.edge_coord = edge_coord;
    f.parent_edge = parent_edge;
    f.build(threads);
    std::vector<uint64_t> S((size_t)N * words, 0);
    for (int j = 0; j < N; j++) S[(size_t)j * words + (j >> 6)] |= 1ULL << (j & 63);
    std::vector<uint8_t> P((size_t)F * n);
    std::vector<uint8_t> removed((size_t)K, 0);
    std::vector<uint64_t> C(words);
    for (int64_t e = 0; e < at; e++) {
        const uint64_t *Se = &S[(size_t)e * words];
        f.labels(Se, P.data(), threads);
        int64_t chosen = -1;
        for (int64_t r = 0; r < K && chosen < 0; r++) {
            if (removed[r]) continue;
            int ed = cand_edge[r];
            uint32_t bit = edge_coord[ed] >= 0 ? getbit(Se, edge_coord[ed]) : 0;
            const uint8_t *lab = &P[(size_t)cand_tree[r] * n];
            if ((bit ^ lab[rows[ed]] ^ lab[cols[ed]]) & 1) chosen = r;
        }
        if (chosen < 0) return -(e + 1);
        removed[chosen] = 1;
        f.cycle_vector(cand_tree[chosen], cand_edge[chosen], words, C.data());
#pragma omp parallel for num_threads(threads) schedule(static)
        for (int64_t j = e + 1; j < N; j++) {
            uint64_t *Sj = &S[(size_t)j * words];
            uint64_t acc = 0;
            for (int w = 0; w < words; w++) acc ^= C[w] & Sj[w];
            if (__builtin_popcountll(acc) & 1)
                for (int w = 0; w < words; w++) Sj[w] ^= Se[w];
        }
    }
    std::memcpy(S_out, &S[(size_t)at * words], sizeof(uint64_t) * words);
    return at;
}

// Cost samples of the loop above, for graphs whose F x n' trees do not fit the
// host (the bench's CPU baseline extrapolates them to a whole solve):
// seconds per label pass over the F trees given (their parent edges only; the
// forest's BFS orders are built first and not timed), the mean of `passes` passes
// with support vectors drawn from `seed`.
double mcbo_label_pass_seconds(int n, int F, int N, const uint32_t *rows, const uint32_t *cols,
                               const int32_t *edge_coord, const int32_t *parent_edge, int passes, int threads,
                               uint64_t seed) {
    if (n <= 0 || F <= 0 || N <= 0 || passes <= 0 || !rows || !cols || !edge_coord || !parent_edge) return -1.0;
    if (threads <= 0) threads = omp_get_max_threads();
    const int words = (N + 63) / 64;
    Forest f;
    f.n = n;
    f.F = F;
    f.rows = rows;
    f.cols = cols;
    f.edge_coord = edge_coord;
    f.parent_edge = parent_edge;
    f.build(threads);
    std::vector<uint8_t> P((size_t)F * n);
    std::vector<uint64_t> S(words);
    uint64_t x = seed | 1;
    double sum = 0;
    for (int k = 0; k < passes; k++) {
        for (auto &w : S) {
            x ^= x << 13;
            x ^= x >> 7;
            x ^= x << 17;
            w = x;
        }
        const double t0 = now_s();
        f.labels(S.data(), P.data(), threads);
        sum += now_s() - t0;
    }
    return sum / passes;
}

// Seconds per row of the independence update (dot product of C with the row over
// all ceil(N/64) words, XOR of S_e into it when odd, as the loop above does for
// every j > e), timed over `rows` rows with random contents, `passes` times.
double mcbo_update_row_seconds(int N, int rows, int passes, int threads, uint64_t seed) {
    if (N <= 0 || rows <= 0 || passes <= 0) return -1.0;
    if (threads <= 0) threads = omp_get_max_threads();
    const int words = (N + 63) / 64;
    std::vector<uint64_t> S((size_t)rows * words), C(words), Se(words);
    uint64_t x = seed | 1;
    auto next = [&]() {
        x ^= x << 13;
        x ^= x >> 7;
        x ^= x << 17;
        return x;
    };
    for (auto &w : S) w = next();
    for (auto &w : C) w = next();
    for (auto &w : Se) w = next();
    const double t0 = now_s();
    for (int k = 0; k < passes; k++) {
#pragma omp parallel for num_threads(threads) schedule(static)
        for (int64_t j = 0; j < rows; j++) {
            uint64_t *Sj = &S[(size_t)j * words];
            uint64_t acc = 0;
            for (int w = 0; w < words; w++) acc ^= C[w] & Sj[w];
            if (__builtin_popcountll(acc) & 1)
                for (int w = 0; w < words; w++) Sj[w] ^= Se[w];
        }
    }
    return (now_s() - t0) / ((double)passes * rows);
}

}  // extern "C"
