// weight_sort (csrc/host/weight_sort.h) against std::sort with the reference's
// weight-only comparison: the two permutations of (weight, index) records must be
// identical, element for element, on random inputs dense in ties, on presorted,
// reversed and constant inputs, and on inputs built by an adversary that makes the
// standard sort exhaust its depth budget (so that its heap-sort fallback runs), at
// sizes below and above the parallel threshold and with 1 to 16 threads.  Exit status
// 0 and "ok" on success.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <numeric>
#include <vector>

#include "weight_sort.h"

static uint64_t state = 0x2545f4914f6cdd1dull;
static uint64_t next_u64() {  // xorshift64*
    state ^= state >> 12;
    state ^= state << 25;
    state ^= state >> 27;
    return state * 0x2545f4914f6cdd1dull;
}

static bool by_weight(const WeightKey &a, const WeightKey &b) { return a.weight < b.weight; }

static bool check(const std::vector<int> &w, int threads, const char *what) {
    std::vector<WeightKey> a(w.size()), b(w.size());
    for (size_t i = 0; i < w.size(); i++) a[i] = b[i] = {w[i], (uint32_t)i};
    std::sort(a.begin(), a.end(), by_weight);
    weight_sort(b.data(), b.size(), threads);
    for (size_t i = 0; i < w.size(); i++)
        if (a[i].index != b[i].index || a[i].weight != b[i].weight) {
            std::printf("FAIL %s n=%zu threads=%d at %zu\n", what, w.size(), threads, i);
            return false;
        }
    return true;
}

// McIlroy's adversary: values are fixed lazily, while std::sort runs, so that its
// pivots are as bad as possible; the values it ends with are an input on which the
// standard sort runs out of depth.
static std::vector<int> adversary(size_t n) {
    const int gas = (int)n;
    std::vector<int> val(n, gas);
    int solid = 0;
    size_t candidate = 0;
    std::vector<size_t> idx(n);
    std::iota(idx.begin(), idx.end(), 0);
    std::sort(idx.begin(), idx.end(), [&](size_t x, size_t y) {
        if (val[x] == gas && val[y] == gas) {
            if (x == candidate)
                val[x] = solid++;
            else
                val[y] = solid++;
        }
        if (val[x] == gas)
            candidate = x;
        else if (val[y] == gas)
            candidate = y;
        return val[x] < val[y];
    });
    for (auto &v : val)
        if (v == gas) v = solid++;
    return val;
}

int main() {
    long long cases = 0;
    const size_t sizes[] = {0, 1, 2, 3, 15, 16, 17, 33, 100, 1000, 4097, 65535, 65536, 70000, 300000, 2000000};
    const int thread_counts[] = {1, 3, 16};
    for (size_t n : sizes) {
        for (int range : {1, 2, 5, 100, 1 << 30}) {
            std::vector<int> w(n);
            for (auto &x : w) x = (int)(next_u64() % (uint64_t)range);
            for (int t : thread_counts) {
                if (!check(w, t, "random")) return 1;
                cases++;
            }
        }
        std::vector<int> up(n), down(n), pipe(n);
        for (size_t i = 0; i < n; i++) {
            up[i] = (int)(i / 3);
            down[i] = (int)((n - i) / 2);
            pipe[i] = (int)std::min(i, n - i);
        }
        for (int t : thread_counts) {
            if (!check(up, t, "ascending") || !check(down, t, "descending") || !check(pipe, t, "organ pipe"))
                return 1;
            cases += 3;
        }
    }
    for (size_t n : {200, 5000, 100000, 400000}) {
        std::vector<int> w = adversary(n);
        for (int t : thread_counts) {
            if (!check(w, t, "adversary")) return 1;
            cases++;
        }
        // few distinct values over the adversary's shape
        for (auto &x : w) x /= 7;
        for (int t : thread_counts) {
            if (!check(w, t, "adversary/7")) return 1;
            cases++;
        }
    }
    std::printf("ok %lld cases\n", cases);
    return 0;
}
