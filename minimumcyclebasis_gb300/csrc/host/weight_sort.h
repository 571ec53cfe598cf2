// The candidate sort of the reference driver, in parallel, with the same result.
//
// The reference orders its candidates with std::sort on the cycle weight alone
// (mcb/mcb_cycle_deg_two_remove.cpp:258, include/cycles.h:25-29).  std::sort is not
// stable, and which of several equal-weight candidates comes first decides which one
// enters the basis, so the order of equal weights has to be the one the standard
// library's sort gives.  That order follows from the sequence of element moves of
// its algorithm, an introsort:
//   - a range longer than 16 elements is split around a pivot: the median of its
//     second, middle and last elements (compared in a fixed sequence) is swapped to
//     the front, and a two-sided scan from the second and the last element swaps
//     pairs (an element not less than the pivot on the left, one not greater on the
//     right) until the scans cross; the right part is then split first, the left
//     part after it, each with the depth budget left after this split;
//   - a range whose depth budget (2 floor(log2 n) at the top) is used up is
//     heap-sorted (std::make_heap + std::sort_heap, the standard's own routines);
//   - ranges of at most 16 elements are left as they are, and a final insertion pass
//     over the whole array moves each element left past the strictly greater ones.
// After the splits every element of a range is not greater than any element of the
// ranges to its right, so the final pass only reorders elements inside each short
// range: it is a stable insertion sort of each of them.  Ranges never interact once
// split, so this code splits the top of the range tree on one thread and finishes
// the sub-ranges in parallel, each with exactly the moves the sequential sort makes
// on it.  tests/weight_sort_check.cpp compares the result with std::sort on random,
// tie-dense and adversarial (depth-exhausting) inputs.
#pragma once

#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <vector>

#include <omp.h>

struct WeightKey {
    int weight;
    uint32_t index;
};

namespace weight_sort_detail {

inline bool less(const WeightKey &a, const WeightKey &b) { return a.weight < b.weight; }

inline int floor_log2(size_t n) {
    int k = 0;
    while (n > 1) {
        n >>= 1;
        k++;
    }
    return k;
}

// Swaps the median of a, b, c (by the standard's comparison sequence) into *result.
inline void median_to_first(WeightKey *result, WeightKey *a, WeightKey *b, WeightKey *c) {
    if (less(*a, *b)) {
        if (less(*b, *c))
            std::swap(*result, *b);
        else if (less(*a, *c))
            std::swap(*result, *c);
        else
            std::swap(*result, *a);
    } else if (less(*a, *c)) {
        std::swap(*result, *a);
    } else if (less(*b, *c)) {
        std::swap(*result, *c);
    } else {
        std::swap(*result, *b);
    }
}

// Two-sided scan of [lo, hi) around the pivot value at *pivot; returns the split.
inline WeightKey *split(WeightKey *lo, WeightKey *hi, const WeightKey *pivot) {
    for (;;) {
        while (less(*lo, *pivot)) ++lo;
        --hi;
        while (less(*pivot, *hi)) --hi;
        if (!(lo < hi)) return lo;
        std::swap(*lo, *hi);
        ++lo;
    }
}

inline WeightKey *split_range(WeightKey *first, WeightKey *last) {
    WeightKey *mid = first + (last - first) / 2;
    median_to_first(first, first + 1, mid, last - 1);
    return split(first + 1, last, first);
}

constexpr ptrdiff_t kShort = 16;

// Stable insertion sort (an element moves left past strictly greater ones only).
inline void insertion(WeightKey *first, WeightKey *last) {
    for (WeightKey *i = first + 1; i < last; ++i) {
        const WeightKey v = *i;
        WeightKey *j = i;
        while (j > first && less(v, *(j - 1))) {
            *j = *(j - 1);
            --j;
        }
        *j = v;
    }
}

// The sequential split loop on one range with its depth budget, then the final
// pass over it.
inline void finish(WeightKey *first, WeightKey *last, int depth) {
    WeightKey *const begin = first, *const end = last;
    struct Range {
        WeightKey *f, *l;
        int d;
    };
    std::vector<Range> todo;
    todo.push_back({first, last, depth});
    while (!todo.empty()) {
        Range r = todo.back();
        todo.pop_back();
        while (r.l - r.f > kShort) {
            if (r.d == 0) {
                std::make_heap(r.f, r.l, less);
                std::sort_heap(r.f, r.l, less);
                break;
            }
            --r.d;
            WeightKey *cut = split_range(r.f, r.l);
            todo.push_back({cut, r.l, r.d});  // the right part (its order of processing is immaterial)
            r.l = cut;
        }
    }
    insertion(begin, end);
}

}  // namespace weight_sort_detail

// Sorts keys by weight with the permutation std::sort gives; `threads` <= 0: all.
inline void weight_sort(WeightKey *keys, size_t n, int threads) {
    using namespace weight_sort_detail;
    if (n < 2) return;
    const int depth0 = 2 * floor_log2(n);
    if (threads <= 0) threads = omp_get_max_threads();
    if (threads <= 1 || n < (size_t)1 << 16) {
        finish(keys, keys + n, depth0);
        return;
    }
    // split the top of the range tree on this thread until there are enough ranges
    struct Range {
        WeightKey *f, *l;
        int d;
    };
    std::vector<Range> ready, work{{keys, keys + n, depth0}};
    const size_t target = (size_t)threads * 8, small = std::max<size_t>(n / ((size_t)threads * 16), 4096);
    while (!work.empty() && ready.size() + work.size() < target) {
        // split the largest range still open
        auto it = std::max_element(work.begin(), work.end(),
                                   [](const Range &a, const Range &b) { return a.l - a.f < b.l - b.f; });
        Range r = *it;
        work.erase(it);
        if ((size_t)(r.l - r.f) <= small || r.d == 0 || r.l - r.f <= kShort) {
            ready.push_back(r);
            continue;
        }
        WeightKey *cut = split_range(r.f, r.l);
        work.push_back({r.f, cut, r.d - 1});
        work.push_back({cut, r.l, r.d - 1});
    }
    ready.insert(ready.end(), work.begin(), work.end());
    std::sort(ready.begin(), ready.end(), [](const Range &a, const Range &b) { return a.l - a.f > b.l - b.f; });
#pragma omp parallel for num_threads(threads) schedule(dynamic, 1)
    for (int64_t i = 0; i < (int64_t)ready.size(); i++) finish(ready[(size_t)i].f, ready[(size_t)i].l, ready[(size_t)i].d);
}
