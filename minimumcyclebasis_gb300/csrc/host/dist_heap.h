// Binary min-heap of (vertex, distance) entries ordered by distance alone, with the
// order of equal distances that the tree searches of the reference rely on: they
// run on std::priority_queue<pair<int,int>> with a distance-only comparator
// (include/Dijkstra.h:37-44), so which of two equally near vertices settles first is
// decided by the binary heap's layout.  This heap moves entries exactly as that
// queue's heap algorithm does, so its pop sequence is the same for any sequence of
// pushes and pops (tests/dist_heap_check.cpp compares the two on random sequences
// dense in ties):
//   push  the new entry rises from the end while its parent is strictly farther;
//   pop   the last entry is taken out, the hole left at the root descends to a leaf
//         along the preferred child (the right one unless the left one is strictly
//         nearer; a lone left child at the bottom when the size is even), and the
//         taken entry rises from there as in push.
// The child choice is arithmetic rather than a branch, which is where the time goes.
#pragma once

#include <cstddef>
#include <utility>
#include <vector>

struct DistHeap {
    std::vector<std::pair<int, int>> h;

    bool empty() const { return h.empty(); }
    size_t size() const { return h.size(); }
    const std::pair<int, int> &top() const { return h[0]; }
    void clear() { h.clear(); }

    void push(std::pair<int, int> v) {
        size_t i = h.size();
        h.push_back(v);
        rise(i, v);
    }

    void pop() {
        const size_t len = h.size() - 1;
        const std::pair<int, int> v = h[len];
        h.pop_back();
        if (len == 0) return;
        std::pair<int, int> *a = h.data();
        size_t hole = 0, c = 0;
        while (c < (len - 1) / 2) {
            c = 2 * (c + 1);
            c -= (size_t)(a[c].second > a[c - 1].second);
            a[hole] = a[c];
            hole = c;
        }
        if ((len & 1) == 0 && c == (len - 2) / 2) {
            c = 2 * (c + 1);
            a[hole] = a[c - 1];
            hole = c - 1;
        }
        rise(hole, v);
    }

  private:
    void rise(size_t i, std::pair<int, int> v) {
        std::pair<int, int> *a = h.data();
        while (i > 0) {
            const size_t p = (i - 1) / 2;
            if (!(a[p].second > v.second)) break;
            a[i] = a[p];
            i = p;
        }
        a[i] = v;
    }
};

// Monotone radix queue (Ahuja, Mehlhorn, Orlin and Tarjan, "Faster algorithms for
// the shortest path problem", 1990): entries are (distance, vertex) with unsigned
// distances that never fall below the last one taken out.  Bucket 0 holds the
// entries at exactly that last distance; bucket i > 0 those whose distance first
// differs from it in bit i - 1 (counting from bit 0).  Taking out refills bucket 0
// from the lowest non-empty bucket by moving its entries down by their new
// difference.  Equal distances come out in no particular order.
struct RadixQueue {
    std::vector<std::pair<unsigned, int>> b[33];
    unsigned last = 0;
    size_t count = 0;

    bool empty() const { return count == 0; }
    void clear() {
        for (auto &v : b) v.clear();
        last = 0;
        count = 0;
    }
    static int bucket_of(unsigned key, unsigned ref) {
        return key == ref ? 0 : 32 - __builtin_clz(key ^ ref);
    }
    void push(unsigned key, int vertex) {
        b[bucket_of(key, last)].push_back(std::make_pair(key, vertex));
        count++;
    }
    // the vertex of an entry at the smallest distance (the queue must not be empty)
    std::pair<unsigned, int> pop() {
        if (b[0].empty()) {
            int i = 1;
            while (b[i].empty()) i++;
            unsigned m = b[i][0].first;
            for (const auto &e : b[i]) m = e.first < m ? e.first : m;
            last = m;
            for (const auto &e : b[i]) b[bucket_of(e.first, last)].push_back(e);
            b[i].clear();
        }
        const std::pair<unsigned, int> e = b[0].back();
        b[0].pop_back();
        count--;
        return e;
    }
};
