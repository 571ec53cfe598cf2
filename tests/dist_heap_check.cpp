// DistHeap against std::priority_queue with a distance-only comparator (the queue of
// the reference's tree searches): random push/pop sequences, distances drawn from
// small ranges so that ties are dense, and Dijkstra-like monotone sequences.  Every
// top() and size() must agree.  RadixQueue on monotone sequences (no push below the
// last distance taken out): the same distances come out in the same order as from
// std::priority_queue, and every pushed vertex comes out exactly once.  Exit status 0
// and "ok" on success.
#include <cstdint>
#include <cstdio>
#include <queue>
#include <vector>

#include "dist_heap.h"

struct ByDistance {
    bool operator()(const std::pair<int, int> &a, const std::pair<int, int> &b) const {
        return a.second > b.second;
    }
};

static uint64_t state = 0x9e3779b97f4a7c15ull;
static uint64_t next_u64() {  // xorshift64*
    state ^= state >> 12;
    state ^= state << 25;
    state ^= state >> 27;
    return state * 0x2545f4914f6cdd1dull;
}

int main() {
    long long checked = 0;
    for (int trial = 0; trial < 3000; trial++) {
        std::priority_queue<std::pair<int, int>, std::vector<std::pair<int, int>>, ByDistance> pq;
        DistHeap dh;
        const int range = 1 + trial % 64;
        const bool monotone = trial % 3 == 0;
        const int ops = 1 + (int)(next_u64() % 4000);
        int base = 0;
        for (int k = 0; k < ops; k++) {
            if (pq.empty() || next_u64() % 3 != 0) {
                int d = (int)(next_u64() % range) + (monotone ? base : 0);
                std::pair<int, int> v((int)(next_u64() % 100000), d);
                pq.push(v);
                dh.push(v);
            } else {
                if (pq.top() != dh.top()) {
                    std::printf("mismatch: trial %d op %d\n", trial, k);
                    return 1;
                }
                base = pq.top().second;
                pq.pop();
                dh.pop();
                checked++;
            }
            if (pq.size() != dh.size()) {
                std::printf("size mismatch: trial %d op %d\n", trial, k);
                return 1;
            }
        }
        while (!pq.empty()) {
            if (pq.top() != dh.top()) {
                std::printf("mismatch while draining: trial %d\n", trial);
                return 1;
            }
            pq.pop();
            dh.pop();
            checked++;
        }
        if (!dh.empty()) return 1;
    }
    for (int trial = 0; trial < 3000; trial++) {
        std::priority_queue<std::pair<int, int>, std::vector<std::pair<int, int>>, ByDistance> pq;
        RadixQueue rq;
        std::vector<int> out_count;
        const int range = 1 + (int)(next_u64() % (trial % 2 ? 8 : 100000));
        const int ops = 1 + (int)(next_u64() % 4000);
        unsigned base = (unsigned)(next_u64() % 1000);
        int id = 0;
        for (int k = 0; k < ops || !pq.empty(); k++) {
            if (k < ops && (pq.empty() || next_u64() % 3 != 0)) {
                unsigned d = base + (unsigned)(next_u64() % range);
                pq.push(std::make_pair(id, (int)d));
                rq.push(d, id);
                out_count.push_back(0);
                id++;
            } else {
                if (rq.empty()) {
                    std::printf("radix queue empty early: trial %d\n", trial);
                    return 1;
                }
                std::pair<unsigned, int> e = rq.pop();
                if ((int)e.first != pq.top().second || out_count[e.second]++ != 0) {
                    std::printf("radix mismatch: trial %d op %d\n", trial, k);
                    return 1;
                }
                base = e.first;
                pq.pop();
                checked++;
            }
        }
        if (!rq.empty()) return 1;
        for (int c : out_count)
            if (c != 1) return 1;
    }
    std::printf("ok %lld pops\n", checked);
    return 0;
}
