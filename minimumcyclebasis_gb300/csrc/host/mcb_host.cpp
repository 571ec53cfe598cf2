// Host-side preprocessing for the minimum-cycle-basis driver (libmcbhost.so).
//
// Every stage reproduces the reference's result exactly, because the reference's
// output (which of several equal-weight cycles enters the basis) depends on all of
// them: edge offsets, the coordinate order of the non-tree edges, which vertices are
// FVS roots, the shortest-path tree chosen among equal-length paths, and the order of
// the candidate list.  Where the reference's result depends on a standard-library
// behaviour (std::sort's permutation of equal keys, std::priority_queue's order of
// equal distances, std::unordered_map's iteration order), this file calls the same
// standard-library routine on the same sequence, which gives the same permutation;
// the tree searches' queue is the one exception: dist_heap.h restates its heap moves
// (faster, same pop order, checked against std::priority_queue by a test).
// The recursive DFS passes of the reference are restated as explicit-stack loops
// that visit edges in the same order (the reference needs `ulimit -s unlimited`).
#include "mcbhost.h"
#include "dist_heap.h"
#include "weight_sort.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <memory>
#include <memory_resource>
#include <new>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <utility>
#include <vector>
#include <omp.h>

namespace {

using u32 = uint32_t;
using u64 = uint64_t;
using i64 = int64_t;

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// One directed edge slot while sorting.  Only (row, col) take part in comparisons,
// so std::sort permutes these exactly as it permutes the reference's edge pointers.
struct EdgeSlot {
    u32 row, col;
    int weight;
    int chain;
    int orig;
    u32 rev;  // index of the reverse slot before sorting
};
struct RowColLess {
    bool operator()(const EdgeSlot &a, const EdgeSlot &b) const {
        return a.row == b.row ? a.col < b.col : a.row < b.row;
    }
};

struct Graph {  // CSR over both directions, sorted by (row, col)
    int n = 0;
    std::vector<u32> rows, cols, ro, deg;
    std::vector<int> w;
    std::vector<u32> rev;  // multigraph only
    size_t slots() const { return rows.size(); }
};

// include/CsrGraph.h:113-174: sort the 2m slots by (row, col), then row offsets.
void finish_simple_csr(Graph &g, std::vector<EdgeSlot> &s) {
    std::sort(s.begin(), s.end(), RowColLess());
    g.rows.resize(s.size());
    g.cols.resize(s.size());
    g.w.resize(s.size());
    for (size_t i = 0; i < s.size(); i++) {
        g.rows[i] = s[i].row;
        g.cols[i] = s[i].col;
        g.w[i] = s[i].weight;
    }
    g.ro.assign(g.n + 1, 0);
    g.deg.assign(g.n, 0);
    for (size_t i = 0; i < s.size(); i++) g.ro[g.rows[i]]++;
    u32 prev = 0;
    for (int i = 0; i <= g.n; i++) {
        u32 c = g.ro[i];
        g.ro[i] = prev;
        prev += c;
    }
    for (int i = 0; i < g.n; i++) g.deg[i] = g.ro[i + 1] - g.ro[i];
}

}  // namespace

struct mcbh_problem {
    // input
    Graph in;
    i64 m_in = 0;
    bool prepared = false;
    bool attempted = false;  // one preparation per problem, successful or not
    bool single_cycle = false;
    i64 total_weight_input = 0;
    // reduced multigraph
    Graph rg;
    std::vector<int> r_chain, r_orig;
    std::vector<int> r_vertex;  // reduced vertex -> input vertex
    int nodes_removed = 0;
    int source_vertex = 0;
    // FVS
    std::vector<int> fvs_array;
    std::vector<u32> fvs_vertices;
    // coordinates
    std::vector<u32> coord_edges;
    std::vector<int> edge_coord;
    // slot pairs of the reduced graph: the lower slot of every pair in ascending
    // order, and each slot's pair index
    std::vector<u32> pair_first, slot_pair;
    std::vector<std::pair<u32, u32>> pair_ends;  // (row, column) of each pair's lower slot
    // the reduced graph's slots as (column, weight) records, for the tree searches
    struct Arc {
        u32 col;
        int w;
    };
    std::vector<Arc> arcs;
    bool fast_search_ok = false;  // every weight >= 1 and no distance can overflow
    bool structure_only = false;  // prepared up to the spanning tree; candidates from mcbh_rank_candidates
    bool ranked = false;          // mcbh_rank_candidates has filled the candidate arrays
    // trees
    std::vector<int> tree_parent;  // F x n'
    std::vector<u32> lay_rows, lay_cols, lay_nodes;
    std::vector<int> lay_edge;
    // candidates in rank order
    std::vector<int> c_root, c_edge, c_weight, c_tree;
    std::vector<i64> c_off;
    std::vector<int> c_coords;
    mcbh_info info{};
};

namespace {

// ---------------------------------------------------------------------------
// Degree-two chains (include/CsrGraphDegreeTwoRemoval.cpp:12-126).
// The reference runs a recursive DFS from the first vertex of degree > 2; on the
// way back from each edge it extends / opens / closes the current chain.  The
// explicit stack below keeps the same edge order and runs the post-edge step when
// a child frame returns.
struct ChainResult {
    std::vector<u32> removal;
    std::vector<std::vector<u32>> chains;
    int src = 0;
    bool bad = false;  // the reference would dereference a null chain here
};

ChainResult mark_degree_two_chains(const Graph &g) {
    ChainResult r;
    const int n = g.n;
    std::vector<char> visited(n, 0);
    std::vector<int> parent(n, -1);
    std::vector<u32> current;  // the chain being assembled
    bool have_current = false;

    auto chain_step = [&](u32 row, u32 offset) {
        u32 column = g.cols[offset];
        bool dc = g.deg[column] == 2, dr = g.deg[row] == 2;
        if (dc && dr) {
            if (!have_current) r.bad = true;
            current.push_back(offset);
            r.removal.push_back(offset);
        } else if (dr) {
            current.clear();
            current.push_back(offset);
            have_current = true;
            r.removal.push_back(offset);
        } else if (dc) {
            if (!have_current) r.bad = true;
            current.push_back(offset);
            r.chains.push_back(current);
            current.clear();
            have_current = false;
            r.removal.push_back(offset);
        }
    };

    int src = -1;
    for (int i = 0; i < n; i++)
        if (g.deg[i] > 2) {
            src = i;
            break;
        }
    if (src < 0) {  // the reference leaves its source uninitialised here
        r.src = 0;
        return r;
    }
    r.src = src;

    struct Frame {
        u32 row, off;
    };
    std::vector<Frame> st;
    visited[src] = 1;
    st.push_back({(u32)src, g.ro[src]});
    while (!st.empty()) {
        Frame &f = st.back();
        if (f.off == g.ro[f.row + 1]) {
            st.pop_back();
            if (!st.empty()) {  // back from dfs(column): finish that tree edge
                Frame &p = st.back();
                chain_step(p.row, p.off);
                p.off++;
            }
            continue;
        }
        u32 row = f.row, offset = f.off;
        u32 column = g.cols[offset];
        if (!visited[column]) {
            visited[column] = 1;
            parent[column] = (int)row;
            st.push_back({column, g.ro[column]});
            continue;
        }
        if ((int)column == parent[row]) {
            if (g.deg[column] == 2 || g.deg[row] == 2) r.removal.push_back(offset);
            f.off++;
            continue;
        }
        if (g.deg[column] == 2) {
            r.removal.push_back(offset);
            f.off++;
            continue;
        }
        chain_step(row, offset);
        f.off++;
    }
    return r;
}

// include/CsrGraphMulti.h:229-300 (get_modified_graph) and :96-168 (sort + reverse).
void build_reduced(mcbh_problem &P, const ChainResult *cr) {
    const Graph &g = P.in;
    std::vector<char> filtered(g.slots(), 0);
    std::vector<std::vector<u32>> new_edges;  // (row, col, weight)
    if (cr) {
        for (u32 o : cr->removal) filtered[o] = 1;
        for (const auto &ch : cr->chains) {
            // csr_graph::sum_edge_weights (include/CsrGraph.h:193-204)
            u32 tot = 0;
            for (u32 o : ch) tot += (u32)g.w[o];
            u32 col = g.cols[ch.front()];
            u32 row = g.rows[ch.back()];
            new_edges.push_back({row, col, tot});
        }
    }
    // Relabel in order of first appearance: kept slots first, then new edges.
    std::vector<int> label(g.n, -1);
    int cnt = 0;
    for (size_t i = 0; i < g.slots(); i++)
        if (!filtered[i]) {
            if (label[g.rows[i]] < 0) label[g.rows[i]] = cnt++;
            if (label[g.cols[i]] < 0) label[g.cols[i]] = cnt++;
        }
    for (const auto &e : new_edges) {
        if (label[e[0]] < 0) label[e[0]] = cnt++;
        if (label[e[1]] < 0) label[e[1]] = cnt++;
    }
    Graph &r = P.rg;
    r.n = cnt;
    P.r_vertex.assign((size_t)cnt, -1);
    for (int v = 0; v < g.n; v++)
        if (label[v] >= 0) P.r_vertex[label[v]] = v;
    std::vector<EdgeSlot> s;
    s.reserve(2 * new_edges.size() + g.slots());
    auto insert_pair = [&](u32 a, u32 b, int wt, int chain, int orig) {
        u32 i0 = (u32)s.size();
        s.push_back({a, b, wt, chain, orig, i0 + 1});
        s.push_back({b, a, wt, chain, orig, i0});
    };
    for (size_t i = 0; i < new_edges.size(); i++)
        insert_pair((u32)label[new_edges[i][0]], (u32)label[new_edges[i][1]], (int)new_edges[i][2], (int)i,
                    -1);
    for (size_t i = 0; i < g.slots(); i++)
        if (!filtered[i] && g.rows[i] < g.cols[i])
            insert_pair((u32)label[g.rows[i]], (u32)label[g.cols[i]], g.w[i], -1, (int)i);

    // Sort slots by (row, col) with std::sort (unstable for parallel edges: the same
    // permutation as the reference's sort of edge pointers), then remap reverses.
    std::vector<EdgeSlot> sorted = s;
    for (size_t i = 0; i < sorted.size(); i++) sorted[i].rev = (u32)i;  // remember origin
    std::sort(sorted.begin(), sorted.end(), RowColLess());
    std::vector<u32> newpos(s.size());
    for (size_t i = 0; i < sorted.size(); i++) newpos[sorted[i].rev] = (u32)i;
    const size_t S2 = sorted.size();
    r.rows.resize(S2);
    r.cols.resize(S2);
    r.w.resize(S2);
    r.rev.resize(S2);
    P.r_chain.resize(S2);
    P.r_orig.resize(S2);
    for (size_t i = 0; i < S2; i++) {
        u32 origin = sorted[i].rev;
        r.rows[i] = sorted[i].row;
        r.cols[i] = sorted[i].col;
        r.w[i] = sorted[i].weight;
        P.r_chain[i] = sorted[i].chain;
        P.r_orig[i] = sorted[i].orig;
        r.rev[i] = newpos[s[origin].rev];
    }
    r.ro.assign(r.n + 1, 0);
    r.deg.assign(r.n, 0);
    for (size_t i = 0; i < S2; i++) r.ro[r.rows[i]]++;
    u32 prev = 0;
    for (int i = 0; i <= r.n; i++) {
        u32 c = r.ro[i];
        r.ro[i] = prev;
        prev += c;
    }
    for (int i = 0; i < r.n; i++) r.deg[i] = r.ro[i + 1] - r.ro[i];
}

// ---------------------------------------------------------------------------
// FVS (include/FVS.cpp:166-262).  MGA's pruning step exits at once (it marks the
// chosen vertex removed before testing it, FVS.cpp:94-104), so W and the degrees
// never change and MGA picks every vertex, by largest degree, lowest id first.  The
// list is then reversed and each vertex is dropped from the FVS if the rest stays
// acyclic (test_fvs: BFS cycle check over non-FVS vertices, FVS.cpp:138-212).  Here
// the same test is answered incrementally with a union-find over the non-FVS
// forest: adding v closes a cycle iff v has a self-loop, or two of its edges
// (parallel edges included) reach the same forest component.
struct DSU {
    std::vector<int> p;
    explicit DSU(int n) : p(n) {
        for (int i = 0; i < n; i++) p[i] = i;
    }
    int find(int x) {
        while (p[x] != x) {
            p[x] = p[p[x]];
            x = p[x];
        }
        return x;
    }
};

void compute_fvs(mcbh_problem &P) {
    const Graph &g = P.rg;
    const int n = g.n;
    // MGA pick order: ratio W/deg ascending with strict '<' (lowest id wins ties).
    // W = 1 for every vertex of the reduced graph (all have degree >= 1).
    std::vector<int> order(n);
    for (int i = 0; i < n; i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        double ra = 1.0 / (double)g.deg[a], rb = 1.0 / (double)g.deg[b];
        return ra < rb;
    });
    std::reverse(order.begin(), order.end());
    std::vector<char> in_fvs(n, 1);
    DSU dsu(n);
    std::vector<int> seen_roots;
    for (int v : order) {
        bool cycle = false;
        seen_roots.clear();
        for (u32 o = g.ro[v]; o < g.ro[v + 1] && !cycle; o++) {
            u32 c = g.cols[o];
            if ((int)c == v) {
                cycle = true;
                break;
            }
            if (in_fvs[c]) continue;
            int rt = dsu.find((int)c);
            for (int x : seen_roots)
                if (x == rt) {
                    cycle = true;
                    break;
                }
            seen_roots.push_back(rt);
        }
        if (!cycle) {
            in_fvs[v] = 0;
            for (int x : seen_roots) dsu.p[dsu.find(x)] = dsu.find(v);
        }
    }
    P.fvs_array.assign(n, -1);
    P.fvs_vertices.clear();
    int cnt = 0;
    for (int v = 0; v < n; v++)
        if (in_fvs[v]) {
            P.fvs_array[v] = cnt++;
            P.fvs_vertices.push_back((u32)v);
        }
}

// ---------------------------------------------------------------------------
// Initial DFS spanning tree (include/CsrGraphMultiSpanningTree.cpp:11-135) and the
// coordinate map (mcb/mcb_cycle_deg_two_remove.cpp:175-187).
bool spanning_tree(mcbh_problem &P, int src) {
    const Graph &g = P.rg;
    const int n = g.n;
    if (src < 0 || src >= n) return false;
    std::vector<char> visited(n, 0);
    std::vector<int> parent(n, -1);
    std::vector<unsigned char> state(g.slots(), 0);  // 0 unseen, 1 tree, 2 non-tree
    std::vector<u32> nte;
    int tree_edges = 0;
    struct Frame {
        u32 row, off;
    };
    std::vector<Frame> st;
    visited[src] = 1;
    st.push_back({(u32)src, g.ro[src]});
    while (!st.empty()) {
        Frame &f = st.back();
        if (f.off == g.ro[f.row + 1]) {
            st.pop_back();
            if (!st.empty()) st.back().off++;
            continue;
        }
        u32 row = f.row, offset = f.off;
        u32 column = g.cols[offset];
        if (!visited[column]) {
            visited[column] = 1;
            tree_edges++;
            parent[column] = (int)row;
            state[offset] = 1;
            st.push_back({column, g.ro[column]});
            continue;
        }
        f.off++;
        if ((int)column == parent[row]) {
            u32 ri = g.rev[offset];
            if (state[ri] == 1) {
                state[offset] = 1;
            } else if (state[ri] == 2) {
                state[offset] = 2;
            } else {
                state[offset] = 2;
                state[ri] = 2;
                nte.push_back(row < column ? offset : ri);
            }
        } else if (state[offset] == 0) {
            u32 ri = g.rev[offset];
            state[offset] = 2;
            state[ri] = 2;
            nte.push_back(row < column ? offset : ri);
        }
    }
    if (tree_edges != n - 1) return false;
    P.coord_edges = nte;
    P.edge_coord.assign(g.slots(), -1);
    for (size_t i = 0; i < nte.size(); i++) P.edge_coord[nte[i]] = (int)i;
    for (size_t i = 0; i < g.slots(); i++)
        if (P.edge_coord[i] < 0 && P.edge_coord[g.rev[i]] >= 0) P.edge_coord[i] = P.edge_coord[g.rev[i]];
    return true;
}

// ---------------------------------------------------------------------------
// Per-root shortest-path tree + candidates (include/Dijkstra.h:78-254,
// include/work_per_thread.h:92-147).
struct LevelItem {  // include/Dijkstra.h:7-21
    int offset, level;
};
struct LevelLess {
    bool operator()(const LevelItem &a, const LevelItem &b) const { return a.level < b.level; }
};

struct LocalCandidate {
    int edge;
    int weight;
    i64 coord_begin;
    int coord_len;
};

struct RootOutput {
    std::vector<LocalCandidate> cands;
    std::vector<int> coords;
    // unordered_map keyed as the reference's, with the same insertion sequence
    // (include/cycle_searcher.h:23-61); only its iteration order is used, and that
    // order depends on the keys and their sequence, not on the mapped values.  Each
    // key maps to the first and last of its candidates, chained in insertion order
    // through `next`.  Its nodes and buckets come from an arena of the root's own
    // (the allocator takes no part in the bucket layout, so not in the order).
    std::unique_ptr<std::pmr::monotonic_buffer_resource> arena =
        std::make_unique<std::pmr::monotonic_buffer_resource>();
    std::pmr::unordered_map<unsigned long long, std::pair<int, int>> groups{arena.get()};
    std::vector<int> next;

    // candidate `local` (just appended to cands) joins the group of its vertex pair
    void group(int local, u32 a, u32 b) {
        next.push_back(-1);
        const unsigned long long key = ((unsigned long long)std::min(a, b) << 32) | std::max(a, b);
        auto it = groups.find(key);
        if (it == groups.end()) {
            groups.insert(std::make_pair(key, std::make_pair(local, local)));
        } else {
            next[it->second.second] = local;
            it->second.second = local;
        }
    }
};

// One vertex of a tree search: distance, parent vertex, slot into it from the
// parent, and flags (bit 0 settled; bit 1, fast search only: the parent has a rival
// at the same distance), one 16-byte record per vertex.
struct VertexState {
    int dist, par, pedge, done;
};

struct TreeWorkspace {
    std::vector<VertexState> vs;
    RadixQueue rq;
    std::vector<int> level;
    std::vector<u32> chain;
    std::vector<u32> pop_order;
    std::vector<unsigned char> pair_tree;
    DistHeap pq;  // include/Dijkstra.h:37-44: min-heap on distance only
    std::vector<LevelItem> lv;
    std::vector<int> tmp;
    void init(int n, size_t pairs) {
        vs.assign(n, VertexState{-1, -1, -1, 0});
        pair_tree.assign(pairs, 0);
        pop_order.clear();
        pop_order.reserve(n);
    }
};

// dijkstra::dijkstra_sp (include/Dijkstra.h:78-124) as the reference runs it: the
// binary heap decides which of two equally near vertices settles first.  (The level
// of a vertex, set with its parent in the reference, is its final parent's level + 1:
// computed after the search, in settle order, where needed.)  kPositive: every
// weight is at least 1 and no distance overflows, so a settled vertex, nearer than
// the one being settled, never passes the distance test and the reference's
// "settled" test before it can be left out without changing the push sequence.
template <bool kPositive>
void search_exact(const mcbh_problem &P, u32 src, TreeWorkspace &ws, std::vector<u32> &tree_edges) {
    const Graph &g = P.rg;
    VertexState *vs = ws.vs.data();
    const mcbh_problem::Arc *arcs = P.arcs.data();
    vs[src].dist = 0;
    ws.pq.clear();
    ws.pq.push(std::make_pair((int)src, 0));
    while (!ws.pq.empty()) {
        std::pair<int, int> val = ws.pq.top();
        ws.pq.pop();
        int x = val.first;
        VertexState &sx = vs[x];
        if (sx.done) continue;
        if ((u32)x != src) tree_edges.push_back((u32)sx.pedge);
        sx.done = 1;
        ws.pop_order.push_back((u32)x);
        const int dx = sx.dist;
        for (u32 o = g.ro[x]; o < g.ro[x + 1]; o++) {
            const mcbh_problem::Arc a = arcs[o];
            VertexState &sc = vs[a.col];
            if (!kPositive && sc.done) continue;
            const int nd = dx + a.w;
            if (kPositive ? (unsigned)nd < (unsigned)sc.dist : (sc.dist == -1 || nd < sc.dist)) {
                sc.dist = nd;
                ws.pq.push(std::make_pair((int)a.col, nd));
                sc.par = x;
                sc.pedge = (int)o;
            }
        }
    }
}

// The same search with a monotone radix queue, for graphs whose weights are all at
// least 1 and whose distances cannot overflow.  Every shortest-path parent of a
// vertex is then strictly nearer than the vertex and settles before it, and the
// parent the reference keeps is the first of them to settle (only a strictly shorter
// path replaces a parent).  Parents at different distances settle in distance order
// under any queue; only two parents at the same distance, each on a shortest path
// through a different vertex, are ordered by the reference's heap.  The search
// counts the vertices whose current parent has such a rival (cleared when a
// strictly shorter path replaces the parent) and returns false if any is left; the
// caller then runs search_exact.  Otherwise distances, parents and parent slots equal
// the reference's; the settle order may differ among equal distances, which only
// the level-ordered layout (built from search_exact alone) depends on.
bool search_fast(const mcbh_problem &P, u32 src, TreeWorkspace &ws, std::vector<u32> &tree_edges) {
    const Graph &g = P.rg;
    VertexState *vs = ws.vs.data();
    const mcbh_problem::Arc *arcs = P.arcs.data();
    long long rivals = 0;
    vs[src].dist = 0;
    ws.rq.clear();
    ws.rq.push(0u, (int)src);
    while (!ws.rq.empty()) {
        const int x = ws.rq.pop().second;
        VertexState &sx = vs[x];
        if (sx.done & 1) continue;
        if ((u32)x != src) tree_edges.push_back((u32)sx.pedge);
        sx.done |= 1;
        ws.pop_order.push_back((u32)x);
        const int dx = sx.dist;
        // with weights >= 1 a settled vertex is nearer than dx < nd, so the distance
        // test alone skips it; unreached (-1) compares as the largest unsigned value
        for (u32 o = g.ro[x]; o < g.ro[x + 1]; o++) {
            const mcbh_problem::Arc a = arcs[o];
            VertexState &sc = vs[a.col];
            const int nd = dx + a.w;
            if ((unsigned)nd < (unsigned)sc.dist) {
                sc.dist = nd;
                ws.rq.push((unsigned)nd, (int)a.col);
                sc.par = x;
                sc.pedge = (int)o;
                if (sc.done & 2) {
                    sc.done = 0;
                    rivals--;
                }
            } else if (nd == sc.dist && sc.par != x && !(sc.done & 2) && vs[sc.par].dist == dx) {
                sc.done |= 2;
                rivals++;
            }
        }
    }
    return rivals == 0;
}

// A root's tree supplied from outside (mcbh_prepare_with_trees: distances and parent
// slots, e.g. computed on the GPU), adopted only if it is the tree the reference's
// search builds.  With every weight at least 1 that is checked in two passes over the
// slots: (1) it is a tree of shortest paths: the root at distance 0, every other
// vertex entered by its parent slot from a vertex whose distance plus the slot's
// weight is its own, and no slot giving any vertex a shorter path; (2) every parent
// is the one the reference keeps: the nearest of the vertex's shortest-path
// neighbours, through that neighbour's first such slot, with no other neighbour as
// near (otherwise the heap's order decides, and the root is searched here).  With
// `structure_only` (a trusted supplier) the parent rule of (2) is not checked; (1)
// is, in full: its first half keeps the later walks up the parent chains finite, its
// second (no slot gives a shorter path) keeps a supplier that stopped short of the
// true distances from yielding a heavier basis.  Returns false, leaving the
// workspace to be reinitialised, if a check fails.
bool take_given_tree(const mcbh_problem &P, u32 src, TreeWorkspace &ws, const int32_t *dist, const int32_t *pedge,
                     std::vector<u32> &tree_edges, bool structure_only) {
    const Graph &g = P.rg;
    const int n = g.n;
    const int64_t slots = (int64_t)g.slots();
    VertexState *vs = ws.vs.data();
    if (dist[src] != 0 || pedge[src] != -1) return false;
    for (int v = 0; v < n; v++) {
        if ((u32)v == src) continue;
        const int64_t o = pedge[v];
        if (o < 0 || o >= slots || g.cols[o] != (u32)v) return false;
        const u32 p = g.rows[o];
        if (dist[p] < 0 || (long long)dist[p] + g.w[o] != (long long)dist[v]) return false;
    }
    for (int c = 0; c < n && structure_only; c++) {
        const long long dc = dist[c];
        for (u32 o = g.ro[c]; o < g.ro[c + 1]; o++)
            if ((long long)dist[g.cols[o]] > dc + g.w[o]) return false;  // a shorter path through c
    }
    for (int c = 0; c < n && !structure_only; c++) {
        const int dc = dist[c];
        int bestd = -1;
        bool rival = false;  // another neighbour as near as the best: the heap decides
        u32 bestx = 0xffffffffu, bests = 0xffffffffu;
        for (u32 o = g.ro[c]; o < g.ro[c + 1]; o++) {
            const u32 x = g.cols[o];
            const long long via = (long long)dc + g.w[o];
            if ((long long)dist[x] > via) return false;  // a shorter path to x through c
            if ((u32)c == src || (long long)dist[x] + g.w[o] != (long long)dc) continue;
            if (bestd < 0 || dist[x] < bestd) {
                bestd = dist[x];
                bestx = x;
                bests = g.rev[o];
                rival = false;
            } else if (dist[x] == bestd) {
                if (x != bestx)
                    rival = true;
                else
                    bests = g.rev[o] < bests ? g.rev[o] : bests;
            }
        }
        if ((u32)c != src && (rival || (int64_t)bests != (int64_t)pedge[c])) return false;
    }
    for (int v = 0; v < n; v++) {
        vs[v].dist = dist[v];
        vs[v].pedge = pedge[v];
        vs[v].par = (u32)v == src ? -1 : (int)g.rows[pedge[v]];
        vs[v].done = 1;
        if ((u32)v != src) tree_edges.push_back((u32)pedge[v]);
    }
    return true;
}

// Which search one root takes, and what it cost.
struct SearchChoice {
    bool try_fast = false;  // in: try search_fast first
    int result = -1;        // out: 1 search_fast kept, 0 it fell back, -1 not tried
    double fast_s = 0, exact_s = 0;
};

// Chooses, root by root, between search_fast (with its fallback) and search_exact
// from their measured costs: search_fast is tried while its mean cost per root, the
// fallbacks' heap searches included, is below the heap search's mean, and on every
// 32nd root regardless, so that the estimate follows the roots.  How often a root's
// search falls back depends on the graph (1% of the roots at weights U[1,1000], a
// quarter at U[1,255], nearly all with small integer weights) and on the root, and
// what search_fast saves depends on the graph too.  Which roots take which search
// changes no output, only the time.
struct SearchPolicy {
    std::atomic<long long> ok_n{0}, fail_n{0}, exact_n{0}, ok_ns{0}, fail_ns{0}, exact_ns{0};

    bool want_fast(int t) const {
        const auto rl = std::memory_order_relaxed;
        const long long okn = ok_n.load(rl), failn = fail_n.load(rl), exn = exact_n.load(rl);
        const long long tries = okn + failn;
        if (tries < 32 || t % 32 == 0 || exn == 0) return true;
        const double exact_mean = (double)exact_ns.load(rl) / (double)exn;
        const double fast_mean =
            ((double)ok_ns.load(rl) + (double)fail_ns.load(rl) + exact_mean * (double)failn) / (double)tries;
        return fast_mean < exact_mean;
    }
    void record(const SearchChoice &c) {
        const auto rl = std::memory_order_relaxed;
        const long long f = (long long)(c.fast_s * 1e9), e = (long long)(c.exact_s * 1e9);
        if (c.result == 1) {
            ok_n.fetch_add(1, rl);
            ok_ns.fetch_add(f, rl);
            return;
        }
        if (c.result == 0) {
            fail_n.fetch_add(1, rl);
            fail_ns.fetch_add(f, rl);
        }
        exact_n.fetch_add(1, rl);
        exact_ns.fetch_add(e, rl);
    }
};

// The slot pairs and the search records of the reduced graph, built once before the
// per-root trees (pairs: the lower slot of every reverse pair in ascending order, the
// order in which the reference's non-tree-edge scan meets them).
void setup_searches(mcbh_problem &P) {
    const Graph &g = P.rg;
    P.pair_first.clear();
    P.pair_first.reserve(g.slots() / 2);
    P.pair_ends.clear();
    P.pair_ends.reserve(g.slots() / 2);
    P.slot_pair.assign(g.slots(), 0);
    P.arcs.resize(g.slots());
    long long wmin = 1, wmax = 0;
    std::vector<long long> pair_w;
    pair_w.reserve(g.slots() / 2);
    for (size_t i = 0; i < g.slots(); i++) {
        P.arcs[i] = {g.cols[i], g.w[i]};
        wmin = std::min(wmin, (long long)g.w[i]);
        wmax = std::max(wmax, (long long)g.w[i]);
        if (i < g.rev[i]) pair_w.push_back(g.w[i]);
    }
    // a shortest path is simple: at most n - 1 edges, so no distance exceeds the sum
    // of the n - 1 heaviest edges, and no tentative one that plus the heaviest edge
    const size_t keep = std::min(pair_w.size(), (size_t)std::max(g.n - 1, 0));
    std::nth_element(pair_w.begin(), pair_w.begin() + keep, pair_w.end(), std::greater<long long>());
    long long path_bound = 0;
    for (size_t i = 0; i < keep; i++) path_bound += pair_w[i];
    P.fast_search_ok = wmin >= 1 && path_bound + wmax < 0x7fffffffLL;
    for (size_t i = 0; i < g.slots(); i++) {
        if (i < g.rev[i]) {
            P.slot_pair[i] = P.slot_pair[g.rev[i]] = (u32)P.pair_first.size();
            P.pair_first.push_back((u32)i);
            P.pair_ends.push_back(std::make_pair(g.rows[i], g.cols[i]));
        }
    }
}

// mcb/mcb_cycle_deg_two_remove.cpp:244-258: the candidates of every root (outs[t]
// for FVS index t, with its group map) into the rank order: roots in vertex-id
// order, each root's map in iteration order, each group in insertion order; then an
// unstable std::sort on total_length alone.  Fills the problem's candidate arrays
// and, with `lists`, its coordinate lists.
int collect_candidates(mcbh_problem *P, std::vector<RootOutput> &outs, bool lists, int threads) {
    mcbh_info &I = P->info;
    const int n = P->rg.n;
    struct Item {
        int weight;
        int tree;
        int local;
        int len;
    };
    // the list in that order, each root's part filled in parallel
    std::vector<int> root_of_rank;  // FVS roots in vertex-id order
    for (int vtx = 0; vtx < n; vtx++)
        if (P->fvs_array[vtx] >= 0) root_of_rank.push_back(P->fvs_array[vtx]);
    std::vector<size_t> base(root_of_rank.size() + 1, 0);
    for (size_t i = 0; i < root_of_rank.size(); i++) base[i + 1] = base[i] + outs[root_of_rank[i]].cands.size();
    const size_t K = base.back();
    if (K > 0xffffffffull) return MCBH_E_NOMEM;  // past the 32-bit index of the sort records
    std::vector<Item> items(K);
#pragma omp parallel for num_threads(threads) schedule(dynamic, 16)
    for (int64_t i = 0; i < (int64_t)root_of_rank.size(); i++) {
        const int t = root_of_rank[i];
        const RootOutput &o = outs[t];
        size_t k = base[i];
        for (auto it = o.groups.begin(); it != o.groups.end(); ++it)
            for (int loc = it->second.first; loc >= 0; loc = o.next[loc])
                items[k++] = {o.cands[loc].weight, t, loc, o.cands[loc].coord_len};
    }
    // std::sort on the weight alone: its permutation follows from the outcomes of
    // its comparisons, so sorting (weight, index) records gives the permutation
    // that sorting the candidates themselves gives; weight_sort gives that
    // permutation with the independent sub-ranges sorted in parallel
    std::vector<WeightKey> keys(K);
#pragma omp parallel for num_threads(threads) schedule(static)
    for (int64_t r = 0; r < (int64_t)K; r++) keys[r] = {items[r].weight, (u32)r};
    weight_sort(keys.data(), K, threads);
    P->c_root.resize(K);
    P->c_edge.resize(K);
    P->c_weight.resize(K);
    P->c_tree.resize(K);
    int64_t nnz = 0;
    if (lists) {
        P->c_off.resize(K + 1);
        P->c_off[0] = 0;
#pragma omp parallel for num_threads(threads) schedule(static)
        for (int64_t r = 0; r < (int64_t)K; r++) P->c_off[r + 1] = items[keys[r].index].len;
        for (size_t r = 0; r < K; r++) {
            nnz += P->c_off[r + 1];
            P->c_off[r + 1] = nnz;
        }
        P->c_coords.resize((size_t)nnz);
    }
#pragma omp parallel for num_threads(threads) schedule(static)
    for (int64_t r = 0; r < (int64_t)K; r++) {
        const Item &it = items[keys[r].index];
        const LocalCandidate &lc = outs[it.tree].cands[it.local];
        P->c_root[r] = (int)P->fvs_vertices[it.tree];
        P->c_edge[r] = lc.edge;
        P->c_weight[r] = lc.weight;
        P->c_tree[r] = it.tree;
        if (lists)
            std::memcpy(&P->c_coords[P->c_off[r]], &outs[it.tree].coords[lc.coord_begin],
                        sizeof(int) * (size_t)lc.coord_len);
    }
    I.num_candidates = (int64_t)K;
    I.cycle_nnz = nnz;
    return MCBH_OK;
}

// given_dist / given_pedge: a supplied tree for this root (or null), adopted after
// take_given_tree's checks; *given_taken says whether it was.
void process_root(const mcbh_problem &P, int tidx, TreeWorkspace &ws, RootOutput &out, bool want_lists,
                  int *tree_parent, u32 *lay_rows, u32 *lay_cols, int *lay_edge, u32 *lay_nodes,
                  SearchChoice &choice, const int32_t *given_dist = nullptr, const int32_t *given_pedge = nullptr,
                  bool *given_taken = nullptr, bool given_trusted = false) {
    const Graph &g = P.rg;
    const int n = g.n;
    const u32 src = P.fvs_vertices[tidx];
    ws.init(n, P.pair_first.size());
    std::vector<u32> tree_edges;
    tree_edges.reserve(n);
    bool fast_done = false;
    choice.result = -1;
    if (given_taken) *given_taken = false;
    if (given_dist && given_pedge && P.fast_search_ok && !lay_rows) {
        if (take_given_tree(P, src, ws, given_dist, given_pedge, tree_edges, given_trusted)) {
            fast_done = true;
            choice.try_fast = false;
            if (given_taken) *given_taken = true;
        } else {
            ws.init(n, P.pair_first.size());
            tree_edges.clear();
        }
    }
    if (!fast_done && choice.try_fast && P.fast_search_ok && !lay_rows) {
        const double t0 = now_s();
        fast_done = search_fast(P, src, ws, tree_edges);
        choice.fast_s = now_s() - t0;
        choice.result = fast_done ? 1 : 0;
        if (!fast_done) {
            ws.init(n, P.pair_first.size());
            tree_edges.clear();
        }
    }
    if (!fast_done) {
        const double t0 = now_s();
        if (P.fast_search_ok)
            search_exact<true>(P, src, ws, tree_edges);
        else
            search_exact<false>(P, src, ws, tree_edges);
        choice.exact_s = now_s() - t0;
    }
    VertexState *vs = ws.vs.data();
    // dijkstra::is_edge_cycle: accepted iff the two root paths meet only at the root
    // and contain no FVS vertex with a smaller id than the root.  Computed here per
    // vertex (vertices in settle order: parents first): the root child a vertex hangs
    // under, or kBlocked if its root path holds such an FVS vertex; -1 for the root
    // (which is never blocked: its id is not smaller than its own).
    constexpr int kBlocked = -2;
    std::vector<int> &branch = ws.tmp;
    branch.assign(n, -1);
    auto code_of = [&](u32 x) {
        const int p = vs[x].par;
        const int bp = ((u32)p == src) ? (int)x : branch[p];
        return (bp == kBlocked || (P.fvs_array[x] >= 0 && src > x)) ? kBlocked : bp;
    };
    if (!ws.pop_order.empty()) {
        for (u32 x : ws.pop_order)
            if (x != src) branch[x] = code_of(x);
    } else {
        // a supplied tree has no settle order: each vertex's chain up to the first
        // vertex already done, then down (distances fall strictly along a chain,
        // checked, so every chain ends)
        constexpr int kUnset = -3;
        branch.assign(n, kUnset);
        branch[src] = -1;
        std::vector<u32> &chain = ws.chain;
        for (int v = 0; v < n; v++) {
            chain.clear();
            for (u32 x = (u32)v; branch[x] == kUnset; x = (u32)vs[x].par) chain.push_back(x);
            for (size_t i = chain.size(); i-- > 0;) branch[chain[i]] = code_of(chain[i]);
        }
    }
    // dijkstra::compute_non_tree_edges (include/Dijkstra.h:129-149): its scan over the
    // slots in ascending order keeps, of every pair that holds no tree slot, the slot
    // met first, i.e. the lower one; the same sequence is the pairs without a tree
    // slot in order of their lower slot.
    for (u32 o : tree_edges) ws.pair_tree[P.slot_pair[o]] = 1;
    const size_t npairs = P.pair_first.size();
    for (size_t k = 0; k < npairs; k++) {
        if (ws.pair_tree[k]) continue;
        const u32 a = P.pair_ends[k].first, b = P.pair_ends[k].second;
        const int ba = branch[a], bb = branch[b];
        if (ba == kBlocked || bb == kBlocked) continue;
        const bool lca_root = (a == src) || (b == src) || (ba != bb);
        if (!lca_root) continue;
        const u32 off = P.pair_first[k];
        int weight = vs[a].dist + vs[b].dist + g.w[off];
        LocalCandidate lc;
        lc.edge = (int)off;
        lc.weight = weight;
        lc.coord_begin = (i64)out.coords.size();
        lc.coord_len = 0;
        if (want_lists) {
            size_t b0 = out.coords.size();
            if (P.edge_coord[off] >= 0) out.coords.push_back(P.edge_coord[off]);
            for (u32 x = a; x != src; x = (u32)vs[x].par) {
                int c = P.edge_coord[vs[x].pedge];
                if (c >= 0) out.coords.push_back(c);
            }
            for (u32 x = b; x != src; x = (u32)vs[x].par) {
                int c = P.edge_coord[vs[x].pedge];
                if (c >= 0) out.coords.push_back(c);
            }
            std::sort(out.coords.begin() + b0, out.coords.end());
            lc.coord_len = (int)(out.coords.size() - b0);
        }
        const int local = (int)out.cands.size();
        out.cands.push_back(lc);
        out.group(local, a, b);
    }
    if (tree_parent) {
        int *tp = tree_parent + (size_t)tidx * n;
        for (int v = 0; v < n; v++) tp[v] = vs[v].pedge;
        tp[src] = -1;
    }
    if (lay_rows) {
        // dijkstra::fill_tree_edges: (offset, level) items, root first, then tree
        // edges in pop order; std::sort by level only.
        ws.level.assign(n, -1);
        ws.level[src] = 0;
        for (u32 x : ws.pop_order)
            if (x != src) ws.level[x] = ws.level[vs[x].par] + 1;
        ws.lv.clear();
        ws.lv.push_back({-1, 0});
        for (u32 o : tree_edges) ws.lv.push_back({(int)o, ws.level[g.cols[o]]});
        std::sort(ws.lv.begin(), ws.lv.end(), LevelLess());
        u32 *R = lay_rows + (size_t)tidx * (n + 1);
        u32 *C = lay_cols + (size_t)tidx * n;
        int *E = lay_edge + (size_t)tidx * n;
        u32 *NI = lay_nodes + (size_t)tidx * n;
        for (int i = 0; i <= n; i++) R[i] = 0;
        for (size_t i = 0; i < ws.lv.size(); i++) {
            R[ws.lv[i].level]++;
            if (ws.lv[i].offset == -1) {
                NI[src] = (u32)i;
                C[i] = 0xFFFFFFFFu;
                E[i] = -1;
            } else {
                u32 r = g.rows[ws.lv[i].offset], c = g.cols[ws.lv[i].offset];
                NI[c] = (u32)i;
                C[i] = NI[r];
                E[i] = ws.lv[i].offset;
            }
        }
        u32 prev = 0;
        for (int i = 0; i <= n; i++) {
            u32 t = R[i];
            R[i] = prev;
            prev += t;
        }
    }
}

}  // namespace

// ===========================================================================
// C ABI
extern "C" {

static int read_mtx(const char *path, int &nodes, std::vector<int> &u, std::vector<int> &v,
                    std::vector<int> &w) {
    FILE *f = fopen(path, "r");
    if (!f) return MCBH_E_IO;
    char line[4096];
    if (!fgets(line, sizeof line, f)) {
        fclose(f);
        return MCBH_E_IO;
    }
    // banner: %%MatrixMarket matrix coordinate <integer|real> <symmetric|general>
    // (the combinations include/FileReader.h:39-44 accepts)
    std::string b(line);
    for (auto &ch : b) ch = (char)tolower(ch);
    if (b.compare(0, 14, "%%matrixmarket") != 0) {
        fclose(f);
        return MCBH_E_FORMAT;
    }
    bool ok = b.find("matrix") != std::string::npos && b.find("coordinate") != std::string::npos &&
              (b.find("integer") != std::string::npos || b.find("real") != std::string::npos) &&
              (b.find("symmetric") != std::string::npos || b.find("general") != std::string::npos);
    if (!ok) {
        fclose(f);
        return MCBH_E_FORMAT;
    }
    long M = 0, Ncol = 0, E = 0;
    while (fgets(line, sizeof line, f)) {
        if (line[0] == '%') continue;
        if (sscanf(line, "%ld %ld %ld", &M, &Ncol, &E) == 3) break;
    }
    if (M <= 0 || E < 0) {
        fclose(f);
        return MCBH_E_IO;
    }
    nodes = (int)M;
    u.resize(E);
    v.resize(E);
    w.resize(E);
    for (long i = 0; i < E; i++) {
        long a, c;
        double wt;
        if (fscanf(f, "%ld %ld %lf", &a, &c, &wt) != 3) {
            fclose(f);
            return MCBH_E_IO;
        }
        if (a < 1 || c < 1 || a > M || c > M) {
            fclose(f);
            return MCBH_E_IO;
        }
        u[i] = (int)(a - 1);
        v[i] = (int)(c - 1);
        w[i] = (int)wt;  // fscanf("%d") of the reference truncates the same way
    }
    fclose(f);
    return MCBH_OK;
}

int mcbh_problem_from_edges(int32_t nodes, int64_t m, const int32_t *u, const int32_t *v, const int32_t *w,
                            mcbh_problem **out) {
    if (!out || nodes <= 0 || m < 0 || (m > 0 && (!u || !v || !w))) return MCBH_E_ARG;
    *out = nullptr;
    mcbh_problem *P = new (std::nothrow) mcbh_problem();
    if (!P) return MCBH_E_NOMEM;
    double t0 = now_s();
    P->in.n = nodes;
    P->m_in = m;
    std::vector<EdgeSlot> s;
    try {
        s.reserve(2 * (size_t)m);
    } catch (...) {
        delete P;
        return MCBH_E_NOMEM;
    }
    for (int64_t i = 0; i < m; i++) {
        if (u[i] < 0 || v[i] < 0 || u[i] >= nodes || v[i] >= nodes) {
            delete P;
            return MCBH_E_ARG;
        }
        // csr_graph::insert(a, b, w, false) pushes (a,b) then (b,a)
        s.push_back({(u32)u[i], (u32)v[i], w[i], -1, -1, 0});
        s.push_back({(u32)v[i], (u32)u[i], w[i], -1, -1, 0});
        P->total_weight_input += w[i];
    }
    finish_simple_csr(P->in, s);
    P->info.t_read = now_s() - t0;
    *out = P;
    return MCBH_OK;
}

int mcbh_problem_from_mtx(const char *path, mcbh_problem **out) {
    if (!path || !out) return MCBH_E_ARG;
    double t0 = now_s();
    int nodes = 0;
    std::vector<int> u, v, w;
    int rc = read_mtx(path, nodes, u, v, w);
    if (rc) return rc;
    rc = mcbh_problem_from_edges(nodes, (int64_t)u.size(), u.data(), v.data(), w.data(), out);
    if (rc == MCBH_OK) (*out)->info.t_read = now_s() - t0;
    return rc;
}

int64_t mcbh_read_mtx(const char *path, int32_t *nodes, int64_t cap, int32_t *u, int32_t *v, int32_t *w) {
    if (!path || !nodes) return MCBH_E_ARG;
    int n = 0;
    std::vector<int> a, b, c;
    const int rc = read_mtx(path, n, a, b, c);
    if (rc) return rc;
    *nodes = n;
    const int64_t m = (int64_t)a.size();
    if (u) {
        if (cap < m || !v || !w) return MCBH_E_ARG;
        std::memcpy(u, a.data(), sizeof(int32_t) * (size_t)m);
        std::memcpy(v, b.data(), sizeof(int32_t) * (size_t)m);
        std::memcpy(w, c.data(), sizeof(int32_t) * (size_t)m);
    }
    return m;
}

void mcbh_problem_free(mcbh_problem *p) { delete p; }

static int prepare_impl(mcbh_problem *P, const mcbh_options *opt, const mcbh_tree_source *source) {
    if (!P || !opt) return MCBH_E_ARG;
    if (P->prepared || P->attempted) return MCBH_E_STATE;
    P->attempted = true;
    mcbh_info &I = P->info;
    I.nodes = P->in.n;
    I.edges2 = (int64_t)P->in.slots();
    I.total_weight_input = P->total_weight_input;
    try {
        // mcb/mcb_cycle_deg_two_remove.cpp:104-113: a graph whose every vertex has
        // degree two is one cycle.
        int deg2 = 0;
        for (int i = 0; i < P->in.n; i++) deg2 += P->in.deg[i] == 2;
        if (opt->contract_chains && deg2 == P->in.n) {
            P->single_cycle = true;
            I.single_cycle = 1;
            I.nodes_removed = P->in.n - 1;
            I.fvs_size = 1;
            I.num_coords = 1;
            I.num_candidates = 1;
            P->prepared = true;
            return MCBH_OK;
        }
        double t0 = now_s();
        if (opt->contract_chains) {
            ChainResult cr = mark_degree_two_chains(P->in);
            if (cr.bad) return MCBH_E_GRAPH;
            int removed = 0;
            for (auto &ch : cr.chains) removed += (int)ch.size() - 1;
            P->nodes_removed = removed;
            P->source_vertex = cr.src;
            build_reduced(*P, &cr);
        } else {
            P->nodes_removed = 0;
            P->source_vertex = 0;  // mcb/mcb_cycle.cpp:110
            build_reduced(*P, nullptr);
        }
        I.nodes_removed = P->nodes_removed;
        I.reduced_nodes = P->rg.n;
        I.reduced_edges2 = (int64_t)P->rg.slots();
        I.source_vertex = P->source_vertex;
        I.t_reduce = now_s() - t0;

        t0 = now_s();
        compute_fvs(*P);
        I.fvs_size = (int)P->fvs_vertices.size();
        I.t_fvs = now_s() - t0;

        t0 = now_s();
        if (!spanning_tree(*P, P->source_vertex)) return MCBH_E_GRAPH;
        I.num_coords = (int)P->coord_edges.size();
        I.t_spanning = now_s() - t0;

        setup_searches(*P);
        if (opt->structure_only) {
            // stop before the per-root trees: the candidates come from
            // mcbh_rank_candidates (a device candidate generation)
            P->structure_only = true;
            P->prepared = true;
            return MCBH_OK;
        }
        t0 = now_s();
        const int F = I.fvs_size;
        const int n = P->rg.n;
        if (opt->keep_trees) P->tree_parent.assign((size_t)F * n, -1);
        if (opt->ref_layout) {
            P->lay_rows.assign((size_t)F * (n + 1), 0);
            P->lay_cols.assign((size_t)F * n, 0);
            P->lay_edge.assign((size_t)F * n, -1);
            P->lay_nodes.assign((size_t)F * n, 0);
        }
        std::vector<RootOutput> outs(F);
        int threads = opt->threads > 0 ? opt->threads : omp_get_max_threads();
        bool lists = opt->cycle_lists != 0;
        SearchPolicy policy;
        I.trees_supplied = 0;
        const bool supplied = source && source->trees && P->fast_search_ok && !opt->ref_layout && F > 0;
        if (supplied) {
            // trees from the supplier, `chunk` roots per call; each adopted after
            // take_given_tree's checks, the others searched here
            const Graph &g = P->rg;
            if (source->begin && source->begin(source->ctx, g.n, (int64_t)g.slots(), g.ro.data(), g.cols.data(),
                                               g.w.data(), g.rev.data()) != 0)
                return MCBH_E_SUPPLIER;
            const int chunk = source->chunk > 0 ? std::min(source->chunk, F) : F;
            std::vector<int32_t> gd((size_t)chunk * n), gp((size_t)chunk * n);
            std::vector<uint8_t> gt((size_t)chunk);
            std::vector<TreeWorkspace> wss((size_t)threads);
            std::atomic<int> taken_count{0};
            for (int t0 = 0; t0 < F; t0 += chunk) {
                const int cnt = std::min(chunk, F - t0);
                std::fill(gt.begin(), gt.begin() + cnt, (uint8_t)1);
                if (source->trees(source->ctx, &P->fvs_vertices[(size_t)t0], cnt, gd.data(), gp.data(), gt.data()) != 0)
                    return MCBH_E_SUPPLIER;
#pragma omp parallel for num_threads(threads) schedule(dynamic, 1)
                for (int i = 0; i < cnt; i++) {
                    const int t = t0 + i;
                    SearchChoice choice;
                    choice.try_fast = policy.want_fast(t);
                    bool taken = false;
                    const bool offer = gt[(size_t)i] == 0;
                    process_root(*P, t, wss[(size_t)omp_get_thread_num()], outs[t], lists,
                                 opt->keep_trees ? P->tree_parent.data() : nullptr, nullptr, nullptr, nullptr, nullptr,
                                 choice, offer ? &gd[(size_t)i * n] : nullptr, offer ? &gp[(size_t)i * n] : nullptr,
                                 &taken, source->trust != 0);
                    if (taken)
                        taken_count.fetch_add(1, std::memory_order_relaxed);
                    else
                        policy.record(choice);
                }
            }
            I.trees_supplied = taken_count.load();
        } else {
#pragma omp parallel num_threads(threads)
            {
                TreeWorkspace ws;
#pragma omp for schedule(dynamic, 1)
                for (int t = 0; t < F; t++) {
                    SearchChoice choice;
                    choice.try_fast = policy.want_fast(t);
                    process_root(*P, t, ws, outs[t], lists, opt->keep_trees ? P->tree_parent.data() : nullptr,
                                 opt->ref_layout ? P->lay_rows.data() : nullptr,
                                 opt->ref_layout ? P->lay_cols.data() : nullptr,
                                 opt->ref_layout ? P->lay_edge.data() : nullptr,
                                 opt->ref_layout ? P->lay_nodes.data() : nullptr, choice);
                    policy.record(choice);
                }
            }
        }
        I.t_trees = now_s() - t0;

        t0 = now_s();
        const int rc = collect_candidates(P, outs, lists, threads);
        if (rc != MCBH_OK) return rc;
        I.t_collect = now_s() - t0;
    } catch (const std::bad_alloc &) {
        return MCBH_E_NOMEM;
    }
    P->prepared = true;
    return MCBH_OK;
}

int mcbh_prepare(mcbh_problem *P, const mcbh_options *opt) { return prepare_impl(P, opt, nullptr); }

int mcbh_prepare_with_trees(mcbh_problem *P, const mcbh_options *opt, const mcbh_tree_source *source) {
    if (!source || !source->trees) return MCBH_E_ARG;
    return prepare_impl(P, opt, source);
}

int mcbh_search_trees(const mcbh_problem *P, const int32_t *trees, int32_t count, int threads, int32_t *dist,
                      int32_t *parent_slot) {
    if (!P || count < 0 || (count > 0 && (!trees || !dist || !parent_slot))) return MCBH_E_ARG;
    if (!P->prepared || P->single_cycle || P->arcs.empty()) return MCBH_E_STATE;
    const int F = (int)P->fvs_vertices.size();
    for (int32_t i = 0; i < count; i++)
        if (trees[i] < 0 || trees[i] >= F) return MCBH_E_ARG;
    const int n = P->rg.n;
    if (threads <= 0) threads = omp_get_max_threads();
    try {
#pragma omp parallel num_threads(threads)
        {
            TreeWorkspace ws;
            std::vector<u32> tree_edges;
#pragma omp for schedule(dynamic, 1)
            for (int32_t i = 0; i < count; i++) {
                const u32 src = P->fvs_vertices[(size_t)trees[i]];
                ws.init(n, 0);
                tree_edges.clear();
                if (P->fast_search_ok)
                    search_exact<true>(*P, src, ws, tree_edges);
                else
                    search_exact<false>(*P, src, ws, tree_edges);
                int32_t *d = dist + (size_t)i * n, *ps = parent_slot + (size_t)i * n;
                for (int v = 0; v < n; v++) {
                    d[v] = ws.vs[v].dist;
                    ps[v] = (u32)v == src ? -1 : ws.vs[v].pedge;
                }
            }
        }
    } catch (const std::bad_alloc &) {
        return MCBH_E_NOMEM;
    }
    return MCBH_OK;
}

int mcbh_get_pairs(const mcbh_problem *P, uint32_t *pair_slot) {
    if (!P || !pair_slot) return MCBH_E_ARG;
    if (!P->prepared || P->single_cycle || P->pair_first.size() * 2 != P->rg.slots()) return MCBH_E_STATE;
    std::memcpy(pair_slot, P->pair_first.data(), sizeof(uint32_t) * P->pair_first.size());
    return MCBH_OK;
}

int mcbh_rank_candidates(mcbh_problem *P, const int64_t *tree_offsets, const uint32_t *pair_index,
                         const int32_t *weight, int threads) {
    if (!P || !tree_offsets) return MCBH_E_ARG;
    if (!P->prepared || !P->structure_only || P->ranked) return MCBH_E_STATE;
    const int F = (int)P->fvs_vertices.size();
    const int64_t total = tree_offsets[F];
    if (tree_offsets[0] != 0 || total < 0 || (total > 0 && (!pair_index || !weight))) return MCBH_E_ARG;
    for (int t = 0; t < F; t++)
        if (tree_offsets[t + 1] < tree_offsets[t]) return MCBH_E_ARG;
    const int64_t npairs = (int64_t)P->pair_first.size();
    if (threads <= 0) threads = omp_get_max_threads();
    const double t0 = now_s();
    try {
        std::vector<RootOutput> outs((size_t)F);
        std::atomic<int> bad{0};
#pragma omp parallel for num_threads(threads) schedule(dynamic, 16)
        for (int t = 0; t < F; t++) {
            RootOutput &o = outs[(size_t)t];
            const int64_t b = tree_offsets[t], e = tree_offsets[t + 1];
            o.cands.reserve((size_t)(e - b));
            o.next.reserve((size_t)(e - b));
            int64_t prev = -1;
            for (int64_t i = b; i < e; i++) {
                const int64_t k = pair_index[i];
                if (k <= prev || k >= npairs) {  // each root's pairs ascending, in range
                    bad.store(1, std::memory_order_relaxed);
                    break;
                }
                prev = k;
                LocalCandidate lc;
                lc.edge = (int)P->pair_first[(size_t)k];
                lc.weight = weight[i];
                lc.coord_begin = 0;
                lc.coord_len = 0;
                const int local = (int)o.cands.size();
                o.cands.push_back(lc);
                o.group(local, P->pair_ends[(size_t)k].first, P->pair_ends[(size_t)k].second);
            }
        }
        if (bad.load()) return MCBH_E_ARG;
        const int rc = collect_candidates(P, outs, false, threads);
        if (rc != MCBH_OK) return rc;
    } catch (const std::bad_alloc &) {
        return MCBH_E_NOMEM;
    }
    P->ranked = true;
    P->info.t_collect = now_s() - t0;
    return MCBH_OK;
}

int mcbh_prepare_many(mcbh_problem **ps, int64_t count, const mcbh_options *opt, int32_t *status) {
    if (count < 0 || (count > 0 && (!ps || !opt))) return MCBH_E_ARG;
    mcbh_options one = *opt;
    one.threads = 1;
    const int threads = opt->threads > 0 ? opt->threads : omp_get_max_threads();
    // the largest problems first, so that the last ones to finish are small
    std::vector<int64_t> order((size_t)count);
    for (int64_t i = 0; i < count; i++) order[(size_t)i] = i;
    auto size_of = [&](int64_t i) { return ps[i] ? (int64_t)ps[i]->in.slots() : 0; };
    std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return size_of(a) > size_of(b); });
    std::vector<int> st((size_t)count, MCBH_OK);
#pragma omp parallel for num_threads(threads) schedule(dynamic, 1)
    for (int64_t k = 0; k < count; k++) {
        const int64_t i = order[(size_t)k];
        st[(size_t)i] = ps[i] ? mcbh_prepare(ps[i], &one) : MCBH_E_ARG;
    }
    int first = MCBH_OK;
    for (int64_t i = 0; i < count; i++) {
        if (status) status[i] = st[(size_t)i];
        if (first == MCBH_OK) first = st[(size_t)i];
    }
    return first;
}

int mcbh_gf2_rank(const mcbh_problem *p, const int64_t *ranks, int64_t count, int threads, int64_t *rank_out) {
    if (!p || !rank_out || count < 0 || (count > 0 && !ranks)) return MCBH_E_ARG;
    if (!p->prepared || p->single_cycle || p->c_off.empty()) return MCBH_E_STATE;
    const int64_t K = (int64_t)p->c_weight.size();
    const int64_t N = (int64_t)p->coord_edges.size();
    for (int64_t i = 0; i < count; i++)
        if (ranks[i] < 0 || ranks[i] >= K) return MCBH_E_ARG;
    if (threads <= 0) threads = omp_get_max_threads();
    const int64_t W = (N + 63) / 64;
    try {
        // one bit row per selected cycle: its coordinates (the cycle vector of
        // include/cycles.h:144-195 over the N coordinates)
        std::vector<u64> M((size_t)(count * W), 0);
#pragma omp parallel for num_threads(threads) schedule(static)
        for (int64_t i = 0; i < count; i++) {
            u64 *row = &M[(size_t)(i * W)];
            for (int64_t k = p->c_off[ranks[i]]; k < p->c_off[ranks[i] + 1]; k++) {
                const int c = p->c_coords[(size_t)k];
                row[c >> 6] ^= 1ull << (c & 63);
            }
        }
        // Gaussian elimination over GF(2), column by column: the first remaining row
        // with the column's bit becomes the pivot and is XORed into every later row
        // that has the bit (only the words from the column's word on change)
        int64_t rank = 0;
        for (int64_t col = 0; col < N && rank < count; col++) {
            const int64_t w = col >> 6;
            const u64 bit = 1ull << (col & 63);
            int64_t piv = -1;
            for (int64_t r = rank; r < count; r++)
                if (M[(size_t)(r * W + w)] & bit) {
                    piv = r;
                    break;
                }
            if (piv < 0) continue;
            if (piv != rank)
                std::swap_ranges(M.begin() + (size_t)(piv * W + w), M.begin() + (size_t)((piv + 1) * W),
                                 M.begin() + (size_t)(rank * W + w));
            const u64 *prow = &M[(size_t)(rank * W)];
#pragma omp parallel for num_threads(threads) schedule(static) if ((count - rank) * (W - w) > 65536)
            for (int64_t r = rank + 1; r < count; r++) {
                u64 *row = &M[(size_t)(r * W)];
                if (row[w] & bit)
                    for (int64_t x = w; x < W; x++) row[x] ^= prow[x];
            }
            rank++;
        }
        *rank_out = rank;
    } catch (const std::bad_alloc &) {
        return MCBH_E_NOMEM;
    }
    return MCBH_OK;
}

int mcbh_get_info(const mcbh_problem *p, mcbh_info *info) {
    if (!p || !info) return MCBH_E_ARG;
    *info = p->info;
    return MCBH_OK;
}

#define NEED_PREPARED(p)                                     \
    do {                                                     \
        if (!(p)) return MCBH_E_ARG;                         \
        if (!(p)->prepared || (p)->single_cycle) return MCBH_E_STATE; \
    } while (0)

int mcbh_get_reduced_graph(const mcbh_problem *p, uint32_t *rows, uint32_t *cols, int32_t *weights,
                           uint32_t *reverse_edge, uint32_t *row_offsets) {
    NEED_PREPARED(p);
    const Graph &g = p->rg;
    if (rows) std::memcpy(rows, g.rows.data(), g.slots() * 4);
    if (cols) std::memcpy(cols, g.cols.data(), g.slots() * 4);
    if (weights) std::memcpy(weights, g.w.data(), g.slots() * 4);
    if (reverse_edge) std::memcpy(reverse_edge, g.rev.data(), g.slots() * 4);
    if (row_offsets) std::memcpy(row_offsets, g.ro.data(), (g.n + 1) * 4);
    return MCBH_OK;
}

int mcbh_get_fvs(const mcbh_problem *p, int32_t *fvs_array, uint32_t *fvs_vertices) {
    NEED_PREPARED(p);
    if (fvs_array) std::memcpy(fvs_array, p->fvs_array.data(), p->fvs_array.size() * 4);
    if (fvs_vertices) std::memcpy(fvs_vertices, p->fvs_vertices.data(), p->fvs_vertices.size() * 4);
    return MCBH_OK;
}

int mcbh_get_vertex_map(const mcbh_problem *p, int32_t *input_vertex) {
    NEED_PREPARED(p);
    if (input_vertex) std::memcpy(input_vertex, p->r_vertex.data(), p->r_vertex.size() * 4);
    return MCBH_OK;
}

int mcbh_get_coords(const mcbh_problem *p, uint32_t *coord_edges, int32_t *edge_coord) {
    NEED_PREPARED(p);
    if (coord_edges) std::memcpy(coord_edges, p->coord_edges.data(), p->coord_edges.size() * 4);
    if (edge_coord) std::memcpy(edge_coord, p->edge_coord.data(), p->edge_coord.size() * 4);
    return MCBH_OK;
}

int mcbh_get_candidates(const mcbh_problem *p, int32_t *root, int32_t *edge_offset, int32_t *weight,
                        int32_t *tree) {
    NEED_PREPARED(p);
    size_t K = p->c_root.size();
    if (root) std::memcpy(root, p->c_root.data(), K * 4);
    if (edge_offset) std::memcpy(edge_offset, p->c_edge.data(), K * 4);
    if (weight) std::memcpy(weight, p->c_weight.data(), K * 4);
    if (tree) std::memcpy(tree, p->c_tree.data(), K * 4);
    return MCBH_OK;
}

int mcbh_get_cycle_lists(const mcbh_problem *p, int64_t *offsets, int32_t *coords) {
    NEED_PREPARED(p);
    if (p->c_off.empty() && !p->c_root.empty()) return MCBH_E_STATE;
    if (p->c_root.empty()) {
        if (offsets) offsets[0] = 0;
        return MCBH_OK;
    }
    if (offsets) std::memcpy(offsets, p->c_off.data(), p->c_off.size() * 8);
    if (coords) std::memcpy(coords, p->c_coords.data(), p->c_coords.size() * 4);
    return MCBH_OK;
}

int mcbh_get_tree_parents(const mcbh_problem *p, int32_t *parent_edge) {
    NEED_PREPARED(p);
    if (p->tree_parent.empty() && p->info.fvs_size > 0) return MCBH_E_STATE;
    if (parent_edge) std::memcpy(parent_edge, p->tree_parent.data(), p->tree_parent.size() * 4);
    return MCBH_OK;
}

int mcbh_get_ref_layout(const mcbh_problem *p, uint32_t *level_offsets, uint32_t *parent_pos,
                        int32_t *edge_offset, uint32_t *nodes_index) {
    NEED_PREPARED(p);
    if (p->lay_rows.empty() && p->info.fvs_size > 0) return MCBH_E_STATE;
    if (level_offsets) std::memcpy(level_offsets, p->lay_rows.data(), p->lay_rows.size() * 4);
    if (parent_pos) std::memcpy(parent_pos, p->lay_cols.data(), p->lay_cols.size() * 4);
    if (edge_offset) std::memcpy(edge_offset, p->lay_edge.data(), p->lay_edge.size() * 4);
    if (nodes_index) std::memcpy(nodes_index, p->lay_nodes.data(), p->lay_nodes.size() * 4);
    return MCBH_OK;
}

// ---------------------------------------------------------------------------
// Seeded generators.  splitmix64 (Steele, Lea, Flood 2014; constants as published
// by Vigna) drives every draw, so the same seed gives the same graph on any host.
struct Rng {
    uint64_t s;
    uint64_t next() {
        uint64_t z = (s += 0x9e3779b97f4a7c15ULL);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
        return z ^ (z >> 31);
    }
    uint64_t below(uint64_t n) { return next() % n; }
    double unit() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

int64_t mcbh_gen_grid(int32_t r, int32_t c, int32_t wlo, int32_t whi, uint64_t seed, int32_t *u, int32_t *v,
                      int32_t *w) {
    if (r <= 0 || c <= 0 || whi < wlo) return MCBH_E_ARG;
    int64_t m = (int64_t)r * (c - 1) + (int64_t)(r - 1) * c;
    if (!u) return m;
    Rng g{seed};
    int64_t k = 0;
    for (int32_t i = 0; i < r; i++)
        for (int32_t j = 0; j < c; j++) {
            int32_t id = i * c + j;
            if (j + 1 < c) {
                u[k] = id;
                v[k] = id + 1;
                w[k] = wlo + (int32_t)g.below((uint64_t)(whi - wlo + 1));
                k++;
            }
            if (i + 1 < r) {
                u[k] = id;
                v[k] = id + c;
                w[k] = wlo + (int32_t)g.below((uint64_t)(whi - wlo + 1));
                k++;
            }
        }
    return k;
}

int64_t mcbh_gen_random(int32_t n, int64_t m, int32_t wlo, int32_t whi, uint64_t seed, int32_t *u, int32_t *v,
                        int32_t *w) {
    if (n <= 1 || m < n - 1 || whi < wlo) return MCBH_E_ARG;
    if (m > (int64_t)n * (n - 1) / 2) return MCBH_E_ARG;
    if (!u) return m;
    Rng g{seed};
    std::vector<int32_t> perm(n);
    for (int32_t i = 0; i < n; i++) perm[i] = i;
    for (int32_t i = n - 1; i > 0; i--) std::swap(perm[i], perm[g.below((uint64_t)i + 1)]);
    std::unordered_set<uint64_t> seen;
    seen.reserve((size_t)m * 2);
    int64_t k = 0;
    auto key = [](int32_t a, int32_t b) {
        return ((uint64_t)(uint32_t)std::min(a, b) << 32) | (uint32_t)std::max(a, b);
    };
    for (int32_t i = 1; i < n; i++) {
        int32_t a = perm[i], b = perm[g.below((uint64_t)i)];
        u[k] = a;
        v[k] = b;
        w[k] = wlo + (int32_t)g.below((uint64_t)(whi - wlo + 1));
        seen.insert(key(a, b));
        k++;
    }
    while (k < m) {
        int32_t a = (int32_t)g.below((uint64_t)n), b = (int32_t)g.below((uint64_t)n);
        if (a == b || seen.count(key(a, b))) continue;
        seen.insert(key(a, b));
        u[k] = a;
        v[k] = b;
        w[k] = wlo + (int32_t)g.below((uint64_t)(whi - wlo + 1));
        k++;
    }
    return k;
}

int64_t mcbh_gen_rgg(int32_t n, int32_t kk, uint64_t seed, int32_t *u, int32_t *v, int32_t *w) {
    if (n <= 1 || kk <= 0 || kk >= n) return MCBH_E_ARG;
    Rng g{seed};
    std::vector<double> x(n), y(n);
    for (int32_t i = 0; i < n; i++) {
        x[i] = g.unit();
        y[i] = g.unit();
    }
    // bucket grid with ~2 points per cell
    int G = std::max(1, (int)std::sqrt((double)n / 2.0));
    std::vector<std::vector<int32_t>> cell((size_t)G * G);
    auto cid = [&](double a) { return std::min(G - 1, (int)(a * G)); };
    for (int32_t i = 0; i < n; i++) cell[(size_t)cid(y[i]) * G + cid(x[i])].push_back(i);
    std::unordered_set<uint64_t> seen;
    std::vector<std::pair<int32_t, int32_t>> edges;
    auto key = [](int32_t a, int32_t b) {
        return ((uint64_t)(uint32_t)std::min(a, b) << 32) | (uint32_t)std::max(a, b);
    };
    auto add = [&](int32_t a, int32_t b) {
        if (a == b) return;
        if (seen.insert(key(a, b)).second) edges.push_back({std::min(a, b), std::max(a, b)});
    };
    // k nearest neighbours by expanding rings (exact: a ring stops only when the
    // k-th distance found is within the ring's guaranteed radius)
    std::vector<std::pair<double, int32_t>> best;
    for (int32_t i = 0; i < n; i++) {
        int cx = cid(x[i]), cy = cid(y[i]);
        best.clear();
        for (int ring = 0;; ring++) {
            for (int dy = -ring; dy <= ring; dy++)
                for (int dx = -ring; dx <= ring; dx++) {
                    if (std::max(std::abs(dx), std::abs(dy)) != ring) continue;
                    int gx = cx + dx, gy = cy + dy;
                    if (gx < 0 || gy < 0 || gx >= G || gy >= G) continue;
                    for (int32_t j : cell[(size_t)gy * G + gx]) {
                        if (j == i) continue;
                        double d = (x[i] - x[j]) * (x[i] - x[j]) + (y[i] - y[j]) * (y[i] - y[j]);
                        best.push_back({d, j});
                    }
                }
            if ((int)best.size() >= kk) {
                std::nth_element(best.begin(), best.begin() + (kk - 1), best.end());
                double r = (double)ring / G;
                if (best[kk - 1].first <= r * r || ring > G) break;
            }
            if (ring > G) break;
        }
        std::sort(best.begin(), best.end());
        for (int t = 0; t < kk && t < (int)best.size(); t++) add(i, best[t].second);
    }
    // connect components: each later component to its nearest outside point
    std::vector<int> comp(n, -1);
    {
        std::vector<std::vector<int32_t>> adj(n);
        for (auto &e : edges) {
            adj[e.first].push_back(e.second);
            adj[e.second].push_back(e.first);
        }
        int nc = 0;
        std::vector<int32_t> stk;
        for (int32_t s = 0; s < n; s++) {
            if (comp[s] >= 0) continue;
            comp[s] = nc;
            stk.push_back(s);
            while (!stk.empty()) {
                int32_t a = stk.back();
                stk.pop_back();
                for (int32_t b : adj[a])
                    if (comp[b] < 0) {
                        comp[b] = nc;
                        stk.push_back(b);
                    }
            }
            nc++;
        }
        if (nc > 1) {
            DSU d(nc);
            for (int32_t i = 0; i < n; i++) {
                if (d.find(comp[i]) == d.find(0)) continue;
                // nearest point in another (merged) component, brute force (rare)
                double bd = 1e300;
                int32_t bj = -1;
                for (int32_t j = 0; j < n; j++) {
                    if (d.find(comp[j]) == d.find(comp[i])) continue;
                    double dd = (x[i] - x[j]) * (x[i] - x[j]) + (y[i] - y[j]) * (y[i] - y[j]);
                    if (dd < bd) {
                        bd = dd;
                        bj = j;
                    }
                }
                if (bj >= 0) {
                    add(i, bj);
                    d.p[d.find(comp[i])] = d.find(comp[bj]);
                }
            }
        }
    }
    int64_t m = (int64_t)edges.size();
    if (!u) return m;
    for (int64_t k = 0; k < m; k++) {
        int32_t a = edges[k].first, b = edges[k].second;
        double len = std::sqrt((x[a] - x[b]) * (x[a] - x[b]) + (y[a] - y[b]) * (y[a] - y[b]));
        u[k] = a;
        v[k] = b;
        w[k] = std::max(1, (int32_t)std::lround(1000.0 * len));
    }
    return m;
}

}  // extern "C"

namespace {

struct EdgeList {
    std::vector<int32_t> u, v, w;
    int32_t nodes = 0;
    void add(int32_t a, int32_t b, int32_t wt) {
        u.push_back(a);
        v.push_back(b);
        w.push_back(wt);
    }
};

int64_t emit(const EdgeList &g, int32_t *u, int32_t *v, int32_t *w, int32_t *nodes) {
    if (nodes) *nodes = g.nodes;
    const int64_t m = (int64_t)g.u.size();
    if (!u) return m;
    std::memcpy(u, g.u.data(), sizeof(int32_t) * (size_t)m);
    std::memcpy(v, g.v.data(), sizeof(int32_t) * (size_t)m);
    std::memcpy(w, g.w.data(), sizeof(int32_t) * (size_t)m);
    return m;
}

}  // namespace

extern "C" {

int64_t mcbh_gen_planar_chains(int32_t points, int32_t delete_pct, int32_t chain_pct, int32_t chain_max, int32_t wlo,
                               int32_t whi, uint64_t seed, int32_t *u, int32_t *v, int32_t *w, int32_t *nodes) {
    if (points < 4 || delete_pct < 0 || delete_pct >= 100 || chain_pct < 0 || chain_pct > 100 || chain_max < 1 ||
        whi < wlo)
        return MCBH_E_ARG;
    Rng g{seed};
    // triangulated grid: r x c points, right and down edges, one diagonal per cell
    // in a random direction (a planar triangulation of a jittered grid)
    const int32_t r = std::max(2, (int32_t)std::lround(std::sqrt((double)points)));
    const int32_t c = std::max(2, (points + r - 1) / r);
    std::vector<std::pair<int32_t, int32_t>> base;
    base.reserve((size_t)3 * r * c);
    for (int32_t i = 0; i < r; i++)
        for (int32_t j = 0; j < c; j++) {
            const int32_t id = i * c + j;
            if (j + 1 < c) base.push_back({id, id + 1});
            if (i + 1 < r) base.push_back({id, id + c});
            if (i + 1 < r && j + 1 < c) {
                if (g.next() & 1)
                    base.push_back({id, id + c + 1});
                else
                    base.push_back({id + 1, id + c});
            }
        }
    const int32_t n0 = r * c;
    // delete delete_pct% of the edges, keeping a random spanning tree
    const size_t E = base.size();
    std::vector<size_t> order(E);
    for (size_t i = 0; i < E; i++) order[i] = i;
    for (size_t i = E - 1; i > 0; i--) std::swap(order[i], order[g.below((uint64_t)i + 1)]);
    std::vector<char> keep(E, 0);
    DSU d(n0);
    size_t kept = 0;
    for (size_t t = 0; t < E; t++) {
        const auto &e = base[order[t]];
        const int a = d.find(e.first), b = d.find(e.second);
        if (a != b) {
            d.p[a] = b;
            keep[order[t]] = 1;
            kept++;
        }
    }
    const size_t target = (size_t)std::llround((double)E * (100 - delete_pct) / 100.0);
    for (size_t t = 0; t < E && kept < target; t++)
        if (!keep[order[t]]) {
            keep[order[t]] = 1;
            kept++;
        }
    // subdivide each kept edge with probability chain_pct% into a chain of
    // 1..chain_max extra vertices; every final edge gets its own weight
    EdgeList out;
    out.nodes = n0;
    for (size_t i = 0; i < E; i++) {
        if (!keep[i]) continue;
        int32_t a = base[i].first;
        const int32_t b = base[i].second;
        if ((int32_t)g.below(100) < chain_pct) {
            const int32_t L = 1 + (int32_t)g.below((uint64_t)chain_max);
            for (int32_t q = 0; q < L; q++) {
                const int32_t x = out.nodes++;
                out.add(a, x, wlo + (int32_t)g.below((uint64_t)(whi - wlo + 1)));
                a = x;
            }
        }
        out.add(a, b, wlo + (int32_t)g.below((uint64_t)(whi - wlo + 1)));
    }
    return emit(out, u, v, w, nodes);
}

int64_t mcbh_gen_block_tree(int32_t blocks, int32_t nmin, int32_t nmax, int32_t deg_lo_x10, int32_t deg_hi_x10,
                            int32_t wlo, int32_t whi, uint64_t seed, int32_t *u, int32_t *v, int32_t *w,
                            int32_t *nodes) {
    if (blocks < 1 || nmin < 3 || nmax < nmin || deg_lo_x10 < 20 || deg_hi_x10 < deg_lo_x10 || whi < wlo)
        return MCBH_E_ARG;
    Rng g{seed};
    EdgeList out;
    std::vector<int32_t> gid;
    std::unordered_set<uint64_t> seen;
    auto key = [](int32_t a, int32_t b) {
        return ((uint64_t)(uint32_t)std::min(a, b) << 32) | (uint32_t)std::max(a, b);
    };
    for (int32_t bi = 0; bi < blocks; bi++) {
        // block size log-uniform in [nmin, nmax], average degree uniform in [lo, hi]
        const double ln = std::log((double)nmin) + g.unit() * (std::log((double)nmax) - std::log((double)nmin));
        const int32_t n = std::min(nmax, std::max(nmin, (int32_t)std::lround(std::exp(ln))));
        const double deg = (deg_lo_x10 + g.unit() * (deg_hi_x10 - deg_lo_x10)) / 10.0;
        int64_t m = std::max<int64_t>(n, std::llround(n * deg / 2.0));
        m = std::min<int64_t>(m, (int64_t)n * (n - 1) / 2);
        // global ids: local vertex 0 is an existing vertex (the articulation point),
        // the others are new
        gid.assign((size_t)n, 0);
        if (bi == 0) {
            for (int32_t q = 0; q < n; q++) gid[q] = out.nodes++;
        } else {
            gid[0] = (int32_t)g.below((uint64_t)out.nodes);
            for (int32_t q = 1; q < n; q++) gid[q] = out.nodes++;
        }
        // a cycle through a random order of the vertices (the block is 2-connected:
        // no cut vertex inside it), then uniform extra edges up to m
        std::vector<int32_t> perm(n);
        for (int32_t q = 0; q < n; q++) perm[q] = q;
        for (int32_t q = n - 1; q > 0; q--) std::swap(perm[q], perm[g.below((uint64_t)q + 1)]);
        seen.clear();
        int64_t k = 0;
        auto add = [&](int32_t a, int32_t b) {
            if (a == b || !seen.insert(key(a, b)).second) return false;
            out.add(gid[a], gid[b], wlo + (int32_t)g.below((uint64_t)(whi - wlo + 1)));
            k++;
            return true;
        };
        for (int32_t q = 0; q < n; q++) add(perm[q], perm[(q + 1) % n]);
        while (k < m) add((int32_t)g.below((uint64_t)n), (int32_t)g.below((uint64_t)n));
    }
    return emit(out, u, v, w, nodes);
}

int64_t mcbh_edge_slot_order(int32_t nodes, int64_t m, const int32_t *u, const int32_t *v, int64_t *order) {
    if (nodes <= 0 || m < 0 || (m > 0 && (!u || !v || !order))) return MCBH_E_ARG;
    for (int64_t i = 0; i < m; i++)
        if (u[i] < 0 || u[i] >= nodes || v[i] < 0 || v[i] >= nodes) return MCBH_E_ARG;
    try {
        // the 2m slots as csr_graph::insert(a, b, w, false) pushes them, sorted by
        // (row, col) with std::sort: the permutation the reference's CSR gets, parallel
        // edges included (only the comparison outcomes decide it)
        std::vector<EdgeSlot> s;
        s.reserve(2 * (size_t)m);
        for (int64_t i = 0; i < m; i++) {
            s.push_back({(u32)u[i], (u32)v[i], 0, -1, (int)i, 0});
            s.push_back({(u32)v[i], (u32)u[i], 0, -1, (int)i, 0});
        }
        std::sort(s.begin(), s.end(), RowColLess());
        int64_t k = 0;
        for (const EdgeSlot &e : s)
            if (e.row > e.col) order[k++] = e.orig;
        return k;
    } catch (const std::bad_alloc &) {
        return MCBH_E_NOMEM;
    }
}

int64_t mcbh_bcc_split(int32_t nodes, int64_t m, const int32_t *u, const int32_t *v, int32_t *comp_of_edge) {
    if (nodes <= 0 || m < 0 || (m > 0 && (!u || !v || !comp_of_edge))) return MCBH_E_ARG;
    for (int64_t i = 0; i < m; i++)
        if (u[i] < 0 || u[i] >= nodes || v[i] < 0 || v[i] >= nodes) return MCBH_E_ARG;
    // adjacency (edge ids) in input order
    std::vector<int64_t> ro((size_t)nodes + 1, 0);
    for (int64_t i = 0; i < m; i++) {
        ro[(size_t)u[i] + 1]++;
        if (v[i] != u[i]) ro[(size_t)v[i] + 1]++;
    }
    for (int32_t x = 0; x < nodes; x++) ro[(size_t)x + 1] += ro[x];
    std::vector<int64_t> adj((size_t)ro[nodes]), fill(ro.begin(), ro.end() - 1);
    for (int64_t i = 0; i < m; i++) {
        adj[(size_t)fill[u[i]]++] = i;
        if (v[i] != u[i]) adj[(size_t)fill[v[i]]++] = i;
    }
    // Hopcroft-Tarjan with an edge stack, as an explicit-stack DFS.  A self-loop is
    // a component of its own.
    std::vector<int64_t> disc((size_t)nodes, -1), low((size_t)nodes, 0);
    std::vector<int64_t> estack;
    std::vector<int32_t> raw(m > 0 ? (size_t)m : 1, -1);
    int32_t ncomp = 0;
    struct Frame {
        int32_t v;
        int64_t pe, it;  // parent edge, next adjacency slot
    };
    std::vector<Frame> st;
    int64_t timer = 0;
    for (int64_t i = 0; i < m; i++)
        if (u[i] == v[i]) raw[i] = ncomp++;
    for (int32_t s = 0; s < nodes; s++) {
        if (disc[s] >= 0 || ro[s] == ro[(size_t)s + 1]) continue;
        disc[s] = low[s] = timer++;
        st.push_back({s, -1, ro[s]});
        while (!st.empty()) {
            Frame &f = st.back();
            if (f.it < ro[(size_t)f.v + 1]) {
                const int64_t e = adj[(size_t)f.it++];
                if (e == f.pe || u[e] == v[e]) continue;
                const int32_t w = u[e] == f.v ? v[e] : u[e];
                if (disc[w] < 0) {
                    estack.push_back(e);
                    disc[w] = low[w] = timer++;
                    st.push_back({w, e, ro[w]});
                } else if (disc[w] < disc[f.v]) {
                    estack.push_back(e);  // back edge
                    low[f.v] = std::min(low[f.v], disc[w]);
                }
                continue;
            }
            const int32_t w = f.v;
            const int64_t pe = f.pe;
            st.pop_back();
            if (st.empty()) break;
            const int32_t p = st.back().v;
            low[p] = std::min(low[p], low[w]);
            if (low[w] >= disc[p]) {  // p separates w's subtree: pop one component
                while (true) {
                    const int64_t e = estack.back();
                    estack.pop_back();
                    raw[e] = ncomp;
                    if (e == pe) break;
                }
                ncomp++;
            }
        }
    }
    // number components by their first input edge
    std::vector<int32_t> ren((size_t)ncomp, -1);
    int32_t next = 0;
    for (int64_t i = 0; i < m; i++) {
        if (ren[raw[i]] < 0) ren[raw[i]] = next++;
        comp_of_edge[i] = ren[raw[i]];
    }
    return next;
}

int mcbh_write_mtx(const char *path, int32_t nodes, int64_t m, const int32_t *u, const int32_t *v,
                   const int32_t *w) {
    if (!path || nodes <= 0 || m < 0) return MCBH_E_ARG;
    FILE *f = fopen(path, "w");
    if (!f) return MCBH_E_IO;
    fprintf(f, "%%%%MatrixMarket matrix coordinate integer symmetric\n");
    fprintf(f, "%d %d %lld\n", nodes, nodes, (long long)m);
    for (int64_t i = 0; i < m; i++) fprintf(f, "%d %d %d\n", u[i] + 1, v[i] + 1, w[i]);
    fclose(f);
    return MCBH_OK;
}

}  // extern "C"
