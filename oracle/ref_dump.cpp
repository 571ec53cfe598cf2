// ref_dump: a small driver of OUR OWN over the reference's host library.
//
// It is compiled (by oracle/Makefile) against the reference's headers where they
// lie, and is only used to produce golden vectors.  It runs the same pipeline as
// the reference CPU driver mcb/mcb_non_cpu_rd.cpp:76-342 (read, degree-2 chain
// contraction, MGA FVS, DFS spanning tree, FVS-rooted shortest-path trees,
// candidate collection + sort, de Pina loop) by calling the reference's classes,
// and prints, in a compact line format:
//   G <n> <2m> <nodes_removed> <reduced_n> <reduced_2m> <F> <N> <K>
//   E <offset> <row> <col> <weight> <reverse>          (reduced multigraph CSR)
//   V <v> <fvs_index>                                  (FVS array)
//   T <coord> <edge offset>                            (coordinate order)
//   C <rank> <root> <edge offset> <weight>             (sorted candidate list)
//   S <iteration> <rank> <root> <edge offset> <weight> (selected basis cycles)
//   W <total weight, 64-bit>
// argv: <in.mtx> <threads> [max_iterations] [flags: any of "noE" "noC"]
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <list>
#include <map>
#include <string>
#include <unordered_map>
#include <algorithm>
#include <omp.h>

#include "FileReader.h"
#include "utils.h"
#include "Host_Timer.h"
#include "CsrGraph.h"
#include "CsrTree.h"
#include "CsrGraphMulti.h"
#include "bit_vector.h"
#include "work_per_thread.h"
#include "cycle_searcher.h"
#include "FVS.h"
#include "compressed_trees.h"

debugger dbg;
HostTimer globalTimer;

int main(int argc, char **argv) {
    if (argc < 3) {
        fprintf(stderr, "usage: ref_dump in.mtx threads [max_iter] [noE] [noC]\n");
        return 1;
    }
    int threads = atoi(argv[2]);
    long max_iter = (argc >= 4) ? atol(argv[3]) : -1;
    bool printE = true, printC = true;
    for (int i = 4; i < argc; i++) {
        if (!strcmp(argv[i], "noE")) printE = false;
        if (!strcmp(argv[i], "noC")) printC = false;
    }
    omp_set_num_threads(threads);

    FileReader reader(argv[1]);
    int nodes, edges;
    reader.get_nodes_edges(nodes, edges);
    csr_graph *g = new csr_graph();
    g->Nodes = nodes;
    g->initial_edge_count = edges;
    for (int i = 0; i < edges; i++) {
        int a, b, w;
        reader.read_edge(a, b, w);
        g->insert(a, b, w, false);
    }
    g->calculateDegreeandRowOffset();
    reader.fileClose();

    if (g->get_num_degree_two_vertices() == g->Nodes) {
        printf("G %d %zu %d %d %d %d %d %d\n", nodes, g->rows->size(), nodes - 1, 0, 0, 1, 1, 1);
        printf("W %d\n", g->get_total_weight());
        return 0;
    }

    std::vector<std::vector<unsigned> > *chains = new std::vector<std::vector<unsigned> >();
    int source_vertex;
    std::vector<unsigned> *removal = g->mark_degree_two_chains(&chains, source_vertex);
    std::vector<std::vector<unsigned> > *new_edges = new std::vector<std::vector<unsigned> >();
    int removed = 0;
    for (size_t i = 0; i < chains->size(); i++) {
        unsigned r, c;
        unsigned w = g->sum_edge_weights(chains->at(i), r, c);
        removed += chains->at(i).size() - 1;
        std::vector<unsigned> ne;
        ne.push_back(r);
        ne.push_back(c);
        ne.push_back(w);
        new_edges->push_back(ne);
    }
    csr_multi_graph *rg = csr_multi_graph::get_modified_graph(g, removal, new_edges, removed);

    FVS fvs(rg);
    fvs.MGA();
    int *fvs_array = fvs.get_copy_fvs_array();
    int F = fvs.get_num_elements();

    csr_tree *st = new csr_tree(rg);
    st->populate_tree_edges(true, source_vertex);
    int N = st->non_tree_edges->size();

    std::vector<int> map(rg->rows->size(), -1);
    for (int i = 0; i < N; i++) map[st->non_tree_edges->at(i)] = i;
    for (size_t i = 0; i < rg->rows->size(); i++)
        if (map[i] < 0 && map[rg->reverse_edge->at(i)] >= 0) map[i] = map[rg->reverse_edge->at(i)];

    compressed_trees trees(F, F, fvs_array, rg);
    cycle_storage *storage = new cycle_storage(rg->Nodes);
    std::vector<worker_thread *> work(threads);
    for (int i = 0; i < threads; i++) work[i] = new worker_thread(rg, storage, fvs_array, &trees);
#pragma omp parallel for
    for (int i = 0; i < trees.fvs_size; ++i) work[omp_get_thread_num()]->produce_sp_tree_and_cycles(i, rg);

    std::vector<cycle *> cand;
    for (size_t j = 0; j < storage->list_cycles.size(); j++)
        for (auto it = storage->list_cycles[j].begin(); it != storage->list_cycles[j].end(); ++it)
            for (size_t k = 0; k < it->second->listed_cycles.size(); k++) {
                cand.push_back(it->second->listed_cycles[k]);
                cand.back()->ID = cand.size() - 1;
            }
    std::sort(cand.begin(), cand.end(), cycle::compare());
    std::map<cycle *, long> rank_of;
    for (size_t i = 0; i < cand.size(); i++) rank_of[cand[i]] = (long)i;

    printf("G %d %zu %d %d %zu %d %d %zu\n", nodes, g->rows->size(), removed, rg->Nodes,
           rg->rows->size(), F, N, cand.size());
    if (printE)
        for (size_t i = 0; i < rg->rows->size(); i++)
            printf("E %zu %u %u %d %u\n", i, rg->rows->at(i), rg->columns->at(i), rg->weights->at(i),
                   rg->reverse_edge->at(i));
    for (int v = 0; v < rg->Nodes; v++)
        if (fvs_array[v] >= 0) printf("V %d %d\n", v, fvs_array[v]);
    for (int i = 0; i < N; i++) printf("T %d %u\n", i, st->non_tree_edges->at(i));
    if (printC)
        for (size_t i = 0; i < cand.size(); i++)
            printf("C %zu %d %u %d\n", i, cand[i]->root, cand[i]->non_tree_edge_index, cand[i]->total_length);

    std::list<cycle *> lst(cand.begin(), cand.end());
    std::vector<bit_vector *> S(N);
    for (int i = 0; i < N; i++) {
        S[i] = new bit_vector(N);
        S[i]->set_bit(i, true);
    }
    long long total = 0;
    long iters = (max_iter >= 0 && max_iter < N) ? max_iter : N;
    for (long e = 0; e < iters; e++) {
#pragma omp parallel for
        for (int i = 0; i < threads; i++) work[i]->precompute_supportVec(map, *S[e]);
        cycle *chosen = NULL;
        for (auto it = lst.begin(); it != lst.end(); ++it) {
            unsigned *ro, *co, *pre;
            int *eo, *pa, *di;
            int idx = trees.vertices_map[(*it)->get_root()];
            trees.get_node_arrays(&ro, &co, &eo, &pa, &di, idx);
            trees.get_precompute_array(&pre, idx);
            unsigned off = (*it)->non_tree_edge_index;
            unsigned bit = 0;
            if (map[off] >= 0) bit = S[e]->get_bit(map[off]);
            bit = (bit + pre[rg->rows->at(off)]) % 2;
            bit = (bit + pre[rg->columns->at(off)]) % 2;
            if (bit == 1) {
                chosen = *it;
                lst.erase(it);
                break;
            }
        }
        if (!chosen) {
            printf("X no odd candidate at iteration %ld\n", e);
            return 2;
        }
        bit_vector *cv = chosen->get_cycle_vector(map, N);
        printf("S %ld %ld %d %u %d\n", e, rank_of[chosen], chosen->root, chosen->non_tree_edge_index,
               chosen->total_length);
        total += chosen->total_length;
#pragma omp parallel for
        for (int j = e + 1; j < N; j++)
            if (cv->dot_product(S[j]) == 1) S[j]->do_xor(S[e]);
        cv->clear_memory();
        delete cv;
    }
    printf("W %lld\n", total);
    return 0;
}
