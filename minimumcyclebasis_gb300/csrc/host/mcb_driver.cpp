// mcb_gb300 — the minimum-cycle-basis driver on this library, a drop-in for the
// reference's GPU driver binary (mcb/mcb_cycle_deg_two_remove.cpp, built as
// mcb_cuda).
//
//   mcb_gb300 <input.mtx> <stats.csv> <threads> [chunk_size] [options]
//
// Same positional arguments as the reference (chunk_size is accepted and ignored:
// every tree stays resident in HBM).  Like the reference it appends one row of
// statistics to stats.csv, writing the header first when the file is new, in the
// column order of the reference's GPU timings row (include/stats.h:256-338).
// Differences: the CSV has no padding whitespace, and Total_Weight is the exact
// 64-bit sum (the reference accumulates it in an int).
//
// Options:
//   --cycles FILE        the basis in selection order, one block per cycle in the
//                        format of cycle::print (include/cycles.h:197-207), reduced
//                        vertex ids + 1 as the reference prints them, then
//                        "Total Weight = W" (mcb/Test_deg_two_remove.cpp:334-341)
//   --cycles-input FILE  the same with the input graph's vertex ids + 1
//   --plain              the per-iteration de Pina loop instead of the blocked one
//   --bcc                split the graph into biconnected components first and solve
//                        each one that has a cycle (in order of its first edge), one
//                        stats row per component, the way the reference's bicc tool +
//                        per-component loop (bicc/, main.sh:19-32) processes a graph,
//                        each component with the tool's edge order and numbering;
//                        the components go through one batched solve (mcbgpu_batch);
//                        the cycle listings give each component's basis in turn
//   --gpu-trees          the per-root shortest-path trees computed on the GPU
//                        (mcbgpu_trees_*, 2048 roots per launch) and handed to the host
//                        preparation, which checks each one and searches any root whose
//                        tree it does not accept itself (the result does not change);
//                        single-graph mode (with --bcc the components are prepared on
//                        the host in parallel)
//   --verify             re-verify every basis over GF(2): the N selected cycles must
//                        have rank N; single-graph blocked solves by the device
//                        certificate (mcbgpu_solver_verify, any N), the others by
//                        Gaussian elimination on the host (mcbh_gf2_rank);
//                        "GF(2) rank R of N" on stderr per problem, an error if R < N
//
// Exit status 0 on success; on any error a message on stderr and status 1 (the
// reference prints and exits on every error too).
#include <cuda_runtime.h>
#include <unistd.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "mcbgpu.h"
#include "mcbhost.h"

namespace {

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

[[noreturn]] void fail(const char *what, const char *detail) {
    std::fprintf(stderr, "mcb_gb300: %s%s%s\n", what, detail ? ": " : "", detail ? detail : "");
    std::exit(1);
}

void check_host(int rc, const char *what) {
    if (rc != MCBH_OK) {
        char code[32];
        std::snprintf(code, sizeof code, "error %d", rc);
        fail(what, code);
    }
}

void check_gpu(int rc, const char *what) {
    if (rc != MCBGPU_OK) fail(what, mcbgpu_last_error());
}

struct Stats {  // the reference's GPU stats row (include/stats.h:256-338)
    long long nodes = 0, edges = 0, new_edges = 0, nodes_removed = 0, fvs = 0, initial = 0, final_ = 0;
    long long total_weight = 0;
    int nchunks = 1, nstreams = 1;
    double total_mb = 0, static_mb = 0, variable_mb = 0;
    bool load_entire = true;
    double t_trees = 0, t_collect = 0, t_inspection = 0, t_gpu = 0, t_hybrid = 0, t_main = 0;

    void append(const char *path) const {
        const bool exists = access(path, F_OK) == 0;
        FILE *f = std::fopen(path, "a");
        if (!f) fail("cannot open the statistics file", path);
        if (!exists)
            std::fprintf(f,
                         "Total_Nodes,Total_Edges,New_Edges,Nodes_removed,Fvs_size,Initial_Cycles,Final_cycles,"
                         "Total_Weight,nchunks,nstreams,total_memory_usage(mb),static_memory_usage(mb),"
                         "variable_memory_usage(mb),load_entire_memory,Construction_trees(s),Collect_cycles(s),"
                         "Inspection_time(s),Gpu_timings,Hybrid_Timings(s),Preprocessing Time(s),Main_loop(s),"
                         "Total_time(s)\n");
        std::fprintf(f, "%lld,%lld,%lld,%lld,%lld,%lld,%lld,%lld,%d,%d,%lf,%lf,%lf,%s,%lf,%lf,%lf,%lf,%lf,%lf,%lf,%lf\n",
                     nodes, edges, new_edges, nodes_removed, fvs, initial, final_, total_weight, nchunks, nstreams,
                     total_mb, static_mb, variable_mb, load_entire ? "YES" : "NO", t_trees, t_collect, t_inspection,
                     t_gpu, t_hybrid, t_trees + t_collect, t_main, t_main + t_trees + t_collect);
        std::fclose(f);
    }
};

// One cycle block per selected candidate, in the format of cycle::print.  vmap: the
// vertex ids to print for each reduced vertex (0-based), or NULL for reduced ids.
void write_cycles(FILE *f, const std::vector<int64_t> &sel, const std::vector<int32_t> &root,
                  const std::vector<int32_t> &edge, const std::vector<int32_t> &weight,
                  const std::vector<uint32_t> &rows, const std::vector<uint32_t> &cols, const int32_t *vmap) {
    const char *bar = "=================================================================================";
    auto id = [&](uint32_t v) { return (unsigned)(vmap ? vmap[v] : (int32_t)v) + 1u; };
    for (int64_t r : sel) {
        std::fprintf(f, "%s\nRoot is %u\nEdge is %u - %u\nTotal weight = %d\n%s\n", bar, id((uint32_t)root[r]),
                     id(rows[edge[r]]), id(cols[edge[r]]), weight[r], bar);
    }
}

struct Outputs {
    const char *stats = nullptr;
    FILE *cycles = nullptr, *cycles_input = nullptr;
    bool plain = false;
    bool verify = false;
    bool gpu_trees = false;
    int threads = 1;
};

// The GPU as the host preparation's tree supplier (mcbh_tree_source).
struct GpuTreeSupplier {
    mcbgpu_trees *t = nullptr;
    int32_t chunk = 2048;
    ~GpuTreeSupplier() { mcbgpu_trees_destroy(t); }
    static int begin(void *ctx, int32_t nodes, int64_t slots, const uint32_t *ro, const uint32_t *cols,
                     const int32_t *w, const uint32_t *rev) {
        GpuTreeSupplier *g = static_cast<GpuTreeSupplier *>(ctx);
        mcbgpu_trees_destroy(g->t);
        g->t = nullptr;
        return mcbgpu_trees_create(&g->t, nodes, slots, ro, cols, w, rev, g->chunk) == MCBGPU_OK ? 0 : 1;
    }
    static int trees(void *ctx, const uint32_t *roots, int32_t count, int32_t *dist, int32_t *pslot,
                     uint8_t *skip) {
        GpuTreeSupplier *g = static_cast<GpuTreeSupplier *>(ctx);
        return mcbgpu_trees_run(g->t, roots, count, dist, pslot, skip, nullptr) == MCBGPU_OK ? 0 : 1;
    }
};

// One problem from preparation to output.
struct Job {
    mcbh_problem *p = nullptr;
    std::vector<int32_t> ids;  // input vertex of every vertex of the problem's graph (empty: the input graph)
    mcbh_info info{};
    Stats st;
    std::vector<int32_t> root, edge, weight, tree, coords;
    std::vector<int64_t> off, sel;
    long long total = 0;
    int64_t device_rank = -1;  // rank certified on the device (--verify, single-problem solver)
};

void init_gpu_once() {
    static bool ready = false;  // first problem that needs the GPU
    if (!ready) {
        int dev = 0, sms = 0;
        size_t mem = 0;
        check_gpu(mcbgpu_init_cuda(&dev, &sms, &mem), "CUDA initialisation");
        ready = true;
    }
}

mcbh_options job_options(const Outputs &o) {
    mcbh_options opt{};
    opt.threads = o.threads > 0 ? o.threads : 1;
    opt.contract_chains = 1;
    opt.cycle_lists = 1;
    return opt;
}

// A prepared problem's rank-ordered candidates and their coordinate lists; the
// stats row's host columns.
void collect_job(Job &j) {
    check_host(mcbh_get_info(j.p, &j.info), "mcbh_get_info");
    const mcbh_info &info = j.info;
    Stats &st = j.st;
    st.nodes = info.nodes;
    st.edges = info.edges2;
    if (info.single_cycle) {  // every vertex has degree two (mcb_cycle_deg_two_remove.cpp:104-111)
        st.fvs = 1;
        st.nodes_removed = info.nodes - 1;
        st.final_ = 1;
        st.initial = 1;
        st.total_weight = info.total_weight_input;
        j.total = info.total_weight_input;
        return;
    }
    st.nodes_removed = info.nodes_removed;
    st.new_edges = info.reduced_edges2;
    st.fvs = info.fvs_size;
    st.initial = info.num_candidates;
    st.t_trees = info.t_trees;
    st.t_collect = info.t_collect;
    const int64_t K = info.num_candidates;
    j.root.resize(K);
    j.edge.resize(K);
    j.weight.resize(K);
    j.tree.resize(K);
    check_host(mcbh_get_candidates(j.p, j.root.data(), j.edge.data(), j.weight.data(), j.tree.data()),
               "mcbh_get_candidates");
    j.off.resize(K + 1);
    j.coords.resize(info.cycle_nnz > 0 ? info.cycle_nnz : 1);
    check_host(mcbh_get_cycle_lists(j.p, j.off.data(), j.coords.data()), "mcbh_get_cycle_lists");
}

// Host preparation of one problem: reduced graph, FVS, trees, candidates.
void prepare_job(Job &j, const Outputs &o) {
    const mcbh_options opt = job_options(o);
    if (o.gpu_trees) {
        init_gpu_once();
        GpuTreeSupplier g;
        mcbh_tree_source src{&g, &GpuTreeSupplier::begin, &GpuTreeSupplier::trees, g.chunk, 0};
        const int rc = mcbh_prepare_with_trees(j.p, &opt, &src);
        if (rc == MCBH_E_SUPPLIER) {
            std::fprintf(stderr, "mcb_gb300: GPU trees: %s\n", mcbgpu_last_error());
            std::exit(1);
        }
        check_host(rc, "preprocessing failed");
    } else {
        check_host(mcbh_prepare(j.p, &opt), "preprocessing failed");
    }
    collect_job(j);
}

bool needs_gpu(const Job &j) { return !j.info.single_cycle && j.info.num_coords > 0; }

// One problem on the single-problem solver (blocked, or per iteration with --plain).
void solve_single(Job &j, const Outputs &o) {
    init_gpu_once();
    const int32_t N = j.info.num_coords;
    const int64_t K = j.info.num_candidates;
    const double t1 = now_s();
    mcbgpu_solver *s = nullptr;
    check_gpu(mcbgpu_solver_create(&s, N, K, j.off[K]), "mcbgpu_solver_create");
    check_gpu(mcbgpu_solver_upload(s, j.weight.data(), j.off.data(), j.coords.data(), nullptr), "mcbgpu_solver_upload");
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, 0);
    check_gpu(o.plain ? mcbgpu_solver_run_plain(s, -1, nullptr) : mcbgpu_solver_run(s, -1, nullptr), "solve");
    cudaEventRecord(b, 0);
    j.sel.assign(N, -1);
    int64_t total = 0;
    check_gpu(mcbgpu_solver_results(s, j.sel.data(), N, &total, nullptr), "mcbgpu_solver_results");
    float gpu_ms = 0;
    cudaEventElapsedTime(&gpu_ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    j.total = total;
    j.st.t_gpu = j.st.t_inspection = gpu_ms / 1000.0;
    j.st.t_main = now_s() - t1;
    j.st.total_mb = (double)mcbgpu_solver_device_bytes(s) / (1024.0 * 1024.0);
    if (o.verify && !o.plain) {
        // the basis against the final support vectors, on the device (exact at any N)
        int64_t bad = 0, bi = -1, bj = -1;
        check_gpu(mcbgpu_solver_verify(s, &bad, &bi, &bj, nullptr), "GF(2) verification on the device");
        if (bad != 0) {
            std::fprintf(stderr, "mcb_gb300: %lld entries of <C_i, S_j> contradict the basis (first (%lld, %lld))\n",
                         (long long)bad, (long long)bi, (long long)bj);
            std::exit(1);
        }
        j.device_rank = N;
    }
    mcbgpu_solver_destroy(s);
}

// Several problems in one batched launch per size class.  The GPU time and the
// main-loop time of the batch are shared out over its problems in proportion to N.
void solve_batched(std::vector<Job *> &jobs) {
    if (jobs.empty()) return;
    init_gpu_once();
    const double t1 = now_s();
    std::vector<int32_t> N;
    std::vector<int64_t> K, off{0};
    std::vector<int32_t> weight, coords;
    for (Job *j : jobs) {
        const int64_t k = j->info.num_candidates, base = off.back();
        N.push_back(j->info.num_coords);
        K.push_back(k);
        weight.insert(weight.end(), j->weight.begin(), j->weight.begin() + k);
        for (int64_t r = 1; r <= k; r++) off.push_back(base + j->off[r]);
        coords.insert(coords.end(), j->coords.begin(), j->coords.begin() + j->off[k]);
    }
    mcbgpu_batch *b = nullptr;
    check_gpu(mcbgpu_batch_create(&b, (int32_t)jobs.size(), N.data(), K.data(), off.back()), "mcbgpu_batch_create");
    check_gpu(mcbgpu_batch_upload(b, weight.data(), off.data(), coords.data(), nullptr), "mcbgpu_batch_upload");
    cudaEvent_t a, e;
    cudaEventCreate(&a);
    cudaEventCreate(&e);
    cudaEventRecord(a, 0);
    check_gpu(mcbgpu_batch_run(b, nullptr), "batched solve");
    cudaEventRecord(e, 0);
    int64_t nsum = 0;
    for (int32_t n : N) nsum += n;
    std::vector<int64_t> sel(nsum > 0 ? nsum : 1), tot(jobs.size());
    check_gpu(mcbgpu_batch_results(b, sel.data(), tot.data(), nullptr, nullptr), "mcbgpu_batch_results");
    float gpu_ms = 0;
    cudaEventElapsedTime(&gpu_ms, a, e);
    cudaEventDestroy(a);
    cudaEventDestroy(e);
    const double main_s = now_s() - t1, mb = (double)mcbgpu_batch_device_bytes(b) / (1024.0 * 1024.0);
    mcbgpu_batch_destroy(b);
    int64_t at = 0;
    for (size_t i = 0; i < jobs.size(); i++) {
        Job &j = *jobs[i];
        const double share = nsum > 0 ? (double)N[i] / (double)nsum : 0.0;
        j.sel.assign(sel.begin() + at, sel.begin() + at + N[i]);
        at += N[i];
        j.total = tot[i];
        j.st.t_gpu = j.st.t_inspection = gpu_ms / 1000.0 * share;
        j.st.t_main = main_s * share;
        j.st.total_mb = mb * share;
    }
}

// Appends the problem's stats row and its cycle blocks.
void emit_job(Job &j, const Outputs &o) {
    if (o.verify && !j.info.single_cycle && j.info.num_coords > 0) {
        int64_t rank = j.device_rank;
        if (rank < 0)
            check_host(mcbh_gf2_rank(j.p, j.sel.data(), (int64_t)j.sel.size(), o.threads, &rank),
                       "GF(2) verification");
        std::fprintf(stderr, "GF(2) rank %lld of %d%s\n", (long long)rank, j.info.num_coords,
                     j.device_rank >= 0 ? " (device certificate)" : "");
        if (rank != j.info.num_coords) {
            std::fprintf(stderr, "mcb_gb300: the basis is not independent\n");
            std::exit(1);
        }
    }
    Stats &st = j.st;
    if (!j.info.single_cycle) {
        const int64_t K = j.info.num_candidates;
        st.final_ = j.info.num_coords;
        st.total_weight = j.total;
        st.static_mb = (double)(sizeof(int32_t) * K + sizeof(int64_t) * (K + 1) +
                                sizeof(int32_t) * (K > 0 ? j.off[K] : 0)) /
                       (1024.0 * 1024.0);
        st.variable_mb = st.total_mb > st.static_mb ? st.total_mb - st.static_mb : 0.0;
    }
    st.append(o.stats);
    if (j.info.single_cycle || !(o.cycles || o.cycles_input)) return;
    const int64_t e2 = j.info.reduced_edges2;
    std::vector<uint32_t> rows(e2), cols(e2), rev(e2), ro(j.info.reduced_nodes + 1);
    std::vector<int32_t> wts(e2), vmap(j.info.reduced_nodes);
    check_host(mcbh_get_reduced_graph(j.p, rows.data(), cols.data(), wts.data(), rev.data(), ro.data()),
               "mcbh_get_reduced_graph");
    check_host(mcbh_get_vertex_map(j.p, vmap.data()), "mcbh_get_vertex_map");
    if (o.cycles) write_cycles(o.cycles, j.sel, j.root, j.edge, j.weight, rows, cols, nullptr);
    if (o.cycles_input) {
        if (!j.ids.empty())
            for (auto &x : vmap) x = j.ids[x];
        write_cycles(o.cycles_input, j.sel, j.root, j.edge, j.weight, rows, cols, vmap.data());
    }
}

}  // namespace

int main(int argc, char **argv) {
    std::vector<const char *> pos;
    const char *cycles_path = nullptr, *cycles_input_path = nullptr;
    bool plain = false, bcc = false, verify = false, gpu_trees = false;
    for (int i = 1; i < argc; i++) {
        if (!std::strcmp(argv[i], "--cycles") && i + 1 < argc)
            cycles_path = argv[++i];
        else if (!std::strcmp(argv[i], "--cycles-input") && i + 1 < argc)
            cycles_input_path = argv[++i];
        else if (!std::strcmp(argv[i], "--plain"))
            plain = true;
        else if (!std::strcmp(argv[i], "--bcc"))
            bcc = true;
        else if (!std::strcmp(argv[i], "--verify"))
            verify = true;
        else if (!std::strcmp(argv[i], "--gpu-trees"))
            gpu_trees = true;
        else
            pos.push_back(argv[i]);
    }
    if (pos.size() < 3) {
        std::printf("Ist Argument should indicate the InputFile\n");
        std::printf("2nd Argument should indicate the OutputFile\n");
        std::printf("3th argument should indicate the number of threads.(Optional) (1 default)\n");
        std::printf("4th Argument is chunk_size.(Optional) (720 default)\n");
        std::printf("options: --cycles FILE, --cycles-input FILE, --plain, --bcc, --verify, --gpu-trees\n");
        return 1;
    }
    const char *input = pos[0];
    Outputs o;
    o.stats = pos[1];
    o.threads = std::atoi(pos[2]);
    o.plain = plain;
    o.verify = verify;
    o.gpu_trees = gpu_trees;
    if (bcc && gpu_trees)
        std::fprintf(stderr, "note: --gpu-trees applies to the single-graph mode; with --bcc the components are "
                             "prepared on the host\n");
    if (cycles_path && !(o.cycles = std::fopen(cycles_path, "w"))) fail("cannot open the cycle file", cycles_path);
    if (cycles_input_path && !(o.cycles_input = std::fopen(cycles_input_path, "w")))
        fail("cannot open the cycle file", cycles_input_path);
    const double t0 = now_s();
    long long total = 0;
    int solved = 0;
    if (!bcc) {
        Job j;
        check_host(mcbh_problem_from_mtx(input, &j.p), "cannot read the input graph");
        prepare_job(j, o);
        if (needs_gpu(j)) solve_single(j, o);
        emit_job(j, o);
        total = j.total;
        solved = 1;
        mcbh_problem_free(j.p);
    } else {
        int32_t nodes = 0;
        const int64_t m = mcbh_read_mtx(input, &nodes, 0, nullptr, nullptr, nullptr);
        if (m < 0) fail("cannot read the input graph", nullptr);
        std::vector<int32_t> u(m > 0 ? m : 1), v(m > 0 ? m : 1), w(m > 0 ? m : 1), comp(m > 0 ? m : 1);
        check_host(mcbh_read_mtx(input, &nodes, m, u.data(), v.data(), w.data()) == m ? MCBH_OK : MCBH_E_IO,
                   "cannot read the input graph");
        const int64_t nc = mcbh_bcc_split(nodes, m, u.data(), v.data(), comp.data());
        if (nc < 0) fail("biconnected split failed", nullptr);
        // every component as the reference's bicc tool writes it and its Relabeller
        // numbers it (bicc/include/bicc.h:220-314, bicc/Relabeller.cpp:72-126): its
        // edges in the input CSR's slot order as (larger, smaller endpoint), its
        // vertices in order of first appearance
        std::vector<int64_t> slot_order(m > 0 ? m : 1);
        const int64_t ns = mcbh_edge_slot_order(nodes, m, u.data(), v.data(), slot_order.data());
        if (ns < 0) fail("slot order failed", nullptr);
        std::vector<int64_t> start(nc + 1, 0);
        for (int64_t k = 0; k < ns; k++) start[comp[slot_order[k]] + 1]++;
        for (int64_t c = 0; c < nc; c++) start[c + 1] += start[c];
        std::vector<int64_t> order(ns > 0 ? ns : 1), fill(start.begin(), start.end() - 1);
        for (int64_t k = 0; k < ns; k++) order[fill[comp[slot_order[k]]]++] = slot_order[k];
        std::vector<int32_t> local(nodes, -1);
        std::vector<Job> jobs;
        jobs.reserve(nc);
        for (int64_t c = 0; c < nc; c++) {
            std::vector<int32_t> cu, cv, cw, ids;
            for (int64_t k = start[c]; k < start[c + 1]; k++) {
                const int64_t e = order[k];
                const int32_t hi = u[e] > v[e] ? u[e] : v[e], lo = u[e] > v[e] ? v[e] : u[e];
                for (int32_t x : {hi, lo})
                    if (local[x] < 0) {
                        local[x] = (int32_t)ids.size();
                        ids.push_back(x);
                    }
                cu.push_back(local[hi]);
                cv.push_back(local[lo]);
                cw.push_back(w[e]);
            }
            for (int32_t x : ids) local[x] = -1;
            if ((int64_t)cu.size() < (int64_t)ids.size()) continue;  // a bridge: no cycle
            jobs.emplace_back();
            Job &j = jobs.back();
            j.ids = ids;
            check_host(mcbh_problem_from_edges((int32_t)ids.size(), (int64_t)cu.size(), cu.data(), cv.data(),
                                               cw.data(), &j.p),
                       "component");
        }
        // the components are independent: prepared in parallel, one thread each
        {
            std::vector<mcbh_problem *> hs;
            for (Job &j : jobs) hs.push_back(j.p);
            const mcbh_options opt = job_options(o);
            check_host(mcbh_prepare_many(hs.data(), (int64_t)hs.size(), &opt, nullptr), "preprocessing failed");
            for (Job &j : jobs) collect_job(j);
        }
        // every component that fits the batch in one batched launch per size class
        // (the per-iteration form with --plain), the rest on the single-problem solver
        std::vector<Job *> batch;
        for (Job &j : jobs) {
            if (!needs_gpu(j)) continue;
            if (!o.plain && j.info.num_coords <= mcbgpu_batch_max_coords())
                batch.push_back(&j);
            else
                solve_single(j, o);
        }
        solve_batched(batch);
        for (Job &j : jobs) {
            emit_job(j, o);
            total += j.total;
            solved++;
            mcbh_problem_free(j.p);
        }
    }
    if (o.cycles) {
        std::fprintf(o.cycles, "Total Weight = %lld\n", total);
        std::fclose(o.cycles);
    }
    if (o.cycles_input) {
        std::fprintf(o.cycles_input, "Total Weight = %lld\n", total);
        std::fclose(o.cycles_input);
    }
    std::printf("mcb_gb300: %s: %d problem(s), total weight %lld, %.3f s\n", input, solved, total, now_s() - t0);
    return 0;
}
