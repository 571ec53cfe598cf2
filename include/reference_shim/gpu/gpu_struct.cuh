/* Drop-in replacement of the reference's gpu/gpu_struct.cuh (gpu_struct.cuh:15-84):
 * the same class name, constructor and member functions that the reference driver
 * calls (mcb/mcb_cycle_deg_two_remove.cpp:282-314,381-382,424), each a thin call into
 * the mcbgpu_struct handle of libmcbgpu.so.  The trees stay resident in HBM after the
 * first upload, so `multiple_transfer` only decides whether process_shortest_path
 * uploads them itself when the driver has not called initialize_memory.  Errors print
 * and exit, as the reference's do (include/utils.h:36-47). */
#ifndef MCBGPU_REFERENCE_SHIM_GPU_STRUCT
#define MCBGPU_REFERENCE_SHIM_GPU_STRUCT

#include <cstdio>
#include <cstdlib>

#include "bit_vector.h"
#include "gpu_task.h"
#include "mcbgpu.h"
#include "stats.h"

struct gpu_struct {
    mcbgpu_struct *h = nullptr;
    bool loaded = false;  // this handle's trees are on the device

    static void check(int rc) {
        if (rc) {
            std::fprintf(stderr, "Error :%s\n", mcbgpu_last_error());
            std::exit(1);
        }
    }
    gpu_struct(int num_edges, int num_non_tree_edges, int size_vector, int original_nodes, int fvs_size,
               int chunk_size, int nstreams, stats *) {
        check(mcbgpu_struct_create(&h, num_edges, num_non_tree_edges, size_vector, original_nodes, fvs_size,
                                   chunk_size, nstreams));
    }
    void initialize_memory(gpu_task *t) {
        compressed_trees *c = t->host_tree;
        check(mcbgpu_struct_initialize_memory(h, t->non_tree_edges_array, (const int32_t *const *)c->edge_offset,
                                              (const uint32_t *const *)c->tree_rows,
                                              (const uint32_t *const *)c->tree_cols));
        loaded = true;
    }
    float copy_support_vector(bit_vector *v) {
        float ms = 0;
        check(mcbgpu_struct_copy_support_vector(h, (const uint64_t *)v->elements, &ms));
        return ms;
    }
    float process_shortest_path(gpu_task *t, bool multiple_transfer) {
        if (!loaded) initialize_memory(t);
        float ms = 0;
        check(mcbgpu_struct_process_shortest_path(h, (uint32_t *const *)t->host_tree->precompute_value,
                                                  multiple_transfer, &ms));
        return ms;
    }
    void clear_memory() {
        check(mcbgpu_struct_clear_memory(h));
        h = nullptr;
        loaded = false;
    }
};

#endif
