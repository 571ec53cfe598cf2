/* Drop-in replacement of the reference's gpu/common.cuh (gpu/common.cuh:1-28) for a
 * driver linked against libmcbgpu.so: the five free functions keep their names and
 * signatures (exported by the library with the reference's print-and-exit error
 * behaviour), and gpu_struct comes from the shim beside this file.  No CUDA header is
 * needed to compile a driver against it.  Put this directory ahead of the reference
 * checkout on the include path so that `#include <gpu/common.cuh>` finds it. */
#ifndef MCBGPU_REFERENCE_SHIM_COMMON
#define MCBGPU_REFERENCE_SHIM_COMMON

#include <stddef.h>

#include "gpu_struct.cuh"

extern "C" void init_cuda();
extern "C" size_t configure_grid(int start, int end);
extern "C" unsigned *allocate_pinned_memory(int chunk, int nodes);
extern "C" void free_pinned_memory(unsigned *);
extern "C" size_t calculate_chunk_size(size_t num_nodes, size_t num_edges, size_t size_vector, size_t nstream);

#endif
