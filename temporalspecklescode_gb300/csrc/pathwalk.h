// pathwalk.h -- launch interface of the per-path random walk (pathwalk.cu).
#pragma once
#include <cuda_runtime.h>

#include "scene.h"

namespace sstmc {

struct WalkParams {
    uint64_t seed;
    uint32_t first_path, paths;
    uint32_t* counts;        // [paths] vertices per path (0: the path hit a limit)
    uint32_t* misses;        // [paths] missed first-vertex attempts
    uint32_t* offsets;       // [paths] exclusive scan of counts
    uint32_t* block_sums;    // [ceil(paths / 1024)]
    unsigned long long* total;  // [1] sum of counts
    float4* verts;           // [total] x, y, z, packed (k << 4 | material), xi = k * 2^-24
    uint32_t* hash;          // [paths] or null
    int* err;
    uint32_t* next;          // [2] path counters of the count and write passes (zeroed by launch_walk_count)
};

// Count pass + exclusive scan of the counts.
int launch_walk_count(const DevScene& S, const WalkParams& W, cudaStream_t stream);
// Write pass (same streams, same vertices).
int launch_walk_write(const DevScene& S, const WalkParams& W, cudaStream_t stream);

__host__ __device__ inline int vertex_material(float w) {
#ifdef __CUDA_ARCH__
    return (int)(__float_as_uint(w) & 15u);
#else
    (void)w; return 0;
#endif
}

}  // namespace sstmc
