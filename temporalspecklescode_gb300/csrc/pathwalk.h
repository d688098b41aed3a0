// pathwalk.h -- launch interface of the per-path random walk (pathwalk.cu).
#pragma once
#include <cuda_runtime.h>

#include "scene.h"

namespace sstmc {

constexpr uint32_t kWalkSlotVerts = 64;   // vertices per path slot and per overflow block

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
    float4* slots;           // [paths][64] or null: single-pass walk (count + first 64 vertices per path)
    uint32_t* list;          // paths longer than the slot (written by launch_walk_compact); write pass: replay only these
    uint32_t* list_count;    // [1] length of list on the device
    uint32_t list_n;         // write pass: length of list
    float4* ovf;             // [ovf_cap][64] overflow blocks: vertices 64 j .. 64 j + 63 of a path longer than its slot
    uint2* ovf_owner;        // [ovf_cap] (path, j >= 1) of each overflow block
    uint32_t* ovf_count;     // [1] overflow blocks taken (past ovf_cap the path is listed for the write pass instead)
    uint32_t ovf_cap;
    uint32_t ovf_n;          // compaction: min(*ovf_count, ovf_cap), read back by the host
    uint32_t* next;          // [2] path counters of the count and write passes (zeroed by launch_walk_count)
    float4* first;           // [paths][2] first vertex of every path (launch_walk_count): (origin, xi),
                             // (x1, ok << 31 | attempts << 4 | material); read by the non-beam walks
    uint32_t* first_next;    // [1] path counter of the first-vertex kernel (zeroed by launch_walk_count)
};

// Count pass (with W.slots: the single pass that also keeps the first 64
// vertices of each path) + exclusive scan of the counts.
int launch_walk_count(const DevScene& S, const WalkParams& W, cudaStream_t stream);
// Single pass: pack the slots and the overflow blocks into verts at the offsets.
int launch_walk_compact(const WalkParams& W, cudaStream_t stream);
// Write pass (same streams, same vertices) over every path, or over W.list.
int launch_walk_write(const DevScene& S, const WalkParams& W, cudaStream_t stream);
size_t walk_slot_bytes_per_path();            // slot + share of the overflow pool + list entry
uint32_t walk_overflow_blocks(uint32_t paths);  // overflow pool size for a chunk of `paths`

__host__ __device__ inline int vertex_material(float w) {
#ifdef __CUDA_ARCH__
    return (int)(__float_as_uint(w) & 15u);
#else
    (void)w; return 0;
#endif
}

}  // namespace sstmc
