// sstmc_internal.h -- render engine state shared by api.cpp and serve.cpp.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <utility>
#include <vector>

#include "scene.h"
#include "pathwalk.h"
#include "trace.h"

namespace sstmc {

constexpr int kMaxSlots = 32;  // view-accumulator slots per lane (8 KB of shared memory per warp)
constexpr size_t kStaticScratchBytes = (size_t)64 << 20;  // per device, sstmc_render_static (static_render.cu)

struct PathDebug {
    uint32_t* hash = nullptr;
    uint32_t* dda = nullptr;
};

// Device buffers of one scene's renders: the per-path rows of a chunk of
// paths, the FP64 accumulator and the far-field single-scattering weights.
struct Engine {
    cudaStream_t stream = nullptr;
    uint32_t cap = 0;
    float2 *a_ms = nullptr, *s_ms = nullptr, *a_ss = nullptr, *b_ss = nullptr, *g2 = nullptr;
    float *pl = nullptr, *x1 = nullptr, *x1t = nullptr;
    unsigned char* m1 = nullptr;
    uint32_t *counts = nullptr, *misses = nullptr, *offsets = nullptr, *block_sums = nullptr;
    unsigned long long* vtotal = nullptr;
    bool rows_real = false;       // the chunk's a_ms / s_ms are real floats (trace_chunk -> contract_chunk)
    float4* slots = nullptr;      // single-pass walk: first 64 vertices of each path of a chunk
    uint32_t* longq = nullptr;    // paths of the chunk that found the overflow pool empty
    float4* first_v = nullptr;    // first vertex of each path of a chunk (two float4 per path)
    float4* ovf = nullptr;        // overflow blocks of 64 vertices (pathwalk.cu)
    uint32_t ovf_blocks = 0;      // overflow blocks allocated
    uint32_t ovf_want = 0;        // learned pool size: a chunk that found the pool short grows it
    float* p2v = nullptr;         // [paths] second-point probability (correlation CBS)
    // far-field x far-field single scattering: the chunk's paths grouped by
    // first-vertex material (contract.cu launch_ss_buckets); null in the
    // static-scratch render, which contracts per material with masks instead
    uint32_t* ss_row = nullptr;   // [paths] row of each path in a_ss / b_ss
    uint32_t* ss_hist = nullptr;  // [ceil(paths / 1024)][kMat] scratch of the partition
    uint32_t* ss_bucket = nullptr;  // [kMat + 1] first row of each material
    bool ss_bucketed = false;     // the chunk's a_ss / b_ss rows are grouped (trace_chunk -> contract_chunk)
    // correlation sampler, general kernel: (path, segment) items of the long
    // paths (trace.cu); grown with the vertex buffer, null in the static render
    uint2* seg_list = nullptr;
    size_t seg_cap = 0;
    uint32_t* seg_ctr = nullptr;  // [2] items in the list, items taken
    uint2* ovf_owner = nullptr;
    float4* verts = nullptr;
    size_t verts_cap = 0;
    unsigned long long* totals = nullptr;
    int* err = nullptr;
    double2* V = nullptr;
    float* W = nullptr;
    // device timing of the last render: events around each kernel class
    cudaEvent_t ev[8] = { nullptr };
    double ms_trace = 0, ms_gemm = 0, ms_ss = 0, ms_total = 0, ms_walk = 0;
    uint64_t launches = 0, chunks = 0;
    bool timing = true;
    size_t budget = 0;    // device bytes for the chunk buffers; 0: min(32 GiB, a quarter of free memory)
    uint32_t tuned_chunk = 0;   // paths per chunk chosen by sstmc_scene_autotune (0: from the budget)
    bool fixed = false;   // buffers carved from a fixed scratch: a chunk that outgrows them fails, nothing is allocated

    static size_t bytes_per_path(const Scene& S);
    int ensure(Scene& S, uint32_t paths);
    void release();
    int prepare_ss_tables(Scene& S);
    void plan(const Scene& S, TraceParams& T, std::vector<std::pair<int, int>>* vchunks,
              std::vector<std::pair<int, int>>* tchunks) const;
    int trace_chunk(Scene& S, uint64_t seed, uint32_t first, uint32_t n, PathDebug* dbg);
    int contract_chunk(Scene& S, uint32_t n);
    // limit: render only the first `limit` paths (0: all), for the autotuner's samples
    int render_one(Scene& S, uint64_t seed, double* u_out, double* iter_out, uint64_t limit = 0);
    int init_events();
    void destroy_events();
};

}  // namespace sstmc

struct sstmc_scene;

namespace sstmc {

// Render entry shared by sstmc_render and the server (api.cpp).
int32_t render_scene(sstmc_scene* s, uint64_t seed, double* u_out, double* iter_out, size_t budget, bool release_after,
                     uint64_t* contributions);
size_t scene_request_bytes(const sstmc_scene* s, size_t cap);
int scene_device(const sstmc_scene* s);

// sstmc_render with every device buffer in a static scratch (static_render.cu).
int render_static(Scene& S, cudaStream_t stream, uint64_t seed, double* u_out, double* iter_out);

int occupancy_blocks(const DevScene& S, int threads, size_t smem);
void set_last_error_text(const std::string& s);

}  // namespace sstmc
