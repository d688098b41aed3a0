// trace.h -- launch interface of the path-tracing kernel (trace.cu).
#pragma once
#include <cuda_runtime.h>

#include "scene.h"

namespace sstmc {

// One launch traces paths [first_path, first_path + paths) of a rendering.
// Path id = wave * batchSize + slot.  Rows are indexed by q = id - first_path.
struct TraceParams {
    uint64_t seed;
    uint32_t first_path, paths;
    int pass0;            // 1: write the illumination rows, single-scattering rows and stats
    int views;            // 1: also sum the view vectors (s_ms); 0: they come from the view-side kernel (viewsum.cu)
    int ss_all_ticks;     // illum_kernel: write the tick-invariant single-scattering rows for every tick (else tick 0 only)
    int v0, vn, t0, tn;   // view / tick chunk accumulated by this pass
    int vw, tg, tpl;      // lanes: view = v0 + lane % vw + vw*j, tick = t0 + lane / vw + tg*k, k < tpl
    int slots;            // accumulator slots per lane (vpl * tpl)
    int lw, lg;           // illumination-side lane split (all ticks)
    int vwa, tga;         // single-scattering view-side lane split (all views, all ticks)
    const float4* verts;      // vertices of the walk (pathwalk.cu), path q at offsets[q]
    const uint32_t* counts;   // [paths] vertices (0: the walk hit a limit)
    const uint32_t* offsets;  // [paths]
    const uint32_t* misses;   // [paths]
    float2* a_ms;         // [paths][Nt][Nl]
    float2* s_ms;         // [paths][Nt][Nv]
    float2* a_ss;         // [paths][Nt][Nl]
    float2* b_ss;         // [paths][Nt][Nv]
    float2* g2;           // [paths][Nt][Nl] (correlation scratch)
    float* pl;            // [paths][Nl] first-point probability terms
    float* x1;            // [paths][3]
    float* x1t;           // [paths][Nt][3] or null
    unsigned char* m1;    // [paths]
    uint32_t* dda;        // [paths] or null (accumulated over passes)
    unsigned long long* totals;  // [0] vertices, [1] dda steps, [2] misses, [3] paths
    int* err;
    uint32_t* work;       // [1] or null: path counter of the warp-per-path kernels (zeroed by their launchers)
    int real_rows;        // illum_kernel / view_kernel: a_ms and s_ms hold real floats [paths][Nt][Nl or Nv]
    int cbs;              // field CBS, reversed pass (trace_kernel): s_ms <- Gv0 [paths][Nt][Nv] (pass0),
                          // a_ms <- GlSum [paths][Nt][Nl]; v0 / vn then index illumination elements
    float* p2;            // [paths] or null: the correlation sampler's second-point probability (CBS)
    const uint32_t* ss_row;   // [paths] or null: row of path q in a_ss / b_ss (paths grouped by first-vertex
                              // material for the far-field x far-field contraction); null: row q
    // view passes: long paths in segments of `seg` vertices (0: whole paths).  A path's own launch sums vertices 2 .. seg + 1; a second
    // launch with seg_mode = 1 takes (path, k) items from seg_list and adds the
    // sums of vertices 2 + k seg .. 1 + (k + 1) seg to the path's rows.
    uint32_t seg;
    int seg_mode;
    const uint2* seg_list;
    const uint32_t* seg_len;  // [1] items in seg_list
    uint32_t* seg_next;       // [1] items taken (zeroed before each segment launch)
};

// The (path, k) items of the paths longer than seg + 1 vertices (trace.cu).
int launch_seg_list(const uint32_t* counts, uint32_t n, uint32_t seg, uint2* list, uint32_t cap, uint32_t* len,
                    cudaStream_t stream);

// Correlation-sampler CBS cross terms (trace.cu, cbs_corr_kernel): V +=
// 0.5 (T2 + T3 + T4) over the paths [0, K) of a chunk.
struct CbsCorrParams {
    const float4* verts;
    const uint32_t* counts;
    const uint32_t* offsets;
    const float* p2;      // [K]
    double2* V;           // [Nt][Nv][Nl]
    int K, kchunk;
};
int launch_cbs_corr(const DevScene& S, const CbsCorrParams& P, cudaStream_t stream);

size_t trace_smem_bytes(int Nt, int slots, int threads);
// Gaussian-beam scenes (3D field sampler): every row of a path in one warp
size_t gauss_trace_smem_bytes(int Nt, int threads);
int launch_gauss_trace(const DevScene& S, const TraceParams& T, int threads, cudaStream_t stream);
int launch_trace(const DevScene& S, const TraceParams& T, int blocks, int threads, cudaStream_t stream);

}  // namespace sstmc
