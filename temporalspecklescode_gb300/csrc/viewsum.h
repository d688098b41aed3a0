// viewsum.h -- launch interface of the view-side kernel (viewsum.cu).
#pragma once
#include <cuda_runtime.h>

#include "scene.h"
#include "trace.h"

namespace sstmc {

// True when the view-side kernel handles the scene: the correlation sampler
// with identical u1 / u2 sources and no drifting material, or the field
// sampler with no moving material (moving_any: some material of the grid moves).
bool view_kernel_covers(const DevScene& S, const bool* moving_any);
// Largest tick and view chunk of one launch.
int view_max_ticks(const DevScene& S);
int view_max_views(const DevScene& S);
size_t view_smem_bytes(int Nt, int threads);
// S[q][t][v] for t in [T.t0, T.t0 + T.tn), v in [T.v0, T.v0 + T.vn).
int launch_view(const DevScene& S, const TraceParams& T, int blocks, int threads, cudaStream_t stream);
// Illumination side (P_l, a_ms, a_ss, b_ss, first-vertex stats) of the
// correlation sampler with identical u1 / u2 sources and static scatterers,
// Nl <= 256.
bool illum_kernel_covers(const DevScene& S);
int launch_illum(const DevScene& S, const TraceParams& T, int blocks, int threads, cudaStream_t stream);

}  // namespace sstmc
