/*
 * sstmc_oracle.h -- TEST INFRASTRUCTURE: the CPU oracle of the NEE speckle
 * path tracer.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline call it, as the checker; the product never links it.
 *
 * It restates the reference estimator (NextEventEstimation::trace,
 * NextEventEstimation.cuh:1461-1637, with the TemporalSampler and
 * TemporalCorrelationSampler of TemporalSampler.cuh / TemporalSamplerCorrelation.cuh)
 * per path: the random walk is sampled in FP32 with the same arithmetic
 * specification as the GPU walk (so vertex positions, materials, voxel
 * steps and termination counts agree bit for bit), and every NEE quantity,
 * attenuation, phase, probability and the illumination x view accumulation
 * is evaluated in FP64 on those vertices.
 *
 * Parity against the reference implementation itself is statistical only:
 * the reference draws from cuRAND XORWOW streams keyed by thread slot,
 * which cannot be reproduced here; the oracle uses Philox4x32-10 keyed by
 * (seed, path, vertex, purpose).  See tests/test_oracle_pins.py for the
 * known-answer checks that pin the oracle.
 */
#ifndef SSTMC_ORACLE_H
#define SSTMC_ORACLE_H

#include "../include/sstmc.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Render `waves` waves of batch_size paths starting at wave `first_wave`
 * for ONE rendering with the given seed.  u_out: 2*Nl*Nv*Nt doubles
 * (accumulated sum, not normalised), iter_out: batch_size*waves + misses.
 * stats (may be NULL): [0] contributions, [1] dda steps, [2] vertices, [3] paths.
 * threads <= 0: all OpenMP threads. */
int32_t oracle_render(const sstmc_config* cfg, uint64_t seed, uint32_t first_wave,
                      uint32_t waves, int32_t threads, double* u_out, double* iter_out,
                      uint64_t* stats);

/* Per-path quantities of paths [first_path, first_path + paths). */
int32_t oracle_trace_paths(const sstmc_config* cfg, uint64_t seed, uint32_t first_path,
                           uint32_t paths, sstmc_path_trace* out);

/* Known-answer helpers. */
/* FP32 voxel traversal from o along d: returns steps, writes optical depth (FP64). */
int32_t oracle_dda(const sstmc_config* cfg, const float* o, const float* d, double* tau32, double* tau64);
/* Scattering amplitude and pdf of material m at cosine c (FP64). */
int32_t oracle_phase(const sstmc_config* cfg, int32_t m, double c, double* amp, double* pdf);
/* complex scattering amplitude of material m at cosine c (tabular: the table entry) */
int32_t oracle_amplitude(const sstmc_config* cfg, int32_t m, double c, double* re, double* im);
/* Sample `n` scattering cosines of material m (FP32 walk arithmetic). */
int32_t oracle_sample_cos(const sstmc_config* cfg, int32_t m, uint64_t seed, uint32_t n, float* out);
/* Field sampler: per-tick positions xt [Nt x 3] and tick weights w [Nt] of a
 * vertex at x of material m (path pid, vertex b >= 1); *r = the tick forced onto
 * x (isForcedInsideBin), -1 when there is none. */
int32_t oracle_tick_positions(const sstmc_config* cfg, uint64_t seed, uint32_t pid, uint32_t b, const float* x,
                              int32_t m, float* xt, float* w, int32_t* r);
/* Gaussian beams (3D): the source terms of illumination beam l and view beam
 * v at scatterer x1 (material m1) with the path on to x2:
 * out[0] P_l(x1), out[1] the second-direction density p_l(x1 -> x2),
 * out[2..3] f_l(x1 -> x2), out[4..5] f_v(x2 -> x1) (x1 the view's vertex),
 * out[6..7] fs(l, v, x1), out[8] g_l(x1), out[9] g_v(x1). */
int32_t oracle_gauss_terms(const sstmc_config* cfg, int32_t l, int32_t v, const float* x1, int32_t m1,
                           const float* x2, double* out);
/* n first vertices of beam-sampled paths (misses included: material 0) and,
 * per vertex, a second direction drawn for its beam at it: xyz[n x 3],
 * mat[n], beam[n], dir[n x 3].  x1_fixed (may be NULL): every draw at this
 * vertex for beam beam_fixed (the second direction only). */
int32_t oracle_gauss_sample(const sstmc_config* cfg, uint64_t seed, uint32_t n, const float* x1_fixed, int32_t beam_fixed,
                            float* xyz, int32_t* mat, int32_t* beam, float* dir);

/* The complex modified Bessel function I0 of the 2D beam amplitudes. */
void oracle_bessel_i0(double re, double im, double* out_re, double* out_im);

/* Portable FP32 math of the decision path, for bit-level tests. */
float oracle_logf(float x);
void oracle_sincospif(float x, float* s, float* c);
void oracle_philox(const uint32_t key[2], const uint32_t ctr[4], uint32_t out[4]);

#ifdef __cplusplus
}
#endif
#endif
