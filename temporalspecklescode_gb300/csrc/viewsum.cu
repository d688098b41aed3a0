// viewsum.cu -- the view side of the multiple-scattering term, summed over
// each path's vertices b >= 2 (multipleResMultiple's GvSum,
// NextEventEstimation.cuh:1138-1395, with the per-vertex view vectors of
// TemporalSampler.cuh:668-719 / TemporalSamplerCorrelation.cuh:384-450):
//
//   field sampler (no material moves, so every tick sees the same vertices):
//     S[v] = sum_b g_v(x_b) f_v(x_{b-1} -> x_b) exp(2 pi i (L_b / lambda + xi_b))
//   correlation sampler with identical u1 / u2 sources and static scatterers:
//     S[v][t] = sum_b |g_v(x_b)|^2 pdf(x_{b-1} -> x_b -> v)
//               exp(-k^2 |t| (D_b |q_bv|^2 + sum_{c<b} D_c |q_c|^2))
//
// One warp per path.  The warp first turns a block of 32 vertices into
// shared-memory records, lane = vertex: position, unit incoming direction,
// material, and either the momentum-transfer prefix (correlation) or the
// path phase L_b / lambda + xi_b reduced modulo one cycle in FP64 (field),
// both prefixes formed with warp scans.  Then each lane owns views
// v0 + lane + 32 j and keeps their tick accumulators in registers while it
// walks the block's records (shared-memory broadcasts), so nothing is read
// or written per (vertex, view, tick) except registers.
//
// The general cases (moving scatterers, distinct u1 / u2 sources) stay in
// the fused trace kernel (trace.cu).
#include <cuda_runtime.h>

#include "nee.cuh"
#include "trace.h"
#include "viewsum.h"

namespace sstmc {

namespace {

constexpr int kVB = 32;     // vertices per block
constexpr int kNT = 8;      // ticks per pass (correlation)
constexpr int kVPL = 4;     // views per lane per pass

struct VRec {
    float x, y, z;
    float ux, uy, uz;       // unit direction x_{b-1} -> x_b
    float mt;               // correlation: k^2 sum_{3 <= c <= b} D_{m(c-1)} |u_{c-1} - u_c|^2
    uint32_t m;             // material | inside << 8
    double ph;              // field: L_b / lambda + xi_b reduced to [-1/2, 1/2] cycles
};

template <bool CORR, bool VWP>
__global__ void __launch_bounds__(128) view_kernel(const __grid_constant__ DevScene S, const __grid_constant__ TraceParams T)
{
    extern __shared__ __align__(16) unsigned char vsm[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    VRec* rec = reinterpret_cast<VRec*>(vsm) + (size_t)wib * kVB;
    float* tk = reinterpret_cast<float*>(reinterpret_cast<VRec*>(vsm) + (size_t)(blockDim.x >> 5) * kVB);
    const int Nt = S.Nt, Nv = S.src[1].n;
    for (int t = threadIdx.x; t < Nt; t += blockDim.x) tk[t] = S.abs_ticks[t];
    __syncthreads();
    const DevSource& vw = S.src[1];
    const bool split = S.precision == SSTMC_PRECISION_SPLIT;
    const bool geo = S.ticks_geometric != 0;
    const int t0 = T.t0, tn = T.tn;
    const int nv = T.vn;
    // ray steps per (vertex, view): one ray per tick (u1 and u2 for the correlation sampler)
    const uint32_t rays = (uint32_t)(CORR ? 2 * tn : tn);

    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t q = gw; q < T.paths; q += nw) {
        const uint32_t B = T.counts[q];
        const float4* vq = T.verts + T.offsets[q];
        float acc[kVPL][CORR ? kNT : 2];
#pragma unroll
        for (int j = 0; j < kVPL; ++j)
#pragma unroll
            for (int k = 0; k < (CORR ? kNT : 2); ++k) acc[j][k] = 0.0f;
        uint32_t steps = 0;
        float mt_carry = 0.0f;
        double l_carry = 0.0;
        for (uint32_t base = 2; base <= B; base += kVB) {
            const int nb = (int)min((uint32_t)kVB, B - base + 1);
            // ---- vertex records, lane = vertex b = base + lane ----
            {
                const uint32_t b = base + (uint32_t)lane;
                const bool act = lane < nb;
                float dmt = 0.0f;
                double seg = 0.0;
                if (act) {
                    const float4 c = vq[b - 1], p = vq[b - 2];
                    const V3 xc = V3{ c.x, c.y, c.z }, xp = V3{ p.x, p.y, p.z };
                    const V3 u = funit(sub3(xc, xp));
                    VRec r;
                    r.x = c.x; r.y = c.y; r.z = c.z; r.ux = u.x; r.uy = u.y; r.uz = u.z;
                    r.m = (__float_as_uint(c.w) & 15u) | (inside(S, xc) ? 256u : 0u);
                    r.mt = 0.0f;
                    r.ph = (double)((float)(__float_as_uint(c.w) >> 4) * (1.0f / 16777216.0f));   // xi_b
                    if (CORR && b >= 3) {
                        const float4 pp = vq[b - 3];
                        const V3 up = funit(sub3(xp, V3{ pp.x, pp.y, pp.z }));
                        const V3 dq = sub3(up, u);
                        dmt = S.D[__float_as_uint(p.w) & 15u] * dot3(dq, dq);
                    }
                    if (!CORR) {
                        if (split) {
                            const double dx = (double)c.x - (double)p.x, dy = (double)c.y - (double)p.y, dz = (double)c.z - (double)p.z;
                            seg = sqrt(fma(dx, dx, fma(dy, dy, dz * dz)));
                        } else {
                            const V3 dd = sub3(xc, xp);
                            seg = (double)sqrtf(dot3(dd, dd));
                        }
                    }
                    rec[lane] = r;
                }
                if constexpr (CORR) {
                    float s = dmt;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) { const float n = __shfl_up_sync(0xffffffffu, s, o); if (lane >= o) s += n; }
                    if (act) rec[lane].mt = S.k2 * (mt_carry + s);
                    mt_carry += __shfl_sync(0xffffffffu, s, 31);
                } else {
                    if (split) {
                        double s = seg;
#pragma unroll
                        for (int o = 1; o < 32; o <<= 1) { const double n = __shfl_up_sync(0xffffffffu, s, o); if (lane >= o) s += n; }
                        if (act) {
                            const double ph = (l_carry + s) * S.inv_lambda + rec[lane].ph;
                            rec[lane].ph = ph - rint(ph);
                        }
                        l_carry += __shfl_sync(0xffffffffu, s, 31);
                    } else {
                        float s = (float)seg;
#pragma unroll
                        for (int o = 1; o < 32; o <<= 1) { const float n = __shfl_up_sync(0xffffffffu, s, o); if (lane >= o) s += n; }
                        if (act) {
                            const float ph = ((float)l_carry + s) * S.inv_lambda_f + (float)rec[lane].ph;
                            rec[lane].ph = (double)(ph - rintf(ph));
                        }
                        l_carry = (double)((float)l_carry + __shfl_sync(0xffffffffu, s, 31));
                    }
                }
            }
            __syncwarp();
            // ---- views of this lane over the block's vertices ----
#pragma unroll
            for (int j = 0; j < kVPL; ++j) {
                const int vi = lane + 32 * j;
                if (vi >= nv) break;
                const int v = T.v0 + vi;
                const V3 sv = load3(vw.p, v);
                for (int i = 0; i < nb; ++i) {
                    const VRec r = rec[i];
                    const V3 xb = V3{ r.x, r.y, r.z };
                    const V3 ub = V3{ r.ux, r.uy, r.uz };
                    const int mb = (int)(r.m & 15u);
                    const bool xin = (r.m & 256u) != 0;
                    // direction to the view and optical depth toward it
                    V3 o;
                    float tau = 0.0f, r2 = 1.0f;
                    uint32_t st = 0;
                    if constexpr (VWP) {
                        const V3 d = sub3(sv, xb);
                        r2 = dot3(d, d);
                        const float ri = rsqrtf(r2);
                        o = V3{ d.x * ri, d.y * ri, d.z * ri };
                        if (S.single) { if (xin) { st = 1; tau = tau_single(S, xb, o); } }
                        else tau = tau_to_point(S, xb, sv, st);
                    } else {
                        o = sv;
                        if (S.single) { if (xin) { st = 1; tau = tau_single(S, xb, o); } }
                        else tau = tau_dir(S, xb, o, st);
                    }
                    steps += st * rays;
                    const V3 df = sub3(ub, o);
                    const float q2 = dot3(df, df);
                    if constexpr (CORR) {
                        // |g|^2 (PointSource.cuh:117-172 / FarField.cuh:223-263) times the pdf
                        float w = __expf(-tau);
                        if constexpr (VWP) {
                            w = S.dims == 3 ? __fdividef(w * kIsoAmp3, r2) : w * rsqrtf(r2);
                            if (vw.is_area) w *= fabsf(S.dims == 3 ? sub3(xb, sv).z : sub3(xb, sv).y) * rsqrtf(r2);
                        }
                        float pdf;
                        if (VWP && S.iso_all) pdf = S.iso_amp * S.iso_amp;
                        else {
                            const int ty = S.scat_type[mb];
                            if (ty == SSTMC_SCATTERING_ISOTROPIC) pdf = S.iso_pdf;
                            else if (ty == SSTMC_SCATTERING_HENYEY_GREENSTEIN) {
                                const float g = S.g[mb], omg = 1.0f - g;
                                const float rr = rsqrtf(fmaf(g, q2, omg * omg));
                                pdf = S.dims == 2 ? S.gup[mb] * rr * rr : S.gup[mb] * rr * rr * rr;
                            } else pdf = 0.0f;
                        }
                        // decorrelation exp(-k^2 |t| (D_b |q|^2 + MT_b)), q = u_b - o (TemporalSamplerCorrelation.cuh:384-450)
                        const float ck = fmaf(S.k2 * S.D[mb], q2, r.mt);
                        const float base_w = w * pdf;
                        if (geo) {
                            const float es = __expf(-ck * tk[0]);
                            float e = t0 == 0 ? es : __expf(-ck * tk[t0]);
#pragma unroll
                            for (int k = 0; k < kNT; ++k)
                                if (k < tn) { acc[j][k] = fmaf(base_w, e, acc[j][k]); e *= es; }
                        } else {
#pragma unroll
                            for (int k = 0; k < kNT; ++k)
                                if (k < tn) acc[j][k] = fmaf(base_w, __expf(-ck * tk[t0 + k]), acc[j][k]);
                        }
                    } else {
                        // g f exp(2 pi i (phase of g + L_b / lambda + xi_b))
                        float a, f;
                        if constexpr (VWP) {
                            float at = __expf(-tau);
                            at = S.dims == 3 ? __fdividef(at * kIsoAmp3, r2) : at * rsqrtf(r2);
                            if (vw.is_area) at *= fabsf(S.dims == 3 ? sub3(xb, sv).z : sub3(xb, sv).y) * rsqrtf(r2);
                            a = sqrtf(at);
                            if (split) {
                                const double dx = (double)xb.x - (double)sv.x, dy = (double)xb.y - (double)sv.y, dz = (double)xb.z - (double)sv.z;
                                const double ph = sqrt(fma(dx, dx, fma(dy, dy, dz * dz))) * S.inv_lambda + r.ph;
                                f = (float)(ph - rint(ph));
                            } else {
                                const float ph = sqrtf(r2) * S.inv_lambda_f + (float)r.ph;
                                f = ph - rintf(ph);
                            }
                        } else {
                            a = sqrtf(__expf(-tau));
                            if (split) {
                                const double dx = fma((double)o.x, (double)xb.x, fma((double)o.y, (double)xb.y, (double)o.z * (double)xb.z));
                                const double ph = r.ph - dx * S.inv_lambda;
                                f = (float)(ph - rint(ph));
                            } else {
                                const float ph = (float)r.ph - (o.x * xb.x + o.y * xb.y + o.z * xb.z) * S.inv_lambda_f;
                                f = ph - rintf(ph);
                            }
                        }
                        float amp;
                        if (VWP && S.iso_all) amp = S.iso_amp;
                        else {
                            const int ty = S.scat_type[mb];
                            if (ty == SSTMC_SCATTERING_ISOTROPIC) amp = S.iso_amp;
                            else if (ty == SSTMC_SCATTERING_HENYEY_GREENSTEIN) {
                                const float g = S.g[mb], omg = 1.0f - g;
                                const float rr = rsqrtf(fmaf(g, q2, omg * omg));
                                amp = S.dims == 2 ? S.sgup[mb] * rr : S.sgup[mb] * rr * sqrtf(rr);
                            } else amp = 0.0f;
                        }
                        float sp, cp;
                        sincospif(2.0f * f, &sp, &cp);
                        const float m = a * amp;
                        acc[j][0] = fmaf(m, cp, acc[j][0]);
                        acc[j][1] = fmaf(m, sp, acc[j][1]);
                    }
                }
            }
            __syncwarp();
        }
        // ---- write S[q][t][v] ----
#pragma unroll
        for (int j = 0; j < kVPL; ++j) {
            const int vi = lane + 32 * j;
            if (vi >= nv) break;
            const int v = T.v0 + vi;
            if constexpr (CORR) {
#pragma unroll
                for (int k = 0; k < kNT; ++k)
                    if (k < tn) T.s_ms[((size_t)q * Nt + t0 + k) * Nv + v] = make_float2(acc[j][k], 0.0f);
            } else {
                const float2 c = make_float2(acc[j][0], acc[j][1]);
                for (int t = t0; t < t0 + tn; ++t) T.s_ms[((size_t)q * Nt + t) * Nv + v] = c;
            }
        }
        const uint32_t ws = warp_sum_u32(steps);
        if (lane == 0 && ws) {
            if (T.dda) atomicAdd(T.dda + q, ws);
            atomicAdd(T.totals + 1, (unsigned long long)ws);
        }
    }
}

}  // namespace

size_t view_smem_bytes(int Nt, int threads)
{
    return (size_t)(threads / 32) * kVB * sizeof(VRec) + (size_t)Nt * sizeof(float);
}

int view_max_ticks(const DevScene& S) { return S.correlation ? kNT : S.Nt; }
int view_max_views() { return 32 * kVPL; }

bool view_kernel_covers(const DevScene& S, const bool* moving_any)
{
    if (S.correlation) return S.sym && S.all_static_corr;
    return !*moving_any;
}

int launch_view(const DevScene& S, const TraceParams& T, int blocks, int threads, cudaStream_t stream)
{
    const size_t smem = view_smem_bytes(S.Nt, threads);
    const bool vp = S.src[1].type == SSTMC_SOURCE_POINT;
    using Fn = void (*)(DevScene, TraceParams);
    Fn f = S.correlation ? (vp ? (Fn)view_kernel<true, true> : (Fn)view_kernel<true, false>)
                         : (vp ? (Fn)view_kernel<false, true> : (Fn)view_kernel<false, false>);
    if (smem > 48 * 1024 && cudaFuncSetAttribute((const void*)f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return SSTMC_KERNEL_ERROR;
    f<<<blocks, threads, smem, stream>>>(S, T);
    return cudaGetLastError() == cudaSuccess ? SSTMC_NO_ERROR : SSTMC_KERNEL_ERROR;
}

}  // namespace sstmc
