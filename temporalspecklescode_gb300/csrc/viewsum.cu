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

#include <algorithm>

#include "nee.cuh"
#include "trace.h"
#include "viewsum.h"

namespace sstmc {

namespace {

constexpr int kVB = 32;     // vertices per block
constexpr int kNT = 8;      // ticks per pass (correlation)
constexpr int kVPL = 4;     // views per lane per pass (field)
constexpr int kVPP = 1;     // view pairs per lane per pass (correlation: 64 views, registers for 5 blocks of 128 threads)
constexpr int kMaxIllum = 8;   // illumination elements per lane (illumination side: Nl <= 256)

struct VRec {
    float x, y, z, mt;      // position; correlation: k^2 sum_{3 <= c <= b} D_{m(c-1)} |u_{c-1} - u_c|^2
    float ux, uy, uz, k2d;  // unit direction x_{b-1} -> x_b; k^2 D_{m(b)}
    float g, omg2, c, sig;  // phase-function constants: pdf or amplitude = c (omg2 + g q^2)^(-e); sig: sigma_t inside the box, else 0
    float nx0, nx1, ny0, ny1;   // distances to the box faces: x - bmin, bmax - x (single-cell media)
    float nz0, nz1;
    uint32_t in;            // 1 inside the box
    float ph_h, ph_l;       // field: L_b / lambda + xi_b reduced to [-1/2, 1/2] cycles, as a float pair
    uint32_t cell;          // packed grid cell of the position (multi-cell media), the start of every view's traversal
};


// Correlation-sampler vertex record: the operands of the packed (two views
// per instruction) inner loop are stored twice, so a 128-bit shared-memory
// broadcast yields f32x2 operands directly.
struct __align__(16) CRec {
    float x, x_, y, y_;         // position
    float z, z_, ux, ux_;       // unit direction x_{b-1} -> x_b
    float uy, uy_, uz, uz_;
    float k2d, k2d_, mt, mt_;   // k^2 D_{m(b)}; k^2 sum_{3 <= c <= b} D_{m(c-1)} |u_{c-1} - u_c|^2
    float g, g_, omg2, omg2_;   // pdf = cw (omg2 + g q^2)^(-(D-1)/2)
    float cw, cw_, sig, sig_;   // cw: pdf coefficient (point views: times the point-source amplitude constant); sig: sigma_t inside
    float nx0, nx1, ny0, ny1;   // distances to the box faces: x - bmin, bmax - x (single-cell media)
    float nz0, nz1;
    uint32_t in, cell;          // cell: packed grid cell of the position (multi-cell media)
};
static_assert(sizeof(CRec) == 128, "CRec layout");

// PTX approximate transcendental instructions (flush-to-zero forms; the
// arguments here are never subnormal)
__device__ __forceinline__ float ex2_ftz(float x)
{
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rsqrt_ftz(float x)
{
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rcp_ftz(float x)
{
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// (face - x) / d along the axis, face = bmin or bmax by the sign of d (the
// reference's bdDistance, HeterogeneousMedium.cuh:269-383, for one cell)
// Packed FP32 pairs (Blackwell f32x2 FMA / MUL)
__device__ __forceinline__ unsigned long long pk2(float lo, float hi)
{
    return (unsigned long long)__float_as_uint(lo) | ((unsigned long long)__float_as_uint(hi) << 32);
}
__device__ __forceinline__ float pk_lo(unsigned long long v) { return __uint_as_float((uint32_t)v); }
__device__ __forceinline__ float pk_hi(unsigned long long v) { return __uint_as_float((uint32_t)(v >> 32)); }
__device__ __forceinline__ unsigned long long fma2(unsigned long long a, unsigned long long b, unsigned long long c)
{
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ unsigned long long mul2(unsigned long long a, unsigned long long b)
{
    unsigned long long d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ unsigned long long add2(unsigned long long a, unsigned long long b)
{
    unsigned long long d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ unsigned long long ex2_2(unsigned long long a) { return pk2(ex2_ftz(pk_lo(a)), ex2_ftz(pk_hi(a))); }
__device__ __forceinline__ unsigned long long rsqrt_2(unsigned long long a) { return pk2(rsqrt_ftz(pk_lo(a)), rsqrt_ftz(pk_hi(a))); }

// distance to the face the direction component d heads for: n0 = x - bmin
// (d < 0) or n1 = bmax - x, over |d| (|d| = 0: +inf, which fminf drops)
__device__ __forceinline__ float face_t(float d, float n0, float n1)
{
    return (d < 0.0f ? n0 : n1) * __fdividef(1.0f, fabsf(d));
}

// Illumination side of the correlation sampler with identical u1 / u2
// sources and static scatterers (the rows are real):
//   P_l   = first-point probability terms (pathProbabilitySingle, NEE.cuh:853-887)
//   a_ss  = |g_l(x1)|^2 / p1                     (single scattering)
//   b_ss  = |g_v(x1)|^2
//   a_ms  = |g_l(x1)|^2 pdf(l -> x1 -> x2) exp(-k^2 D |t| |q|^2) / p2
//           (pathProbabilityMultiple, NEE.cuh:889-1009; C1_l1l2 of
//            TemporalSamplerCorrelation.cuh:384-450)
// Lane l + 32 k of the path's warp.  Each row is written once; the
// single-scattering rows are tick-invariant, so only tick 0 is written
// unless every tick is asked for (T.ss_all_ticks).
// Optical depth from x toward the point s or along the direction d; single
// cell: inside the box, one step to the face the ray heads for.
template <bool SINGLE>
__device__ __forceinline__ float tau_pt(const DevScene& S, const V3& x, const V3& sp, bool xin, uint32_t& st)
{
    if constexpr (SINGLE) {
        if (!xin) return 0.0f;
        st += 1;
        return tau_single(S, x, funit(sub3(sp, x)));
    } else {
        return tau_to_point(S, x, sp, st);
    }
}

template <bool SINGLE>
__device__ __forceinline__ float tau_d(const DevScene& S, const V3& x, const V3& d, bool xin, uint32_t& st)
{
    if constexpr (SINGLE) {
        if (!xin) return 0.0f;
        st += 1;
        return tau_single(S, x, d);
    } else {
        return tau_dir(S, x, d, st);
    }
}

// Per-warp sums of the render statistics (lane 0 adds them to the global
// counters once, when the warp has no paths left).
struct WarpStats {
    unsigned long long vertices = 0, steps = 0, misses = 0, paths = 0;
    __device__ void flush(const TraceParams& T) const
    {
        if (vertices) atomicAdd(T.totals + 0, vertices);
        if (steps) atomicAdd(T.totals + 1, steps);
        if (misses) atomicAdd(T.totals + 2, misses);
        if (paths) atomicAdd(T.totals + 3, paths);
    }
};

template <int NLK, bool ilp, bool vwp, bool SINGLE>
__device__ __forceinline__ void illum_path(const DevScene& S, const TraceParams& T, uint32_t q, int lane,
                                           uint32_t B, const float4* vq, const V3 (&lsrc)[NLK], WarpStats& ws_acc)
{
    const int Nt = S.Nt, Nl = S.src[0].n, Nv = S.src[1].n;
    const DevSource& il = S.src[0];
    const DevSource& vw = S.src[1];
    const bool three = S.dims == 3;
    const bool geo = S.ticks_geometric != 0;
    const int tss = T.ss_all_ticks ? Nt : 1;
    float2* ams = T.a_ms + (size_t)q * Nt * Nl;
    float* amr = reinterpret_cast<float*>(T.a_ms) + (size_t)q * Nt * Nl;   // real rows
    const bool real = T.real_rows != 0;
    auto put_ams = [&](size_t i, float a) { if (real) amr[i] = a; else ams[i] = make_float2(a, 0.f); };
    const uint32_t qs = T.ss_row ? T.ss_row[q] : q;   // row of the single-scattering rows
    float2* ass = T.a_ss + (size_t)qs * Nt * Nl;
    float2* bss = T.b_ss + (size_t)qs * Nt * Nv;
    if (B == 0) {   // the walk hit a limit (error already flagged)
        for (int i = lane; i < Nt * Nl; i += 32) { put_ams(i, 0.f); ass[i] = make_float2(0.f, 0.f); }
        for (int i = lane; i < Nt * Nv; i += 32) bss[i] = make_float2(0.f, 0.f);
        return;
    }
    const float4 v1 = vq[0];
    const float4 v2 = vq[B >= 2 ? 1 : 0];
    const V3 x1 = V3{ v1.x, v1.y, v1.z };
    const int m1 = (int)(__float_as_uint(v1.w) & 15u);
    const bool xin = inside(S, x1);
    uint32_t steps = 0;
    // |g_l|^2 and P_l from one attenuation evaluation per element
    float wl[NLK], pl[NLK];
    float ps = 0.0f;
#pragma unroll
    for (int k = 0; k < NLK; ++k) {
        const int l = lane + 32 * k;
        wl[k] = 0.0f; pl[k] = 0.0f;
        if (32 * k < Nl && l < Nl) {
            uint32_t st = 0;
            float P, w;
            if constexpr (ilp) {
                const V3 sp = lsrc[k];
                const float Ta = __expf(-tau_pt<SINGLE>(S, x1, sp, xin, st));
                const V3 d = sub3(x1, sp);
                const float r2 = dot3(d, d);
                P = three ? __fdividef(Ta, (float)(4.0 * kPi) * r2) : Ta * (float)(8.0 * kPi) * rsqrtf(r2);
                w = three ? __fdividef(Ta * kIsoAmp3, r2) : Ta * rsqrtf(r2);
                if (il.is_area) w *= fabsf(three ? d.z : d.y) * rsqrtf(r2);
            } else {
                const V3 dr = lsrc[k];
                const float Ta = __expf(-tau_d<SINGLE>(S, x1, V3{ -dr.x, -dr.y, -dr.z }, xin, st));
                P = Ta * il.sprob[l];
                w = Ta;
            }
            // u1 and u2 rays (identical sources): the probability and every tick of the rows
            steps += 2 * st + 2 * st * (uint32_t)Nt;
            T.pl[(size_t)q * Nl + l] = P;
            pl[k] = P;
            ps += P;
            wl[k] = w;
        }
    }
    const float p1inv = 1.0f / (warp_sum(ps) / (float)Nl);
#pragma unroll
    for (int k = 0; k < NLK; ++k) {
        const int l = lane + 32 * k;
        if (32 * k < Nl && l < Nl)
            for (int t = 0; t < tss; ++t) ass[(size_t)t * Nl + l] = make_float2(wl[k] * p1inv, 0.f);
    }
    for (int v = lane; v < Nv; v += 32) {
        uint32_t st = 0;
        float w;
        if constexpr (vwp) {
            const V3 sp = load3(vw.p, v);
            const float Ta = __expf(-tau_pt<SINGLE>(S, x1, sp, xin, st));
            const V3 d = sub3(x1, sp);
            const float r2 = dot3(d, d);
            w = three ? __fdividef(Ta * kIsoAmp3, r2) : Ta * rsqrtf(r2);
            if (vw.is_area) w *= fabsf(three ? d.z : d.y) * rsqrtf(r2);
        } else {
            w = __expf(-tau_d<SINGLE>(S, x1, load3(vw.p, v), xin, st));
        }
        steps += 2 * st * (uint32_t)Nt;
        for (int t = 0; t < tss; ++t) bss[(size_t)t * Nv + v] = make_float2(w, 0.f);
    }
    // multiple-scattering illumination vector at x2
    if (B >= 2) {
        const V3 x2 = V3{ v2.x, v2.y, v2.z };
        const V3 x12 = funit(sub3(x2, x1));
        float ps2 = 0.0f;
        V3 i1s[NLK];
        float pdf1[NLK];
#pragma unroll
        for (int k = 0; k < NLK; ++k) {
            const int l = lane + 32 * k;
            i1s[k] = V3{ 0.f, 0.f, 1.f };
            pdf1[k] = 0.0f;
            if (32 * k < Nl && l < Nl) {
                i1s[k] = ilp ? funit(sub3(x1, lsrc[k])) : lsrc[k];
                pdf1[k] = pdf_fast(S, m1, i1s[k], x12);
                ps2 += pl[k] * pdf1[k];
            }
        }
        const float p2inv = 1.0f / (warp_sum(ps2) / (float)Nl);
        const float c1base = S.k2 * S.D[m1];
        const float tau0 = S.abs_ticks[0];
#pragma unroll
        for (int k = 0; k < NLK; ++k) {
            const int l = lane + 32 * k;
            if (!(32 * k < Nl && l < Nl)) continue;
            const V3 qv = sub3(i1s[k], x12);
            const float c1k = c1base * dot3(qv, qv);
            const float f12 = (ilp && S.iso_all) ? S.iso_amp * S.iso_amp : pdf1[k];
            const float base = wl[k] * f12 * p2inv;
            // tick t of element l at l + t Nl (real rows: floats, else (re, 0) pairs)
            if (geo) {
                const float es = __expf(-c1k * tau0);
                float e = es;
                if (real) {
                    float* o = amr + l;
#pragma unroll 4
                    for (int t = 0; t < Nt; ++t, o += Nl) { *o = base * e; e *= es; }
                } else {
                    float2* o = ams + l;
#pragma unroll 4
                    for (int t = 0; t < Nt; ++t, o += Nl) { *o = make_float2(base * e, 0.f); e *= es; }
                }
            } else {
                for (int t = 0; t < Nt; ++t) put_ams((size_t)t * Nl + l, base * __expf(-c1k * S.abs_ticks[t]));
            }
        }
    } else {
        for (int i = lane; i < Nt * Nl; i += 32) put_ams(i, 0.f);
    }
    const uint32_t ws = warp_sum_u32(steps);
    if (lane == 0) {
        if (T.m1) T.m1[q] = (unsigned char)m1;
        if (T.x1) { T.x1[3 * q] = x1.x; T.x1[3 * q + 1] = x1.y; T.x1[3 * q + 2] = x1.z; }
        if (T.dda && ws) atomicAdd(T.dda + q, ws);
        ws_acc.vertices += B;
        ws_acc.misses += T.misses[q];
        ws_acc.paths += 1;
        ws_acc.steps += ws;
    }
}

// One warp per path (a kernel of its own: it needs few registers, so many
// warps hide the latency of its row writes).
template <int NLK, bool ILP, bool VWP, bool SINGLE>
__global__ void __launch_bounds__(128, 8) illum_kernel(const __grid_constant__ DevScene S, const __grid_constant__ TraceParams T)
{
    const int lane = threadIdx.x & 31;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    // this lane's illumination elements (positions or directions), loaded once
    V3 lsrc[NLK];
#pragma unroll
    for (int k = 0; k < NLK; ++k) lsrc[k] = load3(S.src[0].p, min(lane + 32 * k, S.src[0].n - 1));
    WarpStats st;
    // a fixed stride: every path costs about the same here (Nl + Nv rays)
    for (uint32_t q = gw; q < T.paths; q += nw)
        illum_path<NLK, ILP, VWP, SINGLE>(S, T, q, lane, T.counts[q], T.verts + T.offsets[q], lsrc, st);
    if (lane == 0) st.flush(T);
}

// Multi-cell media: 5 blocks per SM (102 registers), measured faster than 6
// (80 registers, a few spills in the traversal) on the 64x64x32-grid workload;
// single-cell media keep 6.
template <bool CORR, bool VWP, bool SINGLE, bool THREE>
__global__ void __launch_bounds__(128, SINGLE ? 6 : 5) view_kernel(const __grid_constant__ DevScene S, const __grid_constant__ TraceParams T)
{
    extern __shared__ __align__(16) unsigned char vsm[];
    constexpr size_t kRecBytes = CORR ? sizeof(CRec) : sizeof(VRec);
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    VRec* rec = reinterpret_cast<VRec*>(vsm + (size_t)wib * kVB * kRecBytes);
    CRec* crec = reinterpret_cast<CRec*>(vsm + (size_t)wib * kVB * kRecBytes);
    float* tk = reinterpret_cast<float*>(vsm + (size_t)(blockDim.x >> 5) * kVB * kRecBytes);
    const int Nt = S.Nt, Nv = S.src[1].n;
    for (int t = threadIdx.x; t < Nt; t += blockDim.x) tk[t] = S.abs_ticks[t];
    __syncthreads();
    const DevSource& vw = S.src[1];
    const bool split = S.precision == SSTMC_PRECISION_SPLIT;
    const bool geo = S.ticks_geometric != 0;
    const bool three = THREE;
    const bool area = vw.is_area != 0;
    const int t0 = T.t0, tn = T.tn;
    const int nv = T.vn;
    const int vpl = (nv + 31) / 32;
    // ray steps per (vertex, view): one ray per tick (u1 and u2 for the correlation sampler)
    const uint32_t rays = (uint32_t)(CORR ? 2 * tn : tn);
    // this lane's views: position or direction, and (far field) the reciprocal direction
    constexpr int kVL = CORR ? 2 * kVPP : kVPL;   // views per lane
    V3 sv[kVL];
    V3 sinv[kVL];
#pragma unroll
    for (int j = 0; j < kVL; ++j) {
        const int vi = min(lane + 32 * j, nv - 1);
        sv[j] = load3(vw.p, T.v0 + vi);
        if (!VWP) sinv[j] = V3{ __fdividef(1.0f, fabsf(sv[j].x)), __fdividef(1.0f, fabsf(sv[j].y)), __fdividef(1.0f, fabsf(sv[j].z)) };
    }
    // correlation: views lane + 32 (2 P) and lane + 32 (2 P + 1) as f32x2 pairs
    unsigned long long pvx[kVPP], pvy[kVPP], pvz[kVPP];
#pragma unroll
    for (int P = 0; P < kVPP; ++P) {
        pvx[P] = pk2(sv[2 * P].x, sv[2 * P + 1].x);
        pvy[P] = pk2(sv[2 * P].y, sv[2 * P + 1].y);
        pvz[P] = pk2(sv[2 * P].z, sv[2 * P + 1].z);
    }
    // exponent constants: exp(-k^2 |t| C) = 2^(C * (-|t| log2 e))
    const float kLog2e = 1.44269504088896341f;
    const unsigned long long neg1 = pk2(-1.0f, -1.0f);
    const unsigned long long nl2e = pk2(-kLog2e, -kLog2e);
    const unsigned long long nt0 = pk2(-tk[0] * kLog2e, -tk[0] * kLog2e);
    const unsigned long long st0 = pk2((float)(t0 + 1), (float)(t0 + 1));   // geometric ticks: |t_t0| = (t0 + 1) |t_0|
    // views of this lane inside the chunk (lanes past its last view count no rays)
    const uint32_t nvalid = (uint32_t)max(0, min(kVL, (nv - lane + 31) / 32));

    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    unsigned long long warp_steps = 0;
    // warps start at their own path and then draw from T.work (path cost grows
    // with its vertex count); the draw for the next path is issued first so
    // its latency hides behind this path's work
    for (uint32_t q = gw; q < T.paths;) {
        uint32_t drawn = 0;
        if (T.work != nullptr && lane == 0) drawn = atomicAdd(T.work, 1u);
        const uint32_t B = T.counts[q];
        const float4* vq = T.verts + T.offsets[q];
        // correlation: ticks of a view pair packed (acc[P][t] = (view 2P, view 2P + 1));
        // field: (re, im) of each view
        unsigned long long acc[CORR ? kVPP : kVPL][CORR ? kNT : 1];
#pragma unroll
        for (int j = 0; j < (CORR ? kVPP : kVPL); ++j)
#pragma unroll
            for (int k = 0; k < (CORR ? kNT : 1); ++k) acc[j][k] = 0ull;
        uint32_t steps = 0;
        float mt_carry = 0.0f;
        double l_carry = 0.0;
        FF lc{ 0.0f, 0.0f };   // split field: path length before this block of vertices, a float pair
        for (uint32_t base = 2; base <= B; base += kVB) {
            const int nb = (int)min((uint32_t)kVB, B - base + 1);
            // ---- vertex records, lane = vertex b = base + lane ----
            {
                const uint32_t b = base + (uint32_t)lane;
                const bool act = lane < nb;
                float dmt = 0.0f;
                double seg = 0.0;
                FF segf{ 0.0f, 0.0f };
                if (act) {
                    const float4 c = vq[b - 1], p = vq[b - 2];
                    const V3 xc = V3{ c.x, c.y, c.z }, xp = V3{ p.x, p.y, p.z };
                    const V3 u = funit(sub3(xc, xp));
                    const int m = (int)(__float_as_uint(c.w) & 15u);
                    // pdf (correlation) or amplitude (field) of the phase function as
                    // c (omg2 + g q^2)^(-e): isotropic is g = 0, omg2 = 1
                    const int ty = S.scat_type[m];
                    float g = 0.0f, omg2 = 1.0f, cc = 0.0f;
                    if (VWP && S.iso_all) cc = CORR ? S.iso_amp * S.iso_amp : S.iso_amp;
                    else if (ty == SSTMC_SCATTERING_ISOTROPIC) cc = CORR ? S.iso_pdf : S.iso_amp;
                    else if (ty == SSTMC_SCATTERING_HENYEY_GREENSTEIN) {
                        g = S.g[m]; omg2 = (1.0f - g) * (1.0f - g); cc = CORR ? S.gup[m] : S.sgup[m];
                    }
                    const bool in = inside(S, xc);
                    const float sig = in ? S.sigt[S.grid_m0] : 0.0f;
                    if constexpr (CORR) {
                        CRec r;
                        r.x = r.x_ = c.x; r.y = r.y_ = c.y; r.z = r.z_ = c.z;
                        r.ux = r.ux_ = u.x; r.uy = r.uy_ = u.y; r.uz = r.uz_ = u.z;
                        r.k2d = r.k2d_ = S.k2 * S.D[m];
                        r.mt = r.mt_ = 0.0f;
                        r.g = r.g_ = g; r.omg2 = r.omg2_ = omg2;
                        // point views: |g_v|^2 = exp(-tau) kIsoAmp3 / r^2 (3D) or exp(-tau) / r (2D)
                        r.cw = r.cw_ = (VWP && THREE) ? cc * kIsoAmp3 : cc;
                        r.sig = r.sig_ = sig;
                        r.nx0 = c.x - S.bmin[0]; r.nx1 = S.bmax[0] - c.x;
                        r.ny0 = c.y - S.bmin[1]; r.ny1 = S.bmax[1] - c.y;
                        r.nz0 = c.z - S.bmin[2]; r.nz1 = S.bmax[2] - c.z;
                        r.in = in ? 1u : 0u;
                        r.cell = SINGLE ? kNoCell : cell_of(S, xc);
                        if (b >= 3) {
                            const float4 pp = vq[b - 3];
                            const V3 up = funit(sub3(xp, V3{ pp.x, pp.y, pp.z }));
                            const V3 dq = sub3(up, u);
                            dmt = S.D[__float_as_uint(p.w) & 15u] * dot3(dq, dq);
                        }
                        crec[lane] = r;
                    } else {
                        VRec r;
                        r.x = c.x; r.y = c.y; r.z = c.z; r.mt = 0.0f;
                        r.ux = u.x; r.uy = u.y; r.uz = u.z; r.k2d = S.k2 * S.D[m];
                        r.g = g; r.omg2 = omg2; r.c = cc;
                        r.in = in ? 1u : 0u;
                        r.cell = SINGLE ? kNoCell : cell_of(S, xc);
                        r.sig = sig;
                        r.nx0 = c.x - S.bmin[0]; r.nx1 = S.bmax[0] - c.x;
                        r.ny0 = c.y - S.bmin[1]; r.ny1 = S.bmax[1] - c.y;
                        r.nz0 = c.z - S.bmin[2]; r.nz1 = S.bmax[2] - c.z;
                        r.ph_h = (float)(__float_as_uint(c.w) >> 4) * (1.0f / 16777216.0f);   // xi_b, replaced below
                        r.ph_l = 0.0f;
                        if (split) {
                            segf = dist_ff(xc, xp);
                        } else {
                            const V3 dd = sub3(xc, xp);
                            seg = (double)sqrtf(dot3(dd, dd));
                        }
                        rec[lane] = r;
                    }
                }
                if constexpr (CORR) {
                    float s = dmt;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) { const float n = __shfl_up_sync(0xffffffffu, s, o); if (lane >= o) s += n; }
                    if (act) crec[lane].mt = crec[lane].mt_ = S.k2 * (mt_carry + s);
                    mt_carry += __shfl_sync(0xffffffffu, s, 31);
                } else {
                    if (split) {
                        // L_b / lambda + xi_b mod 1 in float-float (the path length's warp
                        // scan included): FP64 per vertex would cost more than all views' phases
                        FF s = segf;
#pragma unroll
                        for (int o = 1; o < 32; o <<= 1) {
                            const FF n{ __shfl_up_sync(0xffffffffu, s.h, o), __shfl_up_sync(0xffffffffu, s.l, o) };
                            if (lane >= o) s = add_ff(s, n);
                        }
                        if (act) {
                            const FF t = scale_ff(add_ff(lc, s), S.il_h, S.il_l);
                            const FF v = two_sum(fsb(t.h, rintf(t.h)), rec[lane].ph_h);   // t.h - rint(t.h) is exact; + xi_b
                            float h = fa(v.h, fa(v.l, t.l));
                            const float l = fsb(fa(v.l, t.l), fsb(h, v.h));
                            h = fsb(h, rintf(h));
                            rec[lane].ph_h = h;
                            rec[lane].ph_l = l;
                        }
                        lc = add_ff(lc, FF{ __shfl_sync(0xffffffffu, s.h, 31), __shfl_sync(0xffffffffu, s.l, 31) });
                    } else {
                        float s = (float)seg;
#pragma unroll
                        for (int o = 1; o < 32; o <<= 1) { const float n = __shfl_up_sync(0xffffffffu, s, o); if (lane >= o) s += n; }
                        if (act) {
                            const float ph = ((float)l_carry + s) * S.inv_lambda_f + rec[lane].ph_h;
                            rec[lane].ph_h = ph - rintf(ph);
                        }
                        l_carry = (double)((float)l_carry + __shfl_sync(0xffffffffu, s, 31));
                    }
                }
            }
            __syncwarp();
            if constexpr (CORR) {
                // ---- every vertex of the block against this lane's view pairs ----
                // |g_v|^2 pdf(u_b -> o) exp(-k^2 |t| (D_b |q|^2 + MT_b)), q = u_b - o
                // (PointSource.cuh:117-172 / FarField.cuh:223-263, TemporalSamplerCorrelation.cuh:384-450)
                for (int i = 0; i < nb; ++i) {
                    const CRec* cr = crec + i;
                    const ulonglong2 r0 = *reinterpret_cast<const ulonglong2*>(&cr->x);     // x, y
                    const ulonglong2 r1 = *reinterpret_cast<const ulonglong2*>(&cr->z);     // z, ux
                    const ulonglong2 r2 = *reinterpret_cast<const ulonglong2*>(&cr->uy);    // uy, uz
                    const ulonglong2 r3 = *reinterpret_cast<const ulonglong2*>(&cr->k2d);   // k2d, mt
                    const ulonglong2 r4 = *reinterpret_cast<const ulonglong2*>(&cr->g);     // g, omg2
                    const ulonglong2 r5 = *reinterpret_cast<const ulonglong2*>(&cr->cw);    // cw, sig
                    const float4 nf = *reinterpret_cast<const float4*>(&cr->nx0);
                    const float4 nz = *reinterpret_cast<const float4*>(&cr->nz0);
                    const uint32_t rin = __float_as_uint(nz.z);
                    const uint32_t rcell = __float_as_uint(nz.w);
                    if (SINGLE) steps += rin * rays * nvalid;
#pragma unroll
                    for (int P = 0; P < kVPP; ++P) {
                        if (2 * P >= vpl) break;
                        // direction to the views (unit) and optical depth toward them
                        unsigned long long ox, oy, oz, ri = 0ull;
                        if constexpr (VWP) {
                            const unsigned long long dx = fma2(r0.x, neg1, pvx[P]);
                            const unsigned long long dy = fma2(r0.y, neg1, pvy[P]);
                            const unsigned long long dz = THREE ? fma2(r1.x, neg1, pvz[P]) : 0ull;
                            const unsigned long long d2 = fma2(dx, dx, THREE ? fma2(dy, dy, mul2(dz, dz)) : mul2(dy, dy));
                            ri = rsqrt_2(d2);
                            ox = mul2(dx, ri); oy = mul2(dy, ri); oz = THREE ? mul2(dz, ri) : 0ull;
                        } else {
                            ox = pvx[P]; oy = pvy[P]; oz = pvz[P];
                        }
                        unsigned long long tau2;
                        if constexpr (SINGLE) {
                            float tm[2];
#pragma unroll
                            for (int h = 0; h < 2; ++h) {
                                const float oxh = h ? pk_hi(ox) : pk_lo(ox), oyh = h ? pk_hi(oy) : pk_lo(oy);
                                // distance to the face the direction heads for (|o| = 0: +inf, dropped by fminf)
                                const float ix = VWP ? rcp_ftz(fabsf(oxh)) : sinv[2 * P + h].x;
                                const float iy = VWP ? rcp_ftz(fabsf(oyh)) : sinv[2 * P + h].y;
                                float t = fminf((oxh < 0.0f ? nf.x : nf.y) * ix, (oyh < 0.0f ? nf.z : nf.w) * iy);
                                if (THREE) {
                                    const float ozh = h ? pk_hi(oz) : pk_lo(oz);
                                    const float iz = VWP ? rcp_ftz(fabsf(ozh)) : sinv[2 * P + h].z;
                                    t = fminf(t, (ozh < 0.0f ? nz.x : nz.y) * iz);
                                }
                                tm[h] = t;
                            }
                            tau2 = mul2(pk2(tm[0], tm[1]), r5.y);
                        } else {
                            float tt[2];
#pragma unroll
                            for (int h = 0; h < 2; ++h) {
                                const V3 xb = V3{ pk_lo(r0.x), pk_lo(r0.y), pk_lo(r1.x) };
                                uint32_t st = 0;
                                const V3 oh = V3{ h ? pk_hi(ox) : pk_lo(ox), h ? pk_hi(oy) : pk_lo(oy), h ? pk_hi(oz) : pk_lo(oz) };
                                tt[h] = VWP ? tau_to_point(S, xb, sv[2 * P + h], st, rcell) : tau_dir(S, xb, oh, st, rcell);
                                steps += (lane + 32 * (2 * P + h) < nv) ? st * rays : 0u;
                            }
                            tau2 = pk2(tt[0], tt[1]);
                        }
                        // q = u_b - o, pdf = cw (omg2 + g q^2)^(-(D-1)/2)
                        const unsigned long long qx = fma2(ox, neg1, r1.y);
                        const unsigned long long qy = fma2(oy, neg1, r2.x);
                        const unsigned long long qz = THREE ? fma2(oz, neg1, r2.y) : 0ull;
                        const unsigned long long q2 = fma2(qx, qx, THREE ? fma2(qy, qy, mul2(qz, qz)) : mul2(qy, qy));
                        // factors that do not wait for the rsqrt first, then r^(D-1) c
                        // as (r r)(r c) (3D): two levels of products after the rsqrt
                        unsigned long long cf = r5.x;
                        if constexpr (VWP) {
                            cf = mul2(cf, THREE ? mul2(ri, ri) : ri);
                            if (area) {
                                const unsigned long long oa = THREE ? oz : oy;
                                cf = mul2(cf, pk2(fabsf(pk_lo(oa)), fabsf(pk_hi(oa))));
                            }
                        }
                        const unsigned long long rr = rsqrt_2(fma2(r4.x, q2, r4.y));
                        const unsigned long long wgt = THREE ? mul2(mul2(rr, rr), mul2(rr, cf)) : mul2(mul2(rr, rr), cf);
                        // decorrelation exponent C = D_b |q|^2 + MT_b, exp(-tau) folded into the first factor
                        const unsigned long long ck = fma2(r3.x, q2, r3.y);
                        const unsigned long long tl = mul2(tau2, nl2e);
                        if (geo) {
                            const unsigned long long as = mul2(ck, nt0);
                            const unsigned long long es = ex2_2(as);
                            const unsigned long long e = mul2(wgt, ex2_2(add2(tl, t0 == 0 ? as : mul2(as, st0))));
                            // e es^k for the pass's 8 ticks as a depth-3 product tree
                            // rather than a serial chain of products
                            static_assert(kNT == 8, "tick tree written for 8 ticks");
                            const unsigned long long s2 = mul2(es, es), s4 = mul2(s2, s2);
                            const unsigned long long e1 = mul2(e, es), e2 = mul2(e, s2), e3 = mul2(e1, s2);
                            acc[P][0] = add2(acc[P][0], e); acc[P][1] = add2(acc[P][1], e1);
                            acc[P][2] = add2(acc[P][2], e2); acc[P][3] = add2(acc[P][3], e3);
                            acc[P][4] = add2(acc[P][4], mul2(e, s4)); acc[P][5] = add2(acc[P][5], mul2(e1, s4));
                            acc[P][6] = add2(acc[P][6], mul2(e2, s4)); acc[P][7] = add2(acc[P][7], mul2(e3, s4));
                        } else {
#pragma unroll
                            for (int k = 0; k < kNT; ++k) {
                                const float nt = -tk[t0 + min(k, tn - 1)] * kLog2e;
                                acc[P][k] = fma2(wgt, ex2_2(fma2(ck, pk2(nt, nt), tl)), acc[P][k]);
                            }
                        }
                    }
                }
            } else {
                // ---- field: every vertex of the block against this lane's views ----
                for (int i = 0; i < nb; ++i) {
                    const VRec r = rec[i];
                    const V3 xb = V3{ r.x, r.y, r.z };
                    if (SINGLE) steps += r.in * rays * nvalid;
#pragma unroll
                    for (int j = 0; j < kVPL; ++j) {
                        if (j >= vpl) break;
                        const bool vok = lane + 32 * j < nv;   // lanes past the chunk's last view count no rays
                        // direction to the view and optical depth toward it (to the grid edge)
                        V3 o;
                        float tau, ri = 1.0f;
                        if constexpr (VWP) {
                            const V3 d = sub3(sv[j], xb);
                            const float r2 = dot3(d, d);
                            ri = rsqrtf(r2);
                            o = V3{ d.x * ri, d.y * ri, d.z * ri };
                        } else {
                            o = sv[j];
                        }
                        if constexpr (SINGLE) {
                            float tm;
                            if constexpr (VWP) {
                                tm = fminf(face_t(o.x, r.nx0, r.nx1), face_t(o.y, r.ny0, r.ny1));
                                if (three) tm = fminf(tm, face_t(o.z, r.nz0, r.nz1));
                            } else {
                                tm = fminf((o.x < 0.0f ? r.nx0 : r.nx1) * sinv[j].x, (o.y < 0.0f ? r.ny0 : r.ny1) * sinv[j].y);
                                if (three) tm = fminf(tm, (o.z < 0.0f ? r.nz0 : r.nz1) * sinv[j].z);
                            }
                            tau = tm * r.sig;
                        } else {
                            uint32_t st = 0;
                            tau = VWP ? tau_to_point(S, xb, sv[j], st, r.cell) : tau_dir(S, xb, o, st, r.cell);
                            steps += vok ? st * rays : 0u;
                        }
                        const V3 df = V3{ r.ux - o.x, r.uy - o.y, r.uz - o.z };
                        const float q2 = dot3(df, df);
                        const float rr = rsqrtf(fmaf(r.g, q2, r.omg2));
                        // g f exp(2 pi i (phase of g + L_b / lambda + xi_b))
                        float a, f;
                        if constexpr (VWP) {
                            float at = __expf(-tau);
                            at = three ? at * kIsoAmp3 * ri * ri : at * ri;
                            if (area) at *= fabsf(three ? o.z : o.y);
                            a = sqrtf(at);
                            if (split) {
                                f = frac_ff(r.ph_h, r.ph_l, scale_ff(dist_ff(sv[j], xb), S.il_h, S.il_l));
                            } else {
                                const float ph = __fdividef(1.0f, ri) * S.inv_lambda_f + r.ph_h;
                                f = ph - rintf(ph);
                            }
                        } else {
                            a = sqrtf(__expf(-tau));
                            if (split) {
                                const FF t = scale_ff(dot_ff(o, xb), S.il_h, S.il_l);
                                f = frac_ff(r.ph_h, r.ph_l, FF{ -t.h, -t.l });
                            } else {
                                const float ph = r.ph_h - (o.x * xb.x + o.y * xb.y + o.z * xb.z) * S.inv_lambda_f;
                                f = ph - rintf(ph);
                            }
                        }
                        const float amp = three ? r.c * rr * sqrtf(rr) : r.c * rr;
                        float sp, cp;
                        sincospif(2.0f * f, &sp, &cp);
                        const float m = a * amp;
                        acc[j][0] = fma2(pk2(m, m), pk2(cp, sp), acc[j][0]);
                    }
                }
            }
            __syncwarp();
        }
        // ---- write S[q][t][v] ----
#pragma unroll
        for (int j = 0; j < kVL; ++j) {
            const int vi = lane + 32 * j;
            if (j >= vpl || vi >= nv) break;
            const int v = T.v0 + vi;
            if constexpr (CORR) {
#pragma unroll
                for (int k = 0; k < kNT; ++k)
                    if (k < tn) {
                        const unsigned long long a2 = acc[j >> 1][k];
                        const float a = (j & 1) ? pk_hi(a2) : pk_lo(a2);
                        const size_t o = ((size_t)q * Nt + t0 + k) * Nv + v;
                        if (T.real_rows) reinterpret_cast<float*>(T.s_ms)[o] = a;
                        else T.s_ms[o] = make_float2(a, 0.0f);
                    }
            } else {
                const float2 c = make_float2(pk_lo(acc[j][0]), pk_hi(acc[j][0]));
                for (int t = t0; t < t0 + tn; ++t) T.s_ms[((size_t)q * Nt + t) * Nv + v] = c;
            }
        }
        const uint32_t ws = warp_sum_u32(steps);
        if (lane == 0 && ws) {
            if (T.dda) atomicAdd(T.dda + q, ws);
            warp_steps += ws;
        }
        q = T.work != nullptr ? nw + __shfl_sync(0xffffffffu, drawn, 0) : q + nw;
    }
    if (lane == 0 && warp_steps) atomicAdd(T.totals + 1, warp_steps);
}

}  // namespace

size_t view_smem_bytes(int Nt, int threads)
{
    return (size_t)(threads / 32) * kVB * std::max(sizeof(VRec), sizeof(CRec)) + (size_t)Nt * sizeof(float);
}

int view_max_ticks(const DevScene& S) { return S.correlation ? kNT : S.Nt; }
int view_max_views(const DevScene& S) { return S.correlation ? 64 * kVPP : 32 * kVPL; }

bool view_kernel_covers(const DevScene& S, const bool* moving_any)
{
    if (S.has_amp64) return false;   // tabular / vMF amplitudes from an FP64 angle: trace_kernel
    if (S.correlation) return S.sym && S.all_static_corr;
    return !*moving_any;
}

int launch_view(const DevScene& S, const TraceParams& T, int blocks, int threads, cudaStream_t stream)
{
    const size_t smem = view_smem_bytes(S.Nt, threads);
    const bool vp = S.src[1].type == SSTMC_SOURCE_POINT;
    using Fn = void (*)(DevScene, TraceParams);
    Fn f;
#define SSTMC_VIEW_PICK(C, V, SG)                                                                            \
    (S.dims == 3 ? (Fn)view_kernel<C, V, SG, true> : (Fn)view_kernel<C, V, SG, false>)
    if (S.single)
        f = S.correlation ? (vp ? SSTMC_VIEW_PICK(true, true, true) : SSTMC_VIEW_PICK(true, false, true))
                          : (vp ? SSTMC_VIEW_PICK(false, true, true) : SSTMC_VIEW_PICK(false, false, true));
    else
        f = S.correlation ? (vp ? SSTMC_VIEW_PICK(true, true, false) : SSTMC_VIEW_PICK(true, false, false))
                          : (vp ? SSTMC_VIEW_PICK(false, true, false) : SSTMC_VIEW_PICK(false, false, false));
#undef SSTMC_VIEW_PICK
    if (smem > 48 * 1024 && cudaFuncSetAttribute((const void*)f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return SSTMC_KERNEL_ERROR;
    // one wave of resident blocks (warps stride over the paths)
    int dev = 0, sms = 0, occ = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, (const void*)f, threads, smem) == cudaSuccess && occ > 0)
        blocks = std::max(1, std::min(blocks, occ * sms));
    if (T.work && cudaMemsetAsync(T.work, 0, sizeof(uint32_t), stream) != cudaSuccess) return SSTMC_DEVICE_ERROR;
    f<<<blocks, threads, smem, stream>>>(S, T);
    return cudaGetLastError() == cudaSuccess ? SSTMC_NO_ERROR : SSTMC_KERNEL_ERROR;
}

bool illum_kernel_covers(const DevScene& S)
{
    return S.correlation && S.sym && S.all_static_corr && !S.has_amp64 && S.src[0].n <= 32 * kMaxIllum;
}

int launch_illum(const DevScene& S, const TraceParams& T, int blocks, int threads, cudaStream_t stream)
{
    const bool ip = S.src[0].type == SSTMC_SOURCE_POINT, vp = S.src[1].type == SSTMC_SOURCE_POINT;
    using Fn = void (*)(DevScene, TraceParams);
    Fn f;
    if (S.single) {
        if (S.src[0].n <= 64)
            f = ip ? (vp ? (Fn)illum_kernel<2, true, true, true> : (Fn)illum_kernel<2, true, false, true>)
                   : (vp ? (Fn)illum_kernel<2, false, true, true> : (Fn)illum_kernel<2, false, false, true>);
        else
            f = ip ? (vp ? (Fn)illum_kernel<kMaxIllum, true, true, true> : (Fn)illum_kernel<kMaxIllum, true, false, true>)
                   : (vp ? (Fn)illum_kernel<kMaxIllum, false, true, true> : (Fn)illum_kernel<kMaxIllum, false, false, true>);
    } else {
        if (S.src[0].n <= 64)
            f = ip ? (vp ? (Fn)illum_kernel<2, true, true, false> : (Fn)illum_kernel<2, true, false, false>)
                   : (vp ? (Fn)illum_kernel<2, false, true, false> : (Fn)illum_kernel<2, false, false, false>);
        else
            f = ip ? (vp ? (Fn)illum_kernel<kMaxIllum, true, true, false> : (Fn)illum_kernel<kMaxIllum, true, false, false>)
                   : (vp ? (Fn)illum_kernel<kMaxIllum, false, true, false> : (Fn)illum_kernel<kMaxIllum, false, false, false>);
    }
    f<<<blocks, threads, 0, stream>>>(S, T);
    return cudaGetLastError() == cudaSuccess ? SSTMC_NO_ERROR : SSTMC_KERNEL_ERROR;
}

}  // namespace sstmc
