// trace.cu -- the fused path-tracing kernel: one warp per path.
//
// Replaces the reference's per-bounce wavefront of ~30-60 synchronous launches
// (NextEventEstimation::trace, NextEventEstimation.cuh:1461-1637): sampling
// (TemporalSampler::sampleFirst/Second/Next, TemporalSampler.cuh:1324-1462;
// TemporalCorrelationSampler.cuh:600-760), the per-vertex NEE vectors
// (twoPointsThroughput / threePointsThroughput / pathContribution), the path
// probabilities (pathProbabilitySingle/Multiple, NEE.cuh:853-1009) and the
// per-path view-vector sum (multipleResMultiple's GvSum, NEE.cuh:1138-1395)
// all happen in registers of one warp.  Lanes replay the same warp-uniform
// FP32 walk and split the NEE work over (source element, tick) items, so
// dead paths need no compaction (the reference's P x P permutation GEMMs,
// NEE.cuh:681-759) and nothing per-vertex is written to HBM.  Per path the
// kernel writes four rows -- the illumination and view vectors of the
// multiple- and single-scattering terms -- which the contraction consumes.
#include <cuda_runtime.h>

#include <algorithm>

#include "gauss.cuh"
#include "nee.cuh"
#include "sstmc_internal.h"
#include "trace.h"

namespace sstmc {

namespace {

__device__ __forceinline__ V3 tick_pos(const float* buf, int t) { return V3{ buf[3 * t], buf[3 * t + 1], buf[3 * t + 2] }; }

// Cell index along one axis as the reference's lookup returns it
// (Simulation.cuh:325-367): ax[c] <= x < ax[c+1]; 0 below the first edge and
// n-1 (one past the last cell) at or beyond the last edge.
__device__ __forceinline__ int edge_bin(const float* ax, int n, float x)
{
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(ax + mid) <= x) lo = mid + 1; else hi = mid;
    }
    return lo > 0 ? lo - 1 : 0;
}

// isSameBinKernel (HeterogeneousMedium.cuh:708-735): p inside the box and in
// the grid cell of x
__device__ __forceinline__ bool same_bin(const DevScene& S, const V3& x, const V3& p)
{
    if (!inside(S, p)) return false;
    bool same = edge_bin(S.ax[0], S.n[0], x.x) == edge_bin(S.ax[0], S.n[0], p.x)
             && edge_bin(S.ax[1], S.n[1], x.y) == edge_bin(S.ax[1], S.n[1], p.y);
    if (S.dims == 3) same = same && edge_bin(S.ax[2], S.n[2], x.z) == edge_bin(S.ax[2], S.n[2], p.z);
    return same;
}

// isForcedInsideBin (TemporalSampler.cuh:439-534, 1637-1698): a tick r drawn
// uniformly per vertex (ceil(u Nt) - 1) is moved onto the sampled point by
// shifting the whole tick chain by x - x_t[r]; a tick whose position leaves
// the sampled point's grid cell weighs 0, and so does every tick beyond it on
// the same side of r (in tick order).  The weights go to buf[3 Nt + t].  The
// reference's shift kernel reads x_t[r] while other threads of the path add
// the shift to it (an unordered read); the shift here is the intended one,
// taken from x_t[r] before any tick moves.
__device__ void forced_inside_bin(const DevScene& S, uint64_t seed, uint32_t pid, uint32_t b,
                                  const V3& x, float* buf, int lane)
{
    const int Nt = S.Nt;
    float* w = buf + 3 * Nt;
    Stream rs;
    rs.init(seed, pid, b, kPurposeForcedBin);
    const uint32_t k = (rs.next() >> 8) + 1u;   // u = k 2^-24 in (0, 1]
    const int r = (int)(((uint64_t)k * (uint32_t)Nt - 1u) >> 24);
    const float s0 = __fsub_rn(x.x, buf[3 * r]), s1 = __fsub_rn(x.y, buf[3 * r + 1]), s2 = __fsub_rn(x.z, buf[3 * r + 2]);
    __syncwarp();
    int neg = -1, pos = Nt;
    for (int t = lane; t < Nt; t += 32) {
        buf[3 * t] = fa(buf[3 * t], s0);
        buf[3 * t + 1] = fa(buf[3 * t + 1], s1);
        if (S.dims == 3) buf[3 * t + 2] = fa(buf[3 * t + 2], s2);
        if (!same_bin(S, x, tick_pos(buf, t))) {
            if (t <= r) neg = max(neg, t);
            else pos = min(pos, t);
        }
    }
    neg = __reduce_max_sync(0xffffffffu, neg);
    pos = __reduce_min_sync(0xffffffffu, pos);
    for (int t = lane; t < Nt; t += 32) w[t] = (t > neg && t < pos) ? 1.0f : 0.0f;
    __syncwarp();
}

// Per-tick positions of a vertex of the field sampler (TemporalSampler.cuh:376-436,
// 540-647, 778-937): Brownian displacement N(0, 2 dims D |dt|) along a random
// direction plus dt U per sorted tick, cumulated outward from the mean tick.
// Warp-cooperative; buf holds Nt*3 floats in output-tick order, then (with
// isForcedInsideBin) the Nt tick weights.
__device__ void temporal_positions(const DevScene& S, uint64_t seed, uint32_t pid, uint32_t b,
                                   const V3& x, int m, float* buf, int lane)
{
    const int Nt = S.Nt;
    if (!S.moving[m]) {
        // every tick sits on x: the forced tick does too, and all weights are 1
        for (int t = lane; t < Nt; t += 32) {
            buf[3 * t] = x.x; buf[3 * t + 1] = x.y; buf[3 * t + 2] = x.z;
            if (S.forced_bin) buf[3 * Nt + t] = 1.0f;
        }
        __syncwarp();
        return;
    }
    for (int j = lane; j < Nt; j += 32) {
        const float sc = S.disp_scale[m * Nt + j];
        const float* du = S.disp_u + (m * Nt + j) * 3;
        float dp[3] = { du[0], du[1], du[2] };
        if (sc != 0.0f) {
            Stream ts;
            ts.init(seed, pid, b, kPurposeTemporal | ((uint32_t)j << 8));
            const V3 w = random_direction(S.dims, ts);
            const float u1 = ts.uniform();
            const float u2 = ts.uniform();
            const float r = fsq(fm(-2.0f, walk_logf(u1)));
            float s, c;
            walk_sincospif(fm(2.0f, u2), s, c);
            const float dr = fm(fm(r, c), sc);
            dp[0] = ffma(dr, w.x, du[0]);
            dp[1] = ffma(dr, w.y, du[1]);
            if (S.dims == 3) dp[2] = ffma(dr, w.z, du[2]);
        }
        buf[3 * j] = dp[0]; buf[3 * j + 1] = dp[1]; buf[3 * j + 2] = dp[2];
    }
    __syncwarp();
    if (lane == 0) {
        float c0 = x.x, c1 = x.y, c2 = x.z;
        for (int j = 0; j < Nt; ++j) {
            if (j == 0 || j == S.neg) { c0 = x.x; c1 = x.y; c2 = x.z; }
            c0 = fa(c0, buf[3 * j]);
            c1 = fa(c1, buf[3 * j + 1]);
            if (S.dims == 3) c2 = fa(c2, buf[3 * j + 2]);
            buf[3 * j] = c0; buf[3 * j + 1] = c1; buf[3 * j + 2] = c2;
        }
        // sorted index j -> output tick: the negative group is reversed
        for (int j = 0; j < S.neg / 2; ++j) {
            const int k = S.neg - 1 - j;
            for (int i = 0; i < 3; ++i) { const float tmp = buf[3 * j + i]; buf[3 * j + i] = buf[3 * k + i]; buf[3 * k + i] = tmp; }
        }
    }
    __syncwarp();
    if (S.forced_bin) forced_inside_bin(S, seed, pid, b, x, buf, lane);
}

// weight of tick t of a vertex: 1, or the isForcedInsideBin weight
__device__ __forceinline__ float tick_w(const DevScene& S, const float* buf, int t)
{
    return S.forced_bin ? buf[3 * S.Nt + t] : 1.0f;
}

__device__ void zero_rows(const DevScene& S, const TraceParams& T, uint32_t q, int lane)
{
    const uint32_t qs = T.ss_row ? T.ss_row[q] : q;   // row of the single-scattering rows
    const int Nt = S.Nt, Nl = S.src[0].n, Nv = S.src[1].n;
    if (T.cbs) {   // reversed pass: Gv0 rows (first pass) and this pass's GlSum entries
        if (T.pass0)
            for (int i = lane; i < Nt * Nv; i += 32) T.s_ms[(size_t)q * Nt * Nv + i] = make_float2(0.f, 0.f);
        for (int t = T.t0; t < T.t0 + T.tn; ++t)
            for (int l = T.v0 + lane; l < T.v0 + T.vn; l += 32) T.a_ms[((size_t)q * Nt + t) * Nl + l] = make_float2(0.f, 0.f);
        return;
    }
    if (T.pass0) {
        for (int i = lane; i < Nt * Nl; i += 32) {
            T.a_ms[(size_t)q * Nt * Nl + i] = make_float2(0.f, 0.f);
            T.a_ss[(size_t)qs * Nt * Nl + i] = make_float2(0.f, 0.f);
        }
        for (int i = lane; i < Nt * Nv; i += 32) T.b_ss[(size_t)qs * Nt * Nv + i] = make_float2(0.f, 0.f);
    }
    if (T.views)
        for (int t = T.t0; t < T.t0 + T.tn; ++t)
            for (int v = T.v0 + lane; v < T.v0 + T.vn; v += 32) T.s_ms[((size_t)q * Nt + t) * Nv + v] = make_float2(0.f, 0.f);
}

// ---- NEE vectors, specialised on the source type (PT: point source) ----

// |g|^2 of source element k at x: the attenuation weight T c / r^(D-1)
// (point source, PointSource.cuh:117-172) or T (far field, FarField.cuh:223-263).
template <bool PT>
__device__ __forceinline__ float gweight(const DevScene& S, const DevSource& s, int k, const V3& x, int role, uint32_t& steps,
                                         uint32_t cell = kNoCell)
{
    if constexpr (!PT) {
        const V3 d = load3(s.p, k);
        return expf(-tau_dir(S, x, role == kRoleIllum ? V3{ -d.x, -d.y, -d.z } : d, steps, cell));
    } else {
        const V3 sp = load3(s.p, k);
        const float T = expf(-tau_to_point(S, x, sp, steps, cell));
        const V3 v = sub3(x, sp);
        const float r2 = dot3(v, v);
        float at = S.dims == 3 ? __fdividef(T * kIsoAmp3, r2) : T * rsqrtf(r2);
        if (s.is_area) at *= fabsf(S.dims == 3 ? v.z : v.y) * rsqrtf(r2);
        return at;
    }
}

// g with its phase.  Split precision: the argument d.x / lambda (far field)
// or r / lambda (point source) is formed and reduced modulo one cycle in FP64.
template <bool PT>
__device__ __forceinline__ float2 gcomplex(const DevScene& S, const DevSource& s, int k, const V3& x, int role, uint32_t& steps,
                                           uint32_t cell = kNoCell)
{
    const bool split = S.precision == SSTMC_PRECISION_SPLIT;
    float f, a;
    if constexpr (!PT) {
        const V3 d = load3(s.p, k);
        a = sqrtf(expf(-tau_dir(S, x, role == kRoleIllum ? V3{ -d.x, -d.y, -d.z } : d, steps, cell)));
        if (split) {
            const double dx = fma((double)d.x, (double)x.x, fma((double)d.y, (double)x.y, (double)d.z * (double)x.z));
            f = frac_cycles((role == kRoleIllum ? dx : -dx) * S.inv_lambda);
        } else {
            const float dx = d.x * x.x + d.y * x.y + d.z * x.z;
            const float ph = (role == kRoleIllum ? dx : -dx) * S.inv_lambda_f;
            f = ph - rintf(ph);
        }
    } else {
        const V3 sp = load3(s.p, k);
        const float T = expf(-tau_to_point(S, x, sp, steps, cell));
        const V3 v = sub3(x, sp);
        const float r2 = dot3(v, v);
        float at = S.dims == 3 ? __fdividef(T * kIsoAmp3, r2) : T * rsqrtf(r2);
        if (s.is_area) at *= fabsf(S.dims == 3 ? v.z : v.y) * rsqrtf(r2);
        a = sqrtf(at);
        if (split) {
            const double dx = (double)x.x - (double)sp.x, dy = (double)x.y - (double)sp.y, dz = (double)x.z - (double)sp.z;
            f = frac_cycles(sqrt(fma(dx, dx, fma(dy, dy, dz * dz))) * S.inv_lambda);
        } else {
            const float ph = sqrtf(r2) * S.inv_lambda_f;
            f = ph - rintf(ph);
        }
    }
    return c_scale(unit_phase(f), a);
}

template <bool PT>
__device__ __forceinline__ float pfirst_t(const DevScene& S, const DevSource& s, int l, const V3& x, uint32_t& steps,
                                          uint32_t cell = kNoCell)
{
    if constexpr (!PT) {
        const V3 d = load3(s.p, l);
        return expf(-tau_dir(S, x, V3{ -d.x, -d.y, -d.z }, steps, cell)) * s.sprob[l];
    } else {
        const V3 sp = load3(s.p, l);
        const float T = expf(-tau_to_point(S, x, sp, steps, cell));
        const V3 v = sub3(x, sp);
        const float r2 = dot3(v, v);
        return S.dims == 3 ? __fdividef(T, (float)(4.0 * kPi) * r2) : T * (float)(8.0 * kPi) * rsqrtf(r2);
    }
}

// f: illumination element l -> scatterer pa -> pb (FarField.cuh:546-554, PointSource.cuh:317-345)
template <bool PT>
__device__ __forceinline__ float fillum(const DevScene& S, const DevSource& s, int l, const V3& pa, const V3& pb, int m)
{
    if (PT && S.iso_all) return S.iso_amp;
    return amp_fast(S, m, fsrc_in(s, l, pa), funit(sub3(pb, pa)));
}

// f: pb -> scatterer pa -> view element v
template <bool PT>
__device__ __forceinline__ float fview(const DevScene& S, const DevSource& s, int v, const V3& pa, const V3& pb, int m)
{
    if (PT && S.iso_all) return S.iso_amp;
    return amp_fast(S, m, funit(sub3(pa, pb)), fsrc_out(s, v, pa));
}

// CBS reversed path: view element v as the path's first end, v -> pa -> pb
// (threePointFunction with the view attached at pa, NextEventEstimation.cuh:1533-1537)
template <bool PT>
__device__ __forceinline__ float fview_entry(const DevScene& S, const DevSource& s, int v, const V3& pa, const V3& pb, int m)
{
    if (PT && S.iso_all) return S.iso_amp;
    const V3 o = fsrc_out(s, v, pa);
    return amp_fast(S, m, V3{ -o.x, -o.y, -o.z }, funit(sub3(pb, pa)));
}

// CBS reversed path: illumination element l as the path's last end, pb -> pa -> l
// (NextEventEstimation.cuh:1573-1580)
template <bool PT>
__device__ __forceinline__ float fillum_exit(const DevScene& S, const DevSource& s, int l, const V3& pa, const V3& pb, int m)
{
    if (PT && S.iso_all) return S.iso_amp;
    const V3 i = fsrc_in(s, l, pa);
    return amp_fast(S, m, funit(sub3(pa, pb)), V3{ -i.x, -i.y, -i.z });
}

// f^2 for identical u1 / u2 sources: the pdf (|amplitude|^2 = pdf)
template <bool PT>
__device__ __forceinline__ float fillum2(const DevScene& S, const DevSource& s, int l, const V3& pa, const V3& pb, int m)
{
    if (PT && S.iso_all) return S.iso_amp * S.iso_amp;
    return pdf_fast(S, m, fsrc_in(s, l, pa), funit(sub3(pb, pa)));
}

template <bool PT>
__device__ __forceinline__ float fview2(const DevScene& S, const DevSource& s, int v, const V3& pa, const V3& pb, int m)
{
    if (PT && S.iso_all) return S.iso_amp * S.iso_amp;
    return pdf_fast(S, m, funit(sub3(pa, pb)), fsrc_out(s, v, pa));
}

// CORR: correlation sampler; ILP / VWP: illumination / view sources are point sources.
template <bool CORR, bool ILP, bool VWP>
__global__ void __launch_bounds__(128, 6) trace_kernel(const __grid_constant__ DevScene S, const __grid_constant__ TraceParams T)
{
    extern __shared__ double smem_d[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int Nt = S.Nt, Nl = S.src[0].n, Nv = S.src[1].n, D = S.dims;
    const bool split = S.precision == SSTMC_PRECISION_SPLIT;
    // per-warp shared scratch: L[Nt] doubles, view accumulators [slots][32] float2
    // (lane-major, conflict-free), two Nt*3 float tick-position buffers
    const int nwb = blockDim.x >> 5;
    double* Ls = smem_d + (size_t)wib * Nt;
    float2* accs = reinterpret_cast<float2*>(smem_d + (size_t)nwb * Nt) + (size_t)wib * T.slots * 32 + lane;
    float* fbase = reinterpret_cast<float*>(reinterpret_cast<float2*>(smem_d + (size_t)nwb * Nt) + (size_t)nwb * T.slots * 32);
    float* bufA = fbase + (size_t)wib * 9 * Nt;
    float* bufB = bufA + 4 * Nt;
    float* phs = bufA + 8 * Nt;   // field: the path phase L_t / lambda + xi_b mod 1 of the current vertex per tick
    float* tk_abs = fbase + (size_t)nwb * 9 * Nt;   // block-wide copies of |t| and t
    float* tk_raw = tk_abs + Nt;
    for (int t = threadIdx.x; t < Nt; t += blockDim.x) { tk_abs[t] = S.abs_ticks[t]; tk_raw[t] = S.ticks_f[t]; }
    __syncthreads();
    const DevSource& il = S.src[0];
    const DevSource& vw = S.src[1];
    const DevSource& il2 = S.src[2];
    const DevSource& vw2 = S.src[3];
    const float k2 = S.k2;
    const bool geo = S.ticks_geometric != 0;

    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    unsigned long long acc_v = 0, acc_s = 0, acc_m = 0, acc_p = 0;
    // Work items: a path (its vertices 2 .. B, or with segments 2 .. seg + 1),
    // or in segment mode a (path, k) item of T.seg_list: vertices
    // 2 + k seg .. min(B, 1 + (k + 1) seg) of one long path, its view sums
    // added to the path's rows after the path's own launch wrote them.
    const bool segm = T.seg_mode != 0;
    const bool segf = !CORR && segm;   // field sampler segment: its path-length prefix is replayed
    // path length of tick t across one segment a -> c: FP64 (split) or FP32
    auto path_step = [&](double* L, int t, const V3& a, const V3& c) {
        if (split) {
            const double dx = (double)c.x - (double)a.x, dy = (double)c.y - (double)a.y, dz = (double)c.z - (double)a.z;
            L[t] += sqrt(fma(dx, dx, fma(dy, dy, dz * dz)));
        } else {
            const V3 dd = sub3(c, a);
            L[t] = (double)((float)L[t] + sqrtf(dot3(dd, dd)));
        }
    };
    for (uint32_t it = gw;;) {
        uint32_t q, bs = 2;
        if (segm) {
            uint32_t w = 0;
            if (lane == 0) w = atomicAdd(T.seg_next, 1u);
            w = __shfl_sync(0xffffffffu, w, 0);
            if (w >= *T.seg_len) break;
            const uint2 item = T.seg_list[w];
            q = item.x;
            bs = 2u + item.y * T.seg;
        } else {
            if (it >= T.paths) break;
            q = it;
            it += nw;
        }
        const uint32_t pid = T.first_path + q;
        const uint32_t B = T.counts[q];
        const uint32_t be = T.seg ? min(B, bs + T.seg - 1u) : B;   // last vertex of the item
        const uint32_t qs = T.ss_row ? T.ss_row[q] : q;   // row of the single-scattering rows
        if (B == 0) {  // the walk hit a limit (error already flagged)
            zero_rows(S, T, q, lane);
            continue;
        }
        const float4* vq = T.verts + T.offsets[q];
        const float4 v1 = vq[0];
        const V3 x1 = V3{ v1.x, v1.y, v1.z };
        const int m1 = (int)(__float_as_uint(v1.w) & 15u);
        const float xi1 = (float)(__float_as_uint(v1.w) >> 4) * (1.0f / 16777216.0f);
        const uint32_t c1 = (S.single || segm) ? kNoCell : cell_of(S, x1);   // x1's grid cell, the start of its NEE rays
        float* xtc = bufA;   // tick positions of the current vertex
        float* xtn = bufB;   // tick positions of the new vertex
        bool mov1 = false;
        if constexpr (!CORR) {
            temporal_positions(S, T.seed, pid, 1u, x1, m1, xtc, lane);
            for (int t = lane; t < Nt; t += 32) Ls[t] = 0.0;
            __syncwarp();
            mov1 = S.moving[m1] != 0;
            if (T.pass0 && !T.cbs && T.x1t)
                for (int i = lane; i < 3 * Nt; i += 32) T.x1t[(size_t)q * 3 * Nt + i] = xtc[i];
        }
        uint32_t steps = 0;

        // ---- illumination side at x1: P_l, Gl0, single-scattering rows ----
        if (T.pass0 && !T.cbs && !segm) {
            float ps = 0.0f;
            for (int l = lane; l < Nl; l += 32) {
                uint32_t st = 0;
                float P = pfirst_t<ILP>(S, il, l, x1, st, c1);
                if (CORR) {
                    if (S.sym) st *= 2;
                    else P = 0.5f * (P + pfirst_t<ILP>(S, il2, l, x1, st, c1));
                }
                steps += st;
                T.pl[(size_t)q * Nl + l] = P;
                ps += P;
            }
            const float p1 = warp_sum(ps) / (float)Nl;
            const float p1inv = CORR ? 1.0f / p1 : 1.0f / sqrtf(p1);
            if constexpr (CORR) {
                const bool st1 = S.static_corr[m1] != 0;
                const bool realg = S.sym && st1;
                for (int l = lane % T.lw; l < Nl; l += T.lw) {
                    float w = 0.0f;
                    float2 g1s = make_float2(0.f, 0.f), g2s = make_float2(0.f, 0.f);
                    uint32_t sts = 0;
                    if (realg) { w = gweight<ILP>(S, il, l, x1, kRoleIllum, sts, c1); sts *= 2; }
                    else if (st1) { g1s = gcomplex<ILP>(S, il, l, x1, kRoleIllum, sts, c1); g2s = gcomplex<ILP>(S, il2, l, x1, kRoleIllum, sts, c1); }
                    for (int t = lane / T.lw; t < Nt; t += T.lg) {
                        const size_t o = ((size_t)q * Nt + t) * Nl + l;
                        const size_t os = ((size_t)qs * Nt + t) * Nl + l;
                        if (realg) {
                            steps += sts;
                            T.a_ms[o] = make_float2(w, 0.f);
                            T.a_ss[os] = make_float2(w * p1inv, 0.f);
                        } else {
                            float2 g1 = g1s, g2 = g2s;
                            if (st1) steps += sts;
                            else {
                                const float tau = tk_raw[t];
                                g1 = gcomplex<ILP>(S, il, l, shift_u(S, x1, m1, tau, -1.0f), kRoleIllum, steps);
                                g2 = gcomplex<ILP>(S, il2, l, shift_u(S, x1, m1, tau, 1.0f), kRoleIllum, steps);
                            }
                            T.a_ms[o] = g1;
                            T.g2[o] = g2;
                            T.a_ss[os] = c_scale(c_mulc(g1, g2), p1inv);
                        }
                    }
                }
                for (int v = lane % T.vwa; v < Nv; v += T.vwa) {
                    float w = 0.0f;
                    float2 g1s = make_float2(0.f, 0.f), g2s = make_float2(0.f, 0.f);
                    uint32_t sts = 0;
                    if (realg) { w = gweight<VWP>(S, vw, v, x1, kRoleView, sts, c1); sts *= 2; }
                    else if (st1) { g1s = gcomplex<VWP>(S, vw, v, x1, kRoleView, sts, c1); g2s = gcomplex<VWP>(S, vw2, v, x1, kRoleView, sts, c1); }
                    for (int t = lane / T.vwa; t < Nt; t += T.tga) {
                        float2 b;
                        if (realg) { steps += sts; b = make_float2(w, 0.f); }
                        else if (st1) { steps += sts; b = c_mulc(g1s, g2s); }
                        else {
                            const float tau = tk_raw[t];
                            b = c_mulc(gcomplex<VWP>(S, vw, v, shift_u(S, x1, m1, tau, -1.0f), kRoleView, steps),
                                       gcomplex<VWP>(S, vw2, v, shift_u(S, x1, m1, tau, 1.0f), kRoleView, steps));
                        }
                        T.b_ss[((size_t)qs * Nt + t) * Nv + v] = b;
                    }
                }
            } else {
                const float2 e1 = unit_phase(xi1);
                for (int l = lane % T.lw; l < Nl; l += T.lw) {
                    float2 gs = make_float2(0.f, 0.f);
                    uint32_t sts = 0;
                    if (!mov1) gs = gcomplex<ILP>(S, il, l, x1, kRoleIllum, sts, c1);
                    for (int t = lane / T.lw; t < Nt; t += T.lg) {
                        float2 g = gs;
                        if (!mov1) steps += sts;
                        else g = gcomplex<ILP>(S, il, l, tick_pos(xtc, t), kRoleIllum, steps);
                        T.a_ms[((size_t)q * Nt + t) * Nl + l] = g;
                        T.a_ss[((size_t)qs * Nt + t) * Nl + l] = c_scale(c_mul(g, e1), p1inv * tick_w(S, xtc, t));
                    }
                }
                for (int v = lane % T.vwa; v < Nv; v += T.vwa) {
                    float2 gs = make_float2(0.f, 0.f);
                    uint32_t sts = 0;
                    if (!mov1) gs = gcomplex<VWP>(S, vw, v, x1, kRoleView, sts, c1);
                    for (int t = lane / T.vwa; t < Nt; t += T.tga) {
                        float2 g = gs;
                        if (!mov1) steps += sts;
                        else g = gcomplex<VWP>(S, vw, v, tick_pos(xtc, t), kRoleView, steps);
                        T.b_ss[((size_t)qs * Nt + t) * Nv + v] = g;
                    }
                }
            }
        }

        // ---- later vertices ----
        for (int i = 0; i < T.slots; ++i) accs[32 * i] = make_float2(0.f, 0.f);
        V3 prev = x1, cur = x1;
        int mcur = m1;
        float MT = 0.0f;
        if (CORR && segm) {
            // the segment starts after vertex bs - 1: its two predecessors, and the
            // momentum-transfer sum of the inner vertices before it (lanes over the
            // vertices, then a warp sum)
            const float4 pb = vq[bs - 3], cb = vq[bs - 2];
            prev = V3{ pb.x, pb.y, pb.z };
            cur = V3{ cb.x, cb.y, cb.z };
            mcur = (int)(__float_as_uint(cb.w) & 15u);
            float part = 0.0f;
            for (uint32_t b = 3 + lane; b < bs; b += 32) {
                const float4 a = vq[b - 3], c = vq[b - 2], n = vq[b - 1];
                const V3 xa = V3{ a.x, a.y, a.z }, xc = V3{ c.x, c.y, c.z }, xn = V3{ n.x, n.y, n.z };
                const V3 dq = sub3(funit(sub3(xc, xa)), funit(sub3(xn, xc)));
                part += S.D[__float_as_uint(c.w) & 15u] * dot3(dq, dq);
            }
            MT = warp_sum(part);
        }
        if (segf) {
            // the segment starts after vertex bs - 1: replay the per-tick positions of
            // vertices 2 .. bs - 1 and their path-length sums, the same FP64 additions in
            // the same order as the path's own warp makes them
            const float4 pb = vq[bs - 3], cb = vq[bs - 2];
            prev = V3{ pb.x, pb.y, pb.z };
            cur = V3{ cb.x, cb.y, cb.z };
            mcur = (int)(__float_as_uint(cb.w) & 15u);
            for (uint32_t c = 2; c < bs; ++c) {
                const float4 vc = vq[c - 1];
                temporal_positions(S, T.seed, pid, c, V3{ vc.x, vc.y, vc.z }, (int)(__float_as_uint(vc.w) & 15u), xtn, lane);
                for (int t = lane; t < Nt; t += 32) path_step(Ls, t, tick_pos(xtc, t), tick_pos(xtn, t));
                __syncwarp();
                float* tmp = xtc; xtc = xtn; xtn = tmp;
            }
        }
        for (uint32_t b = bs; b <= be; ++b) {
            if (!T.views && b > 2) break;   // the view-side kernel sums the view vectors
            const float4 vb = vq[b - 1];
            const V3 xn = V3{ vb.x, vb.y, vb.z };
            const int mn = (int)(__float_as_uint(vb.w) & 15u);
            const float xin = (float)(__float_as_uint(vb.w) >> 4) * (1.0f / 16777216.0f);
            const uint32_t cn = (T.views && !S.single) ? cell_of(S, xn) : kNoCell;   // xn's grid cell
            if (CORR && b >= 3) {
                // momentum transfer of the inner vertex cur (TemporalSamplerCorrelation.cuh:144-179)
                const V3 dq = sub3(funit(sub3(cur, prev)), funit(sub3(xn, cur)));
                MT += S.D[mcur] * dot3(dq, dq);
            }
            if constexpr (!CORR) {
                temporal_positions(S, T.seed, pid, b, xn, mn, xtn, lane);
                for (int t = lane; t < Nt; t += 32) {
                    path_step(Ls, t, tick_pos(xtc, t), tick_pos(xtn, t));
                    if (split) {
                        phs[t] = frac_cycles(Ls[t] * S.inv_lambda + (double)xin);
                    } else {
                        const float ph = (float)Ls[t] * S.inv_lambda_f + xin;
                        phs[t] = ph - rintf(ph);
                    }
                }
                __syncwarp();
            }

            // multiple-scattering illumination vector at x2 (NEE.cuh:1525-1559, 889-1009)
            if (b == 2 && T.pass0) {
                const V3 x12 = funit(sub3(xn, x1));
                // tabular or vMF first material: pdf from an FP64 angle (nee.cuh), and
                // the amplitudes unless point sources take the isotropic one
                const bool pdf1 = is_amp64(S, m1);
                const bool tab1 = src_amp64(S, il, m1);
                float ps = 0.0f;
                if (pdf1) {
                    double d12[3];
                    dir64(x1, xn, d12);
                    for (int l = lane; l < Nl; l += 32) {
                        double in[3];
                        src_in64(il, l, x1, in);
                        ps += T.pl[(size_t)q * Nl + l] * pdf64(S, m1, in[0] * d12[0] + in[1] * d12[1] + in[2] * d12[2]);
                    }
                } else {
                    for (int l = lane; l < Nl; l += 32)
                        ps += T.pl[(size_t)q * Nl + l] * pdf_fast(S, m1, fsrc_in(il, l, x1), x12);
                }
                const float p2 = warp_sum(ps) / (float)Nl;
                const float p2inv = CORR ? 1.0f / p2 : 1.0f / sqrtf(p2);
                if (T.p2 && lane == 0) T.p2[q] = p2;
                if constexpr (CORR) {
                    const bool stf = S.static_corr[m1] && S.static_corr[mn];
                    const bool realg = S.sym && S.static_corr[m1];
                    const float c1base = k2 * S.D[m1];
                    for (int l = lane % T.lw; l < Nl; l += T.lw) {
                        const V3 i1 = fsrc_in(il, l, x1);
                        const V3 i2 = S.sym ? i1 : fsrc_in(il2, l, x1);
                        const V3 qv = V3{ 0.5f * (i1.x + i2.x) - x12.x, 0.5f * (i1.y + i2.y) - x12.y, 0.5f * (i1.z + i2.z) - x12.z };
                        const float c1k = c1base * dot3(qv, qv);
                        float f12s = 0.0f;
                        // tabular / vMF: u1 amplitude x conj(u2 amplitude), complex unless u1 == u2
                        auto f12tab = [&](const V3& pa, const V3& pb) {
                            const float2 f1 = amp64(S, m1, f3_cos64(il, l, pa, pb, false));
                            if (S.sym) return make_float2(f1.x * f1.x + f1.y * f1.y, 0.f);
                            return c_mulc(f1, amp64(S, m1, f3_cos64(il2, l, pa, pb, false)));
                        };
                        float2 f12cs = make_float2(0.f, 0.f);
                        if (stf && tab1) f12cs = f12tab(x1, xn);
                        else if (stf) f12s = S.sym ? fillum2<ILP>(S, il, l, x1, xn, m1) : fillum<ILP>(S, il, l, x1, xn, m1) * fillum<ILP>(S, il2, l, x1, xn, m1);
                        const int tfirst = lane / T.lw;
                        float e = tfirst < Nt ? __expf(-c1k * tk_abs[tfirst]) : 0.0f;
                        const float estep = geo ? __expf(-c1k * tk_abs[0] * (float)T.lg) : 0.0f;
                        for (int t = tfirst; t < Nt; t += T.lg) {
                            const size_t o = ((size_t)q * Nt + t) * Nl + l;
                            if (tab1) {
                                float2 f12c = f12cs;
                                if (!stf) {
                                    const float tau = tk_raw[t];
                                    f12c = f12tab(shift_u(S, x1, m1, tau, -1.0f), shift_u(S, xn, mn, tau, -1.0f));
                                }
                                const float sc = p2inv * (geo ? e : __expf(-c1k * tk_abs[t]));
                                e *= estep;
                                if (realg) T.a_ms[o] = make_float2(T.a_ms[o].x * f12c.x * sc, 0.f);
                                else T.a_ms[o] = c_scale(c_mul(c_mulc(T.a_ms[o], T.g2[o]), f12c), sc);
                                continue;
                            }
                            float f12 = f12s;
                            if (!stf) {
                                const float tau = tk_raw[t];
                                const V3 pa = shift_u(S, x1, m1, tau, -1.0f), pb = shift_u(S, xn, mn, tau, -1.0f);
                                f12 = S.sym ? fillum2<ILP>(S, il, l, pa, pb, m1) : fillum<ILP>(S, il, l, pa, pb, m1) * fillum<ILP>(S, il2, l, pa, pb, m1);
                            }
                            const float sc = f12 * p2inv * (geo ? e : __expf(-c1k * tk_abs[t]));
                            e *= estep;
                            if (realg) T.a_ms[o] = make_float2(T.a_ms[o].x * sc, 0.f);
                            else T.a_ms[o] = c_scale(c_mulc(T.a_ms[o], T.g2[o]), sc);
                        }
                    }
                } else if (T.cbs) {
                    // Gv0 = g_v(x1) f(v -> x1 -> x2) / sqrt(p2) from the single-scattering
                    // view rows of the first pass (NextEventEstimation.cuh:995-1004)
                    const bool stf = !S.temporal_amp || (!mov1 && !S.moving[mn]);
                    for (int v = lane % T.vwa; v < Nv; v += T.vwa) {
                        if (tab1) {   // view attached at x1, path on to x2
                            const float2 fs = stf ? amp64(S, m1, f3_cos64(vw, v, x1, xn, true)) : make_float2(0.f, 0.f);
                            for (int t = lane / T.vwa; t < Nt; t += T.tga) {
                                const size_t o = ((size_t)q * Nt + t) * Nv + v;
                                const float2 f = stf ? fs : amp64(S, m1, f3_cos64(vw, v, tick_pos(xtc, t), tick_pos(xtn, t), true));
                                T.s_ms[o] = c_scale(c_mul(T.b_ss[o], f), p2inv);
                            }
                            continue;
                        }
                        const float fs = stf ? fview_entry<VWP>(S, vw, v, x1, xn, m1) : 0.0f;
                        for (int t = lane / T.vwa; t < Nt; t += T.tga) {
                            const size_t o = ((size_t)q * Nt + t) * Nv + v;
                            const float f = stf ? fs : fview_entry<VWP>(S, vw, v, tick_pos(xtc, t), tick_pos(xtn, t), m1);
                            T.s_ms[o] = c_scale(T.b_ss[o], f * p2inv);
                        }
                    }
                } else {
                    const bool stf = !S.temporal_amp || (!mov1 && !S.moving[mn]);
                    for (int l = lane % T.lw; l < Nl; l += T.lw) {
                        if (tab1) {   // illumination attached at x1, path on to x2
                            const float2 fs = stf ? amp64(S, m1, f3_cos64(il, l, x1, xn, false)) : make_float2(0.f, 0.f);
                            for (int t = lane / T.lw; t < Nt; t += T.lg) {
                                const size_t o = ((size_t)q * Nt + t) * Nl + l;
                                const float2 f = stf ? fs : amp64(S, m1, f3_cos64(il, l, tick_pos(xtc, t), tick_pos(xtn, t), false));
                                T.a_ms[o] = c_scale(c_mul(T.a_ms[o], f), p2inv);
                            }
                            continue;
                        }
                        const float fs = stf ? fillum<ILP>(S, il, l, x1, xn, m1) : 0.0f;
                        for (int t = lane / T.lw; t < Nt; t += T.lg) {
                            const size_t o = ((size_t)q * Nt + t) * Nl + l;
                            const float f = stf ? fs : fillum<ILP>(S, il, l, tick_pos(xtc, t), tick_pos(xtn, t), m1);
                            T.a_ms[o] = c_scale(T.a_ms[o], f * p2inv);
                        }
                    }
                }
            }

            // view vectors at vertex b, summed over the path (multipleResMultiple)
            if (!T.views) {
            } else if constexpr (CORR) {
                const bool stn = S.static_corr[mn] != 0;
                const bool realv = S.sym && stn;
                const bool stf = stn && S.static_corr[mcur];
                const float ptk = k2 * MT;
                const float c1base = k2 * S.D[mn];
                const V3 back = funit(sub3(cur, xn));
                const bool tabn = src_amp64(S, vw, mn);
                int j = 0;
                for (int v = T.v0 + lane % T.vw; v < T.v0 + T.vn; v += T.vw, ++j) {
                    const V3 o1 = fsrc_out(vw, v, xn);
                    const V3 o2 = S.sym ? o1 : fsrc_out(vw2, v, xn);
                    const V3 qv = V3{ -0.5f * (o1.x + o2.x) - back.x, -0.5f * (o1.y + o2.y) - back.y, -0.5f * (o1.z + o2.z) - back.z };
                    const float ck = c1base * dot3(qv, qv) + ptk;
                    uint32_t sts = 0;
                    float w = 0.0f;
                    float2 g1s = make_float2(0.f, 0.f), g2s = make_float2(0.f, 0.f);
                    if (realv) { w = gweight<VWP>(S, vw, v, xn, kRoleView, sts, cn); sts *= 2; }
                    else if (stn) { g1s = gcomplex<VWP>(S, vw, v, xn, kRoleView, sts, cn); g2s = gcomplex<VWP>(S, vw2, v, xn, kRoleView, sts, cn); }
                    float f12s = 0.0f;
                    // tabular / vMF: u1 amplitude x conj(u2 amplitude), the view attached at x_b
                    auto f12tab = [&](const V3& pa, const V3& pb) {
                        const float2 f1 = amp64(S, mn, f3_cos64(vw, v, pa, pb, true));
                        if (S.sym) return make_float2(f1.x * f1.x + f1.y * f1.y, 0.f);
                        return c_mulc(f1, amp64(S, mn, f3_cos64(vw2, v, pa, pb, true)));
                    };
                    float2 f12cs = make_float2(0.f, 0.f);
                    if (stf && tabn) f12cs = f12tab(xn, cur);
                    else if (stf) f12s = S.sym ? fview2<VWP>(S, vw, v, xn, cur, mn) : fview<VWP>(S, vw, v, xn, cur, mn) * fview<VWP>(S, vw2, v, xn, cur, mn);
                    int k = 0;
                    const int tfirst = T.t0 + lane / T.vw;
                    float e = tfirst < T.t0 + T.tn ? __expf(-ck * tk_abs[tfirst]) : 0.0f;
                    const float estep = geo ? __expf(-ck * tk_abs[0] * (float)T.tg) : 0.0f;
                    for (int t = tfirst; t < T.t0 + T.tn; t += T.tg, ++k) {
                        const float tau = tk_raw[t];
                        float f12 = f12s;
                        float2 f12c = f12cs;
                        if (!stf) {
                            const V3 pa = shift_u(S, xn, mn, tau, -1.0f), pb = shift_u(S, cur, mcur, tau, -1.0f);
                            if (tabn) f12c = f12tab(pa, pb);
                            else f12 = S.sym ? fview2<VWP>(S, vw, v, pa, pb, mn) : fview<VWP>(S, vw, v, pa, pb, mn) * fview<VWP>(S, vw2, v, pa, pb, mn);
                        }
                        const float decay = geo ? e : __expf(-ck * tk_abs[t]);
                        const float dec = tabn ? decay : f12 * decay;
                        e *= estep;
                        float2 c;
                        if (realv) { steps += sts; c = make_float2(w * (tabn ? f12c.x * dec : dec), 0.f); }
                        else {
                            float2 g1 = g1s, g2 = g2s;
                            if (stn) steps += sts;
                            else {
                                g1 = gcomplex<VWP>(S, vw, v, shift_u(S, xn, mn, tau, -1.0f), kRoleView, steps);
                                g2 = gcomplex<VWP>(S, vw2, v, shift_u(S, xn, mn, tau, 1.0f), kRoleView, steps);
                            }
                            c = tabn ? c_scale(c_mul(c_mulc(g1, g2), f12c), dec) : c_scale(c_mulc(g1, g2), dec);
                        }
                        float2* a = accs + 32 * (j * T.tpl + k);
                        const float2 av = *a;
                        *a = make_float2(av.x + c.x, av.y + c.y);
                    }
                }
            } else {
                const bool stn = !S.moving[mn];
                const bool stf = !S.temporal_amp || (stn && !S.moving[mcur]);
                // the view's vector at x_b (GvSum), or for the CBS reversed pass the
                // illumination's vector at x_b with the illumination as the path's last end (GlSum)
                auto gx = [&](int e, const V3& p, uint32_t& st, uint32_t cell) {
                    return T.cbs ? gcomplex<ILP>(S, il, e, p, kRoleIllum, st, cell) : gcomplex<VWP>(S, vw, e, p, kRoleView, st, cell);
                };
                auto fx = [&](int e, const V3& pa, const V3& pb, int m) {
                    return T.cbs ? fillum_exit<ILP>(S, il, e, pa, pb, m) : fview<VWP>(S, vw, e, pa, pb, m);
                };
                // tabular or vMF vertex material: FP64-angle amplitude, the source attached at x_b
                const bool tabn = src_amp64(S, T.cbs ? il : vw, mn);
                auto fxc = [&](int e, const V3& pa, const V3& pb) {
                    return amp64(S, mn, T.cbs ? f3_cos64(il, e, pa, pb, false) : f3_cos64(vw, e, pa, pb, true));
                };
                int j = 0;
                for (int v = T.v0 + lane % T.vw; v < T.v0 + T.vn; v += T.vw, ++j) {
                    uint32_t sts = 0;
                    float2 gs = make_float2(0.f, 0.f);
                    if (stn) gs = gx(v, xn, sts, cn);
                    const float fs = (stf && !tabn) ? fx(v, xn, cur, mn) : 0.0f;
                    const float2 fsc = (stf && tabn) ? fxc(v, xn, cur) : make_float2(0.f, 0.f);
                    int k = 0;
                    for (int t = T.t0 + lane / T.vw; t < T.t0 + T.tn; t += T.tg, ++k) {
                        float2 g = gs;
                        if (stn) steps += sts;
                        else g = gx(v, tick_pos(xtn, t), steps, kNoCell);
                        const float fr = phs[t];
                        float2 c;
                        if (tabn) {
                            const float2 f = stf ? fsc : fxc(v, tick_pos(xtn, t), tick_pos(xtc, t));
                            c = c_mul(c_mul(g, unit_phase(fr)), f);
                            if (S.forced_bin) c = c_scale(c, tick_w(S, xtn, t));
                        } else {
                            const float f = stf ? fs : fx(v, tick_pos(xtn, t), tick_pos(xtc, t), mn);
                            c = c_scale(c_mul(g, unit_phase(fr)), f * tick_w(S, xtn, t));
                        }
                        float2* a = accs + 32 * (j * T.tpl + k);
                        const float2 av = *a;
                        *a = make_float2(av.x + c.x, av.y + c.y);
                    }
                }
            }
            prev = cur;
            cur = xn;
            mcur = mn;
            float* tmp = xtc; xtc = xtn; xtn = tmp;
        }
        if (T.pass0 && B < 2 && !segm) {
            if (T.cbs) for (int i = lane; i < Nt * Nv; i += 32) T.s_ms[(size_t)q * Nt * Nv + i] = make_float2(0.f, 0.f);
            else for (int i = lane; i < Nt * Nl; i += 32) T.a_ms[(size_t)q * Nt * Nl + i] = make_float2(0.f, 0.f);
        }
        // write the summed view vector of this chunk (a segment adds its part)
        if (T.views) {
            int j = 0;
            for (int v = T.v0 + lane % T.vw; v < T.v0 + T.vn; v += T.vw, ++j) {
                int k = 0;
                for (int t = T.t0 + lane / T.vw; t < T.t0 + T.tn; t += T.tg, ++k) {
                    const float2 a = accs[32 * (j * T.tpl + k)];
                    if (segm) {
                        float2* d = T.s_ms + ((size_t)q * Nt + t) * Nv + v;
                        atomicAdd(&d->x, a.x);
                        atomicAdd(&d->y, a.y);
                    } else if (T.cbs) T.a_ms[((size_t)q * Nt + t) * Nl + v] = a;
                    else T.s_ms[((size_t)q * Nt + t) * Nv + v] = a;
                }
            }
        }
        const uint32_t wsteps = warp_sum_u32(steps);
        if (lane == 0) {
            if (T.pass0 && !T.cbs && !segm) {
                if (T.m1) T.m1[q] = (unsigned char)m1;
                if (T.x1) { T.x1[3 * q] = x1.x; T.x1[3 * q + 1] = x1.y; T.x1[3 * q + 2] = x1.z; }
                acc_v += B;
                acc_m += T.misses[q];
                acc_p += 1;
            }
            if (T.dda && wsteps) atomicAdd(T.dda + q, wsteps);
            acc_s += wsteps;
        }
    }
    // one atomic per counter and warp (per-path atomics on four addresses serialise)
    if (lane == 0) {
        if (acc_v) atomicAdd(T.totals + 0, acc_v);
        if (acc_s) atomicAdd(T.totals + 1, acc_s);
        if (acc_m) atomicAdd(T.totals + 2, acc_m);
        if (acc_p) atomicAdd(T.totals + 3, acc_p);
    }
}

// ---- Gaussian beams: the field sampler's rows with beam sources (gauss.cuh) ----
// Warp per path, lanes over the beams; FP64 source terms.  The rows are the
// ones trace_kernel writes for the field sampler (NextEventEstimation.cuh:
// 1385-1637 with GaussianBeam.cuh's source functions):
//   a_ss(t, l) = g_l(x1_t) e^(2 pi i xi_1) w_t / sqrt(p1),  b_ss(t, v) = g_v(x1_t)
//   a_ms(t, l) = g_l(x1_t) f_l(x1_t -> x2_t) / sqrt(p2)
//   s_ms(t, v) = sum_{b >= 2} g_v(x_b,t) e^(2 pi i (L_t / lambda + xi_b)) f_v(x_{b-1},t -> x_b,t) w_b,t
// with p1 the mean of P_l(x1) and p2 the mean of P_l(x1) p_l(x1 -> x2) (a
// zero product counting 1e20).  The view sums are added into the path's row
// in place (each (t, v) entry is one lane's).
__device__ __forceinline__ float gauss_g(const DevScene& S, const DevSource& s, int k, const V3& x, bool view, uint32_t& steps)
{
    const V3 d = load3(s.gdir, k);
    return sqrtf(expf(-tau_dir(S, x, view ? d : V3{ -d.x, -d.y, -d.z }, steps)));
}

__device__ __forceinline__ double warp_sum_d(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__global__ void __launch_bounds__(128) gauss_trace_kernel(const __grid_constant__ DevScene S, const __grid_constant__ TraceParams T)
{
    extern __shared__ double smem_d[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5, nwb = blockDim.x >> 5;
    const int Nt = S.Nt, Nl = S.src[0].n, Nv = S.src[1].n, D = S.dims;
    const bool split = S.precision == SSTMC_PRECISION_SPLIT;
    double* Ls = smem_d + (size_t)wib * Nt;
    float* fb = reinterpret_cast<float*>(smem_d + (size_t)nwb * Nt) + (size_t)wib * 9 * Nt;
    float* phs = fb + 8 * Nt;
    const DevSource& il = S.src[0];
    const DevSource& vw = S.src[1];
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    unsigned long long acc_v = 0, acc_s = 0, acc_m = 0, acc_p = 0;
    for (uint32_t q = gw; q < T.paths; q += nw) {
        const uint32_t pid = T.first_path + q;
        const uint32_t B = T.counts[q];
        if (B == 0) {   // the walk hit a limit (error already flagged): rows zero, no material
            zero_rows(S, T, q, lane);
            if (lane == 0 && T.m1) T.m1[q] = 0;
            continue;
        }
        float* xtc = fb;
        float* xtn = fb + 4 * Nt;
        const float4* vq = T.verts + T.offsets[q];
        const float4 v1 = vq[0];
        const V3 x1 = V3{ v1.x, v1.y, v1.z };
        const int m1 = (int)(__float_as_uint(v1.w) & 15u);
        const float xi1 = (float)(__float_as_uint(v1.w) >> 4) * (1.0f / 16777216.0f);
        temporal_positions(S, T.seed, pid, 1u, x1, m1, xtc, lane);
        for (int t = lane; t < Nt; t += 32) Ls[t] = 0.0;
        __syncwarp();
        const bool mov1 = S.moving[m1] != 0;
        if (T.x1t)
            for (int i = lane; i < 3 * Nt; i += 32) T.x1t[(size_t)q * 3 * Nt + i] = xtc[i];
        uint32_t steps = 0;

        // first vertex: P_l, p1, the illumination and single-scattering rows
        // 3D beams from their tables; 2D beams as point sources at their focal points
        double ps = 0.0;
        for (int l = lane; l < Nl; l += 32) {
            const double P = D == 3 ? gauss_pfirst(S, il, l, x1, m1) : (double)pfirst_t<true>(S, il, l, x1, steps);
            T.pl[(size_t)q * Nl + l] = (float)P;
            ps += P;
        }
        const double p1 = warp_sum_d(ps) / (double)Nl;
        const float p1inv = (float)(1.0 / sqrt(p1));
        const float2 e1 = unit_phase(xi1);
        for (int l = lane; l < Nl; l += 32) {
            uint32_t sts = 0;
            const float gs = mov1 ? 0.0f : gauss_g(S, il, l, x1, false, sts);
            for (int t = 0; t < Nt; ++t) {
                float g = gs;
                if (!mov1) steps += sts;
                else g = gauss_g(S, il, l, tick_pos(xtc, t), false, steps);
                T.a_ms[((size_t)q * Nt + t) * Nl + l] = make_float2(g, 0.0f);
                T.a_ss[((size_t)q * Nt + t) * Nl + l] = c_scale(e1, g * p1inv * tick_w(S, xtc, t));
            }
        }
        for (int v = lane; v < Nv; v += 32) {
            uint32_t sts = 0;
            const float gs = mov1 ? 0.0f : gauss_g(S, vw, v, x1, true, sts);
            for (int t = 0; t < Nt; ++t) {
                float g = gs;
                if (!mov1) steps += sts;
                else g = gauss_g(S, vw, v, tick_pos(xtc, t), true, steps);
                T.b_ss[((size_t)q * Nt + t) * Nv + v] = make_float2(g, 0.0f);
            }
        }
        for (int i = lane; i < Nt * Nv; i += 32) T.s_ms[(size_t)q * Nt * Nv + i] = make_float2(0.f, 0.f);
        if (B < 2)
            for (int i = lane; i < Nt * Nl; i += 32) T.a_ms[(size_t)q * Nt * Nl + i] = make_float2(0.f, 0.f);
        __syncwarp();

        // later vertices
        V3 cur = x1;
        int mcur = m1;
        for (uint32_t b = 2; b <= B; ++b) {
            const float4 vb = vq[b - 1];
            const V3 xn = V3{ vb.x, vb.y, vb.z };
            const int mn = (int)(__float_as_uint(vb.w) & 15u);
            const float xin = (float)(__float_as_uint(vb.w) >> 4) * (1.0f / 16777216.0f);
            temporal_positions(S, T.seed, pid, b, xn, mn, xtn, lane);
            for (int t = lane; t < Nt; t += 32) {
                const V3 a = tick_pos(xtc, t), c = tick_pos(xtn, t);
                if (split) {
                    const double dx = (double)c.x - (double)a.x, dy = (double)c.y - (double)a.y, dz = (double)c.z - (double)a.z;
                    Ls[t] += sqrt(fma(dx, dx, fma(dy, dy, dz * dz)));
                    phs[t] = frac_cycles(Ls[t] * S.inv_lambda + (double)xin);
                } else {
                    const V3 dd = sub3(c, a);
                    Ls[t] = (double)((float)Ls[t] + sqrtf(dot3(dd, dd)));
                    const float ph = (float)Ls[t] * S.inv_lambda_f + xin;
                    phs[t] = ph - rintf(ph);
                }
            }
            __syncwarp();
            if (b == 2) {
                double qs = 0.0;
                for (int l = lane; l < Nl; l += 32) {
                    if (D == 2) {   // the point-source form: the pdf of the scattering angle at x1
                        qs += (double)T.pl[(size_t)q * Nl + l] * (double)pdf_fast(S, m1, fsrc_in(il, l, x1), funit(sub3(xn, x1)));
                        continue;
                    }
                    const double P = gauss_pfirst(S, il, l, x1, m1);
                    const double pw = S.iso_all ? 0.079577471545947668 : gauss_pw(S, il, l, x1, xn);
                    const double qq = P * pw;
                    qs += qq == 0.0 ? 1e20 : qq;
                }
                const double p2 = warp_sum_d(qs) / (double)Nl;
                const float p2inv = (float)(1.0 / sqrt(p2));
                if (T.p2 && lane == 0) T.p2[q] = (float)p2;
                const bool stf = !S.temporal_amp || (!mov1 && !S.moving[mn]);
                for (int l = lane; l < Nl; l += 32) {
                    CD fs{ 0.0, 0.0 };
                    if (stf) fs = gauss_f(S, il, l, x1, xn, m1, false);
                    for (int t = 0; t < Nt; ++t) {
                        const CD f = stf ? fs : gauss_f(S, il, l, tick_pos(xtc, t), tick_pos(xtn, t), m1, false);
                        const size_t o = ((size_t)q * Nt + t) * Nl + l;
                        const float g = T.a_ms[o].x * p2inv;
                        T.a_ms[o] = make_float2(g * (float)f.re, g * (float)f.im);
                    }
                }
            }
            const bool stn = !S.moving[mn];
            const bool stf = !S.temporal_amp || (stn && !S.moving[mcur]);
            for (int v = lane; v < Nv; v += 32) {
                uint32_t sts = 0;
                const float gs = stn ? gauss_g(S, vw, v, xn, true, sts) : 0.0f;
                CD fs{ 0.0, 0.0 };
                if (stf) fs = gauss_f(S, vw, v, xn, cur, mn, true);
                for (int t = 0; t < Nt; ++t) {
                    float g = gs;
                    if (stn) steps += sts;
                    else g = gauss_g(S, vw, v, tick_pos(xtn, t), true, steps);
                    const CD f = stf ? fs : gauss_f(S, vw, v, tick_pos(xtn, t), tick_pos(xtc, t), mn, true);
                    const float2 c = c_scale(c_mul(unit_phase(phs[t]), make_float2((float)f.re, (float)f.im)), g * tick_w(S, xtn, t));
                    float2* d = T.s_ms + ((size_t)q * Nt + t) * Nv + v;
                    const float2 a = *d;
                    *d = make_float2(a.x + c.x, a.y + c.y);
                }
            }
            cur = xn;
            mcur = mn;
            float* tmp = xtc; xtc = xtn; xtn = tmp;
            __syncwarp();
        }
        const uint32_t wsteps = warp_sum_u32(steps);
        if (lane == 0) {
            if (T.m1) T.m1[q] = (unsigned char)m1;
            if (T.x1) { T.x1[3 * q] = x1.x; T.x1[3 * q + 1] = x1.y; T.x1[3 * q + 2] = x1.z; }
            acc_v += B;
            acc_m += T.misses[q];
            acc_p += 1;
            if (T.dda && wsteps) atomicAdd(T.dda + q, wsteps);
            acc_s += wsteps;
        }
    }
    if (lane == 0) {
        if (acc_v) atomicAdd(T.totals + 0, acc_v);
        if (acc_s) atomicAdd(T.totals + 1, acc_s);
        if (acc_m) atomicAdd(T.totals + 2, acc_m);
        if (acc_p) atomicAdd(T.totals + 3, acc_p);
    }
}

// ---- CBS of the correlation sampler (NextEventEstimation.cuh:1237-1378, 1525-1600) ----
// For every vertex x_b (b >= 2) of every path, the cross terms of the direct
// and reversed paths (SourceInterface.cuh:270-354 for the temporal factors):
//   T2 = Gl_b(l) conj(u2Gv_b(v)) conj(u2Gl0(l)) Gv0(v) exp(-k^2 |t| (D_b |m2b|^2 + D_1 |m21|^2))
//   T3 = conj(u2Gl_b(l)) Gv_b(v) Gl0(l) conj(u2Gv0(v)) exp(-k^2 |t| (D_b |m3b|^2 + D_1 |m31|^2))
//   T4 = Gl_b(l) conj(u2Gl_b(l)) Gv0(v) conj(u2Gv0(v)) exp(-k^2 |t| (D_b |m4b|^2 + D_1 |m41|^2))
// times the u1 path transfer exp(-k^2 |t| MT_b), V += 0.5 (T2 + T3 + T4).
// Gl0 / Gv0 (first vertex, the path on to x2) carry 1 / p2; the vectors at x_b
// are the NEE vector times the amplitude of the source attached at x_b with
// the path back to x_{b-1}; m = (a + b) / 2 - (direction to the other path
// point), a, b the directions from the two ends' sources into the vertex (a
// view's is minus its outgoing direction).  Block = a 16 x 16 (l, v) tile for
// a chunk of ticks and a range of paths; four 16-thread groups stage the u1 /
// u2 illumination and view quantities of the current vertex in shared memory.
// Its rays are not counted in the DDA statistics.
constexpr int kCbT = 16, kCbTicks = 8;

template <bool ILP, bool VWP, bool DRIFT>
__global__ void __launch_bounds__(256) cbs_corr_kernel(const __grid_constant__ DevScene S, const CbsCorrParams P)
{
    // DRIFT: the vectors are staged per tick of the block's chunk (u1 NEE vectors at
    // x - U t/2, u2 ones at x + U t/2, both amplitudes at the u1 positions); static
    // scatterers stage one set for every tick
    constexpr int NE = DRIFT ? kCbTicks : 1;
    __shared__ float2 g0l[2][NE][kCbT], g0v[2][NE][kCbT], gb_l[2][NE][kCbT], gb_v[2][NE][kCbT];   // [u1 / u2][tick][element]
    __shared__ float d0l[2][kCbT][3], d0v[2][kCbT][3], dbl[2][kCbT][3], dbv[2][kCbT][3];
    __shared__ float geo[8];   // d12 (3), back (3), D_b, MT_b
    const int tl = threadIdx.x % kCbT, tv = threadIdx.x / kCbT;
    const int Nt = S.Nt, Nl = S.src[0].n, Nv = S.src[1].n;
    const int l0 = blockIdx.x * kCbT, v0 = blockIdx.y * kCbT;
    const int tchunks = (Nt + kCbTicks - 1) / kCbTicks;
    const int t0 = (blockIdx.z % tchunks) * kCbTicks, tn = min(kCbTicks, Nt - t0);
    const int ks = blockIdx.z / tchunks;
    const int kb = ks * P.kchunk, ke = min(P.K, kb + P.kchunk);
    const int ne = DRIFT ? tn : 1;
    const DevSource* srcl[2] = { &S.src[0], &S.src[2] };
    const DevSource* srcv[2] = { &S.src[1], &S.src[3] };
    // staging role of this thread: group 0 / 1: illumination u1 / u2, 2 / 3: view u1 / u2
    const int grp = threadIdx.x / kCbT, ge = threadIdx.x % kCbT;
    const bool stager = threadIdx.x < 4 * kCbT;
    const bool isl = grp < 2;
    const int u = grp & 1;
    const int el = min((isl ? l0 : v0) + ge, (isl ? Nl : Nv) - 1);
    // the staged vector's positions for slot e: the NEE vector at gp, the
    // amplitude from fa toward fb
    auto positions = [&](int e, const V3& x, int mx, const V3& y, int my, V3& gp, V3& fa, V3& fb) {
        gp = x; fa = x; fb = y;
        if (DRIFT) {
            const float tau = S.ticks_f[t0 + e];
            gp = shift_u(S, x, mx, tau, u == 0 ? -1.0f : 1.0f);
            fa = shift_u(S, x, mx, tau, -1.0f);
            fb = shift_u(S, y, my, tau, -1.0f);
        }
    };
    float2 acc[kCbTicks];
    double accd[kCbTicks][2];
#pragma unroll
    for (int i = 0; i < kCbTicks; ++i) { acc[i] = make_float2(0.f, 0.f); accd[i][0] = accd[i][1] = 0.0; }
    int window = 0;
    for (int p = kb; p < ke; ++p) {
        const uint32_t B = P.counts[p];
        if (B < 2) continue;   // uniform over the block
        const float4* vq = P.verts + P.offsets[p];
        const float4 v1 = vq[0], v2 = vq[1];
        const V3 x1 = V3{ v1.x, v1.y, v1.z }, x2 = V3{ v2.x, v2.y, v2.z };
        const int m1 = (int)(__float_as_uint(v1.w) & 15u), m2 = (int)(__float_as_uint(v2.w) & 15u);
        const float p2inv = 1.0f / P.p2[p];
        __syncthreads();   // the previous path's last vertex is consumed
        if (stager) {
            uint32_t st = 0;
            for (int e = 0; e < ne; ++e) {
                V3 gp, fa, fb;
                positions(e, x1, m1, x2, m2, gp, fa, fb);
                if (isl) {
                    const DevSource& s = *srcl[u];
                    const float2 g = gcomplex<ILP>(S, s, el, gp, kRoleIllum, st);
                    if (src_amp64(S, s, m1)) {   // tabular / vMF: complex amplitude from an FP64 angle
                        g0l[u][e][ge] = c_scale(c_mul(g, amp64(S, m1, f3_cos64(s, el, fa, fb, false))), u == 0 ? p2inv : 1.0f);
                    } else {
                        const float f = fillum<ILP>(S, s, el, fa, fb, m1);
                        g0l[u][e][ge] = c_scale(g, u == 0 ? f * p2inv : f);
                    }
                } else {
                    const DevSource& s = *srcv[u];
                    const float2 g = gcomplex<VWP>(S, s, el, gp, kRoleView, st);
                    if (src_amp64(S, s, m1)) {   // the view attached at x1 as the reversed path's first end
                        g0v[u][e][ge] = c_scale(c_mul(g, amp64(S, m1, f3_cos64(s, el, fa, fb, true))), u == 0 ? p2inv : 1.0f);
                    } else {
                        const float f = fview_entry<VWP>(S, s, el, fa, fb, m1);
                        g0v[u][e][ge] = c_scale(g, u == 0 ? f * p2inv : f);
                    }
                }
            }
            if (isl) {
                const V3 d = fsrc_in(*srcl[u], el, x1);
                d0l[u][ge][0] = d.x; d0l[u][ge][1] = d.y; d0l[u][ge][2] = d.z;
            } else {
                const V3 d = fsrc_out(*srcv[u], el, x1);
                d0v[u][ge][0] = -d.x; d0v[u][ge][1] = -d.y; d0v[u][ge][2] = -d.z;
            }
        }
        if (threadIdx.x == 0) {
            const V3 d = funit(sub3(x2, x1));
            geo[0] = d.x; geo[1] = d.y; geo[2] = d.z;
        }
        float MT = 0.0f;
        V3 prev = x1, cur = x1;
        int mprev = m1, mcur = m1;
        for (uint32_t b = 2; b <= B; ++b) {
            const float4 vb = vq[b - 1];
            const V3 xn = V3{ vb.x, vb.y, vb.z };
            const int mn = (int)(__float_as_uint(vb.w) & 15u);
            if (b >= 3) {   // momentum transfer of the inner vertex cur
                const V3 dq = sub3(funit(sub3(cur, prev)), funit(sub3(xn, cur)));
                MT += S.D[mcur] * dot3(dq, dq);
            }
            prev = cur; mprev = mcur;
            cur = xn; mcur = mn;
            __syncthreads();   // the previous vertex's records are consumed
            if (stager) {
                uint32_t st = 0;
                for (int e = 0; e < ne; ++e) {
                    V3 gp, fa, fb;
                    positions(e, xn, mn, prev, mprev, gp, fa, fb);
                    if (isl) {
                        const DevSource& s = *srcl[u];
                        const float2 g = gcomplex<ILP>(S, s, el, gp, kRoleIllum, st);
                        gb_l[u][e][ge] = src_amp64(S, s, mn) ? c_mul(g, amp64(S, mn, f3_cos64(s, el, fa, fb, false)))
                                                         : c_scale(g, fillum_exit<ILP>(S, s, el, fa, fb, mn));
                    } else {
                        const DevSource& s = *srcv[u];
                        const float2 g = gcomplex<VWP>(S, s, el, gp, kRoleView, st);
                        gb_v[u][e][ge] = src_amp64(S, s, mn) ? c_mul(g, amp64(S, mn, f3_cos64(s, el, fa, fb, true)))
                                                         : c_scale(g, fview<VWP>(S, s, el, fa, fb, mn));
                    }
                }
                if (isl) {
                    const V3 d = fsrc_in(*srcl[u], el, xn);
                    dbl[u][ge][0] = d.x; dbl[u][ge][1] = d.y; dbl[u][ge][2] = d.z;
                } else {
                    const V3 d = fsrc_out(*srcv[u], el, xn);
                    dbv[u][ge][0] = -d.x; dbv[u][ge][1] = -d.y; dbv[u][ge][2] = -d.z;
                }
            }
            if (threadIdx.x == 0) {
                const V3 d = funit(sub3(prev, xn));
                geo[3] = d.x; geo[4] = d.y; geo[5] = d.z;
                geo[6] = S.D[mn];
                geo[7] = MT;
            }
            __syncthreads();
            auto q2 = [&](const float* a, const float* c, int o) {
                float r = 0.0f;
#pragma unroll
                for (int i = 0; i < 3; ++i) { const float d = 0.5f * (a[i] + c[i]) - geo[o + i]; r = fmaf(d, d, r); }
                return r;
            };
            const float D1 = S.D[m1], Db = geo[6];
            const float a2 = S.k2 * (Db * q2(dbl[0][tl], dbv[1][tv], 3) + D1 * q2(d0v[0][tv], d0l[1][tl], 0));
            const float a3 = S.k2 * (Db * q2(dbv[0][tv], dbl[1][tl], 3) + D1 * q2(d0l[0][tl], d0v[1][tv], 0));
            const float a4 = S.k2 * (Db * q2(dbl[0][tl], dbl[1][tl], 3) + D1 * q2(d0v[0][tv], d0v[1][tv], 0));
            auto terms = [&](int e, float2& c2, float2& c3, float2& c4) {
                c2 = c_mul(c_mulc(gb_l[0][e][tl], gb_v[1][e][tv]), c_mulc(g0v[0][e][tv], g0l[1][e][tl]));
                c3 = c_mul(c_mulc(gb_v[0][e][tv], gb_l[1][e][tl]), c_mulc(g0l[0][e][tl], g0v[1][e][tv]));
                c4 = c_mul(c_mulc(gb_l[0][e][tl], gb_l[1][e][tl]), c_mulc(g0v[0][e][tv], g0v[1][e][tv]));
            };
            float2 c2, c3, c4;
            if (!DRIFT) terms(0, c2, c3, c4);
            const float ptk = S.k2 * geo[7];
#pragma unroll
            for (int tt = 0; tt < kCbTicks; ++tt) {
                if (tt >= tn) break;
                if (DRIFT) terms(tt, c2, c3, c4);
                const float at = S.abs_ticks[t0 + tt];
                const float e2 = __expf(-at * a2), e3 = __expf(-at * a3), e4 = __expf(-at * a4);
                const float w = 0.5f * __expf(-at * ptk);
                acc[tt].x = fmaf(w, c2.x * e2 + c3.x * e3 + c4.x * e4, acc[tt].x);
                acc[tt].y = fmaf(w, c2.y * e2 + c3.y * e3 + c4.y * e4, acc[tt].y);
            }
            if (++window == 64) {   // FP32 windows folded into FP64 registers
                window = 0;
#pragma unroll
                for (int tt = 0; tt < kCbTicks; ++tt) {
                    accd[tt][0] += acc[tt].x; accd[tt][1] += acc[tt].y;
                    acc[tt] = make_float2(0.f, 0.f);
                }
            }
        }
    }
    const int l = l0 + tl, v = v0 + tv;
    if (l >= Nl || v >= Nv) return;
#pragma unroll
    for (int tt = 0; tt < kCbTicks; ++tt) {
        if (tt >= tn) break;
        const size_t o = ((size_t)(t0 + tt) * Nv + v) * Nl + l;
        atomicAdd(&P.V[o].x, accd[tt][0] + (double)acc[tt].x);
        atomicAdd(&P.V[o].y, accd[tt][1] + (double)acc[tt].y);
    }
}

}  // namespace

int launch_cbs_corr(const DevScene& S, const CbsCorrParams& P, cudaStream_t stream)
{
    if (P.K <= 0) return SSTMC_NO_ERROR;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int tchunks = (S.Nt + kCbTicks - 1) / kCbTicks;
    const int tiles = ((S.src[0].n + kCbT - 1) / kCbT) * ((S.src[1].n + kCbT - 1) / kCbT) * tchunks;
    const int want = std::max(1, (8 * sms + tiles - 1) / tiles);
    CbsCorrParams Q = P;
    Q.kchunk = std::max(1, (P.K + want - 1) / want);
    const int ksplit = (P.K + Q.kchunk - 1) / Q.kchunk;
    dim3 grid((S.src[0].n + kCbT - 1) / kCbT, (S.src[1].n + kCbT - 1) / kCbT, tchunks * ksplit);
    const bool ip = S.src[0].type == SSTMC_SOURCE_POINT, vp = S.src[1].type == SSTMC_SOURCE_POINT;
    using Fn = void (*)(DevScene, CbsCorrParams);
    const Fn fns[2][2][2] = {
        { { cbs_corr_kernel<false, false, false>, cbs_corr_kernel<false, false, true> },
          { cbs_corr_kernel<false, true, false>, cbs_corr_kernel<false, true, true> } },
        { { cbs_corr_kernel<true, false, false>, cbs_corr_kernel<true, false, true> },
          { cbs_corr_kernel<true, true, false>, cbs_corr_kernel<true, true, true> } } };
    fns[ip][vp][S.all_static_corr ? 0 : 1]<<<grid, 256, 0, stream>>>(S, Q);
    return cudaGetLastError() == cudaSuccess ? SSTMC_NO_ERROR : SSTMC_KERNEL_ERROR;
}

namespace {

// The long paths' extra segments: for every path of more than seg + 1
// vertices, the items (path, k) for k = 1 .. (B - 2) / seg.  The list's order
// is that of the atomic appends; capacity cap >= total vertices / seg.
__global__ void seg_list_kernel(const uint32_t* counts, uint32_t n, uint32_t seg, uint2* list, uint32_t cap, uint32_t* len)
{
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const uint32_t B = counts[q];
        if (B <= seg + 1u) continue;
        const uint32_t extra = (B - 2u) / seg;
        const uint32_t at = atomicAdd(len, extra);
        for (uint32_t k = 1; k <= extra && at + k - 1u < cap; ++k) list[at + k - 1u] = make_uint2(q, k);
    }
}

}  // namespace

int launch_seg_list(const uint32_t* counts, uint32_t n, uint32_t seg, uint2* list, uint32_t cap, uint32_t* len, cudaStream_t stream)
{
    if (cudaMemsetAsync(len, 0, sizeof(uint32_t), stream) != cudaSuccess) return SSTMC_DEVICE_ERROR;
    const int blocks = (int)std::min<uint32_t>(4096, (n + 255) / 256);
    seg_list_kernel<<<std::max(1, blocks), 256, 0, stream>>>(counts, n, seg, list, cap, len);
    return cudaGetLastError() == cudaSuccess ? SSTMC_NO_ERROR : SSTMC_KERNEL_ERROR;
}

size_t trace_smem_bytes(int Nt, int slots, int threads)
{
    const int warps = threads / 32;
    return (size_t)warps * Nt * sizeof(double) + (size_t)warps * slots * 32 * sizeof(float2)
         + (size_t)warps * 9 * Nt * sizeof(float) + 2 * (size_t)Nt * sizeof(float);
}

using TraceFn = void (*)(DevScene, TraceParams);

static TraceFn pick(const DevScene& S)
{
    const bool ip = S.src[0].type == SSTMC_SOURCE_POINT, vp = S.src[1].type == SSTMC_SOURCE_POINT;
    if (S.correlation) {
        if (ip) return vp ? (TraceFn)trace_kernel<true, true, true> : (TraceFn)trace_kernel<true, true, false>;
        return vp ? (TraceFn)trace_kernel<true, false, true> : (TraceFn)trace_kernel<true, false, false>;
    }
    if (ip) return vp ? (TraceFn)trace_kernel<false, true, true> : (TraceFn)trace_kernel<false, true, false>;
    return vp ? (TraceFn)trace_kernel<false, false, true> : (TraceFn)trace_kernel<false, false, false>;
}

int occupancy_blocks(const DevScene& S, int threads, size_t smem)
{
    TraceFn f = pick(S);
    if (smem > 48 * 1024) cudaFuncSetAttribute((const void*)f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, f, threads, smem) != cudaSuccess) n = 1;
    return n > 0 ? n : 1;
}

size_t gauss_trace_smem_bytes(int Nt, int threads)
{
    const size_t nwb = (size_t)threads / 32;
    return nwb * (size_t)Nt * sizeof(double) + nwb * 9 * (size_t)Nt * sizeof(float);
}

int launch_gauss_trace(const DevScene& S, const TraceParams& T, int threads, cudaStream_t stream)
{
    const size_t smem = gauss_trace_smem_bytes(S.Nt, threads);
    if (smem > 48 * 1024) {
        if (cudaFuncSetAttribute((const void*)gauss_trace_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
            return SSTMC_KERNEL_ERROR;
    }
    // four paths per block, at most one wave of resident blocks
    int dev = 0, sms = 0, occ = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, gauss_trace_kernel, threads, smem) != cudaSuccess || occ < 1) occ = 1;
    const int blocks = (int)std::max<uint32_t>(1u, std::min<uint32_t>((T.paths + 3) / 4, (uint32_t)(sms * occ)));
    gauss_trace_kernel<<<blocks, threads, smem, stream>>>(S, T);
    return cudaGetLastError() == cudaSuccess ? SSTMC_NO_ERROR : SSTMC_KERNEL_ERROR;
}

int launch_trace(const DevScene& S, const TraceParams& T, int blocks, int threads, cudaStream_t stream)
{
    const size_t smem = trace_smem_bytes(S.Nt, T.slots, threads);
    TraceFn f = pick(S);
    if (smem > 48 * 1024) {
        if (cudaFuncSetAttribute((const void*)f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
            return SSTMC_KERNEL_ERROR;
    }
    f<<<blocks, threads, smem, stream>>>(S, T);
    return cudaGetLastError() == cudaSuccess ? SSTMC_NO_ERROR : SSTMC_KERNEL_ERROR;
}

}  // namespace sstmc
