// nee.cuh -- per-vertex NEE quantities (value path: FP32, with the phase
// argument reduction in FP64 in the split-precision form).
//
//   g, far field      FarField.cuh:223-263   sqrt(T) exp(+/- 2 pi i d.x / lambda)
//   g, point source   PointSource.cuh:117-172 sqrt(T c / r^(D-1)) exp(2 pi i r / lambda)
//   P_l (first point) FarField.cuh:469-499, PointSource.cuh:92-115, 263-294
//   f (three points)  FarField.cuh:546-554, PointSource.cuh:317-345, Scattering.cuh:895-955
//   pdf               Scattering.cuh:959-1023
// Henyey-Greenstein amplitudes are evaluated from the difference of the two
// unit directions, 1 + g^2 - 2 g cos = (1 - g)^2 + g |a - b|^2, which keeps
// full FP32 relative accuracy for strongly forward scattering (g = 0.9).
#pragma once
#include "walk.cuh"

namespace sstmc {

constexpr int kRoleIllum = 0;
constexpr int kRoleView = 1;

__device__ __forceinline__ float2 c_mul(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ float2 c_mulc(float2 a, float2 b) { return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y); }  // a * conj(b)
__device__ __forceinline__ float2 c_scale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }

__device__ __forceinline__ V3 sub3(const V3& a, const V3& b) { return V3{ a.x - b.x, a.y - b.y, a.z - b.z }; }
__device__ __forceinline__ float dot3(const V3& a, const V3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 unit3(const V3& v)
{
    const float s = dot3(v, v);
    if (!(s > 0.0f)) return V3{ 0.f, 0.f, 1.f };
    const float r = rsqrtf(s);
    return V3{ v.x * r, v.y * r, v.z * r };
}

// exp(2 pi i f)
__device__ __forceinline__ float2 unit_phase(float f)
{
    float s, c;
    sincospif(2.0f * f, &s, &c);
    return make_float2(c, s);
}

// reduce a phase measured in cycles: FP64 in the split form, FP32 in the plain form
__device__ __forceinline__ float frac_cycles(double ph) { return (float)(ph - rint(ph)); }

// ---- float-float phases (split precision) ----
// GB300 runs FP64 at a small fraction of the FP32 rate, and the field
// sampler needs a phase per (vertex, view): the phase of a far-field view
// o . x / lambda or of a point view |v - x| / lambda, modulo 1, to about
// 1e-7 cycles at positions of up to ~1e5 wavelengths.  It is formed from
// exact FP32 products and sums (FMA error terms, two-sums: Dekker / Knuth
// error-free transformations), about 2^-48 relative, in FP32 instructions.
// Every product and sum is explicitly rounded, so nothing is fused.
struct FF { float h, l; };
__device__ __forceinline__ FF two_sum(float a, float b)
{
    const float s = fa(a, b), bb = fsb(s, a);
    return FF{ s, fa(fsb(a, fsb(s, bb)), fsb(b, bb)) };
}
__device__ __forceinline__ FF two_prod(float a, float b)
{
    const float p = fm(a, b);
    return FF{ p, __fmaf_rn(a, b, -p) };
}
// a . b (three products) as a float pair
__device__ __forceinline__ FF dot_ff(const V3& a, const V3& b)
{
    const FF p0 = two_prod(a.x, b.x), p1 = two_prod(a.y, b.y), p2 = two_prod(a.z, b.z);
    const FF s1 = two_sum(p0.h, p1.h), s2 = two_sum(s1.h, p2.h);
    return FF{ s2.h, fa(fa(fa(s1.l, s2.l), fa(p0.l, p1.l)), p2.l) };
}
// x (a float pair) times 1 / lambda (a float pair)
__device__ __forceinline__ FF scale_ff(const FF& x, float ih, float il)
{
    const FF p = two_prod(x.h, ih);
    return FF{ p.h, fa(p.l, fa(fm(x.h, il), fm(x.l, ih))) };
}
// (ph + t) mod 1 in [-1/2, 1/2], ph and t float pairs (|ph| <= 1/2)
__device__ __forceinline__ float frac_ff(float ph_h, float ph_l, const FF& t)
{
    const float k = rintf(t.h);
    const float f = fa(fa(ph_h, fsb(t.h, k)), fa(ph_l, t.l));   // t.h - k is exact
    return fsb(f, rintf(f));
}
// a + b for float pairs (two-sum of the high parts, renormalised)
__device__ __forceinline__ FF add_ff(const FF& a, const FF& b)
{
    const FF s = two_sum(a.h, b.h);
    const float e = fa(s.l, fa(a.l, b.l));
    const float h = fa(s.h, e);
    return FF{ h, fsb(e, fsb(h, s.h)) };
}
// |v - x| (float pair): exact differences, a float-pair sum of squares and
// one Newton correction of the FP32 square root
__device__ __forceinline__ FF dist_ff(const V3& v, const V3& x)
{
    const FF dx = two_sum(v.x, -x.x), dy = two_sum(v.y, -x.y), dz = two_sum(v.z, -x.z);
    const FF qx = two_prod(dx.h, dx.h), qy = two_prod(dy.h, dy.h), qz = two_prod(dz.h, dz.h);
    const FF s1 = two_sum(qx.h, qy.h), s2 = two_sum(s1.h, qz.h);
    const float cross = fm(2.0f, fa(fa(fm(dx.h, dx.l), fm(dy.h, dy.l)), fm(dz.h, dz.l)));
    const float sl = fa(fa(fa(s1.l, s2.l), fa(fa(qx.l, qy.l), qz.l)), cross);
    const float r0 = __fsqrt_rn(s2.h);
    if (!(r0 > 0.0f)) return FF{ 0.0f, 0.0f };
    const FF r2 = two_prod(r0, r0);
    const float res = fa(fsb(fsb(s2.h, r2.h), r2.l), sl);
    return FF{ r0, __fdiv_rn(res, fm(2.0f, r0)) };
}

__device__ __forceinline__ float amp_dirs(const DevScene& S, int m, const V3& a, const V3& b)
{
    const int ty = S.scat_type[m];
    if (ty == SSTMC_SCATTERING_ISOTROPIC) return S.iso_amp;
    if (ty != SSTMC_SCATTERING_HENYEY_GREENSTEIN) return 0.0f;
    const float g = S.g[m];
    const V3 d = sub3(a, b);
    const float omg = 1.0f - g;
    const float dn = fmaf(g, dot3(d, d), omg * omg);
    return S.dims == 2 ? sqrtf(S.gup[m] / dn) : sqrtf(S.gup[m] / (dn * sqrtf(dn)));
}

__device__ __forceinline__ float pdf_dirs(const DevScene& S, int m, const V3& a, const V3& b)
{
    const int ty = S.scat_type[m];
    if (ty == SSTMC_SCATTERING_ISOTROPIC) return S.iso_pdf;
    if (ty != SSTMC_SCATTERING_HENYEY_GREENSTEIN) return 0.0f;
    const float g = S.g[m];
    const V3 d = sub3(a, b);
    const float omg = 1.0f - g;
    const float dn = fmaf(g, dot3(d, d), omg * omg);
    return S.dims == 2 ? S.gup[m] / dn : S.gup[m] / (dn * sqrtf(dn));
}

// ---- tabular scattering: nearest table entry of the scattering angle ----
// The angle is formed in FP64 from the FP32 positions (as the oracle does), so
// the rounding to a table index agrees with the CPU restatement.

// normalize(b - a) in FP64
__device__ __forceinline__ void dir64(const V3& a, const V3& b, double o[3])
{
    const double x = (double)b.x - (double)a.x, y = (double)b.y - (double)a.y, z = (double)b.z - (double)a.z;
    const double r = sqrt(x * x + y * y + z * z);
    o[0] = x / r; o[1] = y / r; o[2] = z / r;
}

// round_num(safeAcos(c) (N - 1) / pi, N), 2 pi in 2D (Scattering.cuh:907-917,
// Simulation.cuh:274-298; the FP64 safeAcos clamps within 1e-12 of +-1)
__device__ __forceinline__ int tab_index(const DevScene& S, int m, double c)
{
    const double th = c < -1.0 + 1e-12 ? kPi : (c > 1.0 - 1e-12 ? 0.0 : acos(c));
    const int N = S.tab_n[m];
    const int n = __double2int_rn(th * (double)(N - 1) / (S.dims == 2 ? 2.0 * kPi : kPi));
    return n < 0 ? 0 : (n >= N ? N - 1 : n);
}

// vMF mixture in 3D: amplitude sum_k exp(c mu_k + C'_k) (Scattering.cuh:933-946)
// and pdf sum_j w_j exp(c kappa_j + logN_j) (Scattering.cuh:997-1012), in FP64
__device__ __forceinline__ double vmf_amp(const DevScene& S, int m, double c)
{
    const double* p = S.vmf_mc + 2 * S.vmf_off[m];
    double r = 0.0;
    for (int k = 0; k < S.vmf_n[m]; ++k) r += exp(fma(c, p[2 * k], p[2 * k + 1]));
    return r;
}

__device__ __forceinline__ double vmf_pdf(const DevScene& S, int m, double c)
{
    const double* p = S.vmf_pd + 3 * S.vmf_poff[m];
    const int P = S.vmf_n[m] * S.vmf_n[m];
    double r = 0.0;
    for (int j = 0; j < P; ++j) r += p[3 * j + 1] * exp(fma(c, p[3 * j], p[3 * j + 2]));
    return r;
}

// Amplitude and pdf of a tabular or vMF material at scattering cosine c
__device__ __forceinline__ float2 amp64(const DevScene& S, int m, double c)
{
    if (S.scat_type[m] == SSTMC_SCATTERING_VMF_MIXTURE) return make_float2((float)vmf_amp(S, m, c), 0.0f);
    return S.tab_f[S.tab_off[m] + tab_index(S, m, c)];
}
__device__ __forceinline__ float pdf64(const DevScene& S, int m, double c)
{
    if (S.scat_type[m] == SSTMC_SCATTERING_VMF_MIXTURE) return (float)vmf_pdf(S, m, c);
    return S.tab_pdf[S.tab_off[m] + tab_index(S, m, c)];
}
__device__ __forceinline__ bool is_amp64(const DevScene& S, int m)
{
    return S.has_amp64 && (S.scat_type[m] == SSTMC_SCATTERING_TABULAR || S.scat_type[m] == SSTMC_SCATTERING_VMF_MIXTURE);
}

// The amplitude a source attached at a material-m vertex takes from an FP64
// angle (amp64): a point source in a scene whose materials are all isotropic
// takes the isotropic amplitude instead, also where a vMF mixture scatters
// (PointSource.cuh:347-360, 365-399); far-field sources evaluate the mixture
// (FarField.cuh:546-599).  The pdf of the vertex is the mixture's either way.
__device__ __forceinline__ bool src_amp64(const DevScene& S, const DevSource& s, int m)
{
    return is_amp64(S, m) && !(s.type == SSTMC_SOURCE_POINT && S.iso_all);
}

// Scattering cosine of source element k attached at pa with the path
// continuing to pb (threePointFunction, FarField.cuh:546-554,
// PointSource.cuh:317-345): a far-field direction d (views: -d) against the
// segment, or the direction from the point source into pa.
__device__ __forceinline__ double f3_cos64(const DevSource& s, int k, const V3& pa, const V3& pb, bool view)
{
    double ab[3];
    dir64(pa, pb, ab);
    if (s.type == SSTMC_SOURCE_FARFIELD) {
        const V3 d = load3(s.p, k);
        const double c = (double)d.x * ab[0] + (double)d.y * ab[1] + (double)d.z * ab[2];
        return view ? -c : c;
    }
    double in[3];
    dir64(load3(s.p, k), pa, in);
    return in[0] * ab[0] + in[1] * ab[1] + in[2] * ab[2];
}

// Incoming direction of illumination element l at x in FP64 (a far-field
// direction as stored, or normalize(x - s_l))
__device__ __forceinline__ void src_in64(const DevSource& s, int l, const V3& x, double o[3])
{
    if (s.type == SSTMC_SOURCE_FARFIELD) {
        const V3 d = load3(s.p, l);
        o[0] = d.x; o[1] = d.y; o[2] = d.z;
        return;
    }
    dir64(load3(s.p, l), x, o);
}

// Outgoing direction toward view element v from x in FP64
__device__ __forceinline__ void src_out64(const DevSource& s, int v, const V3& x, double o[3])
{
    if (s.type == SSTMC_SOURCE_FARFIELD) {
        const V3 d = load3(s.p, v);
        o[0] = d.x; o[1] = d.y; o[2] = d.z;
        return;
    }
    dir64(x, load3(s.p, v), o);
}

// Direction of travel from source element k into scatterer x (illumination side).
__device__ __forceinline__ V3 src_in(const DevSource& s, int k, const V3& x)
{
    if (s.type == SSTMC_SOURCE_FARFIELD) return load3(s.p, k);
    return unit3(sub3(x, load3(s.p, k)));
}

// Direction of travel from scatterer x toward view element k.
__device__ __forceinline__ V3 src_out(const DevSource& s, int k, const V3& x)
{
    if (s.type == SSTMC_SOURCE_FARFIELD) return load3(s.p, k);
    return unit3(sub3(load3(s.p, k), x));
}

// ---- value-path helpers (fast intrinsics; no decision depends on them) ----

__device__ __forceinline__ V3 funit(const V3& v)
{
    const float s = dot3(v, v);
    if (!(s > 0.0f)) return V3{ 0.f, 0.f, 1.f };
    const float r = rsqrtf(s);
    return V3{ v.x * r, v.y * r, v.z * r };
}

// Optical depth to the box edge of a single-cell medium.  The traversal of a
// single cell always takes exactly one step, so the step count does not
// depend on the arithmetic and fast reciprocals are used.
__device__ __forceinline__ float tau_single(const DevScene& S, const V3& o, const V3& d)
{
    float best = 3.0e38f;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        if (i == 2 && S.dims == 2) break;
        const float di = comp(d, i);
        const float inv = fabsf(di) < 1e-12f ? (di >= 0.0f ? 1e12f : -1e12f) : __fdividef(1.0f, di);
        const float face = di < 0.0f ? S.bmin[i] : S.bmax[i];
        best = fminf(best, (face - comp(o, i)) * inv);
    }
    return best * S.sigt[S.grid_m0];
}

// Optical depth from x along the exact direction d (a table direction), with
// the voxel-step count of the bit-exact traversal.
// cell: x's packed grid cell (cell_of) when the caller has it.
__device__ __forceinline__ float tau_dir(const DevScene& S, const V3& x, const V3& d, uint32_t& steps, uint32_t cell = kNoCell)
{
    if (S.single) {
        if (!inside(S, x)) return 0.0f;
        steps += 1;
        return tau_single(S, x, d);
    }
    return dda(S, x, d, steps, cell);
}

// Optical depth from x toward the point s.  Multi-cell media traverse along
// the IEEE-normalised direction (decision path); a single cell needs no exact
// direction.
__device__ __forceinline__ float tau_to_point(const DevScene& S, const V3& x, const V3& s, uint32_t& steps, uint32_t cell = kNoCell)
{
    if (S.single) {
        if (!inside(S, x)) return 0.0f;
        steps += 1;
        return tau_single(S, x, funit(sub3(s, x)));
    }
    const V3 dir = normalize32(S.dims, V3{ fsb(s.x, x.x), fsb(s.y, x.y), fsb(s.z, x.z) });
    return dda(S, x, dir, steps, cell);
}

// Henyey-Greenstein pdf / amplitude from two unit directions with fast
// intrinsics: dn = (1 - g)^2 + g |a - b|^2, pdf = gup dn^(-(D-1)/2... )
__device__ __forceinline__ float pdf_fast(const DevScene& S, int m, const V3& a, const V3& b)
{
    const int ty = S.scat_type[m];
    if (ty == SSTMC_SCATTERING_ISOTROPIC) return S.iso_pdf;
    if (ty != SSTMC_SCATTERING_HENYEY_GREENSTEIN) return 0.0f;
    const float g = S.g[m];
    const V3 d = sub3(a, b);
    const float omg = 1.0f - g;
    const float dn = fmaf(g, dot3(d, d), omg * omg);
    const float r = rsqrtf(dn);
    return S.dims == 2 ? S.gup[m] * r * r : S.gup[m] * r * r * r;
}

__device__ __forceinline__ float amp_fast(const DevScene& S, int m, const V3& a, const V3& b)
{
    const int ty = S.scat_type[m];
    if (ty == SSTMC_SCATTERING_ISOTROPIC) return S.iso_amp;
    if (ty != SSTMC_SCATTERING_HENYEY_GREENSTEIN) return 0.0f;
    const float g = S.g[m];
    const V3 d = sub3(a, b);
    const float omg = 1.0f - g;
    const float dn = fmaf(g, dot3(d, d), omg * omg);
    const float r = rsqrtf(dn);
    return S.dims == 2 ? S.sgup[m] * r : S.sgup[m] * r * sqrtf(r);
}

// P_l(x): attenuation toward illumination element l times its sampling density.
__device__ inline float pfirst(const DevScene& S, const DevSource& s, int l, const V3& x, uint32_t& steps)
{
    if (s.type == SSTMC_SOURCE_FARFIELD) {
        const V3 d = load3(s.p, l);
        const V3 nd = V3{ -d.x, -d.y, -d.z };
        return expf(-dda(S, x, nd, steps)) * s.sprob[l];
    }
    const V3 sp = load3(s.p, l);
    const V3 dir = normalize32(S.dims, V3{ fsb(sp.x, x.x), fsb(sp.y, x.y), fsb(sp.z, x.z) });
    const float T = expf(-dda(S, x, dir, steps));
    const V3 v = sub3(x, sp);
    const float r2 = dot3(v, v);
    const float k4pi = (float)(4.0 * kPi), k8pi = (float)(8.0 * kPi);
    return S.dims == 3 ? T / (k4pi * r2) : T * k8pi / sqrtf(r2);
}

// NEE vector of source element k at scatterer x.  with_phase = false returns
// the real amplitude sqrt(attenuation): used where the phase cancels exactly
// (u1 * conj(u2) with both fields evaluated at the same point and source).
__device__ inline float2 gvec(const DevScene& S, const DevSource& s, int k, const V3& x, int role, bool with_phase, uint32_t& steps)
{
    if (s.type == SSTMC_SOURCE_FARFIELD) {
        const V3 d = load3(s.p, k);
        const V3 dir = role == kRoleIllum ? V3{ -d.x, -d.y, -d.z } : d;
        const float a = sqrtf(expf(-dda(S, x, dir, steps)));
        if (!with_phase) return make_float2(a, 0.0f);
        float f;
        if (S.precision == SSTMC_PRECISION_SPLIT) {
            const FF t = scale_ff(dot_ff(d, x), S.il_h, S.il_l);
            f = role == kRoleIllum ? frac_ff(0.0f, 0.0f, t) : frac_ff(0.0f, 0.0f, FF{ -t.h, -t.l });
        } else {
            const float dx = d.x * x.x + d.y * x.y + d.z * x.z;
            const float ph = (role == kRoleIllum ? dx : -dx) * S.inv_lambda_f;
            f = ph - rintf(ph);
        }
        return c_scale(unit_phase(f), a);
    }
    const V3 sp = load3(s.p, k);
    const V3 dir = normalize32(S.dims, V3{ fsb(sp.x, x.x), fsb(sp.y, x.y), fsb(sp.z, x.z) });
    const float T = expf(-dda(S, x, dir, steps));
    FF r{ 0.0f, 0.0f };
    float rf;
    if (S.precision == SSTMC_PRECISION_SPLIT) {
        r = dist_ff(sp, x);
        rf = r.h;
    } else {
        const V3 v = sub3(x, sp);
        rf = sqrtf(dot3(v, v));
    }
    float at = S.dims == 3 ? T * kIsoAmp3 / (rf * rf) : T / rf;
    if (s.is_area) at *= fabsf(S.dims == 3 ? x.z - sp.z : x.y - sp.y) / rf;
    const float a = sqrtf(at);
    if (!with_phase) return make_float2(a, 0.0f);
    float f;
    if (S.precision == SSTMC_PRECISION_SPLIT) f = frac_ff(0.0f, 0.0f, scale_ff(r, S.il_h, S.il_l));
    else { const float ph = rf * S.inv_lambda_f; f = ph - rintf(ph); }
    return c_scale(unit_phase(f), a);
}

// f for the illumination side: element l -> scatterer pa -> point pb.
__device__ __forceinline__ V3 fsrc_in(const DevSource& s, int k, const V3& x)
{
    if (s.type == SSTMC_SOURCE_FARFIELD) return load3(s.p, k);
    return funit(sub3(x, load3(s.p, k)));
}

__device__ __forceinline__ V3 fsrc_out(const DevSource& s, int k, const V3& x)
{
    if (s.type == SSTMC_SOURCE_FARFIELD) return load3(s.p, k);
    return funit(sub3(load3(s.p, k), x));
}

__device__ __forceinline__ float famp_illum(const DevScene& S, const DevSource& s, int l, const V3& pa, const V3& pb, int m)
{
    if (s.type == SSTMC_SOURCE_POINT && S.iso_all) return S.iso_amp;
    return amp_dirs(S, m, src_in(s, l, pa), unit3(sub3(pb, pa)));
}

// f for the view side: point pb (previous vertex) -> scatterer pa -> view element v.
__device__ __forceinline__ float famp_view(const DevScene& S, const DevSource& s, int v, const V3& pa, const V3& pb, int m)
{
    if (s.type == SSTMC_SOURCE_POINT && S.iso_all) return S.iso_amp;
    return amp_dirs(S, m, unit3(sub3(pa, pb)), src_out(s, v, pa));
}

// Correlation-sampler shift x + h U(m), h = -/+ tau/2 (TemporalSamplerCorrelation.cuh:229-255).
__device__ __forceinline__ V3 shift_u(const DevScene& S, const V3& x, int m, float tau, float sign)
{
    const float h = fm(tau, fm(0.5f, sign));
    return V3{ ffma(h, S.U[m][0], x.x), ffma(h, S.U[m][1], x.y), S.dims == 3 ? ffma(h, S.U[m][2], x.z) : 0.0f };
}

__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ uint32_t warp_sum_u32(uint32_t v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

}  // namespace sstmc
