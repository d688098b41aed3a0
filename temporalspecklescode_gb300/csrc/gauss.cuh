// gauss.cuh -- focused Gaussian-beam sources (GaussianBeam.cuh).  3D beams
// sample from their own tables; 2D beams sample and weigh as point sources at
// their focal points, with Bessel-I0 amplitudes.
//
//   first vertex from a beam        GaussianBeam.cuh:357-418 (sampleFirstBeam)
//   first-point probability P_l     GaussianBeam.cuh:420-487
//   second direction, lobe pairs    GaussianBeam.cuh:489-690 (computeCdfBuffer, sampleCdfBuffer)
//   second-point probability        GaussianBeam.cuh:693-753
//   NEE vector g                    GaussianBeam.cuh:795-816
//   three-point amplitude f         GaussianBeam.cuh:818-892
//   single-scattering amplitude fs  GaussianBeam.cuh:894-999
//   complex helpers                 ComplexType.cuh:84-215
//
// Everything is FP64.  The sampling arithmetic (the first vertex, the lobe
// pairs' mean directions) uses explicitly rounded operations in the order of
// the CPU oracle's restatement, so the vertices agree bit for bit; only the
// lobe-pair weights go through exp / log, whose last-ulp differences move a
// pick only when a uniform lands within that distance of a cdf boundary.
#pragma once
#include "nee.cuh"

namespace sstmc {

__device__ __forceinline__ double dA(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dS(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dM(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dD(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ double dQ(double a) { return __dsqrt_rn(a); }

struct CD { double re, im; };

__device__ __forceinline__ CD cd_add(CD a, CD b) { return CD{ dA(a.re, b.re), dA(a.im, b.im) }; }
__device__ __forceinline__ CD cd_sub(CD a, CD b) { return CD{ dS(a.re, b.re), dS(a.im, b.im) }; }
__device__ __forceinline__ CD cd_mul(CD a, CD b)
{
    return CD{ dS(dM(a.re, b.re), dM(a.im, b.im)), dA(dM(a.re, b.im), dM(a.im, b.re)) };
}
__device__ __forceinline__ double cd_abs(CD a) { return dQ(dA(dM(a.re, a.re), dM(a.im, a.im))); }
__device__ __forceinline__ CD cd_div(CD a, CD b)
{
    const double d = dA(dM(b.re, b.re), dM(b.im, b.im));
    return CD{ dD(dA(dM(a.re, b.re), dM(a.im, b.im)), d), dD(dS(dM(a.im, b.re), dM(a.re, b.im)), d) };
}
__device__ __forceinline__ CD cd_exp(CD a)
{
    const double e = exp(a.re);
    double s, c;
    sincos(a.im, &s, &c);
    return CD{ e * c, e * s };
}
// principal root: s = sqrt((|re| + |z|) / 2); (s, im / 2s) for re >= 0, else (|im| / 2s, +-s)
__device__ __forceinline__ CD cd_sqrt(CD a)
{
    if (a.re == 0.0 && a.im == 0.0) return CD{ 0.0, 0.0 };
    const double s = dQ(dM(dA(fabs(a.re), cd_abs(a)), 0.5));
    if (a.re >= 0.0) return CD{ s, dD(a.im, dM(2.0, s)) };
    return CD{ dD(fabs(a.im), dM(2.0, s)), copysign(s, a.im) };
}
// 1 / sqrt(z): the conjugate of the root over |root|^2
__device__ __forceinline__ CD cd_rsqrt(CD a)
{
    const double s2 = dM(dA(fabs(a.re), cd_abs(a)), 0.5);
    const double mult = dD(1.0, dA(s2, dD(dM(a.im, a.im), dM(4.0, s2))));
    const double s = dQ(s2);
    if (a.re >= 0.0) return CD{ dM(s, mult), dD(dM(-a.im, mult), dM(2.0, s)) };
    return CD{ dD(dM(fabs(a.im), mult), dM(2.0, s)), copysign(dM(s, mult), -a.im) };
}
// e^(c + z) - e^(c - z), each exponential dropped at or below a real part of -10
__device__ __forceinline__ CD cd_2sinh(CD z, CD c)
{
    const CD p = cd_add(c, z), n = cd_sub(c, z);
    CD r{ 0.0, 0.0 };
    if (p.re > -10.0) r = cd_add(r, cd_exp(p));
    if (n.re > -10.0) r = cd_sub(r, cd_exp(n));
    return r;
}

__device__ __forceinline__ CD cd_log(CD a) { return CD{ log(cd_abs(a)), atan2(a.im, a.re) }; }

// Complex modified Bessel function I0 by the reference's algorithm
// (SpecialFunctions.cuh:42-178, besseli with nu = 0): the power series
// sum_k ((z/2)^2)^k / (k!)^2 to k = 20 for |z| < 5, else J0(iz) in the
// modulus-phase asymptotic form of Abramowitz & Stegun 9.2.28-9.2.31 (the
// modulus series to k = 10, stopping once |(2y)^(2k)| or the coefficient
// product exceeds 1e20; four phase terms).  I0(0) = 1.
__device__ inline CD bessel_i0(CD z)
{
    const double az = cd_abs(z);
    if (az == 0.0) return CD{ 1.0, 0.0 };
    if (az < 5.0) {
        const CD h{ 0.5 * z.re, 0.5 * z.im };
        const CD Y{ (h.re - h.im) * (h.re + h.im), 2.0 * h.re * h.im };
        CD Bk{ 1.0, 0.0 }, res{ 1.0, 0.0 };
        for (int k = 1; k <= 20; ++k) {
            const double d = (double)k * (double)k;
            Bk = cd_mul(CD{ Y.re / d, Y.im / d }, Bk);
            res = cd_add(res, Bk);
        }
        return res;
    }
    const CD y{ -z.im, z.re };   // i z
    CD den{ 4.0 * y.re, 4.0 * y.im };
    const CD den2 = cd_mul(den, den);
    CD th{ y.re - 0.25 * kPi, y.im };
    const double tc[4] = { -1.0 / 2.0, 25.0 / 6.0, -1073.0 / 5.0, 375733.0 / 14.0 };
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        th = cd_add(th, cd_div(CD{ tc[i], 0.0 }, den));
        den = cd_mul(den, den2);
    }
    const CD ct{ cos(th.re) * cosh(th.im), -sin(th.re) * sinh(th.im) };
    CD M2{ 1.0, 0.0 };
    const CD t2{ 2.0 * y.re, 2.0 * y.im };
    CD tq = cd_mul(t2, t2);
    const CD tq1 = tq;
    double mm = -1.0, ck = 1.0;
    for (int k = 1; k <= 10; ++k) {
        ck = ck * (2.0 * k - 1.0) / (2.0 * k);
        M2 = cd_add(M2, cd_div(CD{ ck * mm, 0.0 }, tq));
        tq = cd_mul(tq, tq1);
        mm *= -(2.0 * k + 1.0) * (2.0 * k + 1.0);
        if (cd_abs(tq) > 1e20 || mm > 1e20) break;
    }
    CD q = cd_div(M2, y);
    q.re *= 2.0 / kPi; q.im *= 2.0 / kPi;
    return cd_mul(cd_sqrt(q), ct);
}

// ---- per-element arithmetic of the NEE and single-scattering sums ----
// Complex operations contracted to FMAs (the sampling code above keeps the
// explicitly rounded forms).
__device__ __forceinline__ CD cf_add(CD a, CD b) { return CD{ a.re + b.re, a.im + b.im }; }
__device__ __forceinline__ CD cf_sub(CD a, CD b) { return CD{ a.re - b.re, a.im - b.im }; }
__device__ __forceinline__ CD cf_mul(CD a, CD b) { return CD{ a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re }; }
__device__ __forceinline__ float g_ex2_32(float x)
{
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float g_rcp32(float x)
{
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
// e^x = 2^kk p for |x| < 700: x log2(e) split into an integer kk and a
// fraction in FP64 (log2(e) in two parts), p = 2^fraction by the FP32
// exponential instruction (relative error a few 1e-7)
__device__ __forceinline__ void exp_split(double x, float& p, double& kk)
{
    kk = rint(x * 1.4426950408889634);
    const double fr = fma(x, 1.4426950408889634, -kk) + x * 2.0355273740931033e-17;
    p = g_ex2_32((float)fr);
}
// e^z = 2^kk p (c, s): the magnitude by exp_split, the angle reduced to
// [-pi, pi] in FP64 (Cody and Waite's reduction with 2 pi in two parts) and
// (c, s) its FP32 cosine and sine
__device__ __forceinline__ void exp_parts(CD z, float& p, double& kk, float& c, float& s)
{
    exp_split(z.re, p, kk);
    const double n = rint(z.im * 0.15915494309189535);
    const double r = fma(-n, 2.4492935982947064e-16, fma(-n, 6.283185307179586, z.im));
    __sincosf((float)r, &s, &c);
}
// 2^kk for an integer-valued kk in [-1022, 1023], by the exponent field
__device__ __forceinline__ double pow2i(double kk)
{
    return __longlong_as_double((long long)((int)kk + 1023) << 52);
}
// principal square root: s = sqrt((|re| + |z|) / 2); (s, im / 2s) for re >= 0,
// else (|im| / 2s, +-s), with 1 / s from one reciprocal square root
__device__ __forceinline__ CD cf_sqrt(CD a)
{
    if (a.re == 0.0 && a.im == 0.0) return CD{ 0.0, 0.0 };
    const double h = 0.5 * (fabs(a.re) + sqrt(a.re * a.re + a.im * a.im));
    const double ri = rsqrt(h), s = h * ri;
    if (a.re >= 0.0) return CD{ s, 0.5 * a.im * ri };
    return CD{ 0.5 * fabs(a.im) * ri, copysign(s, a.im) };
}

// sum_i (a v_i + T_i)^2 over the three axes (a, v real; T complex)
__device__ __forceinline__ CD g_sumsq(double a, const double v[3], const CD T[3])
{
    CD r{ 0.0, 0.0 };
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const double x = dA(dM(a, v[i]), T[i].re), y = T[i].im;
        r.re = dA(r.re, dS(dM(x, x), dM(y, y)));
        r.im = dA(r.im, dM(dM(2.0, x), y));
    }
    return r;
}

// the beam's complex throughput ga d + i k (x - f)
__device__ __forceinline__ void g_throughput(const DevSource& s, int l, const double x[3], double k, CD T[3])
{
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        T[i].re = dM((double)s.gdir[3 * l + i], s.ga);
        T[i].im = dM(k, dS(x[i], (double)s.p[3 * l + i]));
    }
}

// vMFnormalizationLog in 3D (SpecialFunctions.cuh:187-203)
__device__ __forceinline__ double g_vmf_log_norm(double x)
{
    if (x < 1e-12) return -log(4.0 * kPi);
    if (x < 5.0) return log(x) - log(4.0 * kPi * sinh(x));
    return log(x) - log(2.0 * kPi) - x;
}

// Per lobe i of the focal material of beam l at x1: its c_i and real mean
// direction lv_i (computeCdfBuffer, GaussianBeam.cuh:530-583).  M <= 8.
struct GLobes {
    int M;
    double ga;
    double lc[8];
    double lv[8][3];
};

__device__ inline void g_lobes(const DevScene& S, const DevSource& s, int l, const V3& x1, GLobes& L)
{
    const int fmat = s.gfm[l];
    const int M = S.gmix_n[fmat];
    const double* mix = S.gmix + 2 * S.gmix_off[fmat];
    const double x[3] = { (double)x1.x, (double)x1.y, (double)x1.z };
    CD T[3];
    g_throughput(s, l, x, S.gk, T);
    L.M = M;
    L.ga = s.ga;
    for (int i = 0; i < M; ++i) {
        const double mu = mix[2 * i];
        if (fabs(mu) < 1e-9) {
            const double z0[3] = { 0.0, 0.0, 0.0 };
            const CD C = cd_sqrt(g_sumsq(0.0, z0, T));
            L.lc[i] = dA(dS(C.re, log(cd_abs(C))), mix[2 * i + 1]);
            L.lv[i][0] = L.lv[i][1] = L.lv[i][2] = 0.0;
        } else {
            CD g0 = cd_rsqrt(g_sumsq(mu, S.gmean, T));
            g0.re = dM(g0.re, mu); g0.im = dM(g0.im, mu);
            double cv[3];
#pragma unroll
            for (int a = 0; a < 3; ++a) cv[a] = dS(dM(g0.re, T[a].re), dM(g0.im, T[a].im));
            const double r = dD(1.0, dQ(dA(dA(dM(cv[0], cv[0]), dM(cv[1], cv[1])), dM(cv[2], cv[2]))));
            const double wv[3] = { dM(r, cv[0]), dM(r, cv[1]), dM(r, cv[2]) };
            const CD C = cd_sqrt(g_sumsq(mu, wv, T));
            const double wc = dA(dA(dM(wv[0], cv[0]), dM(wv[1], cv[1])), dM(wv[2], cv[2]));
            L.lc[i] = dS(dA(dS(C.re, log(cd_abs(C))), mix[2 * i + 1]), wc);
            L.lv[i][0] = cv[0]; L.lv[i][1] = cv[1]; L.lv[i][2] = cv[2];
        }
    }
}

// Lobe pair j = i1 + M i2: the summed mean direction, its log C (1 / (4 pi)
// below kappa = 1e-4, as the reference), and the unnormalised weight.
__device__ __forceinline__ double g_pair(const GLobes& L, int j, double cv[3], double& logC)
{
    const int i1 = j % L.M, i2 = j / L.M;
#pragma unroll
    for (int a = 0; a < 3; ++a) cv[a] = dA(L.lv[i1][a], L.lv[i2][a]);
    const double kap = dQ(dA(dA(dM(cv[0], cv[0]), dM(cv[1], cv[1])), dM(cv[2], cv[2])));
    logC = kap < 1e-4 ? 1.0 / (4.0 * kPi) : g_vmf_log_norm(kap);
    return exp(L.lc[i1] + L.lc[i2] - logC - 2.0 * L.ga);
}

__device__ __forceinline__ double g_pair_sum(const GLobes& L)
{
    double sum = 0.0, cv[3], lc;
    for (int j = 0; j < L.M * L.M; ++j) sum += g_pair(L, j, cv, lc);
    return sum;
}

// largest i < n with cdf[i] <= u (cdf[0] = 0)
__device__ __forceinline__ int g_cdf_pick(const double* cdf, int n, double u)
{
    int lo = 0, hi = n;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(cdf + mid) <= u) lo = mid; else hi = mid;
    }
    return lo;
}

// standard normal, Box-Muller's cosine branch in the walk's portable functions
__device__ __forceinline__ float g_normal(Stream& rs)
{
    const float u1 = rs.uniform(), u2 = rs.uniform();
    const float r = fsq(fm(-2.0f, walk_logf(u1)));
    float s, c;
    walk_sincospif(fm(2.0f, u2), s, c);
    return fm(r, c);
}

// First vertex from a beam: a beam uniformly, a lobe of its focal material, a
// distance bin and a uniform offset in it, a transverse Gaussian offset of
// variance w^2(dz) = (ga + |mu|) / k^2 + dz^2 / ga; x0 one unit back along the beam.
__device__ inline void gauss_first(const DevScene& S, const DevSource& s, Stream& rs, V3& x0, V3& x1, int& beam)
{
    const int n = s.n;
    int l = (int)ceilf(fm(rs.uniform(), (float)n)) - 1;
    l = l < 0 ? 0 : (l > n - 1 ? n - 1 : l);
    beam = l;
    const int fmat = s.gfm[l];
    const double* mix = S.gmix + 2 * S.gmix_off[fmat];
    const double* tb = s.gtab + 9 * l;
    const int m = g_cdf_pick(s.gaicdf + (size_t)l * s.gM, S.gmix_n[fmat], (double)rs.uniform());
    const int b = g_cdf_pick(s.gicdf + ((size_t)l * s.gM + m) * kGaussBins, kGaussBins, (double)rs.uniform());
    const double uo = (double)rs.uniform();
    double d[3], f[3], z[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) { d[i] = (double)s.gdir[3 * l + i]; f[i] = (double)s.p[3 * l + i]; }
    const double t = dA(tb[0], dM((double)b, tb[2]));
    const double step = dM(uo, tb[2]);
#pragma unroll
    for (int i = 0; i < 3; ++i) z[i] = dA(dA(f[i], dM(t, d[i])), dM(step, d[i]));
    const double k = S.gk;
    const double dz = dA(dA(dM(dS(z[0], f[0]), d[0]), dM(dS(z[1], f[1]), d[1])), dM(dS(z[2], f[2]), d[2]));
    const double wz = dQ(dA(dD(dA(s.ga, fabs(mix[2 * m])), dM(k, k)), dD(dM(dz, dz), s.ga)));
    const double n1 = (double)g_normal(rs), n2 = (double)g_normal(rs);
    float o[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) o[i] = __double2float_rn(dA(z[i], dM(wz, dA(dM(n1, tb[3 + i]), dM(n2, tb[6 + i])))));
    x1 = V3{ o[0], o[1], o[2] };
    x0 = V3{ fsb(o[0], s.gdir[3 * l]), fsb(o[1], s.gdir[3 * l + 1]), fsb(o[2], s.gdir[3 * l + 2]) };
}

// Second direction for beam l at x1: a lobe pair by the running-sum scan whose
// step back after the loop is kept, then a vMF direction about the pair's mean
// (the exact inverse cdf of the cosine, as for vMF scattering).
__device__ inline V3 gauss_second_dir(const DevScene& S, const DevSource& s, int l, const V3& x1, Stream& rs)
{
    GLobes L;
    g_lobes(S, s, l, x1, L);
    const double sum = g_pair_sum(L);
    const float u = rs.uniform();
    double cdf = 0.0, cv[3], lc;
    int j;
    for (j = 0; j < L.M * L.M; ++j) {
        if ((double)u < cdf) break;
        cdf += g_pair(L, j, cv, lc) / sum;
    }
    j--;
    g_pair(L, j, cv, lc);
    const double kap = dQ(dA(dA(dM(cv[0], cv[0]), dM(cv[1], cv[1])), dM(cv[2], cv[2])));
    V3 cen;
    if (kap < 1e-4) cen = V3{ 0.0f, 0.0f, 1.0f };
    else cen = V3{ __double2float_rn(dD(cv[0], kap)), __double2float_rn(dD(cv[1], kap)), __double2float_rn(dD(cv[2], kap)) };
    const float kf = __double2float_rn(kap);
    const float v = rs.uniform();
    float c;
    if (kf < 1e-4f) {
        c = fsb(fm(v, 2.0f), 1.0f);
    } else {
        const float e2k = __double2float_rn(exp(-2.0 * (double)kf));
        c = fa(1.0f, fdv(walk_logf(fa(v, fm(fsb(1.0f, v), e2k))), kf));
        if (c < -1.0f) c = -1.0f;
    }
    return rotate_dir(S, cen, c, rs);
}

// P_l(x1): the bin pdf at x1's axial offset times the transverse Gaussian,
// summed over the focal material's lobes, over sigs(x1) times the box depth.
__device__ inline double gauss_pfirst(const DevScene& S, const DevSource& s, int l, const V3& x1, int m1)
{
    const int fmat = s.gfm[l], M = S.gmix_n[fmat];
    const double* mix = S.gmix + 2 * S.gmix_off[fmat];
    const double* tb = s.gtab + 9 * l;
    double d[3], f[3], x[3] = { (double)x1.x, (double)x1.y, (double)x1.z };
#pragma unroll
    for (int i = 0; i < 3; ++i) { d[i] = (double)s.gdir[3 * l + i]; f[i] = (double)s.p[3 * l + i]; }
    double o[3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
        o[i] = d[i] * d[0] * (x[0] - f[0]) + d[i] * d[1] * (x[1] - f[1]) + d[i] * d[2] * (x[2] - f[2]);
    const double dz = o[0] * d[0] + o[1] * d[1] + o[2] * d[2];
    double dxy2 = 0.0;
#pragma unroll
    for (int i = 0; i < 3; ++i) { const double e = f[i] + dz * d[i] - x[i]; dxy2 += e * e; }
    int zi;
    if (dz < tb[0]) zi = 0;
    else if (dz > tb[1]) zi = kGaussBins - 1;
    else { zi = (int)((dz - tb[0]) / tb[2]); zi = zi < 0 ? 0 : (zi > kGaussBins - 1 ? kGaussBins - 1 : zi); }
    const double k2 = S.gk * S.gk;
    double pdf = 0.0;
    for (int m = 0; m < M; ++m) {
        const double pz = __ldg(s.gpdf + ((size_t)l * s.gM + m) * kGaussBins + zi);
        const double w2 = (s.ga + fabs(mix[2 * m])) / k2 + dz * dz / s.ga;
        const double pxy = exp(-dxy2 / (2.0 * w2)) / ((2.0 * w2) * kPi);
        pdf += __ldg(s.gapdf + (size_t)l * s.gM + m) * pz * pxy;
    }
    return pdf / (S.gsigs[m1] * S.glz);
}

// p2 factor of beam l for the direction x1 -> x2: sum_j w_j exp(conv_j . o + log C_j)
__device__ inline double gauss_pw(const DevScene& S, const DevSource& s, int l, const V3& x1, const V3& x2)
{
    GLobes L;
    g_lobes(S, s, l, x1, L);
    const double sum = g_pair_sum(L);
    double o[3];
    dir64(x1, x2, o);
    double r = 0.0, cv[3], lc;
    for (int j = 0; j < L.M * L.M; ++j) {
        const double w = g_pair(L, j, cv, lc) / sum;
        r += w * exp(cv[0] * o[0] + cv[1] * o[1] + cv[2] * o[2] + lc);
    }
    return r;
}

// f: beam k -> scatterer pa -> pb (illumination) or pb -> pa -> beam k (view,
// k negative): sum over pa's lobes of 2 sinh(sqrt(mu)) e^(log nu) / sqrt(mu).
__device__ inline CD gauss_f(const DevScene& S, const DevSource& s, int k, const V3& pa, const V3& pb, int m, bool view)
{
    CD acc{ 0.0, 0.0 };
    if (m <= 0) return acc;
    double w0[3];
    if (!view) dir64(pa, pb, w0);
    else dir64(pb, pa, w0);
    const double kk = view ? -S.gk : S.gk;
    const double x[3] = { (double)pa.x, (double)pa.y, (double)pa.z };
    CD T[3];
    g_throughput(s, k, x, kk, T);
    const double tc = s.gnorm + log(2.0 * kPi);
    const double* mix = S.gmix + 2 * S.gmix_off[m];
    for (int i = 0; i < S.gmix_n[m]; ++i) {
        const CD lnu{ tc + mix[2 * i + 1], 0.0 };
        if (S.dims == 2) {
            const CD sm = cd_sqrt(g_sumsq(mix[2 * i], w0, T));
            acc = cd_add(acc, cd_exp(cd_add(cd_log(bessel_i0(sm)), lnu)));
            continue;
        }
        const CD sm = cf_sqrt(g_sumsq(mix[2 * i], w0, T));
        const double lr = lnu.re, posre = lr + sm.re, negre = lr - sm.re;
        if (fabs(sm.re) < 0.0001 && fabs(sm.im) < 0.0001) {
            acc.re += 2.0 * exp(lr);
        } else if (fabs(lr) < 300.0 && fabs(posre) < 300.0 && fabs(negre) < 600.0 && fabs(sm.re) + fabs(sm.im) > 0.05) {
            // 2 sinh(sm) e^lnu / sm: e^(lnu + sm) = 2^kk p (c, s), e^(lnu - sm) =
            // e^(2 lnu) / e^(lnu + sm) = 2^(k2 - kk) (p2 / p) (c, -s); each dropped
            // at a real part of -10 or below
            float pf, c, s, p2;
            double kk, k2;
            exp_parts(CD{ posre, sm.im }, pf, kk, c, s);
            exp_split(2.0 * lr, p2, k2);
            CD r{ 0.0, 0.0 };
            if (posre > -10.0) {
                const double mg = (double)pf * pow2i(kk);
                r = CD{ mg * (double)c, mg * (double)s };
            }
            if (negre > -10.0) {
                const double mg = (double)(p2 * g_rcp32(pf)) * pow2i(k2 - kk);
                r.re -= mg * (double)c;
                r.im += mg * (double)s;
            }
            // / sm: the reciprocal of |sm|^2 to FP32 accuracy
            const double iw = (double)g_rcp32((float)(sm.re * sm.re + sm.im * sm.im));
            acc = cf_add(acc, CD{ (r.re * sm.re + r.im * sm.im) * iw, (r.im * sm.re - r.re * sm.im) * iw });
        } else {
            acc = cd_add(acc, cd_div(cd_2sinh(sm, lnu), sm));
        }
    }
    return acc;
}

// fs: illumination beam l -> x -> view beam v: the lobe convolved with the
// illumination throughput, then integrated against the view's.
__device__ inline CD gauss_fs(const DevScene& S, const DevSource& il, int l, const DevSource& vw, int v, const V3& xf, int m)
{
    CD acc{ 0.0, 0.0 };
    if (m <= 0) return acc;
    const double k = S.gk;
    const double x[3] = { (double)xf.x, (double)xf.y, (double)xf.z };
    CD aT[3], bT[3];
    g_throughput(il, l, x, k, aT);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        bT[i].re = dM((double)vw.gdir[3 * v + i], vw.ga);
        bT[i].im = dM(k, dS((double)vw.p[3 * v + i], x[i]));
    }
    const double vd[3] = { (double)vw.gdir[3 * v], (double)vw.gdir[3 * v + 1], (double)vw.gdir[3 * v + 2] };
    const double tc = il.gnorm + vw.gnorm + 2.0 * log(2.0 * kPi);
    const double* mix = S.gmix + 2 * S.gmix_off[m];
    const double z0[3] = { 0.0, 0.0, 0.0 };
    for (int i = 0; i < S.gmix_n[m]; ++i) {
        const double gs = mix[2 * i];
        const CD lnu{ tc + mix[2 * i + 1], 0.0 };
        CD C, sm, c{ 0.0, 0.0 };
        if (fabs(gs) < 0.000001) {
            C = cd_sqrt(g_sumsq(0.0, z0, aT));
            sm = cd_sqrt(g_sumsq(0.0, z0, bT));
        } else {
            CD g0 = cd_rsqrt(g_sumsq(gs, vd, aT));
            g0.re = dM(g0.re, gs); g0.im = dM(g0.im, gs);
            CD q{ 0.0, 0.0 }, aw{ 0.0, 0.0 };
            double wv[3];
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const CD e = cd_add(cd_mul(g0, aT[a]), bT[a]);
                q = cd_add(q, cd_mul(e, e));
                wv[a] = dS(dM(g0.re, aT[a].re), dM(g0.im, aT[a].im));
            }
            sm = cd_sqrt(q);
            const double ra = dD(1.0, dQ(dA(dA(dM(wv[0], wv[0]), dM(wv[1], wv[1])), dM(wv[2], wv[2]))));
            C = cd_sqrt(g_sumsq(dM(gs, ra), wv, aT));
#pragma unroll
            for (int a = 0; a < 3; ++a) { aw.re = dA(aw.re, dM(aT[a].re, wv[a])); aw.im = dA(aw.im, dM(aT[a].im, wv[a])); }
            c = cd_mul(g0, aw);
            c.re = dM(c.re, -ra); c.im = dM(c.im, -ra);
        }
        const CD cl = cd_add(c, lnu);
        if (S.dims == 2) {
            acc = cd_add(acc, cd_exp(cd_add(cd_add(cd_log(bessel_i0(C)), cd_log(bessel_i0(sm))), cl)));
            continue;
        }
        const bool sbig = fabs(sm.re) > 0.0001 || fabs(sm.im) > 0.0001;
        const bool cbig = fabs(C.re) > 0.0001 || fabs(C.im) > 0.0001;
        if (sbig && cbig) {
            acc = cd_add(acc, cd_div(cd_2sinh(cd_add(C, sm), cl), cd_mul(C, sm)));
        } else if (!sbig && !cbig) {
            const CD e = cd_exp(cl);
            acc.re += 4.0 * e.re; acc.im += 4.0 * e.im;
        } else if (!sbig) {
            const CD e = cd_div(cd_2sinh(C, cl), C);
            acc.re += 2.0 * e.re; acc.im += 2.0 * e.im;
        } else {
            const CD e = cd_div(cd_2sinh(sm, lnu), sm);
            acc.re += 2.0 * e.re; acc.im += 2.0 * e.im;
        }
    }
    return acc;
}

}  // namespace sstmc
