// scene.cpp -- config validation and scene tables (host side).
//
// Config semantics follow MatlabInterface.cu:712-1372 (buildScattering,
// buildMedium, buildSource, buildSampler): a single scattering cell is
// duplicated into material 1 (:750-760), material 0 may not appear inside the
// grid (:979-991), D must be non-negative (:1278-1283), correlation sources
// must come in same-size pairs (:1304-1320).  Far-field tables restate
// FarField.cuh:71-127 (fillBuffers) and MediumInterface.cuh:138-199
// (projectBoxToLine) in double precision and are stored as float; the field
// sampler's tick ordering restates TemporalSampler.cuh:958-1150.
//
// Compiled with -ffp-contract=off: the float tables must be bit-identical to
// any other host restatement of the same formulas.
#include "scene.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <functional>

namespace sstmc {

Scene::~Scene()
{
    for (void* p : dev_allocs) cudaFree(p);
}

namespace {

// The scene's device tables, packed into one allocation and one copy: tables
// are appended at 256-byte offsets, and each table's device pointer is set
// once the block exists (a scene of a few dozen tables is created with one
// cudaMalloc and one cudaMemcpy, and destroyed with one cudaFree).
struct TablePack {
    std::vector<unsigned char> host;
    std::vector<std::pair<size_t, std::function<void(const unsigned char*)>>> fix;

    void add_bytes(const void* data, size_t bytes, std::function<void(const unsigned char*)> set)
    {
        if (bytes == 0) return;
        const size_t off = (host.size() + 255) & ~size_t(255);
        host.resize(off + bytes);
        std::memcpy(host.data() + off, data, bytes);
        fix.emplace_back(off, std::move(set));
    }

    template <class T>
    void add(const std::vector<T>& v, const T** out)
    {
        *out = nullptr;
        add_bytes(v.data(), v.size() * sizeof(T), [out](const unsigned char* base) { *out = reinterpret_cast<const T*>(base); });
    }

    int commit(Scene* s)
    {
        if (host.empty()) return SSTMC_NO_ERROR;
        void* d = nullptr;
        if (cudaMalloc(&d, host.size()) != cudaSuccess) return SSTMC_ALLOCATION_ERROR;
        s->dev_allocs.push_back(d);
        if (cudaMemcpy(d, host.data(), host.size(), cudaMemcpyHostToDevice) != cudaSuccess) return SSTMC_ALLOCATION_ERROR;
        for (auto& f : fix) f.second(static_cast<const unsigned char*>(d) + f.first);
        return SSTMC_NO_ERROR;
    }
};

int prep_farfield(Scene::HostSource* s, const sstmc_source_cfg* c, int dims, const double bmin[3], const double bmax[3])
{
    const int n = (int)c->count;
    s->p.assign(3 * n, 0.f); s->inv.assign(3 * n, 0.f); s->tang.assign(3 * n, 0.f);
    s->pt.assign(3 * n, 0.f); s->ps.assign(3 * n, 0.f);
    s->mint.assign(n, 0.f); s->maxt.assign(n, 0.f); s->mins.assign(n, 0.f); s->maxs.assign(n, 0.f);
    s->sprob.assign(n, 0.f); s->sprob_d.assign(n, 0.0);
    double center[3], radius[3];
    for (int i = 0; i < 3; ++i) { center[i] = (bmax[i] + bmin[i]) * 0.5; radius[i] = (bmax[i] - bmin[i]) * 0.5; }
    double rc = radius[0] > radius[1] ? radius[0] : radius[1];
    if (dims == 3 && radius[2] > rc) rc = radius[2];
    rc = rc + 1e-12;
    for (int k = 0; k < n; ++k) {
        double v[3] = { c->xyz[3 * k], c->xyz[3 * k + 1], dims == 3 ? c->xyz[3 * k + 2] : 0.0 };
        double nrm = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        if (!(nrm > 0.0)) return SSTMC_INVALID_CONFIG;
        double inr = 1.0 / nrm;
        double d[3] = { v[0] * inr, v[1] * inr, v[2] * inr };
        double op[3] = { -d[0], -d[1], -d[2] };
        double tg[3], T[3], S[3] = { 0, 0, 0 };
        for (int i = 0; i < 3; ++i) tg[i] = center[i] + rc * op[i];
        if (dims == 3) {
            if (std::fabs(1.0 - std::fabs(op[2])) <= 1e-12) {
                T[0] = 1; T[1] = 0; T[2] = 0; S[0] = 0; S[1] = 1; S[2] = 0;
            } else {
                T[0] = -op[1]; T[1] = op[0]; T[2] = 0.0;
                double tn = 1.0 / std::sqrt(T[0] * T[0] + T[1] * T[1]);
                T[0] = T[0] * tn; T[1] = T[1] * tn;
                S[0] = T[1] * op[2] - T[2] * op[1];
                S[1] = T[2] * op[0] - T[0] * op[2];
                S[2] = T[0] * op[1] - T[1] * op[0];
            }
        } else {
            T[0] = -op[1]; T[1] = op[0]; T[2] = 0.0;
        }
        double mnT = 0, mxT = 0, mnS = 0, mxS = 0;
        const int corners = dims == 3 ? 8 : 4;
        for (int q = 0; q < corners; ++q) {
            double cc[3] = { (q & 1) ? bmax[0] : bmin[0], (q & 2) ? bmax[1] : bmin[1],
                             dims == 3 ? ((q & 4) ? bmax[2] : bmin[2]) : 0.0 };
            double pT = (cc[0] - tg[0]) * T[0] + (cc[1] - tg[1]) * T[1] + (cc[2] - tg[2]) * T[2];
            double pS = (cc[0] - tg[0]) * S[0] + (cc[1] - tg[1]) * S[1] + (cc[2] - tg[2]) * S[2];
            if (q == 0 || pT < mnT) mnT = pT;
            if (q == 0 || pT > mxT) mxT = pT;
            if (q == 0 || pS < mnS) mnS = pS;
            if (q == 0 || pS > mxS) mxS = pS;
        }
        for (int i = 0; i < 3; ++i) {
            s->p[3 * k + i] = (float)d[i];
            s->inv[3 * k + i] = (float)(std::fabs(d[i]) < 1e-12 ? 1e12 : 1.0 / d[i]);
            s->tang[3 * k + i] = (float)tg[i];
            s->pt[3 * k + i] = (float)T[i];
            s->ps[3 * k + i] = (float)S[i];
        }
        s->mint[k] = (float)mnT; s->maxt[k] = (float)mxT;
        s->mins[k] = (float)mnS; s->maxs[k] = (float)mxS;
        s->sprob_d[k] = dims == 3 ? 1.0 / ((mxT - mnT) * (mxS - mnS)) : 1.0 / (mxT - mnT);
        s->sprob[k] = (float)s->sprob_d[k];
    }
    return SSTMC_NO_ERROR;
}

int prep_source(Scene::HostSource* s, const sstmc_source_cfg* c, int dims, const double bmin[3], const double bmax[3])
{
    s->type = c->type; s->n = (int)c->count; s->is_area = c->is_area_source ? 1 : 0;
    if (c->type == SSTMC_SOURCE_NONE) { s->n = 0; return SSTMC_NO_ERROR; }
    if (c->count == 0 || c->xyz == nullptr) return SSTMC_INVALID_CONFIG;
    if (c->type == SSTMC_SOURCE_FARFIELD) return prep_farfield(s, c, dims, bmin, bmax);
    if (c->type == SSTMC_SOURCE_GAUSSIANBEAM) {
        // focal points in p, beam directions as given, ga = 1 / aperture^2
        // (GaussianBeam.cuh:1056-1068); the tables follow in prep_gauss
        if (!c->focal_direction || !(c->aperture > 0.0) || !std::isfinite(c->aperture)) return SSTMC_INVALID_CONFIG;
        s->gdir.resize(3 * s->n);
        for (int k = 0; k < 3 * s->n; ++k) s->gdir[k] = (float)c->focal_direction[k];
        for (int k = 0; k < s->n; ++k) {   // a beam needs a direction
            const float* d = s->gdir.data() + 3 * k;
            if (!(d[0] != 0.0f || d[1] != 0.0f || d[2] != 0.0f) || !std::isfinite(d[0]) || !std::isfinite(d[1]) || !std::isfinite(d[2]))
                return SSTMC_INVALID_CONFIG;
        }
        s->ga = 1.0 / (c->aperture * c->aperture);
        if (dims == 2) for (int k = 0; k < s->n; ++k) s->gdir[3 * k + 2] = 0.0f;
    } else if (c->type != SSTMC_SOURCE_POINT) {
        return SSTMC_NOT_SUPPORTED;
    }
    s->p.assign(3 * s->n, 0.f);
    for (int k = 0; k < s->n; ++k) {
        s->p[3 * k] = (float)c->xyz[3 * k];
        s->p[3 * k + 1] = (float)c->xyz[3 * k + 1];
        s->p[3 * k + 2] = dims == 3 ? (float)c->xyz[3 * k + 2] : 0.0f;
    }
    return SSTMC_NO_ERROR;
}

bool same_source(const Scene::HostSource& a, const Scene::HostSource& b)
{
    return a.type == b.type && a.n == b.n && a.is_area == b.is_area && a.p == b.p;
}

}  // namespace

// Tables of one tabular material (Scattering.cuh:272-384), in FP64 in the
// reference's order of operations: the sampling weights |f_i|^2 (x sin(theta_i)
// in 3D, theta_i = i pi / (N - 1)), their sum S, the cross section
// (S / N) 2 pi (x pi in 3D), the amplitude scaled by sqrt(1 / cross section),
// the inverse cdf by a lower bound of j / (N - 1) on the running sum of the
// normalised weights (angle = index x pi / (N - 1), or 2 pi / (N - 1) in 2D),
// and the evaluation pdf |f_n|^2 (x sin(theta_i) in 3D).
static void tabular_tables(const double* f, uint32_t N, int dims, std::vector<double>& fn, std::vector<double>& pdf,
                           std::vector<float>& cosv)
{
    std::vector<double> raw(N), cdf(N);
    auto theta = [&](uint32_t i) { return ((double)i / (double)(N - 1)) * kPi; };
    double sum = 0.0;
    for (uint32_t i = 0; i < N; ++i) {
        const double a2 = f[2 * i] * f[2 * i] + f[2 * i + 1] * f[2 * i + 1];
        raw[i] = dims == 2 ? a2 : a2 * std::sin(theta(i));
        sum += raw[i];
    }
    const double inv = 1.0 / sum;
    double run = 0.0;
    for (uint32_t i = 0; i < N; ++i) { run += raw[i] * inv; cdf[i] = run; }
    const double cross = (sum / (double)N) * 2.0 * kPi * (dims == 3 ? kPi : 1.0);
    const double sc = std::sqrt(1.0 / cross);
    fn.resize(2 * N);
    pdf.resize(N);
    for (uint32_t i = 0; i < N; ++i) {
        fn[2 * i] = f[2 * i] * sc;
        fn[2 * i + 1] = f[2 * i + 1] * sc;
        const double a2 = fn[2 * i] * fn[2 * i] + fn[2 * i + 1] * fn[2 * i + 1];
        pdf[i] = dims == 2 ? a2 : a2 * std::sin(theta(i));
    }
    cosv.resize(N);
    const double step = (dims == 2 ? 2.0 * kPi : kPi) / (double)(N - 1);
    for (uint32_t j = 0; j < N; ++j) {
        const double th = (double)j / (double)(N - 1);
        const uint32_t idx = (uint32_t)(std::lower_bound(cdf.begin(), cdf.end(), th) - cdf.begin());
        cosv[j] = (float)std::cos((double)idx * step);
    }
}

// vMFnormalizationLog in 3D (SpecialFunctions.cuh:187-203): the log of the
// normalisation kappa / (4 pi sinh kappa) of a vMF lobe; a kappa below 1e-12
// (negative ones included) takes the isotropic value.
static double vmf_log_norm(double x)
{
    if (x < 1e-12) return -std::log(4.0 * kPi);
    if (x < 5.0) return std::log(x) - std::log(4.0 * kPi * std::sinh(x));
    return std::log(x) - std::log(2.0 * kPi) - x;
}

// |I0(x)| of a real x >= 0, the modified Bessel function by the reference's
// algorithm (SpecialFunctions.cuh:42-178): the power series to k = 20 below 5,
// else the modulus-phase asymptotic form of J0(ix) (Abramowitz & Stegun
// 9.2.28-9.2.31), on the real axis where that form holds.
static double bessel_i0_real(double x)
{
    if (x == 0.0) return 1.0;
    if (x < 5.0) {
        const double Y = (0.5 * x) * (0.5 * x);
        double Bk = 1.0, res = 1.0;
        for (int k = 1; k <= 20; ++k) { Bk = (Y / ((double)k * (double)k)) * Bk; res += Bk; }
        return res;
    }
    // J0(y), y = i x: M cos(theta), the phase and modulus series in y
    const std::complex<double> y(0.0, x);
    std::complex<double> den = 4.0 * y;
    const std::complex<double> den2 = den * den;
    std::complex<double> th = y - 0.25 * kPi;
    const double tc[4] = { -1.0 / 2.0, 25.0 / 6.0, -1073.0 / 5.0, 375733.0 / 14.0 };
    for (int i = 0; i < 4; ++i) { th += tc[i] / den; den *= den2; }
    const std::complex<double> ct(std::cos(th.real()) * std::cosh(th.imag()), -std::sin(th.real()) * std::sinh(th.imag()));
    std::complex<double> M2(1.0, 0.0);
    const std::complex<double> t2 = 2.0 * y;
    std::complex<double> tq = t2 * t2;
    const std::complex<double> tq1 = tq;
    double mm = -1.0, ck = 1.0;
    for (int k = 1; k <= 10; ++k) {
        ck = ck * (2.0 * k - 1.0) / (2.0 * k);
        M2 += ck * mm / tq;
        tq *= tq1;
        mm *= -(2.0 * k + 1.0) * (2.0 * k + 1.0);
        if (std::abs(tq) > 1e20 || mm > 1e20) break;
    }
    return std::abs(std::sqrt((2.0 / kPi) * (M2 / y)) * ct);
}

// vMFnormalizationLog in 2D (SpecialFunctions.cuh:187-203): -log(2 pi) - log I0(x)
static double vmf_log_norm2(double x) { return -std::log(2.0 * kPi) - std::log(bessel_i0_real(x)); }

// Tables of one 3D vMF mixture (Scattering.cuh:636-774): the amplitude's
// components (mu_k, C_k + log alpha_k); the pdf's component pairs j = k1 + N k2
// with kappa_j = mu_k1 + mu_k2, weight exp(C'_k1 + C'_k2 - logN(kappa_j))
// normalised to sum 1, and the sampler's exclusive cdf of the weights.
static void vmf_tables(const double* mu, const double* c, const double* alpha, uint32_t N,
                       std::vector<double>& mc, std::vector<double>& pd, std::vector<float>& pf)
{
    for (uint32_t k = 0; k < N; ++k) { mc.push_back(mu[k]); mc.push_back(c[k] + std::log(alpha[k])); }
    const uint32_t P = N * N;
    std::vector<double> w(P), kap(P), ln(P);
    double sum = 0.0;
    for (uint32_t j = 0; j < P; ++j) {
        const uint32_t k1 = j % N, k2 = j / N;
        kap[j] = mu[k1] + mu[k2];
        ln[j] = vmf_log_norm(kap[j]);
        w[j] = std::exp(c[k1] + std::log(alpha[k1]) + c[k2] + std::log(alpha[k2]) - ln[j]);
        sum += w[j];
    }
    double cdf = 0.0;
    for (uint32_t j = 0; j < P; ++j) {
        const double pj = w[j] / sum;
        pd.push_back(kap[j]); pd.push_back(pj); pd.push_back(ln[j]);
        pf.push_back((float)cdf); pf.push_back((float)kap[j]); pf.push_back((float)std::exp(-2.0 * std::fabs(kap[j])));
        cdf += pj;
    }
}

// FP64 optical depth from o along d to the box edge, the parametric traversal
// of the walk (HeterogeneousMedium.cuh:386-573) in double: the attenuation of
// the Gaussian beams' distance bins, computed once per scene.
static double tau64_host(const Scene* S, const double o[3], const double d[3])
{
    const int D = S->dims;
    const DevScene& G = S->dev;
    for (int i = 0; i < D; ++i)
        if (!(o[i] >= (double)S->ax[i].front() && o[i] <= (double)S->ax[i].back())) return 0.0;
    double inv[3] = { 0, 0, 0 };
    int sg[3] = { 1, 1, 1 }, bin[3] = { 0, 0, 0 }, n[3] = { 0, 0, 0 };
    for (int i = 0; i < D; ++i) {
        n[i] = (int)S->ax[i].size();
        inv[i] = std::fabs(d[i]) < 1e-12 ? (d[i] >= 0.0 ? 1e12 : -1e12) : 1.0 / d[i];
        sg[i] = d[i] < 0.0 ? -1 : 1;
        int lo = 0, hi = n[i];
        while (lo < hi) { const int mid = (lo + hi) >> 1; if ((double)S->ax[i][mid] <= o[i]) lo = mid + 1; else hi = mid; }
        int c = lo - 1;
        c = c < 0 ? 0 : (c > n[i] - 2 ? n[i] - 2 : c);
        bin[i] = c;
    }
    double t = 0.0, acc = 0.0;
    for (int guard = 0; guard < (1 << 24); ++guard) {
        double tn[3] = { 0, 0, 0 };
        for (int i = 0; i < D; ++i) tn[i] = ((double)S->ax[i][bin[i] + (sg[i] > 0 ? 1 : 0)] - o[i]) * inv[i];
        int a;
        if (D == 2) a = tn[0] < tn[1] ? 0 : 1;
        else a = (tn[0] < tn[1] && tn[0] < tn[2]) ? 0 : (tn[1] < tn[2] ? 1 : 2);
        size_t idx = (size_t)bin[0] + (size_t)bin[1] * (n[0] - 1);
        if (D == 3) idx += (size_t)bin[2] * (n[0] - 1) * (n[1] - 1);
        const double seg = tn[a] - t;
        if (seg > 0) acc += seg * (double)G.sigt[S->grid[idx]];
        if (tn[a] > t) t = tn[a];
        if ((sg[a] < 0 && bin[a] == 0) || (sg[a] > 0 && bin[a] == n[a] - 2)) break;
        bin[a] += sg[a];
    }
    return acc;
}

// Projection distance of p on the line f + t d (MediumInterface.cuh:138-153)
static double gproj(const double p[3], const double f[3], const double d[3])
{
    double o[3];
    for (int i = 0; i < 3; ++i)
        o[i] = d[i] * d[0] * (p[0] - f[0]) + d[i] * d[1] * (p[1] - f[1]) + d[i] * d[2] * (p[2] - f[2]);
    return o[0] * d[0] + o[1] * d[1] + o[2] * d[2];
}

// Gaussian-beam scene tables (GaussianBeam.cuh:1029-1228, 1284-1566).
// Requirements (as the reference, or refused where it is undefined): 3D, the
// field sampler without CBS, illumination and view both GaussianBeam, every
// defined material a vMF mixture (of at most 8 lobes), each focal point inside
// the medium in a vMF material, a mean view direction of norm >= 1e-4 (the
// reference draws a random one below).  Per illumination beam: its focal
// material, the axial range [tmin, tmax] of the box on the beam line, the xy
// base, per lobe of the focal material the pdf and exclusive cdf of 1000
// distance bins, attenuation at the bin point over the squared beam width
// (T / ((ga + |mu|) / k^2 + dz^2 / ga)), normalised as the reference does (pdf
// times (B - 1) / sum), and the lobe weights exp(C' + l(|mu|)).  The bin
// attenuation runs along the first beam's backward direction for every beam,
// as the reference's attenuationDirection call with one direction computes it.
static int prep_gauss(Scene* S, bool cbs)
{
    DevScene& D = S->dev;
    Scene::HostSource& il = S->hsrc[0];
    Scene::HostSource& vw = S->hsrc[1];
    if (il.type != SSTMC_SOURCE_GAUSSIANBEAM || vw.type != SSTMC_SOURCE_GAUSSIANBEAM) return SSTMC_NOT_SUPPORTED;
    if (S->correlation || cbs) return SSTMC_NOT_SUPPORTED;
    for (int m = 0; m < kMat; ++m)
        if (D.gmix_n[m] == 0 && D.scat_type[m] != SSTMC_SCATTERING_NOT_DEFINED) return SSTMC_NOT_SUPPORTED;
    il.gnorm = S->dims == 3 ? vmf_log_norm(il.ga) : vmf_log_norm2(il.ga);
    vw.gnorm = S->dims == 3 ? vmf_log_norm(vw.ga) : vmf_log_norm2(vw.ga);
    if (S->dims == 2) return SSTMC_NO_ERROR;   // 2D beams sample and weigh as point sources: no tables
    double mv[3] = { 0, 0, 0 };
    const double inv = 1.0 / vw.n;
    for (int v = 0; v < vw.n; ++v)
        for (int a = 0; a < 3; ++a) mv[a] = mv[a] + inv * (double)vw.gdir[3 * v + a];
    const double r = std::sqrt(mv[0] * mv[0] + mv[1] * mv[1] + mv[2] * mv[2]);
    if (r < 0.0001) return SSTMC_NOT_SUPPORTED;
    for (int a = 0; a < 3; ++a) D.gmean[a] = mv[a] * (1.0 / r);
    const int n = il.n;
    int gM = 0;
    il.gfm.assign(n, 0);
    il.gtab.assign((size_t)9 * n, 0.0);
    for (int l = 0; l < n; ++l) {
        const float* f = il.p.data() + 3 * l;
        bool in = true;
        for (int a = 0; a < 3; ++a) in = in && f[a] >= S->ax[a].front() && f[a] <= S->ax[a].back();
        int fm = 0;
        if (in) {
            int c[3];
            for (int a = 0; a < 3; ++a) {
                const int na = (int)S->ax[a].size();
                int lo = 0, hi = na;
                while (lo < hi) { const int mid = (lo + hi) >> 1; if (S->ax[a][mid] <= f[a]) lo = mid + 1; else hi = mid; }
                int cc = lo - 1;
                c[a] = cc < 0 ? 0 : (cc > na - 2 ? na - 2 : cc);
            }
            const size_t nx = S->ax[0].size() - 1, ny = S->ax[1].size() - 1;
            fm = S->grid[(size_t)c[0] + (size_t)c[1] * nx + (size_t)c[2] * nx * ny];
        }
        if (fm <= 0 || D.gmix_n[fm] < 1 || D.gmix_n[fm] > 8) return SSTMC_NOT_SUPPORTED;
        il.gfm[l] = fm;
        gM = std::max(gM, D.gmix_n[fm]);
    }
    il.gM = gM;
    const size_t nb = (size_t)n * gM * kGaussBins;
    il.gpdf.assign(nb, 0.0); il.gicdf.assign(nb, 0.0);
    il.gapdf.assign((size_t)n * gM, 0.0); il.gaicdf.assign((size_t)n * gM, 0.0);
    const double k = 2.0 * kPi / S->cfg_copy.lambda;
    const double back0[3] = { -(double)il.gdir[0], -(double)il.gdir[1], -(double)il.gdir[2] };
    const double lo[3] = { (double)S->ax[0].front(), (double)S->ax[1].front(), (double)S->ax[2].front() };
    const double hi[3] = { (double)S->ax[0].back(), (double)S->ax[1].back(), (double)S->ax[2].back() };
    for (int l = 0; l < n; ++l) {
        double d[3], f[3];
        for (int i = 0; i < 3; ++i) { d[i] = il.gdir[3 * l + i]; f[i] = il.p[3 * l + i]; }
        double* tb = il.gtab.data() + 9 * l;
        double tmin = 0, tmax = 0;   // projectBoxToLine, MediumInterface.cuh:156-200
        for (int c = 0; c < 8; ++c) {
            const double cp[3] = { (c & 1) ? hi[0] : lo[0], (c & 2) ? hi[1] : lo[1], (c & 4) ? hi[2] : lo[2] };
            const double t = gproj(cp, f, d);
            if (c == 0 || t < tmin) tmin = t;
            if (c == 0 || t > tmax) tmax = t;
        }
        tb[0] = tmin; tb[1] = tmax; tb[2] = (tmax - tmin) / (double)kGaussBins;
        if (std::fabs(1.0 - std::fabs(d[2])) <= 1e-12) {   // orthogonalBase, VectorType.cuh:293-314
            tb[3] = 1; tb[4] = 0; tb[5] = 0; tb[6] = 0; tb[7] = 1; tb[8] = 0;
        } else {
            double b0[3] = { -d[1], d[0], 0.0 };
            const double rb = std::sqrt(b0[0] * b0[0] + b0[1] * b0[1]);
            b0[0] /= rb; b0[1] /= rb;
            tb[3] = b0[0]; tb[4] = b0[1]; tb[5] = 0.0;
            tb[6] = b0[1] * d[2] - b0[2] * d[1];
            tb[7] = b0[2] * d[0] - b0[0] * d[2];
            tb[8] = b0[0] * d[1] - b0[1] * d[0];
        }
        const int fm = il.gfm[l], M = D.gmix_n[fm];
        const double* mix = S->gmix.data() + 2 * D.gmix_off[fm];
        for (int b = 0; b < kGaussBins; ++b) {
            const double t = tmin + (double)b * tb[2];
            const double z[3] = { f[0] + t * d[0], f[1] + t * d[1], f[2] + t * d[2] };
            const double T = std::exp(-tau64_host(S, z, back0));
            const double dz = (z[0] - f[0]) * d[0] + (z[1] - f[1]) * d[1] + (z[2] - f[2]) * d[2];
            for (int m = 0; m < M; ++m)
                il.gpdf[((size_t)l * gM + m) * kGaussBins + b] = T / ((il.ga + std::fabs(mix[2 * m])) / (k * k) + dz * dz / il.ga);
        }
        for (int m = 0; m < M; ++m) {
            double* pdf = il.gpdf.data() + ((size_t)l * gM + m) * kGaussBins;
            double* cdf = il.gicdf.data() + ((size_t)l * gM + m) * kGaussBins;
            double run = 0.0;
            for (int b = 0; b < kGaussBins; ++b) { cdf[b] = run; run += pdf[b]; }
            const double tot = pdf[kGaussBins - 1] + cdf[kGaussBins - 1];
            for (int b = 0; b < kGaussBins; ++b) { pdf[b] *= (double)(kGaussBins - 1) / tot; cdf[b] /= tot; }
        }
        // lobe weights, alphaPdfIcdfKernel (GaussianBeam.cuh:254-295)
        double* ap = il.gapdf.data() + (size_t)l * gM;
        double* ac = il.gaicdf.data() + (size_t)l * gM;
        double asum = 0.0;
        for (int m = 0; m < M; ++m) {
            const double kap = std::fabs(mix[2 * m]);
            const double ln = kap < 1e-5 ? -std::log(4.0 * kPi)
                                         : std::log(kap) - (kap > 10.0 ? std::log(2.0 * kPi) * kap : std::log(4.0 * kPi * std::sinh(kap)));
            ap[m] = std::exp(mix[2 * m + 1] + ln);
            asum += ap[m];
        }
        for (int m = 0; m < M; ++m) ap[m] /= asum;
        double run = 0.0;
        for (int m = 0; m < M; ++m) { ac[m] = run; run += ap[m]; }
    }
    return SSTMC_NO_ERROR;
}

int build_scene(const sstmc_config* cfg, Scene* S, std::string* why)
{
    auto fail = [&](int code, const char* msg) { if (why) *why = msg; return code; };
    if (cfg->dims != 2 && cfg->dims != 3) return fail(SSTMC_INVALID_CONFIG, "dims must be 2 or 3");
    const int dims = S->dims = (int)cfg->dims;
    if (cfg->batch_size == 0 || cfg->full_iteration == 0 || cfg->renderings_num == 0)
        return fail(SSTMC_INVALID_CONFIG, "batchSize, fullIteration and renderingsNum must be positive");
    if (!(cfg->lambda > 0)) return fail(SSTMC_INVALID_CONFIG, "lambda must be positive");
    S->cfg_copy = *cfg;
    S->P = cfg->batch_size; S->full_iter = cfg->full_iteration; S->renders = cfg->renderings_num;
    S->seed = cfg->seed; S->device = cfg->device_number; S->precision = cfg->precision;
    DevScene& D = S->dev;
    std::memset(&D, 0, sizeof(D));
    D.dims = dims; D.P = S->P; D.precision = cfg->precision;

    // scattering
    if (cfg->scattering_num == 0 || cfg->scattering_num > (uint32_t)kMat || !cfg->scattering_type)
        return fail(SSTMC_INVALID_CONFIG, "scattering.type must have 1..10 cells");
    int M = (int)cfg->scattering_num;
    for (int m = 0; m < kMat; ++m) D.scat_type[m] = SSTMC_SCATTERING_NOT_DEFINED;
    size_t tab_pos = 0;   // running offset into cfg->tabular_f (entries)
    size_t vmf_pos = 0;   // running offset into cfg->vmf_* (components)
    bool iso_m[kMat] = { false };   // isIsotropicScattering per material (Scattering.cuh:1484-1512)
    for (int m = 0; m < M; ++m) {
        const int ty = cfg->scattering_type[m];
        const double g = (ty == SSTMC_SCATTERING_HENYEY_GREENSTEIN && cfg->scattering_g) ? cfg->scattering_g[m] : 0.0;
        if (ty != SSTMC_SCATTERING_ISOTROPIC && ty != SSTMC_SCATTERING_HENYEY_GREENSTEIN && ty != SSTMC_SCATTERING_TABULAR
            && ty != SSTMC_SCATTERING_VMF_MIXTURE)
            return fail(SSTMC_INVALID_CONFIG, "scattering types are Isotropic, Tabular, HenyeyGreenstein (HG) and VonMisesFisher (vMF)");
        if (ty == SSTMC_SCATTERING_HENYEY_GREENSTEIN && !(std::fabs(g) < 1.0)) return fail(SSTMC_INVALID_CONFIG, "|g| must be < 1");
        int toff = 0, tn = 0;
        if (ty == SSTMC_SCATTERING_TABULAR) {
            if (!cfg->tabular_n || !cfg->tabular_f || cfg->tabular_n[m] < 2)
                return fail(SSTMC_INVALID_CONFIG, "a tabular material needs an amplitude table of at least 2 entries");
            tn = (int)cfg->tabular_n[m];
            std::vector<double> fn, pdf;
            std::vector<float> cosv;
            tabular_tables(cfg->tabular_f + 2 * tab_pos, (uint32_t)tn, dims, fn, pdf, cosv);
            tab_pos += (size_t)tn;
            toff = (int)S->tab_pdf.size();
            for (int i = 0; i < tn; ++i) {
                S->tab_f.push_back((float)fn[2 * i]); S->tab_f.push_back((float)fn[2 * i + 1]);
                S->tab_f_d.push_back(fn[2 * i]); S->tab_f_d.push_back(fn[2 * i + 1]);
                S->tab_pdf.push_back((float)pdf[i]);
                S->tab_cos.push_back(cosv[i]);
            }
            D.has_amp64 = 1;
        }
        int voff = 0, vpoff = 0, vn = 0, goff = 0;
        bool iso = ty == SSTMC_SCATTERING_ISOTROPIC || (ty == SSTMC_SCATTERING_HENYEY_GREENSTEIN && std::fabs(g) < 0.0001);
        if (ty == SSTMC_SCATTERING_VMF_MIXTURE) {
            if (!cfg->vmf_n || !cfg->vmf_mu || !cfg->vmf_c || !cfg->vmf_alpha || cfg->vmf_n[m] < 1)
                return fail(SSTMC_INVALID_CONFIG, "a vMF material needs mixtureMu, mixtureC and mixtureAlpha with at least one component");
            vn = (int)cfg->vmf_n[m];
            const double* mu = cfg->vmf_mu + vmf_pos;
            const double* cc = cfg->vmf_c + vmf_pos;
            const double* al = cfg->vmf_alpha + vmf_pos;
            vmf_pos += (size_t)vn;
            // the lobes the Gaussian-beam terms read, mixtureMu and mixtureC + log(alpha)
            // (Scattering.cuh:703-721), in 2D too
            goff = (int)(S->gmix.size() / 2);
            for (int k = 0; k < vn; ++k) { S->gmix.push_back(mu[k]); S->gmix.push_back(cc[k] + std::log(al[k])); }
            double asum = 0.0;
            iso = true;   // isIsotropicScatteringVonMisesFisher: every |mu| <= 1e-4 (Scattering.cuh:744-751)
            for (int k = 0; k < vn; ++k) {
                if (!std::isfinite(mu[k]) || !std::isfinite(cc[k]) || !std::isfinite(al[k]) || al[k] < 0.0)
                    return fail(SSTMC_INVALID_CONFIG, "vMF mixtures need finite values and mixtureAlpha >= 0");
                asum += al[k];
                if (std::fabs(mu[k]) > 0.0001) iso = false;
            }
            if (!(asum > 0.0)) return fail(SSTMC_INVALID_CONFIG, "vMF mixtureAlpha must not be all zero");
            if (dims == 3) {   // in 2D the reference scatters vMF materials isotropically (Scattering.cuh:899-905, 1093-1100)
                voff = (int)(S->vmf_mc.size() / 2);
                vpoff = (int)(S->vmf_pd.size() / 3);
                vmf_tables(mu, cc, al, (uint32_t)vn, S->vmf_mc, S->vmf_pd, S->vmf_pf);
                D.has_amp64 = 1;
            }
        }
        const int targets[2] = { m, 1 };
        const int nt = (M == 1) ? 2 : 1;
        for (int q = 0; q < nt; ++q) {
            const int mm = targets[q];
            D.tab_off[mm] = toff;
            D.tab_n[mm] = tn;
            D.vmf_n[mm] = dims == 3 ? vn : 0;
            D.vmf_off[mm] = voff;
            D.vmf_poff[mm] = vpoff;
            D.gmix_n[mm] = vn;
            D.gmix_off[mm] = goff;
            iso_m[mm] = iso;
            D.scat_type[mm] = (ty == SSTMC_SCATTERING_VMF_MIXTURE && dims == 2) ? SSTMC_SCATTERING_ISOTROPIC : ty;
            S->g_d[mm] = g;
            D.g[mm] = (float)g;
            D.gup[mm] = (float)(dims == 2 ? 2.0 * ((1.0 - g * g) / (4.0 * kPi)) : (1.0 - g * g) / (4.0 * kPi));
            D.sgup[mm] = (float)std::sqrt(dims == 2 ? 2.0 * ((1.0 - g * g) / (4.0 * kPi)) : (1.0 - g * g) / (4.0 * kPi));
            D.gd1[mm] = (float)(1.0 + g * g);
            D.gd2[mm] = (float)(-2.0 * g);
        }
    }
    if (M == 1) M = 2;
    S->M = M;
    // isIsotropicScattering over every defined material (Scattering.cuh:1514-1528)
    D.iso_all = 1;
    for (int m = 0; m < kMat; ++m)
        if (D.scat_type[m] != SSTMC_SCATTERING_NOT_DEFINED && !iso_m[m]) D.iso_all = 0;
    D.iso_amp = dims == 2 ? kIsoAmp2 : kIsoAmp3;
    D.iso_pdf = dims == 2 ? kIsoPdf2 : kIsoPdf3;

    // medium
    double bmin[3] = { 0, 0, 0 }, bmax[3] = { 0, 0, 0 };
    double sigs[kMat] = { 0 }, siga[kMat] = { 0 };
    if (cfg->medium_type == SSTMC_MEDIUM_HOMOGENEOUS) {
        if (M != 2) return fail(SSTMC_INVALID_CONFIG, "Homogeneous medium cannot have heterogeneous material.");
        for (int a = 0; a < dims; ++a) {
            if (!(cfg->box_max[a] > cfg->box_min[a])) return fail(SSTMC_INVALID_CONFIG, "boxMax must exceed boxMin");
            S->ax[a] = { (float)cfg->box_min[a], (float)cfg->box_max[a] };
        }
        S->grid = { 1 };
        sigs[1] = cfg->homogeneous_sigs;
    } else if (cfg->medium_type == SSTMC_MEDIUM_HETEROGENEOUS) {
        const double* axes[3] = { cfg->x_axis, cfg->y_axis, cfg->z_axis };
        const uint32_t sizes[3] = { cfg->x_axis_size, cfg->y_axis_size, cfg->z_axis_size };
        size_t cells = 1;
        for (int a = 0; a < dims; ++a) {
            if (!axes[a] || sizes[a] < 2) return fail(SSTMC_INVALID_CONFIG, "medium axes need at least 2 edges");
            S->ax[a].resize(sizes[a]);
            for (uint32_t i = 0; i < sizes[a]; ++i) {
                S->ax[a][i] = (float)axes[a][i];
                if (i > 0 && !(S->ax[a][i] > S->ax[a][i - 1])) return fail(SSTMC_INVALID_CONFIG, "medium axes must increase");
            }
            cells *= (size_t)(sizes[a] - 1);
        }
        if (!cfg->material_grid || !cfg->sigs) return fail(SSTMC_INVALID_CONFIG, "materialGrid and sigs are required");
        S->grid.resize(cells);
        for (size_t i = 0; i < cells; ++i) {
            const uint32_t m = cfg->material_grid[i];
            if (m == 0) return fail(SSTMC_INVALID_CONFIG, "Material 0 is only allowed outside the grid.");
            if (m >= (uint32_t)M) return fail(SSTMC_INVALID_CONFIG, "materialGrid names an undefined material.");
            S->grid[i] = (unsigned char)m;
        }
        for (int m = 0; m < M; ++m) { sigs[m] = cfg->sigs[m]; siga[m] = cfg->siga ? cfg->siga[m] : 0.0; }
    } else {
        return fail(SSTMC_NOT_SUPPORTED, "unsupported medium type");
    }
    {
        bool seen[kMat] = { false };
        for (unsigned char m : S->grid) seen[m] = true;
        S->materials_present.clear();
        for (int m = 1; m < kMat; ++m) if (seen[m]) S->materials_present.push_back(m);
    }
    for (int a = 0; a < dims; ++a) {
        D.n[a] = (int)S->ax[a].size();
        D.bmin[a] = S->ax[a].front(); D.bmax[a] = S->ax[a].back();
        bmin[a] = (double)S->ax[a].front(); bmax[a] = (double)S->ax[a].back();
        const double c = (bmax[a] + bmin[a]) * 0.5, r = (bmax[a] - bmin[a]) * 0.5;
        D.center[a] = (float)c; D.radius[a] = (float)r;
        D.inv_radius[a] = std::fabs(D.radius[a]) < 1e-12f ? 1e12f : 1.0f / D.radius[a];
    }
    D.single = (S->grid.size() == 1) ? 1 : 0;
    D.grid_m0 = S->grid[0];
    float maxsigt = 0.0f;
    for (int m = 0; m < kMat; ++m) {
        if (sigs[m] < 0 || siga[m] < 0) return fail(SSTMC_INVALID_CONFIG, "sigs and siga must be non-negative");
        const float ss = (float)sigs[m], sa = (float)siga[m];
        D.sigt[m] = ss + sa;
        D.survive[m] = D.sigt[m] > 0.0f ? ss / D.sigt[m] : 1.0f;
        if (D.sigt[m] > maxsigt) maxsigt = D.sigt[m];
    }
    if (!(maxsigt > 0.0f)) return fail(SSTMC_INVALID_CONFIG, "the medium has no extinction (max sigt = 0)");
    D.inv_maxsigt = 1.0f / maxsigt;
    for (int m = 0; m < kMat; ++m) D.accept[m] = D.sigt[m] / maxsigt;

    // sources
    const sstmc_source_cfg* sc[4] = { &cfg->illumination, &cfg->view, &cfg->illumination2, &cfg->view2 };
    for (int i = 0; i < 4; ++i) {
        const int e = prep_source(&S->hsrc[i], sc[i], dims, bmin, bmax);
        if (e) return fail(e, "invalid source");
    }
    if (S->hsrc[0].type == SSTMC_SOURCE_NONE || S->hsrc[1].type == SSTMC_SOURCE_NONE)
        return fail(SSTMC_INVALID_CONFIG, "illumination and view are required");
    S->Nl = S->hsrc[0].n; S->Nv = S->hsrc[1].n;
    D.gauss = (S->hsrc[0].type == SSTMC_SOURCE_GAUSSIANBEAM || S->hsrc[1].type == SSTMC_SOURCE_GAUSSIANBEAM) ? 1 : 0;
    for (int m = 0; m < kMat; ++m) D.gsigs[m] = sigs[m];
    D.glz = dims == 3 ? bmax[2] - bmin[2] : 0.0;
    D.gk = 2.0 * kPi / cfg->lambda;

    // sampler
    if (!cfg->t || cfg->t_num == 0) return fail(SSTMC_INVALID_CONFIG, "sampler.t is required");
    S->correlation = cfg->sampler_type == SSTMC_SAMPLER_TEMPORAL_CORRELATION;
    if (cfg->sampler_type != SSTMC_SAMPLER_TEMPORAL && !S->correlation) return fail(SSTMC_INVALID_CONFIG, "unsupported sampler");
    D.correlation = S->correlation ? 1 : 0;
    if (S->correlation) {
        if (S->hsrc[2].type == SSTMC_SOURCE_NONE || S->hsrc[3].type == SSTMC_SOURCE_NONE)
            return fail(SSTMC_INVALID_CONFIG, "For correlation sampler, illumination2 and view2 must be entered");
        if (S->hsrc[2].n != S->hsrc[0].n || S->hsrc[3].n != S->hsrc[1].n)
            return fail(SSTMC_INVALID_CONFIG, "illumination2 / view2 must have the sizes of illumination / view");
        if (S->hsrc[2].type != S->hsrc[0].type || S->hsrc[3].type != S->hsrc[1].type)
            return fail(SSTMC_NOT_SUPPORTED, "illumination2 / view2 must have the types of illumination / view");
        D.sym = same_source(S->hsrc[0], S->hsrc[2]) && same_source(S->hsrc[1], S->hsrc[3]);
    }
    D.temporal_amp = cfg->is_temporal_amplitude ? 1 : 0;
    const int Nt = S->Nt = D.Nt = (int)cfg->t_num;
    S->ticks.assign(cfg->t, cfg->t + Nt);
    S->ticks_f.resize(Nt); S->abs_ticks.resize(Nt);
    for (int t = 0; t < Nt; ++t) { S->ticks_f[t] = (float)S->ticks[t]; S->abs_ticks[t] = std::fabs(S->ticks_f[t]); }
    double Dm[kMat];
    double Um[kMat][3];
    for (int m = 0; m < kMat; ++m) {
        Dm[m] = (m < M && cfg->D) ? cfg->D[m] : 0.0;
        if (Dm[m] < 0) return fail(SSTMC_INVALID_CONFIG, "D values in temporal sampler must be non-negative");
        for (int i = 0; i < 3; ++i) Um[m][i] = (m < M && cfg->U && i < dims) ? cfg->U[3 * m + i] : 0.0;
        D.D[m] = (float)Dm[m];
        S->D_d[m] = Dm[m];
        for (int i = 0; i < 3; ++i) D.U[m][i] = (float)Um[m][i];
        D.static_corr[m] = D.U[m][0] == 0.0f && D.U[m][1] == 0.0f && D.U[m][2] == 0.0f;
    }
    D.all_static_corr = 1;
    for (int m = 0; m < kMat; ++m) if (!D.static_corr[m]) D.all_static_corr = 0;
    // isForcedInsideBin belongs to the field sampler; the correlation sampler has no
    // such option and the reference ignores the field there (MatlabInterface.cu:1245-1282)
    D.forced_bin = (cfg->is_forced_inside_bin && !S->correlation) ? 1 : 0;
    if (D.gauss) {
        const int e = prep_gauss(S, cfg->is_cbs != 0);
        if (e) return fail(e, "GaussianBeam sources: 3D field sampler without CBS, both illumination and view GaussianBeam, "
                              "every material vMF, focal points inside vMF materials, a mean view direction");
    }
    D.ticks_geometric = S->abs_ticks[0] > 0.0f;
    for (int t = 0; t < Nt; ++t)
        if (S->abs_ticks[t] != (float)(t + 1) * S->abs_ticks[0]) D.ticks_geometric = 0;
    // field sampler: ticks sorted around their mean (TemporalSampler.cuh:958-1150)
    {
        double mean = 0;
        for (int t = 0; t < Nt; ++t) mean += S->ticks[t];
        mean = mean / Nt;
        std::vector<int> used(Nt, 0), negl, posl;
        int nn = 0, np = 0;
        for (int t = 0; t < Nt; ++t) { if (S->ticks[t] - mean < 0) nn++; else np++; }
        for (int a = 0; a < nn; ++a) {
            bool first = true; int idx = 0; double best = 0;
            for (int t = 0; t < Nt; ++t) if (!used[t] && S->ticks[t] - mean < 0) {
                if (first || mean - S->ticks[t] < best) { first = false; best = mean - S->ticks[t]; idx = t; }
            }
            used[idx] = 1; negl.push_back(idx);
        }
        for (int a = 0; a < np; ++a) {
            bool first = true; int idx = 0; double best = 0;
            for (int t = 0; t < Nt; ++t) if (!used[t] && S->ticks[t] - mean >= 0) {
                if (first || S->ticks[t] - mean < best) { first = false; best = S->ticks[t] - mean; idx = t; }
            }
            used[idx] = 1; posl.push_back(idx);
        }
        D.neg = nn;
        std::vector<double> dt(Nt);
        int cn = 0, cp = 0, prev = -1;
        for (int j = 0; j < Nt; ++j) {
            int tick;
            if (j < nn) { tick = negl[cn]; if (cn == 0) prev = -1; cn++; }
            else { tick = posl[cp]; if (cp == 0) prev = -1; cp++; }
            dt[j] = prev < 0 ? S->ticks[tick] - mean : S->ticks[tick] - S->ticks[prev];
            prev = tick;
        }
        S->disp_scale.assign((size_t)kMat * Nt, 0.f);
        S->disp_u.assign((size_t)kMat * Nt * 3, 0.f);
        for (int m = 0; m < kMat; ++m) {
            D.moving[m] = (Dm[m] != 0.0) || D.U[m][0] != 0.0f || D.U[m][1] != 0.0f || D.U[m][2] != 0.0f;
            for (int j = 0; j < Nt; ++j) {
                S->disp_scale[m * Nt + j] = (float)std::sqrt(2.0 * dims * Dm[m] * std::fabs(dt[j]));
                for (int i = 0; i < 3; ++i) S->disp_u[(m * Nt + j) * 3 + i] = (float)(dt[j] * Um[m][i]);
            }
        }
    }
    D.inv_lambda = 1.0 / cfg->lambda;
    D.inv_lambda_f = (float)D.inv_lambda;
    D.il_h = D.inv_lambda_f;
    D.il_l = (float)(D.inv_lambda - (double)D.il_h);
    D.k2 = (float)((2.0 * kPi / cfg->lambda) * (2.0 * kPi / cfg->lambda));

    // upload
    if (cudaSetDevice(S->device) != cudaSuccess) return fail(SSTMC_DEVICE_ERROR, "cudaSetDevice failed");
    TablePack pk;
    for (int a = 0; a < dims; ++a) pk.add(S->ax[a], &D.ax[a]);
    if (D.has_amp64) {
        D.tab_f = nullptr;
        pk.add_bytes(S->tab_f.data(), S->tab_f.size() * sizeof(float),
                     [&D](const unsigned char* base) { D.tab_f = reinterpret_cast<const float2*>(base); });
        pk.add(S->tab_pdf, &D.tab_pdf);
        pk.add(S->tab_cos, &D.tab_cos);
        pk.add(S->vmf_mc, &D.vmf_mc);
        pk.add(S->vmf_pd, &D.vmf_pd);
        pk.add(S->vmf_pf, &D.vmf_pf);
    }
    if (D.gauss) pk.add(S->gmix, &D.gmix);
    pk.add(S->grid, &D.grid);
    pk.add(S->disp_scale, &D.disp_scale);
    pk.add(S->disp_u, &D.disp_u);
    pk.add(S->ticks_f, &D.ticks_f);
    pk.add(S->abs_ticks, &D.abs_ticks);
    for (int i = 0; i < 4; ++i) {
        Scene::HostSource& h = S->hsrc[i];
        DevSource& d = D.src[i];
        d.type = h.type; d.n = h.n; d.is_area = h.is_area;
        if (h.type == SSTMC_SOURCE_NONE) continue;
        pk.add(h.p, &d.p);
        if (h.type == SSTMC_SOURCE_GAUSSIANBEAM) {
            d.ga = h.ga; d.gnorm = h.gnorm; d.gM = h.gM;
            d.gsame = 1;
            for (int k = 1; k < h.n; ++k)
                for (int a = 0; a < 3; ++a) if (h.gdir[3 * k + a] != h.gdir[a]) d.gsame = 0;
            pk.add(h.gdir, &d.gdir);
            if (!h.gfm.empty()) {
                pk.add(h.gfm, &d.gfm);
                pk.add(h.gtab, &d.gtab);
                pk.add(h.gpdf, &d.gpdf);
                pk.add(h.gicdf, &d.gicdf);
                pk.add(h.gapdf, &d.gapdf);
                pk.add(h.gaicdf, &d.gaicdf);
            }
        }
        if (h.type == SSTMC_SOURCE_FARFIELD) {
            pk.add(h.inv, &d.inv);
            pk.add(h.tang, &d.tang);
            pk.add(h.pt, &d.pt);
            pk.add(h.ps, &d.ps);
            pk.add(h.mint, &d.mint);
            pk.add(h.maxt, &d.maxt);
            pk.add(h.mins, &d.mins);
            pk.add(h.maxs, &d.maxs);
            pk.add(h.sprob, &d.sprob);
        }
    }
    const int e = pk.commit(S);
    if (e) return fail(e, "device allocation failed");
    return SSTMC_NO_ERROR;
}

}  // namespace sstmc
