// walk.cuh -- FP32 random walk and voxel traversal (decision path).
//
// Restates, per path and on the GPU:
//   Woodcock free flight + absorption roulette  HeterogeneousMedium.cuh:576-678
//   outside-point "ray hits box" test           HeterogeneousMedium.cuh:269-383 (bdDistance)
//   voxel lookup                                Simulation.cuh:325-367, HeterogeneousMedium.cuh:260-267
//   voxel traversal (attenuation)               HeterogeneousMedium.cuh:386-573
//   far-field / point first-vertex sampling     FarField.cuh:129-205, PointSource.cuh:72-90
//   phase-function sampling (Iso, HG)           Scattering.cuh:1039-1115
//   direction rotation, random direction        VectorType.cuh:207-283, 316-362
// The traversal is parametric (face distances from the ray origin, not from
// an advanced point) so rounding does not accumulate along long rays.
#pragma once
#include "device_math.cuh"
#include "scene.h"

namespace sstmc {

struct V3 { float x, y, z; };

__device__ __forceinline__ float comp(const V3& v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }
__device__ __forceinline__ V3 load3(const float* p, int k) { return V3{ p[3 * k], p[3 * k + 1], p[3 * k + 2] }; }

__device__ __forceinline__ bool inside(const DevScene& S, const V3& p)
{
    bool in = p.x >= S.bmin[0] && p.x <= S.bmax[0] && p.y >= S.bmin[1] && p.y <= S.bmax[1];
    if (S.dims == 3) in = in && p.z >= S.bmin[2] && p.z <= S.bmax[2];
    return in;
}

// cell c with ax[c] <= x < ax[c+1], clamped to [0, n-2]
__device__ __forceinline__ int bin_of(const float* ax, int n, float x)
{
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(ax + mid) <= x) lo = mid + 1; else hi = mid;
    }
    int c = lo - 1;
    c = c < 0 ? 0 : c;
    c = c > n - 2 ? n - 2 : c;
    return c;
}

__device__ __forceinline__ int material_at(const DevScene& S, const V3& p)
{
    const int ix = bin_of(S.ax[0], S.n[0], p.x);
    const int iy = bin_of(S.ax[1], S.n[1], p.y);
    int idx = ix + iy * (S.n[0] - 1);
    if (S.dims == 3) idx += bin_of(S.ax[2], S.n[2], p.z) * (S.n[0] - 1) * (S.n[1] - 1);
    return __ldg(S.grid + idx);
}

// Whether the ray from p along d hits the box; *hit = distance to the face it
// enters (or leaves, from inside) first.
__device__ inline bool points_toward(const DevScene& S, const V3& p, const V3& d, float* hit = nullptr)
{
    const int D = S.dims;
    float o[3], inv[3], dist[3];
    float mx = 0.0f;
    for (int i = 0; i < D; ++i) {
        o[i] = fsb(comp(p, i), S.center[i]);
        const float a = fm(fabsf(o[i]), S.inv_radius[i]);
        if (i == 0 || a > mx) mx = a;
        const float di = comp(d, i);
        inv[i] = fabsf(di) < 1e-12f ? 1e12f : fdv(1.0f, di);
    }
    const float winding = mx <= 1.0f ? -1.0f : 1.0f;
    for (int i = 0; i < D; ++i) {
        const float sg = comp(d, i) < 0.0f ? 1.0f : -1.0f;
        dist[i] = fm(inv[i], fsb(fm(S.radius[i], winding * sg), o[i]));
    }
    for (int i = 0; i < D; ++i) {
        if (!(dist[i] >= 0.0f)) continue;
        bool ok = true;
        for (int j = 0; j < D; ++j) {
            if (j == i) continue;
            if (!(fabsf(ffma(comp(d, j), dist[i], o[j])) < S.radius[j])) ok = false;
        }
        if (ok) { if (hit) *hit = dist[i]; return true; }
    }
    return false;
}

__device__ __forceinline__ V3 normalize32(int dims, const V3& v)
{
    const float s = dims == 3 ? ffma(v.x, v.x, ffma(v.y, v.y, fm(v.z, v.z))) : ffma(v.x, v.x, fm(v.y, v.y));
    if (!(s > 0.0f)) return dims == 3 ? V3{ 0.f, 0.f, 1.f } : V3{ 0.f, 1.f, 0.f };
    const float inv = fdv(1.0f, fsq(s));
    return V3{ fm(v.x, inv), fm(v.y, inv), dims == 3 ? fm(v.z, inv) : 0.0f };
}

__device__ __forceinline__ V3 random_direction(int dims, Stream& rs)
{
    if (dims == 2) {
        float s, c;
        walk_sincospif(fm(2.0f, rs.uniform()), s, c);
        return V3{ s, c, 0.0f };
    }
    float sp, cp;
    walk_sincospif(fm(2.0f, rs.uniform()), sp, cp);
    const float ct = ffma(rs.uniform(), 2.0f, -1.0f);
    const float st = fsq(fmaxf(0.0f, fsb(1.0f, fm(ct, ct))));
    return V3{ fm(st, cp), fm(st, sp), ct };
}

// vMF mixture cosine: a component pair j by the exclusive cdf of the pair
// weights (Scattering.cuh:1065-1077), then the cosine of a vMF lobe of
// concentration kappa_j.  The reference draws that cosine with Wood's
// rejection loop (VectorType.cuh:169-203); here it is the exact inverse cdf of
// the density ~ exp(kappa w) on [-1, 1]:
// w = 1 + log(v + (1 - v) exp(-2 |kappa|)) / |kappa|, negated for kappa < 0.
__device__ __forceinline__ float vmf_cosine(const DevScene& S, int m, Stream& rs)
{
    const float* pf = S.vmf_pf + 3 * S.vmf_poff[m];
    const int P = S.vmf_n[m] * S.vmf_n[m];
    const float u = rs.uniform();
    int lo = 0, hi = P;   // pairs whose cdf is <= u
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(pf + 3 * mid) <= u) lo = mid + 1; else hi = mid;
    }
    const int j = lo > 0 ? lo - 1 : 0;
    const float kap = __ldg(pf + 3 * j + 1), e2k = __ldg(pf + 3 * j + 2);
    const float v = rs.uniform();
    const float ak = fabsf(kap);
    if (ak < 1e-4f) return fsb(fm(v, 2.0f), 1.0f);
    const float w = fmaxf(-1.0f, fa(1.0f, fdv(walk_logf(fa(v, fm(fsb(1.0f, v), e2k))), ak)));
    return kap < 0.0f ? -w : w;
}

// VMF: the scene has vMF materials (3D).  Without it the vMF branch is not
// compiled, so scenes without vMF run the walk code they ran before vMF existed.
__device__ inline V3 rotate_dir(const DevScene& S, const V3& din, float c, Stream& rs);

template <bool VMF>
__device__ inline V3 sample_direction(const DevScene& S, int m, const V3& din, Stream& rs)
{
    const int ty = S.scat_type[m];
    if (ty != SSTMC_SCATTERING_HENYEY_GREENSTEIN && ty != SSTMC_SCATTERING_TABULAR && !(VMF && ty == SSTMC_SCATTERING_VMF_MIXTURE))
        return random_direction(S.dims, rs);
    const float g = S.g[m];
    float c;
    if (VMF && ty == SSTMC_SCATTERING_VMF_MIXTURE) {
        c = vmf_cosine(S, m, rs);
    } else if (ty == SSTMC_SCATTERING_TABULAR) {
        // inverse-cdf table entry round_num(xi N, N) (Scattering.cuh:1030-1037,
        // Simulation.cuh:287-298: nearest, ties to even, clamped to N - 1)
        const int N = S.tab_n[m];
        int k = (int)rintf(fm(rs.uniform(), (float)N));
        k = k < 0 ? 0 : (k >= N ? N - 1 : k);
        c = S.tab_cos[S.tab_off[m] + k];
    } else if (fabsf(g) < 0.001f) {
        c = fsb(fm(rs.uniform(), 2.0f), 1.0f);
    } else {
        const float xi = rs.uniform();
        if (S.dims == 2) {
            const float a = fdv(fsb(1.0f, g), fa(1.0f, g));
            float sp, cp;
            walk_sincospif(xi, sp, cp);
            const float s2 = fm(sp, sp);
            const float ac = fm(a, cp);
            const float ac2 = fm(ac, ac);
            c = fdv(fsb(s2, ac2), fa(s2, ac2));
        } else {
            const float gg = fm(g, g);
            const float s = fdv(fsb(1.0f, gg), ffma(fm(2.0f, g), xi, fsb(1.0f, g)));
            c = fdv(fsb(fa(1.0f, gg), fm(s, s)), fm(2.0f, g));
        }
    }
    return rotate_dir(S, din, c, rs);
}

// The direction at cosine c to din (VectorType.cuh:207-283, vector_rotation):
// a side (2D) or an azimuth (3D) from the stream.
__device__ inline V3 rotate_dir(const DevScene& S, const V3& din, float c, Stream& rs)
{
    const float sgn = rs.uniform() < 0.5f ? -1.0f : 1.0f;
    const float sa = fm(sgn, fsq(fmaxf(0.0f, fsb(1.0f, fm(c, c)))));
    if (S.dims == 2) {
        return V3{ fsb(fm(din.x, c), fm(din.y, sa)), fa(fm(din.x, sa), fm(din.y, c)), 0.0f };
    }
    float sphi, cphi;
    walk_sincospif(fm(2.0f, rs.uniform()), sphi, cphi);
    if (fabsf(din.z) > 1.0f - 1e-6f) {
        return V3{ fm(sa, cphi), fm(sa, sphi), fm(c, signbit(din.z) ? -1.0f : 1.0f) };
    }
    const float st = fsq(fsb(1.0f, fm(din.z, din.z)));
    const float nx = fsb(fm(fm(din.x, din.z), cphi), fm(din.y, sphi));
    const float ny = fa(fm(fm(din.y, din.z), cphi), fm(din.x, sphi));
    return V3{ fa(fdv(fm(sa, nx), st), fm(din.x, c)),
               fa(fdv(fm(sa, ny), st), fm(din.y, c)),
               fa(fm(fm(-sa, cphi), st), fm(din.z, c)) };
}

// Woodcock free flight from o along d (HeterogeneousMedium.cuh:576-678);
// returns false if the step limit ran out.  A tentative point outside the box
// on a ray that still enters it moves on to the entry face: flight lengths
// are memoryless, so the first point inside is the entry plus an exponential
// step, as with further steps outside, but one lane no longer spins alone
// through many small steps toward a far or grazing entry.  A flight that
// starts inside the (convex) box ends at its first point outside.
__device__ inline bool woodcock(const DevScene& S, const V3& o, const V3& d, Stream& rs, V3& out, int& mat)
{
    float dist = 0.0f;
    V3 p = o;
    int m = 0;
    uint32_t steps = 0;
    const bool from_inside = inside(S, o);
    for (;;) {
        if (++steps > kMaxWoodcock) return false;
        const float u = rs.uniform();
        dist = fa(dist, fm(-walk_logf(u), S.inv_maxsigt));
        p.x = ffma(dist, d.x, o.x);
        p.y = ffma(dist, d.y, o.y);
        if (S.dims == 3) p.z = ffma(dist, d.z, o.z);
        if (!inside(S, p)) {
            float te = 0.0f;
            if (from_inside || !points_toward(S, p, d, &te)) break;
            dist = fa(dist, te);
        } else {
            m = material_at(S, p);
            if (rs.uniform() <= S.accept[m]) break;
        }
    }
    if (S.dims == 2) p.z = 0.0f;
    out = p;
    if (inside(S, p)) mat = (rs.uniform() > S.survive[m]) ? 0 : m;
    else mat = 0;
    return true;
}

__device__ inline void sample_source(const DevScene& S, const DevSource& src, Stream& rs, V3& x0, V3& d0)
{
    const int D = S.dims;
    int l = (int)ceilf(fm(rs.uniform(), (float)src.n)) - 1;
    l = l < 0 ? 0 : (l > src.n - 1 ? src.n - 1 : l);
    if (src.type != SSTMC_SOURCE_FARFIELD) {   // point sources, and 2D beams from their focal points
        x0 = load3(src.p, l);
        d0 = random_direction(D, rs);
        return;
    }
    const V3 dir = load3(src.p, l);
    const float mnt = src.mint[l], mxt = src.maxt[l];
    const float st = fa(mnt, fm(rs.uniform(), fsb(mxt, mnt)));
    const V3 tg = load3(src.tang, l), pt = load3(src.pt, l);
    float p[3] = { fa(tg.x, fm(st, pt.x)), fa(tg.y, fm(st, pt.y)), fa(tg.z, fm(st, pt.z)) };
    if (D == 3) {
        const float mns = src.mins[l], mxs = src.maxs[l];
        const float ss = fa(mns, fm(rs.uniform(), fsb(mxs, mns)));
        const V3 ps = load3(src.ps, l);
        p[0] = fa(p[0], fm(ss, ps.x)); p[1] = fa(p[1], fm(ss, ps.y)); p[2] = fa(p[2], fm(ss, ps.z));
    }
    const V3 inv = load3(src.inv, l);
    float sh[3], dist[3];
    for (int i = 0; i < D; ++i) {
        sh[i] = fsb(p[i], S.center[i]);
        const float sg = comp(dir, i) < 0.0f ? 1.0f : -1.0f;
        dist[i] = fm(comp(inv, i), fsb(fm(S.radius[i], sg), sh[i]));
    }
    float bd = 0.0f;
    for (int i = 0; i < D; ++i) {
        bool ok = dist[i] >= 0.0f;
        for (int j = 0; j < D && ok; ++j) {
            if (j == i) continue;
            if (!(fabsf(ffma(comp(dir, j), dist[i], sh[j])) < S.radius[j])) ok = false;
        }
        if (ok) { bd = dist[i]; break; }
    }
    const float step = fa(bd, 1e-12f);
    x0 = V3{ fa(p[0], fm(step, dir.x)), fa(p[1], fm(step, dir.y)), D == 3 ? fa(p[2], fm(step, dir.z)) : 0.0f };
    d0 = V3{ dir.x, dir.y, D == 3 ? dir.z : 0.0f };
}

// Voxel traversal from o along d, starting in cell (b0, b1, b2), in D
// dimensions.  Every per-axis quantity lives in its own register (an array
// indexed by the crossing axis would be placed in local memory): per step the
// three face distances, the axis crossed first and the cell's extinction.
// All face distances are recomputed per step: keeping the two unchanged ones
// and updating only the crossed axis (a branch on the axis) measured 14 %
// slower on the 64x64x32-grid workload than the branch-free recomputation.
// Arithmetic identical to the oracle's traversal (the same IEEE operations in
// the same order), so the optical depth and the step count are too.
template <int D>
__device__ __forceinline__ float dda_cells(const DevScene& S, const V3& o, const V3& d, int b0, int b1, int b2,
                                           uint32_t& steps)
{
    auto inv_of = [](float di) { return fabsf(di) < 1e-12f ? (di >= 0.0f ? 1e12f : -1e12f) : fdv(1.0f, di); };
    const float i0 = inv_of(d.x), i1 = inv_of(d.y), i2 = D == 3 ? inv_of(d.z) : 0.0f;
    const int s0 = d.x < 0.0f ? -1 : 1, s1 = d.y < 0.0f ? -1 : 1, s2 = (D == 3 && d.z < 0.0f) ? -1 : 1;
    // the last cell index along each axis in the direction of travel (0 going down)
    const int e0 = s0 > 0 ? S.n[0] - 2 : 0, e1 = s1 > 0 ? S.n[1] - 2 : 0, e2 = D == 3 ? (s2 > 0 ? S.n[2] - 2 : 0) : 0;
    const float* ax0 = S.ax[0] + (s0 > 0 ? 1 : 0);
    const float* ax1 = S.ax[1] + (s1 > 0 ? 1 : 0);
    const float* ax2 = D == 3 ? S.ax[2] + (s2 > 0 ? 1 : 0) : nullptr;
    const int sx = S.n[0] - 1, sxy = (S.n[0] - 1) * (S.n[1] - 1);
    float t = 0.0f, acc = 0.0f;
    uint32_t n = 0;
    const uint32_t limit = (uint32_t)(S.n[0] + S.n[1] + (D == 3 ? S.n[2] : 0)) + 4u;
    for (;;) {
        const int idx = b0 + b1 * sx + (D == 3 ? b2 * sxy : 0);
        const unsigned char m = __ldg(S.grid + idx);
        const float t0 = fm(fsb(__ldg(ax0 + b0), o.x), i0);
        const float t1 = fm(fsb(__ldg(ax1 + b1), o.y), i1);
        int a;
        float tna;
        if (D == 2) {
            a = t0 < t1 ? 0 : 1;
            tna = a == 0 ? t0 : t1;
        } else {
            const float t2 = fm(fsb(__ldg(ax2 + b2), o.z), i2);
            a = (t0 < t1 && t0 < t2) ? 0 : (t1 < t2 ? 1 : 2);
            tna = a == 0 ? t0 : (a == 1 ? t1 : t2);
        }
        acc = ffma(fsb(tna, t), S.sigt[m], acc);
        t = tna;
        ++n;
        const bool last = a == 0 ? b0 == e0 : (a == 1 ? b1 == e1 : b2 == e2);
        if (last || n >= limit) break;
        b0 += a == 0 ? s0 : 0;
        b1 += a == 1 ? s1 : 0;
        if (D == 3) b2 += a == 2 ? s2 : 0;
    }
    steps += n;
    return acc;
}

// Packed start cell of a point (10 bits per axis), or kNoCell when an axis
// has more than 1024 cells: a point's cell is the same for every ray leaving
// it, so the view-side kernels look it up once per vertex.
constexpr uint32_t kNoCell = 0xffffffffu;

__device__ __forceinline__ uint32_t cell_of(const DevScene& S, const V3& p)
{
    if (S.n[0] > 1025 || S.n[1] > 1025 || (S.dims == 3 && S.n[2] > 1025)) return kNoCell;
    const uint32_t c0 = (uint32_t)bin_of(S.ax[0], S.n[0], p.x);
    const uint32_t c1 = (uint32_t)bin_of(S.ax[1], S.n[1], p.y);
    const uint32_t c2 = S.dims == 3 ? (uint32_t)bin_of(S.ax[2], S.n[2], p.z) : 0u;
    return c0 | (c1 << 10) | (c2 << 20);
}

// FP32 parametric voxel traversal from o along d.  Returns the optical depth;
// `steps` counts the voxels crossed.  Termination: every iteration moves one
// axis' cell index monotonically toward that axis' far edge.  cell: o's packed
// cell (cell_of), or kNoCell to look it up here.
__device__ inline float dda(const DevScene& S, const V3& o, const V3& d, uint32_t& steps, uint32_t cell = kNoCell)
{
    const int D = S.dims;
    if (!inside(S, o)) return 0.0f;
    // single cell: one step (same arithmetic as the general loop's first step)
    if (S.n[0] == 2 && S.n[1] == 2 && (D == 2 || S.n[2] == 2)) {
        auto face_t = [&](float di, float oi, float lo, float hi) {
            const float inv = fabsf(di) < 1e-12f ? (di >= 0.0f ? 1e12f : -1e12f) : fdv(1.0f, di);
            return fm(fsb(di < 0.0f ? lo : hi, oi), inv);
        };
        const float t0 = face_t(d.x, o.x, S.bmin[0], S.bmax[0]);
        const float t1 = face_t(d.y, o.y, S.bmin[1], S.bmax[1]);
        float tna;
        if (D == 2) tna = t0 < t1 ? t0 : t1;
        else {
            const float t2 = face_t(d.z, o.z, S.bmin[2], S.bmax[2]);
            tna = (t0 < t1 && t0 < t2) ? t0 : (t1 < t2 ? t1 : t2);
        }
        steps += 1;
        return ffma(tna, S.sigt[__ldg(S.grid)], 0.0f);
    }
    int b0, b1, b2;
    if (cell != kNoCell) {
        b0 = (int)(cell & 1023u); b1 = (int)((cell >> 10) & 1023u); b2 = (int)(cell >> 20);
    } else {
        b0 = bin_of(S.ax[0], S.n[0], o.x);
        b1 = bin_of(S.ax[1], S.n[1], o.y);
        b2 = D == 3 ? bin_of(S.ax[2], S.n[2], o.z) : 0;
    }
    return D == 3 ? dda_cells<3>(S, o, d, b0, b1, b2, steps) : dda_cells<2>(S, o, d, b0, b1, 0, steps);
}

}  // namespace sstmc
