// contract.cu -- illumination x view contractions over paths (SIMT forms).
//
// The reference materialises the Nl x Nv x P broadcast product and sums it
// with cublasZgemv against a ones vector (multipleResSingle / multipleResFinal,
// NextEventEstimation.cuh:1016-1136, 1397-1458; MatrixOperations.cuh:192-516).
// Here the sum over paths is a complex GEMM per tick,
//     V[t][v][l] += sum_p A[p][t][l] * B[p][t][v],
// with the paths as the K dimension.
//
// gemm_kernel: 32 x 32 output tile per CTA, K split across CTAs, FP32 partial
// sums over 256-path windows folded into a compensated two-float accumulator
// (Knuth TwoSum), FP64 atomic add of the CTA result.  The optional material
// filter and weight table give the single-scattering term of far-field x
// far-field scenes, whose amplitude depends only on (material, l, v, t).
//
// ss_kernel: the single-scattering term when the amplitude depends on the
// scatterer position (point sources):
//     V[t][v][l] += sum_p a[p][t][l] * b[p][t][v] * W(l, v, t, p).
#include <cuda_runtime.h>

#include <algorithm>

#include "contract.h"
#include "gauss.cuh"
#include "nee.cuh"

namespace sstmc {

namespace {

__device__ __forceinline__ void two_sum_add(float& hi, float& lo, float x)
{
    const float s = hi + x;
    const float bb = s - hi;
    const float e = (hi - (s - bb)) + (x - bb);
    hi = s;
    lo += e;
}

constexpr int kTile = 32;
constexpr int kKc = 32;
constexpr int kFlush = 8;  // chunks per compensated flush (256 paths)

__global__ void __launch_bounds__(256) gemm_kernel(const GemmParams G)
{
    __shared__ float2 As[kKc][kTile + 1];
    __shared__ float2 Bs[kKc][kTile + 1];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int l0 = blockIdx.x * kTile, v0 = blockIdx.y * kTile;
    const int t = blockIdx.z % G.Nt, ks = blockIdx.z / G.Nt;
    const int kb = ks * G.kchunk;
    const int ke = min(G.K, kb + G.kchunk);
    float2 acc[2][2];
    float hr[2][2], lr[2][2], hi_[2][2], li[2][2];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) { acc[i][j] = make_float2(0.f, 0.f); hr[i][j] = lr[i][j] = hi_[i][j] = li[i][j] = 0.f; }
    int chunk = 0;
    for (int k = kb; k < ke; k += kKc, ++chunk) {
        for (int idx = threadIdx.x; idx < kKc * kTile; idx += 256) {
            const int pp = idx / kTile, c = idx % kTile;
            const int p = k + pp;
            float2 a = make_float2(0.f, 0.f), b = make_float2(0.f, 0.f);
            if (p < ke && (G.mat == nullptr || G.mat[p] == G.mat_sel)) {
                if (l0 + c < G.Nl) a = G.A[((size_t)p * G.Nt + t) * G.Nl + l0 + c];
                if (v0 + c < G.Nv) b = G.B[((size_t)p * G.Nt + t) * G.Nv + v0 + c];
            }
            As[pp][c] = a;
            Bs[pp][c] = b;
        }
        __syncthreads();
#pragma unroll 4
        for (int pp = 0; pp < kKc; ++pp) {
            const float2 a0 = As[pp][tx], a1 = As[pp][tx + 16];
            const float2 b0 = Bs[pp][ty], b1 = Bs[pp][ty + 16];
            const float2 av[2] = { a0, a1 }, bv[2] = { b0, b1 };
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 2; ++j) {
                    acc[i][j].x = fmaf(av[i].x, bv[j].x, fmaf(-av[i].y, bv[j].y, acc[i][j].x));
                    acc[i][j].y = fmaf(av[i].x, bv[j].y, fmaf(av[i].y, bv[j].x, acc[i][j].y));
                }
        }
        __syncthreads();
        if (G.compensated && (chunk + 1) % kFlush == 0) {
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 2; ++j) {
                    two_sum_add(hr[i][j], lr[i][j], acc[i][j].x);
                    two_sum_add(hi_[i][j], li[i][j], acc[i][j].y);
                    acc[i][j] = make_float2(0.f, 0.f);
                }
        }
    }
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const int l = l0 + tx + 16 * i, v = v0 + ty + 16 * j;
            if (l >= G.Nl || v >= G.Nv) continue;
            double re = (double)hr[i][j] + (double)lr[i][j] + (double)acc[i][j].x;
            double im = (double)hi_[i][j] + (double)li[i][j] + (double)acc[i][j].y;
            const size_t o = ((size_t)t * G.Nv + v) * G.Nl + l;
            if (G.W) { const double w = G.W[o]; re *= w; im *= w; }
            if (G.scale != 0.0) { re *= G.scale; im *= G.scale; }
            atomicAdd(&G.V[o].x, re);
            atomicAdd(&G.V[o].y, im);
        }
}

constexpr int kSsL = 16, kSsV = 16, kSsK = 16, kSsT = 8;

// Single-scattering weight W(l, v, t) of one path.
struct SsGeom {
    V3 in1, in2, out1, out2;
};

__global__ void __launch_bounds__(256) ss_kernel(const __grid_constant__ DevScene S, const SsParams G)
{
    __shared__ float2 as[kSsK][kSsT][kSsL];
    __shared__ float2 bs[kSsK][kSsT][kSsV];
    __shared__ float inx[kSsK][kSsL][6];
    __shared__ float outx[kSsK][kSsV][6];
    __shared__ float x1s[kSsK][3];
    __shared__ int m1s[kSsK];
    const int tl = threadIdx.x % kSsL, tv = threadIdx.x / kSsL;
    const int l0 = blockIdx.x * kSsL, v0 = blockIdx.y * kSsV;
    const int Nt = S.Nt, Nl = S.src[0].n, Nv = S.src[1].n;
    const int tchunks = (Nt + kSsT - 1) / kSsT;
    const int t0 = (blockIdx.z % tchunks) * kSsT;
    const int tn = min(kSsT, Nt - t0);
    const int ks = blockIdx.z / tchunks;
    const int kb = ks * G.kchunk, ke = min(G.K, kb + G.kchunk);
    const bool corr = S.correlation != 0;
    const DevSource& il = S.src[0];
    const DevSource& vw = S.src[1];
    const DevSource& il2 = corr ? S.src[2] : S.src[0];
    const DevSource& vw2 = corr ? S.src[3] : S.src[1];
    const bool scalar_fs = il.type == SSTMC_SOURCE_POINT && vw.type == SSTMC_SOURCE_POINT && S.iso_all;
    float2 acc[kSsT];
    float hr[kSsT], lr[kSsT], hi_[kSsT], li[kSsT];
#pragma unroll
    for (int i = 0; i < kSsT; ++i) { acc[i] = make_float2(0.f, 0.f); hr[i] = lr[i] = hi_[i] = li[i] = 0.f; }
    int chunk = 0;
    for (int k = kb; k < ke; k += kSsK, ++chunk) {
        // stage rows and geometry
        for (int idx = threadIdx.x; idx < kSsK * kSsT * kSsL; idx += 256) {
            const int pp = idx / (kSsT * kSsL), r = idx % (kSsT * kSsL);
            const int tt = r / kSsL, c = r % kSsL;
            const int p = k + pp;
            float2 a = make_float2(0.f, 0.f), b = make_float2(0.f, 0.f);
            if (p < ke && tt < tn) {
                if (l0 + c < Nl) a = G.a[((size_t)p * Nt + t0 + tt) * Nl + l0 + c];
                if (v0 + c < Nv) b = G.b[((size_t)p * Nt + t0 + tt) * Nv + v0 + c];
            }
            as[pp][tt][c] = a;
            bs[pp][tt][c] = b;
        }
        if (threadIdx.x < kSsK) {
            const int p = k + threadIdx.x;
            if (p < ke) {
                x1s[threadIdx.x][0] = G.x1[3 * p]; x1s[threadIdx.x][1] = G.x1[3 * p + 1]; x1s[threadIdx.x][2] = G.x1[3 * p + 2];
                m1s[threadIdx.x] = G.m1[p];
            } else {
                x1s[threadIdx.x][0] = x1s[threadIdx.x][1] = x1s[threadIdx.x][2] = 0.f;
                m1s[threadIdx.x] = 0;
            }
        }
        __syncthreads();
        for (int idx = threadIdx.x; idx < kSsK * kSsL; idx += 256) {
            const int pp = idx / kSsL, c = idx % kSsL;
            const V3 x = V3{ x1s[pp][0], x1s[pp][1], x1s[pp][2] };
            const int l = min(l0 + c, Nl - 1), v = min(v0 + c, Nv - 1);
            const V3 i1 = src_in(il, l, x), i2 = src_in(il2, l, x);
            const V3 o1 = src_out(vw, v, x), o2 = src_out(vw2, v, x);
            inx[pp][c][0] = i1.x; inx[pp][c][1] = i1.y; inx[pp][c][2] = i1.z;
            inx[pp][c][3] = i2.x; inx[pp][c][4] = i2.y; inx[pp][c][5] = i2.z;
            outx[pp][c][0] = o1.x; outx[pp][c][1] = o1.y; outx[pp][c][2] = o1.z;
            outx[pp][c][3] = o2.x; outx[pp][c][4] = o2.y; outx[pp][c][5] = o2.z;
        }
        __syncthreads();
        for (int pp = 0; pp < kSsK; ++pp) {
            const int m = m1s[pp];
            if (m == 0) continue;
            const V3 i1 = V3{ inx[pp][tl][0], inx[pp][tl][1], inx[pp][tl][2] };
            const V3 i2 = V3{ inx[pp][tl][3], inx[pp][tl][4], inx[pp][tl][5] };
            const V3 o1 = V3{ outx[pp][tv][0], outx[pp][tv][1], outx[pp][tv][2] };
            const V3 o2 = V3{ outx[pp][tv][3], outx[pp][tv][4], outx[pp][tv][5] };
            float w0, c = 0.0f;
            if (scalar_fs) {
                w0 = corr ? S.iso_amp * S.iso_amp : S.iso_amp;
            } else if (!corr) {
                w0 = (il.type == SSTMC_SOURCE_POINT && S.iso_all) ? S.iso_amp : amp_dirs(S, m, i1, o1);
            } else {
                const bool pi = il.type == SSTMC_SOURCE_POINT && S.iso_all;
                w0 = (pi ? S.iso_amp : amp_dirs(S, m, i1, o1)) * (pi ? S.iso_amp : amp_dirs(S, m, i2, o2));
                const V3 qv = V3{ 0.5f * (i1.x + i2.x - o1.x - o2.x), 0.5f * (i1.y + i2.y - o1.y - o2.y), 0.5f * (i1.z + i2.z - o1.z - o2.z) };
                c = S.k2 * S.D[m] * dot3(qv, qv);
            }
            // scatterer evaluation point that moves with the tick: field sampler with
            // temporal amplitude (TemporalSampler.cuh:272-300) or correlation-sampler
            // drift U (TemporalSamplerCorrelation.cuh:293-315)
            const bool vary = !scalar_fs && (corr ? S.static_corr[m] == 0 : (S.temporal_amp && S.moving[m]));
            const V3 xp = V3{ x1s[pp][0], x1s[pp][1], x1s[pp][2] };
            const int lg = min(l0 + tl, Nl - 1), vg = min(v0 + tv, Nv - 1);
            if (src_amp64(S, il, m)) {
                // tabular or vMF scattering: amplitude (FP64 angle) between the
                // incoming and outgoing directions (FP64, nee.cuh); correlation:
                // u1 amplitude x conj(u2 amplitude) x the temporal factor
                auto fs_tab = [&](const DevSource& a, const DevSource& bsrc, const V3& x) {
                    double in[3], out[3];
                    src_in64(a, lg, x, in);
                    src_out64(bsrc, vg, x, out);
                    return amp64(S, m, in[0] * out[0] + in[1] * out[1] + in[2] * out[2]);
                };
                for (int tt = 0; tt < kSsT; ++tt) {
                    if (tt >= tn) break;
                    V3 xq = xp;
                    if (vary) {
                        if (corr) xq = shift_u(S, xp, m, S.ticks_f[t0 + tt], -1.0f);
                        else {
                            const float* q = G.x1t + ((size_t)(k + pp) * Nt + t0 + tt) * 3;
                            xq = V3{ q[0], q[1], q[2] };
                        }
                    }
                    const float2 f1 = fs_tab(il, vw, xq);
                    const float2 w = corr ? c_scale(c_mulc(f1, fs_tab(il2, vw2, xq)), expf(-c * S.abs_ticks[t0 + tt])) : f1;
                    const float2 cv = c_mul(c_mul(as[pp][tt][tl], bs[pp][tt][tv]), w);
                    acc[tt].x += cv.x;
                    acc[tt].y += cv.y;
                }
                continue;
            }
#pragma unroll
            for (int tt = 0; tt < kSsT; ++tt) {
                if (tt >= tn) break;
                float w = (corr && !scalar_fs) ? w0 * expf(-c * S.abs_ticks[t0 + tt]) : w0;
                if (vary) {
                    V3 xt;
                    if (corr) xt = shift_u(S, xp, m, S.ticks_f[t0 + tt], -1.0f);
                    else {
                        const float* q = G.x1t + ((size_t)(k + pp) * Nt + t0 + tt) * 3;
                        xt = V3{ q[0], q[1], q[2] };
                    }
                    const bool pi = il.type == SSTMC_SOURCE_POINT && S.iso_all;
                    const float f1 = pi ? S.iso_amp : amp_dirs(S, m, src_in(il, lg, xt), src_out(vw, vg, xt));
                    if (!corr) w = f1;
                    else {
                        const float f2 = pi ? S.iso_amp : amp_dirs(S, m, src_in(il2, lg, xt), src_out(vw2, vg, xt));
                        w = f1 * f2 * expf(-c * S.abs_ticks[t0 + tt]);
                    }
                }
                const float2 ab = c_mul(as[pp][tt][tl], bs[pp][tt][tv]);
                acc[tt].x = fmaf(ab.x, w, acc[tt].x);
                acc[tt].y = fmaf(ab.y, w, acc[tt].y);
            }
        }
        __syncthreads();
        if (G.compensated && (chunk + 1) % 16 == 0) {
#pragma unroll
            for (int tt = 0; tt < kSsT; ++tt) {
                two_sum_add(hr[tt], lr[tt], acc[tt].x);
                two_sum_add(hi_[tt], li[tt], acc[tt].y);
                acc[tt] = make_float2(0.f, 0.f);
            }
        }
    }
    const int l = l0 + tl, v = v0 + tv;
    if (l >= Nl || v >= Nv) return;
#pragma unroll
    for (int tt = 0; tt < kSsT; ++tt) {
        if (tt >= tn) break;
        const size_t o = ((size_t)(t0 + tt) * Nv + v) * Nl + l;
        atomicAdd(&G.V[o].x, (double)hr[tt] + (double)lr[tt] + (double)acc[tt].x);
        atomicAdd(&G.V[o].y, (double)hi_[tt] + (double)li[tt] + (double)acc[tt].y);
    }
}

// Single-scattering term of the correlation sampler when the u1 and u2
// sources are identical and every scatterer is static (U = 0): the rows are
// real (|g|^2) and Fs1 Fs2 TS = pdf(in, out) exp(-k^2 D |tau| |in - out|^2)
// (SourceInterface.cuh:221-270 with q = in - out).  Each thread owns a 2 x 2
// (illumination, view) block and all ticks of a chunk.  Per path the block
// stages one float4 per illumination element (direction into the scatterer,
// row value), one per view element (-2 x direction out, row value) and one
// per path with the material constants, so the inner loop is branch-free:
//   q^2 = 2 - 2 in . out                   (unit directions)
//   pdf = gup (omg2 + g q^2)^(-D/2)        (isotropic: g = 0, omg2 = 1)
//   e_t = exp2(-c q^2 |tau_t|), c = k^2 D log2(e)
// and the pdf's power is folded into the first tick's exponential:
//   pdf e_0 = gup exp2(-(D/2) log2(omg2 + g q^2) - c q^2 |tau_0|).
// The scalar single-scattering amplitude of point x point isotropic scenes
// (no temporal factor, NextEventEstimation.cuh:1024-1032) is g = 0, c = 0.
// The tick chain runs on packed FP32 pairs (the thread's two views per FMA / MUL).
constexpr int kFl = 32, kFv = 32, kFk = 16, kFt = 8;

// staging tiles double-buffered (one barrier per chunk) + the compensated window sums
constexpr size_t kFastStage = sizeof(float4) * (2 * kFk * kFl + kFk * kFv + kFk);
constexpr size_t kFastSmem = 2 * kFastStage + sizeof(float2) * 4 * kFt * 256;

// Rows here are tick-invariant (static scatterers, identical u1 / u2
// sources), so only the first tick's rows are read; the tick dependence is
// the decay exp(-c |t|), chained multiplicatively for geometric ticks.
// Packed FP32 pairs (Blackwell f32x2 FMA / MUL): two values per instruction.
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

__device__ __forceinline__ float ex2_fast(float x)
{
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float lg2_fast(float x)
{
    float y;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rsqrt_fast(float x)
{
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ unsigned long long ex2_2(unsigned long long a) { return pk2(ex2_fast(pk_lo(a)), ex2_fast(pk_hi(a))); }

// Accumulators are packed over the thread's view pair, so the whole tick
// chain runs on f32x2 values: per (path, illumination element, view pair)
// 2 lg2 + 4 ex2 and 22 packed FP32 instructions for 8 ticks.
// FIRST: the block's first tick is tick 0 (GEO chain starts at e_s).
template <bool THREE, bool GEO, bool FIRST>
__global__ void __launch_bounds__(256, 2) ss_fast_kernel(const __grid_constant__ DevScene S, const SsParams G)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* accc = reinterpret_cast<float2*>(smem_raw);                       // [4*kFt][256] compensated (hi, lo) window sums
    unsigned char* stage0 = reinterpret_cast<unsigned char*>(accc + 4 * kFt * 256);
    // staging buffer b of a chunk:
    //   sI [kFk][kFl][2] (x x y y) (z z w w), w = row x pdf coefficient
    //   sO [kFk][4][kFv] (x, y, z, row), views contiguous
    //   sM [kFk] (g, omg2, cn, 0), 2^(cn q^2) = decay of the first tick
    auto sI_of = [&](int b) { return reinterpret_cast<float4*>(stage0 + (size_t)b * kFastStage); };
    auto sO_of = [&](int b) { return reinterpret_cast<float*>(sI_of(b) + 2 * kFk * kFl); };
    auto sM_of = [&](int b) { return reinterpret_cast<float4*>(sO_of(b) + kFk * 4 * kFv); };
    // thread: view pair v0 + 2 tx + (0, 1), illumination elements l0 + ty + 16 i.
    // A warp reads two illumination records (broadcast) and 16 consecutive
    // view pairs (one 128-byte wavefront) from shared memory.
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int l0 = blockIdx.x * kFl, v0 = blockIdx.y * kFv;
    const int Nt = S.Nt, Nl = S.src[0].n, Nv = S.src[1].n;
    const int tchunks = (Nt + kFt - 1) / kFt;
    const int t0 = (blockIdx.z % tchunks) * kFt;
    const int tn = min(kFt, Nt - t0);
    const int ks = blockIdx.z / tchunks;
    const int kb = ks * G.kchunk, ke = min(G.K, kb + G.kchunk);
    const DevSource& il = S.src[0];
    const DevSource& vw = S.src[1];
    const bool scalar_fs = S.iso_all && il.type == SSTMC_SOURCE_POINT && vw.type == SSTMC_SOURCE_POINT;
    const float tau0 = S.abs_ticks[0];
    const float start_scale = (float)(t0 + 1);   // GEO: |t_t0| = (t0 + 1) |t_0|
    unsigned long long acc[2][kFt];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int t = 0; t < kFt; ++t) acc[i][t] = 0ull;
#pragma unroll
    for (int t = 0; t < 4 * kFt; ++t) accc[t * 256 + threadIdx.x] = make_float2(0.f, 0.f);
    // staging items of a chunk: 4 per thread, idx = threadIdx.x + 256 u
    // (u = 0, 1: illumination elements; u = 2, 3: view elements).  The next
    // chunk's global loads are issued before the current chunk is computed.
    float px[4], py[4], pz[4], pv[4];
    int pm[4];
    int mm = 0;
    auto prefetch = [&](int k) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int idx = threadIdx.x + 256 * u;
            const bool isI = u < 2;
            const int r = isI ? idx : idx - kFk * kFl;
            const int pp = r / kFl, c = r % kFl;
            const int p = k + pp;
            const int pc = min(p, ke - 1);
            px[u] = G.x1[3 * pc]; py[u] = G.x1[3 * pc + 1]; pz[u] = G.x1[3 * pc + 2];
            pm[u] = (int)G.m1[pc];
            pv[u] = 0.f;
            if (isI) { if (p < ke && l0 + c < Nl) pv[u] = G.a[(size_t)p * Nt * Nl + l0 + c].x; }
            else if (p < ke && v0 + c < Nv) pv[u] = G.b[(size_t)p * Nt * Nv + v0 + c].x;
        }
        mm = (threadIdx.x < kFk && k + (int)threadIdx.x < ke) ? (int)G.m1[k + threadIdx.x] : 0;
    };
    prefetch(kb);
    int chunk = 0;
    for (int k = kb; k < ke; k += kFk, ++chunk) {
        // double-buffered: this chunk's buffer was last read two chunks ago, before
        // the previous chunk's barrier, so one barrier per chunk suffices
        float4* sI = sI_of(chunk & 1);
        float* sO = sO_of(chunk & 1);
        float4* sM = sM_of(chunk & 1);
        if (threadIdx.x < kFk) {
            const int m = mm;
            const int ty_ = S.scat_type[m];
            float g = 0.f, omg2 = 1.f, c = 0.f;
            if (m != 0 && !scalar_fs) {
                c = S.k2 * S.D[m];
                if (ty_ == SSTMC_SCATTERING_HENYEY_GREENSTEIN) { g = S.g[m]; omg2 = (1.0f - g) * (1.0f - g); }
            }
            // exp(-c q^2 |t|) = 2^(cn q^2 |t| / |t_0|) (GEO) or 2^(cn q^2 |t|)
            const float cn = -(GEO ? c * tau0 : c) * 1.44269504088896341f;
            sM[threadIdx.x] = make_float4(g, omg2, cn, 0.f);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int idx = threadIdx.x + 256 * u;
            const bool isI = u < 2;
            const int r = isI ? idx : idx - kFk * kFl;
            const int pp = r / kFl, c = r % kFl;
            const int p = k + pp;
            const V3 x = V3{ px[u], py[u], pz[u] };
            if (isI) {
                // row value times the material's pdf coefficient
                const int m = pm[u];
                const int ty_ = S.scat_type[m];
                const float coef = (p >= ke || m == 0) ? 0.0f
                                 : scalar_fs ? S.iso_amp * S.iso_amp
                                 : ty_ == SSTMC_SCATTERING_HENYEY_GREENSTEIN ? S.gup[m]
                                 : ty_ == SSTMC_SCATTERING_ISOTROPIC ? S.iso_pdf : 0.0f;
                const V3 dir = fsrc_in(il, min(l0 + c, Nl - 1), x);
                const float w = pv[u] * coef;
                sI[2 * r] = make_float4(dir.x, dir.x, dir.y, dir.y);
                sI[2 * r + 1] = make_float4(dir.z, dir.z, w, w);
            } else {
                // -2 out, so that q^2 = 2 + (-2 out) . in
                const V3 dir = fsrc_out(vw, min(v0 + c, Nv - 1), x);
                float* o = sO + (size_t)pp * 4 * kFv + c;
                o[0] = -2.0f * dir.x; o[kFv] = -2.0f * dir.y; o[2 * kFv] = -2.0f * dir.z; o[3 * kFv] = pv[u];
            }
        }
        if (k + kFk < ke) prefetch(k + kFk);
        __syncthreads();
#pragma unroll 2
        for (int pp = 0; pp < kFk; ++pp) {
            const float4 mc = sM[pp];
            const unsigned long long* op = reinterpret_cast<const unsigned long long*>(sO + (size_t)pp * 4 * kFv + 2 * tx);
            const unsigned long long ox = op[0], oy = op[kFv / 2], oz = op[kFv], ob = op[3 * kFv / 2];
            const unsigned long long g2 = pk2(mc.x, mc.x), omg = pk2(mc.y, mc.y), cn2 = pk2(mc.z, mc.z);
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const ulonglong2 ia = reinterpret_cast<const ulonglong2*>(sI)[2 * (pp * kFl + ty + 16 * i)];
                const ulonglong2 ib = reinterpret_cast<const ulonglong2*>(sI)[2 * (pp * kFl + ty + 16 * i) + 1];
                // q^2 = |in - out|^2 = 2 - 2 in . out for unit directions, both views
                // packed, z first (the largest product's cancellation against 2 is
                // exact inside the FMA); pdf = c dn^(-D/2), dn = omg2 + g q^2, as
                // exp2(-(D/2) log2 dn) inside the first tick's exponential
                const unsigned long long q2 = fma2(ox, ia.x, fma2(oy, ia.y, fma2(oz, ib.x, pk2(2.0f, 2.0f))));
                const unsigned long long dn = fma2(g2, q2, omg);
                const unsigned long long w = mul2(ob, ib.y);
                const unsigned long long L = pk2(lg2_fast(pk_lo(dn)), lg2_fast(pk_hi(dn)));
                const unsigned long long arg = mul2(cn2, q2);
                if (GEO) {
                    // e_t = e_s^(t + 1), e_s = exp(-c q^2 |t_0|): per view one ex2 for e_s
                    // and one for the first tick's term with the pdf's power
                    const unsigned long long es = ex2_2(arg);
                    const unsigned long long beta = THREE ? pk2(-1.5f, -1.5f) : pk2(-1.0f, -1.0f);
                    const unsigned long long e = ex2_2(fma2(beta, L, FIRST ? arg : mul2(arg, pk2(start_scale, start_scale))));
                    // the 8 terms b0 es^k: the even ones by products in a depth-2
                    // tree, the odd ones as FMAs of their even neighbour (13 packed
                    // instructions; a serial product chain stalled on latency, and
                    // 8 products and 8 packed adds measured 1 % slower)
                    static_assert(kFt == 8, "tick tree written for 8 ticks");
                    const unsigned long long s2 = mul2(es, es), s4 = mul2(s2, s2);
                    const unsigned long long b0 = mul2(w, e);
                    const unsigned long long b2 = mul2(b0, s2), b4 = mul2(b0, s4), b6 = mul2(b2, s4);
                    acc[i][0] = add2(acc[i][0], b0); acc[i][1] = fma2(b0, es, acc[i][1]);
                    acc[i][2] = add2(acc[i][2], b2); acc[i][3] = fma2(b2, es, acc[i][3]);
                    acc[i][4] = add2(acc[i][4], b4); acc[i][5] = fma2(b4, es, acc[i][5]);
                    acc[i][6] = add2(acc[i][6], b6); acc[i][7] = fma2(b6, es, acc[i][7]);
                } else {
#pragma unroll
                    for (int tt = 0; tt < kFt; ++tt) {
                        const float ta = S.abs_ticks[min(t0 + tt, Nt - 1)];
                        const unsigned long long beta = THREE ? pk2(-1.5f, -1.5f) : pk2(-1.0f, -1.0f);
                        acc[i][tt] = fma2(w, ex2_2(fma2(beta, L, mul2(arg, pk2(ta, ta)))), acc[i][tt]);
                    }
                }
            }
        }
        if ((chunk + 1) % 16 == 0) {
            // fold the 256-path window into the compensated (hi, lo) pairs
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int t = 0; t < kFt; ++t) {
                    float2* c0 = accc + ((i * 2 + 0) * kFt + t) * 256 + threadIdx.x;
                    float2* c1 = accc + ((i * 2 + 1) * kFt + t) * 256 + threadIdx.x;
                    float2 a0 = *c0, a1 = *c1;
                    two_sum_add(a0.x, a0.y, pk_lo(acc[i][t]));
                    two_sum_add(a1.x, a1.y, pk_hi(acc[i][t]));
                    *c0 = a0; *c1 = a1;
                    acc[i][t] = 0ull;
                }
        }
    }
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const int l = l0 + ty + 16 * i, v = v0 + 2 * tx + j;
            if (l >= Nl || v >= Nv) continue;
#pragma unroll
            for (int tt = 0; tt < kFt; ++tt) {
                if (tt >= tn) break;
                const size_t o = ((size_t)(t0 + tt) * Nv + v) * Nl + l;
                const float last = j ? pk_hi(acc[i][tt]) : pk_lo(acc[i][tt]);
                const float2 c = accc[((i * 2 + j) * kFt + tt) * 256 + threadIdx.x];
                atomicAdd(&G.V[o].x, (double)c.x + (double)c.y + (double)last);
            }
        }
}


// ---- paths grouped by first-vertex material (far-field x far-field single scattering) ----
// The far-field x far-field single-scattering term weighs each (l, v) by a
// table of the first vertex's material, so its contraction runs once per
// material over that material's paths.  A stable partition of the chunk's
// paths by material gives each path its row in the single-scattering rows and
// each material a contiguous row range: ss_row[q] and bucket[m] .. bucket[m + 1].
// Three launches: per-block counts, one block scanning them, per-block ranks.
constexpr int kBucketBlock = 1024;

__device__ __forceinline__ int first_material(const SsBucketParams& P, uint32_t q)
{
    return P.counts[q] ? (int)(__float_as_uint(P.verts[P.offsets[q]].w) & 15u) : 0;
}

__global__ void __launch_bounds__(kBucketBlock) bucket_count_kernel(const SsBucketParams P)
{
    __shared__ uint32_t h[kMat];
    if (threadIdx.x < kMat) h[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t q = blockIdx.x * kBucketBlock + threadIdx.x;
    if (q < P.n) atomicAdd(&h[first_material(P, q)], 1u);
    __syncthreads();
    if (threadIdx.x < kMat) P.hist[blockIdx.x * kMat + threadIdx.x] = h[threadIdx.x];
}

// One block: per material the exclusive scan of the per-block counts, offset
// by the rows of the lower materials; hist becomes each block's first row per
// material, bucket[m] the first row of material m, bucket[kMat] = n.
__global__ void __launch_bounds__(kBucketBlock) bucket_scan_kernel(const SsBucketParams P)
{
    __shared__ uint32_t warp_sums[kBucketBlock / 32];
    __shared__ uint32_t carry;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t base = 0;
    for (int m = 0; m < kMat; ++m) {
        if (threadIdx.x == 0) carry = base;
        __syncthreads();
        for (uint32_t b0 = 0; b0 < P.nblocks; b0 += kBucketBlock) {
            const uint32_t b = b0 + threadIdx.x;
            const uint32_t v = b < P.nblocks ? P.hist[b * kMat + m] : 0u;
            uint32_t x = v;   // inclusive warp scan
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            if (lane == 31) warp_sums[w] = x;
            __syncthreads();
            if (w == 0) {
                uint32_t s = warp_sums[lane];
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
                    if (lane >= o) s += y;
                }
                warp_sums[lane] = s;   // inclusive over warps
            }
            __syncthreads();
            const uint32_t before = carry + (w ? warp_sums[w - 1] : 0u) + x - v;
            if (b < P.nblocks) P.hist[b * kMat + m] = before;
            __syncthreads();
            if (threadIdx.x == kBucketBlock - 1) carry = before + v;
            __syncthreads();
        }
        if (threadIdx.x == 0) P.bucket[m] = base;
        base = carry;
        __syncthreads();
    }
    if (threadIdx.x == 0) P.bucket[kMat] = base;
}

// Rank of each path among the earlier paths of its block with the same
// material (warp match masks, then the earlier warps' counts): the partition
// is stable, so the rows keep the paths' order within a material.
__global__ void __launch_bounds__(kBucketBlock) bucket_scatter_kernel(const SsBucketParams P)
{
    __shared__ uint32_t wc[kBucketBlock / 32][kMat];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint32_t q = blockIdx.x * kBucketBlock + threadIdx.x;
    for (int i = threadIdx.x; i < (kBucketBlock / 32) * kMat; i += kBucketBlock) (&wc[0][0])[i] = 0;
    __syncthreads();
    const bool in = q < P.n;
    const int m = in ? first_material(P, q) : kMat;   // kMat: no path
    const uint32_t same = __match_any_sync(0xffffffffu, m);
    const uint32_t rank = __popc(same & ((1u << lane) - 1u));
    if (in && rank == 0) wc[w][m] = __popc(same);
    __syncthreads();
    if (in) {
        uint32_t before = 0;
        for (int j = 0; j < w; ++j) before += wc[j][m];
        P.ss_row[q] = P.hist[blockIdx.x * kMat + m] + before + rank;
    }
}

}  // namespace

int launch_ss_buckets(const SsBucketParams& P, cudaStream_t stream)
{
    if (P.n == 0) return SSTMC_NO_ERROR;
    SsBucketParams Q = P;
    Q.nblocks = (P.n + kBucketBlock - 1) / kBucketBlock;
    bucket_count_kernel<<<Q.nblocks, kBucketBlock, 0, stream>>>(Q);
    bucket_scan_kernel<<<1, kBucketBlock, 0, stream>>>(Q);
    bucket_scatter_kernel<<<Q.nblocks, kBucketBlock, 0, stream>>>(Q);
    return cudaGetLastError() == cudaSuccess ? SSTMC_NO_ERROR : SSTMC_KERNEL_ERROR;
}

namespace {
}  // namespace

int launch_gemm(const GemmParams& G, cudaStream_t stream)
{
    if (G.K <= 0) return SSTMC_NO_ERROR;
    const int ksplit = (G.K + G.kchunk - 1) / G.kchunk;
    dim3 grid((G.Nl + kTile - 1) / kTile, (G.Nv + kTile - 1) / kTile, G.Nt * ksplit);
    gemm_kernel<<<grid, 256, 0, stream>>>(G);
    return cudaGetLastError() == cudaSuccess ? SSTMC_NO_ERROR : SSTMC_CUBLAS_ERROR;
}

// Gaussian beams: V[t][v][l] += sum_p a[p][t][l] b[p][t][v] fs(l, v, x_p,t)
// (threePointFunctionSingle, GaussianBeam.cuh:894-999).  fs depends on the
// scatterer's position, so it is evaluated per (path, l, v) -- once for a
// static vertex, per tick for a moving one with the temporal amplitude -- in
// FP64 (gauss.cuh), and the products are summed in FP64.  Thread per (l, v) of
// a 16 x 16 tile, a chunk of kSsT ticks and a range of paths.
__global__ void __launch_bounds__(256, 1) gauss_ss_kernel(const __grid_constant__ DevScene S, const SsParams G)
{
    const int Nt = S.Nt, Nl = S.src[0].n, Nv = S.src[1].n;
    const int l = blockIdx.x * kSsL + threadIdx.x % kSsL, v = blockIdx.y * kSsV + threadIdx.x / kSsL;
    const int tchunks = (Nt + kSsT - 1) / kSsT;
    const int t0 = (blockIdx.z % tchunks) * kSsT;
    const int tn = min(kSsT, Nt - t0);
    const int ks = blockIdx.z / tchunks;
    const int kb = ks * G.kchunk, ke = min(G.K, kb + G.kchunk);
    if (l >= Nl || v >= Nv) return;
    const DevSource& il = S.src[0];
    const DevSource& vw = S.src[1];
    double ar[kSsT], ai[kSsT];
#pragma unroll
    for (int i = 0; i < kSsT; ++i) { ar[i] = 0.0; ai[i] = 0.0; }
    for (int p = kb; p < ke; ++p) {
        const int m = G.m1[p];
        if (m <= 0 || m >= kMat) continue;
        const bool stat = !S.temporal_amp || !S.moving[m];
        CD f0{ 0.0, 0.0 };
        if (stat) f0 = gauss_fs(S, il, l, vw, v, V3{ G.x1[3 * p], G.x1[3 * p + 1], G.x1[3 * p + 2] }, m);
#pragma unroll
        for (int i = 0; i < kSsT; ++i) {
            if (i >= tn) break;
            const int t = t0 + i;
            CD f = f0;
            if (!stat) {
                const float* xt = G.x1t + ((size_t)p * Nt + t) * 3;
                f = gauss_fs(S, il, l, vw, v, V3{ xt[0], xt[1], xt[2] }, m);
            }
            const float2 a = G.a[((size_t)p * Nt + t) * Nl + l];
            const float2 b = G.b[((size_t)p * Nt + t) * Nv + v];
            const double abr = (double)a.x * b.x - (double)a.y * b.y, abi = (double)a.x * b.y + (double)a.y * b.x;
            ar[i] += abr * f.re - abi * f.im;
            ai[i] += abr * f.im + abi * f.re;
        }
    }
    for (int i = 0; i < tn; ++i) {
        const size_t o = ((size_t)(t0 + i) * Nv + v) * Nl + l;
        atomicAdd(&G.V[o].x, ar[i]);
        atomicAdd(&G.V[o].y, ai[i]);
    }
}

// The same sum when every view beam shares one direction (the confocal
// geometry): the lobe's convolution with the illumination throughput -- g0,
// C, c of fsGaussianBeam -- then depends on (vertex, illumination) only.  Per
// vertex (per path, or per path and tick for a moving scatterer) one thread
// per illumination element stages it, one thread per view element the view
// throughput, and each (l, v) thread finishes with one complex square root,
// one complex exponential and one reciprocal per lobe: 2 sinh(z) e^cl / (C sm)
// with e^(cl + z) = 2^kk p (c, s) from exp_parts and e^(cl - z) as e^(2 cl)
// 2^-kk p^-1 (c, -s), each exponential dropped at a real part of -10 or below
// as in gauss_fs (gauss.cuh), whose FP64 form runs where |Re cl| or
// |Re(cl + z)| reaches 300 or |z| is below 0.05 (the difference of the two
// exponentials cancels there).  3D, at most 8 lobes per material.
__global__ void __launch_bounds__(256, 1) gauss_ss_shared_kernel(const __grid_constant__ DevScene S, const SsParams G)
{
    __shared__ CD sA[kSsL][3], sB[kSsV][3], sBi[kSsV];
    __shared__ CD sG0[kSsL][8], sC[kSsL][8], sCl[kSsL][8], sE2[kSsL][8];
    const int Nt = S.Nt, Nl = S.src[0].n, Nv = S.src[1].n;
    const int tl = threadIdx.x % kSsL, tv = threadIdx.x / kSsL;
    const int l = blockIdx.x * kSsL + tl, v = blockIdx.y * kSsV + tv;
    const int lc = min(l, Nl - 1), vc = min(v, Nv - 1);
    const bool act = l < Nl && v < Nv;
    const int tchunks = (Nt + kSsT - 1) / kSsT;
    const int t0 = (blockIdx.z % tchunks) * kSsT;
    const int tn = min(kSsT, Nt - t0);
    const int ks = blockIdx.z / tchunks;
    const int kb = ks * G.kchunk, ke = min(G.K, kb + G.kchunk);
    const DevSource& il = S.src[0];
    const DevSource& vw = S.src[1];
    const double k = S.gk;
    const double vd[3] = { (double)vw.gdir[0], (double)vw.gdir[1], (double)vw.gdir[2] };
    const double tc = il.gnorm + vw.gnorm + 2.0 * log(2.0 * kPi);
    const double z0[3] = { 0.0, 0.0, 0.0 };
    double ar[kSsT], ai[kSsT];
#pragma unroll
    for (int i = 0; i < kSsT; ++i) { ar[i] = 0.0; ai[i] = 0.0; }
    for (int p = kb; p < ke; ++p) {
        const int m = G.m1[p];
        if (m <= 0 || m >= kMat) continue;
        const int M = S.gmix_n[m];
        const double* mix = S.gmix + 2 * S.gmix_off[m];
        const bool stat = !S.temporal_amp || !S.moving[m];
        // a static vertex is staged once for every tick, a moving one per tick
        for (int s = 0; s < (stat ? 1 : tn); ++s) {
            const float* xf = stat ? G.x1 + 3 * p : G.x1t + ((size_t)p * Nt + t0 + s) * 3;
            const double x[3] = { (double)xf[0], (double)xf[1], (double)xf[2] };
            __syncthreads();   // the previous vertex's staged values are consumed
            if (tv < M) {   // thread (l, lobe)
                CD aT[3];
                g_throughput(il, lc, x, k, aT);
                if (tv == 0)
                    for (int a = 0; a < 3; ++a) sA[tl][a] = aT[a];
                {
                    const int i = tv;
                    const double gs = mix[2 * i];
                    CD C, c{ 0.0, 0.0 }, g0{ 0.0, 0.0 };
                    if (fabs(gs) < 0.000001) {
                        C = cd_sqrt(g_sumsq(0.0, z0, aT));
                    } else {
                        g0 = cd_rsqrt(g_sumsq(gs, vd, aT));
                        g0.re = dM(g0.re, gs); g0.im = dM(g0.im, gs);
                        double wv[3];
                        CD aw{ 0.0, 0.0 };
#pragma unroll
                        for (int a = 0; a < 3; ++a) wv[a] = dS(dM(g0.re, aT[a].re), dM(g0.im, aT[a].im));
                        const double ra = dD(1.0, dQ(dA(dA(dM(wv[0], wv[0]), dM(wv[1], wv[1])), dM(wv[2], wv[2]))));
                        C = cd_sqrt(g_sumsq(dM(gs, ra), wv, aT));
#pragma unroll
                        for (int a = 0; a < 3; ++a) { aw.re = dA(aw.re, dM(aT[a].re, wv[a])); aw.im = dA(aw.im, dM(aT[a].im, wv[a])); }
                        c = cd_mul(g0, aw);
                        c.re = dM(c.re, -ra); c.im = dM(c.im, -ra);
                    }
                    const CD cl = cd_add(c, CD{ tc + mix[2 * i + 1], 0.0 });
                    sG0[tl][i] = g0; sC[tl][i] = C; sCl[tl][i] = cl;
                    sE2[tl][i] = fabs(cl.re) < 300.0 ? cd_exp(CD{ 2.0 * cl.re, 2.0 * cl.im }) : CD{ 0.0, 0.0 };
                }
            }
            if (tl == 0) {
                // the view throughput, and the isotropic lobes' root sqrt(sum_a B_a^2)
                CD q{ 0.0, 0.0 };
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    const CD b = CD{ dM((double)vw.gdir[3 * vc + a], vw.ga), dM(k, dS((double)vw.p[3 * vc + a], x[a])) };
                    sB[tv][a] = b;
                    q = cf_add(q, cf_mul(b, b));
                }
                sBi[tv] = cf_sqrt(q);
            }
            __syncthreads();
            if (!act) continue;
            CD f{ 0.0, 0.0 };
            for (int i = 0; i < M; ++i) {
                const double gs = mix[2 * i];
                const CD C = sC[tl][i], cl = sCl[tl][i];
                CD sm;
                if (fabs(gs) < 0.000001) {
                    sm = sBi[tv];
                } else {
                    const CD g0 = sG0[tl][i];
                    CD q{ 0.0, 0.0 };
#pragma unroll
                    for (int a = 0; a < 3; ++a) {
                        const CD e = cf_add(cf_mul(g0, sA[tl][a]), sB[tv][a]);
                        q = cf_add(q, cf_mul(e, e));
                    }
                    sm = cf_sqrt(q);
                }
                const bool sbig = fabs(sm.re) > 0.0001 || fabs(sm.im) > 0.0001;
                const bool cbig = fabs(C.re) > 0.0001 || fabs(C.im) > 0.0001;
                if (sbig && cbig) {
                    const CD z = cf_add(C, sm);
                    const CD pos = cf_add(cl, z);
                    const double negre = cl.re - z.re;
                    if (fabs(cl.re) < 300.0 && fabs(pos.re) < 300.0 && fabs(negre) < 600.0 && fabs(z.re) + fabs(z.im) > 0.05) {
                        // (e^(cl + z) - e^(cl - z)) / (C sm) with e^(cl + z) = 2^kk p (cos, sin)
                        // and e^(cl - z) = e^(2 cl) / e^(cl + z) = e^(2 cl) 2^-kk p^-1 (cos, -sin)
                        float pf, cf, sf;
                        double kk;
                        exp_parts(pos, pf, kk, cf, sf);
                        CD r{ 0.0, 0.0 };
                        if (pos.re > -10.0) {
                            const double m = (double)pf * pow2i(kk);
                            r = CD{ m * (double)cf, m * (double)sf };
                        }
                        if (negre > -10.0) {
                            const CD e2 = sE2[tl][i];
                            const double im = (double)g_rcp32(pf) * pow2i(-kk);
                            const CD q{ im * (double)cf, -im * (double)sf };
                            r = cf_sub(r, cf_mul(e2, q));
                        }
                        // / (C sm): the reciprocal of |C sm|^2 to FP32 accuracy (the
                        // factor scales the term; |C sm| is far from FP32's range ends)
                        const CD w = cf_mul(C, sm);
                        const double iw = (double)g_rcp32((float)(w.re * w.re + w.im * w.im));
                        f = cf_add(f, CD{ (r.re * w.re + r.im * w.im) * iw, (r.im * w.re - r.re * w.im) * iw });
                    } else {
                        f = cd_add(f, cd_div(cd_2sinh(z, cl), cd_mul(C, sm)));
                    }
                } else if (!sbig && !cbig) {
                    const CD e = cd_exp(cl);
                    f.re += 4.0 * e.re; f.im += 4.0 * e.im;
                } else if (!sbig) {
                    const CD e = cd_div(cd_2sinh(C, cl), C);
                    f.re += 2.0 * e.re; f.im += 2.0 * e.im;
                } else {
                    const CD e = cd_div(cd_2sinh(sm, CD{ tc + mix[2 * i + 1], 0.0 }), sm);
                    f.re += 2.0 * e.re; f.im += 2.0 * e.im;
                }
            }
#pragma unroll
            for (int i = 0; i < kSsT; ++i) {
                if (i >= tn) break;
                if (!stat && i != s) continue;
                const int t = t0 + i;
                const float2 a = G.a[((size_t)p * Nt + t) * Nl + l];
                const float2 b = G.b[((size_t)p * Nt + t) * Nv + v];
                const double abr = (double)a.x * b.x - (double)a.y * b.y, abi = (double)a.x * b.y + (double)a.y * b.x;
                ar[i] += abr * f.re - abi * f.im;
                ai[i] += abr * f.im + abi * f.re;
            }
        }
    }
    if (!act) return;
    for (int i = 0; i < tn; ++i) {
        const size_t o = ((size_t)(t0 + i) * Nv + v) * Nl + l;
        atomicAdd(&G.V[o].x, ar[i]);
        atomicAdd(&G.V[o].y, ai[i]);
    }
}

int launch_ss(const DevScene& S, const SsParams& G, cudaStream_t stream)
{
    if (G.K <= 0) return SSTMC_NO_ERROR;
    if (S.gauss) {
        const int tchunks = (S.Nt + kSsT - 1) / kSsT;
        const int ksplit = (G.K + G.kchunk - 1) / G.kchunk;
        dim3 grid((S.src[0].n + kSsL - 1) / kSsL, (S.src[1].n + kSsV - 1) / kSsV, tchunks * ksplit);
        bool lobes8 = true;
        for (int m = 0; m < kMat; ++m) lobes8 = lobes8 && S.gmix_n[m] <= 8;
        if (S.dims == 3 && S.src[1].gsame && lobes8) gauss_ss_shared_kernel<<<grid, 256, 0, stream>>>(S, G);
        else gauss_ss_kernel<<<grid, 256, 0, stream>>>(S, G);
        return cudaGetLastError() == cudaSuccess ? SSTMC_NO_ERROR : SSTMC_CUBLAS_ERROR;
    }
    if (S.correlation && S.sym && S.all_static_corr && !S.has_amp64) {
        // two resident blocks per SM: split the paths so the grid fills them
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const int tchunks = (S.Nt + kFt - 1) / kFt;
        const int tiles = ((S.src[0].n + kFl - 1) / kFl) * ((S.src[1].n + kFv - 1) / kFv) * tchunks;
        using Fn = void (*)(DevScene, SsParams);
        const bool geo = S.ticks_geometric != 0, first = tchunks == 1;
        Fn f = S.dims == 3
            ? (geo ? (first ? (Fn)ss_fast_kernel<true, true, true> : (Fn)ss_fast_kernel<true, true, false>) : (Fn)ss_fast_kernel<true, false, false>)
            : (geo ? (first ? (Fn)ss_fast_kernel<false, true, true> : (Fn)ss_fast_kernel<false, true, false>) : (Fn)ss_fast_kernel<false, false, false>);
        if (cudaFuncSetAttribute((const void*)f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFastSmem) != cudaSuccess)
            return SSTMC_CUBLAS_ERROR;
        // resident blocks per SM (two, by registers and shared memory): split the paths so the grid fills them
        int occ = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, (const void*)f, 256, kFastSmem) != cudaSuccess || occ < 1) occ = 1;
        const int want = std::max(1, (occ * sms) / tiles);
        SsParams P = G;
        P.kchunk = ((G.K + want - 1) / want + kFk - 1) / kFk * kFk;
        const int ksplit = (G.K + P.kchunk - 1) / P.kchunk;
        dim3 grid((S.src[0].n + kFl - 1) / kFl, (S.src[1].n + kFv - 1) / kFv, tchunks * ksplit);
        f<<<grid, 256, kFastSmem, stream>>>(S, P);
        return cudaGetLastError() == cudaSuccess ? SSTMC_NO_ERROR : SSTMC_CUBLAS_ERROR;
    }
    const int ksplit = (G.K + G.kchunk - 1) / G.kchunk;
    const int tchunks = (S.Nt + kSsT - 1) / kSsT;
    dim3 grid((S.src[0].n + kSsL - 1) / kSsL, (S.src[1].n + kSsV - 1) / kSsV, tchunks * ksplit);
    ss_kernel<<<grid, 256, 0, stream>>>(S, G);
    return cudaGetLastError() == cudaSuccess ? SSTMC_NO_ERROR : SSTMC_CUBLAS_ERROR;
}

}  // namespace sstmc
