// device_math.cuh -- FP32 decision-path arithmetic of the tracer.
//
// Every operation on the random walk (free flight, voxel lookup, direction
// sampling, roulette, voxel traversal) uses round-to-nearest intrinsics that
// nvcc never fuses (__fmul_rn, __fadd_rn, __fmaf_rn, __fdiv_rn, __fsqrt_rn),
// so a walk replayed on the host with the same IEEE operations gives the same
// bits.  The natural log and sin/cos(pi x) below are written from their
// Taylor / atanh series; the RNG is Philox4x32-10 (Salmon et al., SC'11)
// keyed by (seed, path, vertex, purpose) instead of the reference's per-thread
// cuRAND XORWOW pool (TracerInterface.cuh:56-117), so any path can be
// replayed on its own and a request gives the same result alone or batched.
#pragma once
#include <cstdint>

namespace sstmc {

__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsb(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float ffma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ float fdv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float fsq(float a) { return __fsqrt_rn(a); }

// Stream purposes (low byte of counter word 3).
constexpr uint32_t kPurposeWalk = 1u;
constexpr uint32_t kPurposeTemporal = 2u;
constexpr uint32_t kPurposeWave = 3u;
constexpr uint32_t kPurposeForcedBin = 4u;

__device__ __forceinline__ void philox4x32_10(uint32_t k0, uint32_t k1, uint32_t c0, uint32_t c1,
                                              uint32_t c2, uint32_t c3, uint32_t out[4])
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t lo0 = 0xD2511F53u * c0, hi0 = __umulhi(0xD2511F53u, c0);
        const uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = __umulhi(0xCD9E8D57u, c2);
        const uint32_t n0 = hi1 ^ c1 ^ k0;
        const uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

// Sequential words of one (path, vertex, purpose) stream:
// block j = Philox(key = seed, counter = (j, a, b, tag)).  The walk primes the
// first two blocks (8 words) at one point of its loop so that all lanes of a
// warp run the two Philox evaluations together; later blocks are generated
// on demand, 4 words at a time.  Priming changes when words are generated,
// never which words a draw returns.
struct Stream {
    uint32_t k0, k1, a, b, tag, block;
    uint32_t w0, w1, w2, w3, w4, w5, w6, w7;
    int idx, n;

    __device__ __forceinline__ void init(uint64_t seed, uint32_t a_, uint32_t b_, uint32_t tag_)
    {
        k0 = (uint32_t)seed; k1 = (uint32_t)(seed >> 32);
        a = a_; b = b_; tag = tag_; block = 0; idx = 0; n = 0;
    }
    __device__ __forceinline__ void prime2()
    {
        uint32_t o[4];
        philox4x32_10(k0, k1, 0u, a, b, tag, o);
        w0 = o[0]; w1 = o[1]; w2 = o[2]; w3 = o[3];
        philox4x32_10(k0, k1, 1u, a, b, tag, o);
        w4 = o[0]; w5 = o[1]; w6 = o[2]; w7 = o[3];
        block = 2; idx = 0; n = 8;
    }
    __device__ __forceinline__ uint32_t next()
    {
        if (idx == n) {
            uint32_t o[4];
            philox4x32_10(k0, k1, block, a, b, tag, o);
            w0 = o[0]; w1 = o[1]; w2 = o[2]; w3 = o[3];
            block++;
            idx = 0; n = 4;
        }
        const int i = idx++;
        const uint32_t lo = i & 2 ? (i & 1 ? w3 : w2) : (i & 1 ? w1 : w0);
        const uint32_t hi = i & 2 ? (i & 1 ? w7 : w6) : (i & 1 ? w5 : w4);
        return i & 4 ? hi : lo;
    }
    // Uniform in (0, 1]: ((x >> 8) + 1) * 2^-24 (exact).
    __device__ __forceinline__ float uniform()
    {
        return fm((float)((next() >> 8) + 1u), 1.0f / 16777216.0f);
    }
};

// log(x), x normal positive: x = 2^e m, m in [sqrt(1/2), sqrt(2)),
// log(m) = 2 atanh((m - 1)/(m + 1)) as an odd series.
__device__ __forceinline__ float walk_logf(float x)
{
    uint32_t bits = __float_as_uint(x);
    int e = (int)((bits >> 23) & 0xffu) - 127;
    float m = __uint_as_float((bits & 0x007fffffu) | 0x3f800000u);
    if (m > 1.41421356f) { m = fm(m, 0.5f); e = e + 1; }
    const float f = fdv(fsb(m, 1.0f), fa(m, 1.0f));
    const float s = fm(f, f);
    float p = 0.0909090909f;
    p = ffma(p, s, 0.111111111f);
    p = ffma(p, s, 0.142857143f);
    p = ffma(p, s, 0.2f);
    p = ffma(p, s, 0.333333333f);
    p = fm(p, s);
    const float f2 = fm(2.0f, f);
    const float lm = ffma(f2, p, f2);
    const float fe = (float)e;
    return ffma(fe, 0.693145752f, ffma(fe, 1.42860677e-06f, lm));
}

// sin(pi x), cos(pi x): x = n/2 + r, |r| <= 1/4, Taylor series in r.
__device__ __forceinline__ void walk_sincospif(float x, float& sp, float& cp)
{
    const float n = rintf(fm(x, 2.0f));
    const float r = ffma(n, -0.5f, x);
    const float r2 = fm(r, r);
    float ps = 0.0821458866f;
    ps = ffma(ps, r2, -0.599264529f);
    ps = ffma(ps, r2, 2.55016404f);
    ps = ffma(ps, r2, -5.16771278f);
    ps = ffma(ps, r2, 3.14159265f);
    const float s = fm(ps, r);
    float pc = -0.0258068914f;
    pc = ffma(pc, r2, 0.235330630f);
    pc = ffma(pc, r2, -1.33526277f);
    pc = ffma(pc, r2, 4.05871213f);
    pc = ffma(pc, r2, -4.93480220f);
    const float c = ffma(pc, r2, 1.0f);
    const int q = ((int)n) & 3;
    if (q == 0) { sp = s; cp = c; }
    else if (q == 1) { sp = c; cp = -s; }
    else if (q == 2) { sp = -s; cp = -c; }
    else { sp = -c; cp = s; }
}

__device__ __forceinline__ uint32_t hash_mix(uint32_t h, uint32_t v)
{
    h ^= v;
    h *= 0x01000193u;
    h ^= h >> 15;
    return h;
}

}  // namespace sstmc
