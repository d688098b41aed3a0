/*
 * oracle_math.h -- TEST INFRASTRUCTURE (part of the CPU oracle).  Only the
 * tests, __graft_entry__.smoke() and bench.py's CPU baseline use it.
 *
 * Portable FP32 building blocks of the decision path: Philox4x32-10 counter
 * RNG (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as
 * 1, 2, 3", SC'11) and a natural logarithm and sin/cos(pi x) written from
 * their Taylor / atanh series with only +, -, *, / and fmaf, so that the
 * same inputs give the same bits on the host and on the GPU.  The GPU
 * library carries its own restatement of the same specification.
 *
 * Compile with -ffp-contract=off: every fused multiply-add is explicit.
 */
#ifndef SSTMC_ORACLE_MATH_H
#define SSTMC_ORACLE_MATH_H

#include <stdint.h>
#include <string.h>
#include <math.h>

static inline float o_u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static inline uint32_t o_f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }

/* ---------------- Philox4x32-10 ---------------- */
static inline void o_philox(const uint32_t key_in[2], const uint32_t ctr_in[4], uint32_t out[4])
{
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* Stream purposes (counter word 3, low byte). */
#define O_PURPOSE_WALK      1u
#define O_PURPOSE_TEMPORAL  2u
#define O_PURPOSE_WAVE      3u
#define O_PURPOSE_FORCED    4u

/* A sequential stream of 32-bit words for one (path, vertex, purpose):
 * block j = Philox(key = seed, counter = (j, a, b, tag)). */
typedef struct {
    uint32_t key[2];
    uint32_t a, b, tag;
    uint32_t block;
    uint32_t buf[4];
    int idx;
} o_stream;

static inline void o_stream_init(o_stream* s, uint64_t seed, uint32_t a, uint32_t b, uint32_t tag)
{
    s->key[0] = (uint32_t)seed; s->key[1] = (uint32_t)(seed >> 32);
    s->a = a; s->b = b; s->tag = tag; s->block = 0; s->idx = 4;
}

static inline uint32_t o_next_u32(o_stream* s)
{
    if (s->idx == 4) {
        uint32_t ctr[4] = { s->block, s->a, s->b, s->tag };
        o_philox(s->key, ctr, s->buf);
        s->block++;
        s->idx = 0;
    }
    return s->buf[s->idx++];
}

/* Uniform in (0, 1] with 24 random bits: ((x >> 8) + 1) * 2^-24, exact. */
static inline float o_uniform(o_stream* s)
{
    return (float)((o_next_u32(s) >> 8) + 1u) * (1.0f / 16777216.0f);
}

/* ---------------- portable FP32 log ---------------- */
/* log(x) for normal positive x: x = 2^e m, m in [sqrt(1/2), sqrt(2)),
 * log(m) = 2 atanh(f), f = (m - 1)/(m + 1), odd series in f. */
static inline float o_logf(float x)
{
    uint32_t bits = o_f2u(x);
    int e = (int)((bits >> 23) & 0xffu) - 127;
    float m = o_u2f((bits & 0x007fffffu) | 0x3f800000u);
    if (m > 1.41421356f) { m = m * 0.5f; e = e + 1; }
    float f = (m - 1.0f) / (m + 1.0f);
    float s = f * f;
    float p = 0.0909090909f;                 /* 1/11 */
    p = fmaf(p, s, 0.111111111f);            /* 1/9  */
    p = fmaf(p, s, 0.142857143f);            /* 1/7  */
    p = fmaf(p, s, 0.2f);                    /* 1/5  */
    p = fmaf(p, s, 0.333333333f);            /* 1/3  */
    p = p * s;
    float lm = fmaf(2.0f * f, p, 2.0f * f);  /* 2f(1 + s/3 + ...) */
    float fe = (float)e;
    return fmaf(fe, 0.693145752f, fmaf(fe, 1.42860677e-06f, lm));
}

/* ---------------- portable FP32 sin(pi x), cos(pi x) ---------------- */
/* x = n/2 + r, |r| <= 1/4; Taylor series of sin(pi r) and cos(pi r). */
static inline void o_sincospif(float x, float* sp, float* cp)
{
    float n = rintf(x * 2.0f);
    float r = fmaf(n, -0.5f, x);
    float r2 = r * r;
    /* sin(pi r) = r (pi - pi^3 r^2/3! + pi^5 r^4/5! - pi^7 r^6/7! + pi^9 r^8/9!) */
    float ps = 0.0821458866f;                /*  pi^9/9! */
    ps = fmaf(ps, r2, -0.599264529f);        /* -pi^7/7! */
    ps = fmaf(ps, r2, 2.55016404f);          /*  pi^5/5! */
    ps = fmaf(ps, r2, -5.16771278f);         /* -pi^3/3! */
    ps = fmaf(ps, r2, 3.14159265f);          /*  pi      */
    float s = ps * r;
    /* cos(pi r) = 1 - pi^2 r^2/2! + pi^4 r^4/4! - pi^6 r^6/6! + pi^8 r^8/8! - pi^10 r^10/10! */
    float pc = -0.0258068914f;               /* -pi^10/10! */
    pc = fmaf(pc, r2, 0.235330630f);         /*  pi^8/8!  */
    pc = fmaf(pc, r2, -1.33526277f);         /* -pi^6/6!  */
    pc = fmaf(pc, r2, 4.05871213f);          /*  pi^4/4!  */
    pc = fmaf(pc, r2, -4.93480220f);         /* -pi^2/2!  */
    float c = fmaf(pc, r2, 1.0f);
    int q = ((int)n) & 3;
    if (q == 0) { *sp = s;  *cp = c;  }
    else if (q == 1) { *sp = c;  *cp = -s; }
    else if (q == 2) { *sp = -s; *cp = -c; }
    else { *sp = -c; *cp = s; }
}

/* ---------------- hash of a vertex sequence ---------------- */
static inline uint32_t o_hash_mix(uint32_t h, uint32_t v)
{
    h ^= v;
    h *= 0x01000193u;
    h ^= h >> 15;
    return h;
}

#endif
