// gemm_tc.cu -- the illumination x view contraction on the 5th-generation
// tensor cores (tcgen05, sm_103a), 3xTF32 with FP32 accumulation.
//
//     V[t][v][l] += sum_p A[p][t][l] * B[p][t][v]      (complex, FP64 V)
//
// replaces multipleResFinal's broadcast product + cublasZgemv
// (NextEventEstimation.cuh:1397-1458, MatrixOperations.cuh:192-516).
//
// The complex product is a real GEMM over interleaved (re, im) rows:
// D[m][n] = sum_p a[p][m] b[p][n] with m = 2l + re/im, n = 2v + re/im, then
// Re V = D[2l][2v] - D[2l+1][2v+1], Im V = D[2l][2v+1] + D[2l+1][2v].
// Real rows (G.real, the correlation sampler with identical u1 / u2 sources
// and static scatterers): two ticks of a path are 2 Nl (or 2 Nv) consecutive
// floats, so the same 128-row tiles span a tick pair and D's diagonal blocks
// (tick of m == tick of n) are the two ticks' products; the row bytes read
// from HBM are half the complex form's.
// Each FP32 operand x is split into TF32 parts hi = rna(x), lo = rna(x - hi),
// and D accumulates hi*hi + hi*lo + lo*hi.
//
// One CTA owns a 128 x 128 tile of D for one tick and a range of paths:
//   warp 0      allocates tensor memory; one thread issues the TMA box loads
//               (cp.async.bulk.tensor, 32 paths x 128 rows of A and of B)
//               into a 3-deep raw ring and the tcgen05.mma (M = N = 128,
//               K = 8) into one of two TMEM accumulators;
//   warps 1-8   split each raw box into TF32 hi / lo tiles stored in the
//               128-byte-swizzled K-major layout the MMA descriptors
//               describe (2-deep ring), one 8-path group per warp;
//   warps 9-12  drain an accumulator every 256 paths into compensated FP32
//               (hi, lo) pairs kept in tensor memory too (TwoSum), so FP32
//               rounding grows with a 256-path window rather than with the
//               whole path range, and add the tile to V with FP64 atomics
//               at the end.
// Every mbarrier wait is bounded; a wait that runs out sets SSTMC_TIMEOUT in
// the error word, and every role then leaves its loop, waits for the MMAs it
// issued and frees the tensor memory.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "contract.h"

namespace sstmc {

namespace {

constexpr int kTM = 128;          // D rows per CTA (64 illumination entries, re / im)
constexpr int kTN = 128;          // D columns per CTA (64 view entries, re / im)
constexpr int kKS = 32;           // paths per step: one 128-byte swizzle row of TF32
constexpr int kStages = 2;        // hi / lo tiles in flight to the MMA
constexpr int kRaw = 3;           // raw TMA boxes in flight from global memory
constexpr int kWinSteps = 8;      // steps per accumulation window (256 paths)
constexpr int kSplitWarps = 8;
constexpr int kEpiWarps = 4;
constexpr int kThreads = (1 + kSplitWarps + kEpiWarps) * 32;  // 416
constexpr int kSplitThreads = kSplitWarps * 32;
constexpr int kEpiThreads = kEpiWarps * 32;
constexpr uint32_t kATile = kTM * kKS * 4;                   // 16 KB
constexpr uint32_t kBTile = kTN * kKS * 4;                   // 16 KB
constexpr uint32_t kStageBytes = 2 * kATile + 2 * kBTile;    // 64 KB: A hi, A lo, B hi, B lo
constexpr uint32_t kRawA = kKS * kTM * 4;                    // 16 KB: 32 paths x 128 floats
constexpr uint32_t kRawBytes = kRawA + kKS * kTN * 4;        // + 16 KB: 32 paths x 128 floats
constexpr uint32_t kBarBytes = 256;
constexpr size_t kSmemBytes = (size_t)kStages * kStageBytes + (size_t)kRaw * kRawBytes + kBarBytes + 1024;
// tensor memory: two accumulators, then the compensated hi and lo sums
constexpr uint32_t kColD = 0, kColHi = 2 * kTN, kColLo = 3 * kTN;
constexpr uint32_t kTmemCols = 4 * kTN;                      // 512: all of it
constexpr unsigned long long kWaitNs = 2000000000ull;        // 2 s per wait

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// try_wait with a suspend-time hint: the thread sleeps until the phase
// completes or the hint runs out, so waiting warps take no issue slots from
// the warps that share their scheduler.
__device__ __forceinline__ bool mbar_try_sleep(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity), "r"(1000000u)
        : "memory");
    return ok != 0;
}

// Bounded wait for the phase with the given parity; false if it ran out or
// (when honor_abort) another role gave up.  The final waits for in-flight
// copies and MMAs pass honor_abort = false: they must end before the CTA
// frees its tensor memory and exits, and they are bounded all the same.
// sleep = true for the long waits (a whole accumulation window): the waiting
// warp is suspended instead of polling; the short pipeline waits poll.
__device__ __noinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int* abort, int* err,
                                       bool honor_abort = true, bool sleep = false)
{
    if (mbar_try(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    for (;;) {
        if (sleep ? mbar_try_sleep(bar, parity) : mbar_try(bar, parity)) return true;
        if (honor_abort && *abort) return false;
        if (global_ns() - t0 > kWaitNs) {
            *abort = 1;
            atomicExch(err, SSTMC_TIMEOUT);
            return false;
        }
    }
}

__device__ __forceinline__ void fence_proxy_async()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart (tcgen05 descriptor format, version 1).
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr)
{
    return (uint64_t)((saddr & 0x3FFFFu) >> 4)
         | ((uint64_t)1 << 16)               // leading byte offset (unused for swizzled K-major)
         | ((uint64_t)(1024u >> 4) << 32)    // stride byte offset
         | ((uint64_t)1 << 46)               // descriptor version
         | ((uint64_t)2 << 61);              // SWIZZLE_128B
}

// Instruction descriptor of kind::tf32: D F32, A and B TF32, both K-major.
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(kTN >> 3) << 17) | ((uint32_t)(kTM >> 4) << 24);

__device__ __forceinline__ void mma_tf32(uint32_t d, uint64_t a, uint64_t b, uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(d), "l"(a), "l"(b), "r"(kIdesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&r)[16])
{
    uint32_t u[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(u[0]), "=r"(u[1]), "=r"(u[2]), "=r"(u[3]), "=r"(u[4]), "=r"(u[5]), "=r"(u[6]), "=r"(u[7]),
          "=r"(u[8]), "=r"(u[9]), "=r"(u[10]), "=r"(u[11]), "=r"(u[12]), "=r"(u[13]), "=r"(u[14]), "=r"(u[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) r[i] = __uint_as_float(u[i]);
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ void tmem_st16(uint32_t taddr, const float (&r)[16])
{
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};"
        ::"r"(taddr), "r"(__float_as_uint(r[0])), "r"(__float_as_uint(r[1])), "r"(__float_as_uint(r[2])), "r"(__float_as_uint(r[3])),
          "r"(__float_as_uint(r[4])), "r"(__float_as_uint(r[5])), "r"(__float_as_uint(r[6])), "r"(__float_as_uint(r[7])),
          "r"(__float_as_uint(r[8])), "r"(__float_as_uint(r[9])), "r"(__float_as_uint(r[10])), "r"(__float_as_uint(r[11])),
          "r"(__float_as_uint(r[12])), "r"(__float_as_uint(r[13])), "r"(__float_as_uint(r[14])), "r"(__float_as_uint(r[15]))
        : "memory");
}

__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// byte offset of (row, 16-byte chunk) in a K-major 128-byte-swizzled tile
__device__ __forceinline__ uint32_t sw128(uint32_t row, uint32_t chunk)
{
    return (row >> 3) * 1024u + (row & 7u) * 128u + ((chunk ^ (row & 7u)) << 4);
}

// x = hi + lo with hi = x rounded to the nearest TF32 and lo = x - hi (exact
// in FP32, |lo| <= 2^-12 |x|) also rounded to TF32, so the three products
// hi*hi + hi*lo + lo*hi carry FP32-level error (the dropped lo*lo and the
// rounding of lo are below 2^-23 |x y|).
// round to nearest TF32, ties away from zero (the rna rounding): add half of
// the 13 dropped bits to the magnitude, then clear them
__device__ __forceinline__ float round_tf32(float x)
{
    return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
}

__device__ __forceinline__ void split_tf32(float x, float& hi, float& lo)
{
    hi = round_tf32(x);
    lo = round_tf32(x - hi);
}

__device__ __forceinline__ void two_sum(float& hi, float& lo, float x)
{
    const float s = hi + x;
    const float bb = s - hi;
    const float e = (hi - (s - bb)) + (x - bb);
    hi = s;
    lo += e;
}

struct TcParams {
    GemmParams G;
    int ksplit;        // path ranges per tile (per material with G.bucket)
    int tiles_m, tiles_n;
    int tdim;          // middle tensor dimension: Nt ticks (complex) or Nt / 2 tick pairs (real)
    CUtensorMap tmA;   // A viewed as [K paths][tdim][2 Nl floats], box 32 x 1 x 128
    CUtensorMap tmB;   // B viewed as [K paths][tdim][2 Nv floats], box 32 x 1 x 128
};

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* tm, int x, int y, int z, uint32_t bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(dst), "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(z), "r"(bar)
        : "memory");
}

// One thread's share of a step: 4 rows (row0 + 32 r) of one 8-path group
// kq, read from the raw box (128 floats per path), split into TF32 hi / lo
// and stored as two 16-byte chunks of the swizzled hi and lo tiles.
__device__ __forceinline__ void split_group(const float* raw, unsigned char* hi_tile, uint32_t lo_delta, uint32_t valid,
                                            int row0, int kq)
{
    const uint32_t vq = (valid >> (8 * kq)) & 0xffu;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int row = row0 + 32 * r;
        const float* src = raw + kq * 8 * 128 + row;
        float x[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) x[j] = src[j * 128];
        if (vq != 0xffu) {
#pragma unroll
            for (int j = 0; j < 8; ++j) x[j] = ((vq >> j) & 1u) ? x[j] : 0.0f;
        }
        float h[8], l[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) split_tf32(x[j], h[j], l[j]);
        const uint32_t o0 = sw128((uint32_t)row, (uint32_t)(2 * kq));
        unsigned char* d0 = hi_tile + o0;
        unsigned char* d1 = hi_tile + (o0 ^ 16u);
        *reinterpret_cast<float4*>(d0) = make_float4(h[0], h[1], h[2], h[3]);
        *reinterpret_cast<float4*>(d1) = make_float4(h[4], h[5], h[6], h[7]);
        *reinterpret_cast<float4*>(d0 + lo_delta) = make_float4(l[0], l[1], l[2], l[3]);
        *reinterpret_cast<float4*>(d1 + lo_delta) = make_float4(l[4], l[5], l[6], l[7]);
    }
}

__global__ void __launch_bounds__(kThreads, 1) gemm_tc_kernel(const __grid_constant__ TcParams P)
{
    extern __shared__ unsigned char tc_smem_raw[];
    const GemmParams& G = P.G;
    // 1024-byte aligned tiles (the swizzle pattern is taken from address bits
    // 4-9).  The offset is added to the shared array itself so every derived
    // pointer stays a shared-memory pointer (ld.shared / st.shared, not generic).
    const uint32_t pad = ((smem_u32(tc_smem_raw) + 1023u) & ~1023u) - smem_u32(tc_smem_raw);
    unsigned char* smem = tc_smem_raw + pad;
    const uint32_t split_base = smem_u32(smem);                                  // kStages x (A hi, A lo, B hi, B lo)
    const uint32_t raw_base = split_base + (uint32_t)kStages * kStageBytes;      // kRaw x (A raw, B raw)
    unsigned char* bars = smem + (size_t)kStages * kStageBytes + (size_t)kRaw * kRawBytes;
    const uint32_t bar0 = smem_u32(bars);
    auto full_bar = [&](int s) { return bar0 + 8u * (uint32_t)s; };
    auto empty_bar = [&](int s) { return bar0 + 8u * (uint32_t)(kStages + s); };
    auto rfull_bar = [&](int r) { return bar0 + 8u * (uint32_t)(2 * kStages + r); };
    auto rempty_bar = [&](int r) { return bar0 + 8u * (uint32_t)(2 * kStages + kRaw + r); };
    auto accfull_bar = [&](int b) { return bar0 + 8u * (uint32_t)(2 * kStages + 2 * kRaw + b); };
    auto accempty_bar = [&](int b) { return bar0 + 8u * (uint32_t)(2 * kStages + 2 * kRaw + 2 + b); };
    const uint32_t done_bar = bar0 + 8u * (uint32_t)(2 * kStages + 2 * kRaw + 4);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 8 * (2 * kStages + 2 * kRaw + 5));
    volatile int* abort = reinterpret_cast<volatile int*>(bars + 8 * (2 * kStages + 2 * kRaw + 5) + 4);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    // tile of this CTA
    int bid = blockIdx.x;
    const int tn = bid % P.tiles_n; bid /= P.tiles_n;
    const int tm = bid % P.tiles_m; bid /= P.tiles_m;
    const int t = bid % P.tdim; bid /= P.tdim;
    int kb, ke;
    const float* W = G.W;
    if (G.bucket) {
        // material mats[bid % nmat]: its rows bucket[m] .. bucket[m + 1], split in
        // ksplit ranges of whole accumulation windows, and its weight table
        const int m = G.mats[bid % G.nmat];
        const int ks = bid / G.nmat;
        const int rb = (int)G.bucket[m], re = (int)G.bucket[m + 1];
        const int win = kKS * kWinSteps;
        const int kc = ((re - rb + P.ksplit - 1) / P.ksplit + win - 1) / win * win;
        kb = rb + ks * kc;
        ke = min(re, kb + kc);
        W = G.W + (size_t)m * G.wstride;
    } else {
        kb = bid * G.kchunk;
        ke = min(G.K, kb + G.kchunk);
    }
    const int nsteps = ke > kb ? (ke - kb + kKS - 1) / kKS : 0;
    const int m0 = tm * kTM, n0 = tn * kTN;

    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) { mbar_init(full_bar(s), kSplitThreads); mbar_init(empty_bar(s), 1); }
        for (int r = 0; r < kRaw; ++r) { mbar_init(rfull_bar(r), 1); mbar_init(rempty_bar(r), kSplitThreads); }
        for (int b = 0; b < 2; ++b) { mbar_init(accfull_bar(b), 1); mbar_init(accempty_bar(b), kEpiThreads); }
        mbar_init(done_bar, 1);
        *abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        fence_proxy_async();
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&P.tmA)) : "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&P.tmB)) : "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)), "r"(kTmemCols) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        // ---------------- TMA producer + MMA issuer (one thread) ----------------
        if (lane == 0) {
            int issued_raw = 0, issued = 0;
            bool ok = true;
            auto issue_raw = [&](int j) -> bool {
                const int r = j % kRaw;
                if (j >= kRaw && !mbar_wait(rempty_bar(r), (uint32_t)((j / kRaw) - 1) & 1u, abort, G.err)) return false;
                const uint32_t dst = raw_base + (uint32_t)r * kRawBytes;
                mbar_expect_tx(rfull_bar(r), kRawBytes);
                const int p0 = kb + j * kKS;
                tma_load_3d(dst, &P.tmA, m0, t, p0, rfull_bar(r));
                tma_load_3d(dst + kRawA, &P.tmB, n0, t, p0, rfull_bar(r));
                issued_raw = j + 1;
                return true;
            };
            for (int j = 0; j < min(kRaw - 1, nsteps) && ok; ++j) ok = issue_raw(j);
            for (int i = 0; i < nsteps && ok; ++i) {
                if (i + kRaw - 1 < nsteps && !issue_raw(i + kRaw - 1)) { ok = false; break; }
                const int s = i % kStages;
                if (!mbar_wait(full_bar(s), (uint32_t)(i / kStages) & 1u, abort, G.err)) { ok = false; break; }
                const int w = i / kWinSteps, b = w & 1;
                const bool first = (i % kWinSteps) == 0;
                if (first && w >= 2 && !mbar_wait(accempty_bar(b), (uint32_t)((w >> 1) - 1) & 1u, abort, G.err)) { ok = false; break; }
                tc_fence_after();
                const uint32_t st = split_base + (uint32_t)s * kStageBytes;
                const uint32_t d = tmem + kColD + (uint32_t)(b * kTN);
#pragma unroll
                for (int k = 0; k < kKS / 8; ++k) {
                    const uint64_t ah = sdesc(st + 32u * k), al = sdesc(st + kATile + 32u * k);
                    const uint64_t bh = sdesc(st + 2u * kATile + 32u * k), bl = sdesc(st + 2u * kATile + kBTile + 32u * k);
                    mma_tf32(d, al, bh, (first && k == 0) ? 0u : 1u);
                    mma_tf32(d, ah, bl, 1u);
                    mma_tf32(d, ah, bh, 1u);
                }
                issued = 1;
                mma_commit(empty_bar(s));
                if ((i % kWinSteps) == kWinSteps - 1 || i == nsteps - 1) mma_commit(accfull_bar(b));
            }
            // every MMA issued here has completed once done_bar flips; every raw
            // box issued here has landed once its rfull phase completed
            if (issued) {
                mma_commit(done_bar);
                mbar_wait(done_bar, 0u, abort, G.err, false);
            }
            for (int j = max(0, issued_raw - kRaw); j < issued_raw; ++j)
                mbar_wait(rfull_bar(j % kRaw), (uint32_t)(j / kRaw) & 1u, abort, G.err, false);
        }
        __syncwarp();
    } else if (warp <= kSplitWarps) {
        // ---------------- split warps: one 8-path group of A or B each ----------------
        const int sw = warp - 1;
        const bool isA = sw < 4;
        const int kq = sw & 3;
        for (int i = 0; i < nsteps; ++i) {
            const int r = i % kRaw, s = i % kStages;
            if (!mbar_wait(rfull_bar(r), (uint32_t)(i / kRaw) & 1u, abort, G.err)) break;
            if (i >= kStages && !mbar_wait(empty_bar(s), (uint32_t)((i / kStages) - 1) & 1u, abort, G.err)) break;
            const int pbase = kb + i * kKS;
            // paths of this step that count: inside [kb, ke) and of the selected material
            const int nin = min(kKS, ke - pbase);
            uint32_t valid = nin >= kKS ? 0xffffffffu : ((1u << nin) - 1u);
            if (G.mat)
                for (int j = 0; j < nin; ++j)
                    if (G.mat[pbase + j] != G.mat_sel) valid &= ~(1u << j);
            const float* rawf = reinterpret_cast<const float*>(smem + (size_t)kStages * kStageBytes + (size_t)r * kRawBytes);
            unsigned char* stp = smem + (size_t)s * kStageBytes;
            if (isA) split_group(rawf, stp, kATile, valid, lane, kq);
            else split_group(rawf + kRawA / 4, stp + 2 * kATile, kBTile, valid, lane, kq);
            fence_proxy_async();
            mbar_arrive(full_bar(s));
            mbar_arrive(rempty_bar(r));
        }
    } else {
        // ---------------- accumulator drain (lane quadrant warp & 3) ----------------
        const int q = warp & 3;
        const uint32_t row_addr = tmem + ((uint32_t)(32 * q) << 16);
        {
            float z[16];
#pragma unroll
            for (int c = 0; c < 16; ++c) z[c] = 0.0f;
#pragma unroll
            for (int c = 0; c < kTN / 16; ++c) { tmem_st16(row_addr + kColHi + 16u * c, z); tmem_st16(row_addr + kColLo + 16u * c, z); }
            tmem_wait_st();
        }
        const int nwin = (nsteps + kWinSteps - 1) / kWinSteps;
        bool ok = true;
        for (int w = 0; w < nwin && ok; ++w) {
            const int b = w & 1;
            ok = mbar_wait(accfull_bar(b), (uint32_t)(w >> 1) & 1u, abort, G.err, true, true);
            ok = __all_sync(0xffffffffu, ok);   // tcgen05.ld / st and the final shuffles need the whole warp
            if (!ok) break;
            tc_fence_after();
#pragma unroll 1
            for (int c = 0; c < kTN / 16; ++c) {
                float dv[16], hv[16], lv[16];
                tmem_ld16(row_addr + kColD + (uint32_t)(b * kTN) + 16u * c, dv);
                tmem_ld16(row_addr + kColHi + 16u * c, hv);
                tmem_ld16(row_addr + kColLo + 16u * c, lv);
                tmem_wait_ld();
                if (c == kTN / 16 - 1) {   // the accumulator has been read: the MMA may reuse it
                    tc_fence_before();
                    mbar_arrive(accempty_bar(b));
                }
#pragma unroll
                for (int e = 0; e < 16; ++e) two_sum(hv[e], lv[e], dv[e]);
                tmem_st16(row_addr + kColHi + 16u * c, hv);
                tmem_st16(row_addr + kColLo + 16u * c, lv);
            }
            tmem_wait_st();
        }
        if (ok && nwin > 0 && G.real) {
            // real rows: row m = tick (2 t + mt) of illumination l, column n = tick
            // (2 t + nt) of view v; the same-tick blocks are the two ticks' sums
            const int gm = m0 + 32 * q + lane;
            const int mt = gm / G.Nl, l = gm - mt * G.Nl;
            const int tick = 2 * t + mt;
#pragma unroll 1
            for (int c = 0; c < kTN / 16; ++c) {
                float hv[16], lv[16];
                tmem_ld16(row_addr + kColHi + 16u * c, hv);
                tmem_ld16(row_addr + kColLo + 16u * c, lv);
                tmem_wait_ld();
#pragma unroll
                for (int e = 0; e < 16; ++e) {
                    const int gn = n0 + 16 * c + e;
                    const int nt = gn / G.Nv, v = gn - nt * G.Nv;
                    if (nt == mt && mt < 2 && tick < G.Nt) {
                        const size_t o = ((size_t)tick * G.Nv + v) * G.Nl + l;
                        const double wv = (W ? (double)W[o] : 1.0) * (G.scale != 0.0 ? G.scale : 1.0);
                        atomicAdd(&G.V[o].x, ((double)hv[e] + (double)lv[e]) * wv);
                    }
                }
            }
        } else if (ok && nwin > 0) {
            // rows m (even: Re a, odd: Im a) pair up across adjacent lanes
            const int m = 32 * q + lane;
            const int gm = m0 + m;
            const int l = gm >> 1;
            const bool odd = (gm & 1) != 0;
#pragma unroll 1
            for (int c = 0; c < kTN / 16; ++c) {
                float hv[16], lv[16];
                tmem_ld16(row_addr + kColHi + 16u * c, hv);
                tmem_ld16(row_addr + kColLo + 16u * c, lv);
                tmem_wait_ld();
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const double own = (double)hv[2 * j] + (double)lv[2 * j];
                    const double send = (double)hv[2 * j + 1] + (double)lv[2 * j + 1];
                    const double r = __shfl_xor_sync(0xffffffffu, send, 1);
                    const double val = odd ? own + r : own - r;   // odd: Im V = D[2l][2v+1] + D[2l+1][2v]; even: Re V
                    const int v = (n0 + 16 * c + 2 * j) >> 1;
                    if (l < G.Nl && v < G.Nv) {
                        const size_t o = ((size_t)t * G.Nv + v) * G.Nl + l;
                        const double wv = (W ? (double)W[o] : 1.0) * (G.scale != 0.0 ? G.scale : 1.0);
                        atomicAdd(odd ? &G.V[o].y : &G.V[o].x, val * wv);
                    }
                }
            }
        }
    }

    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
    }
}

}  // namespace

// TMA needs 16-byte row strides: Nl and Nv even (odd counts use gemm_kernel);
// real rows pair ticks: Nt even.
bool gemm_tc_eligible(const GemmParams& G)
{
    return G.compensated != 0 && G.K > 0 && G.Nl > 0 && G.Nv > 0 && G.Nl % 2 == 0 && G.Nv % 2 == 0
        && (!G.real || G.Nt % 2 == 0)
        && reinterpret_cast<uintptr_t>(G.A) % 16 == 0 && reinterpret_cast<uintptr_t>(G.B) % 16 == 0;
}

// cuTensorMapEncodeTiled, resolved through the runtime so the library does
// not link the driver library itself (it still loads on a host without one).
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess
            || q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}

// [K paths][Nt ticks][rows floats] as a 3D tensor (rows fastest), box
// box_rows x 1 x kKS; boxes past the tensor's edge are filled with zeros.
static bool encode_rows(CUtensorMap* tm, const void* base, int rows, int Nt, int K, int box_rows)
{
    const PFN_cuTensorMapEncodeTiled_v12000 encode = encode_fn();
    if (!encode) return false;
    cuuint64_t dims[3] = { (cuuint64_t)rows, (cuuint64_t)Nt, (cuuint64_t)K };
    cuuint64_t strides[2] = { (cuuint64_t)rows * 4u, (cuuint64_t)rows * 4u * (cuuint64_t)Nt };
    cuuint32_t box[3] = { (cuuint32_t)box_rows, 1u, (cuuint32_t)kKS };
    cuuint32_t estr[3] = { 1u, 1u, 1u };
    return encode(tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void*>(base), dims, strides, box, estr,
                                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int launch_gemm_tc(const GemmParams& G, cudaStream_t stream)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    TcParams P;
    P.G = G;
    if (G.real && G.Nt % 2 != 0) return SSTMC_CUBLAS_ERROR;
    P.tiles_m = (2 * G.Nl + kTM - 1) / kTM;
    P.tiles_n = (2 * G.Nv + kTN - 1) / kTN;
    P.tdim = G.real ? G.Nt / 2 : G.Nt;
    const long long tiles = (long long)P.tiles_m * P.tiles_n * P.tdim * (G.bucket ? G.nmat : 1);
    // K split: fewer tiles than SMs take sms / tiles ranges each; more tiles take
    // the smallest split (up to 8) whose CTAs fill their last wave to 95 % (one
    // CTA per SM: a partly filled last wave idles the rest of the SMs)
    int ksplit = (int)std::max<long long>(1, sms / std::max<long long>(1, tiles));
    if (tiles >= sms) {
        double best = 0.0;
        for (int ks = 1; ks <= 8; ++ks) {
            const long long ctas = tiles * ks, waves = (ctas + sms - 1) / sms;
            const double eff = (double)ctas / (double)(waves * sms);
            if (eff > best + 0.02) { best = eff; ksplit = ks; }
            if (eff >= 0.95) break;
        }
    }
    const int win = kKS * kWinSteps;
    if (G.bucket) {
        // the materials' row counts are on the device: at most K / nmat rows on
        // average, at least one window per range
        const int avg = std::max(1, G.K / std::max(1, G.nmat));
        ksplit = std::max(1, std::min(ksplit, (avg + win - 1) / win));
        if (G.nmat < 1 || G.nmat > kMat) return SSTMC_CUBLAS_ERROR;
    } else {
        int kchunk = (G.K + ksplit - 1) / ksplit;
        kchunk = ((kchunk + win - 1) / win) * win;
        ksplit = (G.K + kchunk - 1) / kchunk;
        P.G.kchunk = kchunk;
    }
    P.ksplit = ksplit;
    // complex: 2 Nl floats (re, im) per tick; real: 2 Nl floats per tick pair
    if (!encode_rows(&P.tmA, G.A, 2 * G.Nl, P.tdim, G.K, kTM) || !encode_rows(&P.tmB, G.B, 2 * G.Nv, P.tdim, G.K, kTN))
        return SSTMC_CUBLAS_ERROR;
    const long long grid = tiles * ksplit;
    if (grid <= 0 || grid > 0x7fffffffLL) return SSTMC_CUBLAS_ERROR;
    if (cudaFuncSetAttribute((const void*)gemm_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBytes) != cudaSuccess)
        return SSTMC_CUBLAS_ERROR;
    gemm_tc_kernel<<<(unsigned)grid, kThreads, kSmemBytes, stream>>>(P);
    return cudaGetLastError() == cudaSuccess ? SSTMC_NO_ERROR : SSTMC_CUBLAS_ERROR;
}

}  // namespace sstmc
