// pathwalk.cu -- the random walk, one thread per path.
//
// Samples the first vertex with miss resampling (NextEventEstimation.cuh:643-679,
// FarField.cuh:129-205 / PointSource.cuh:72-90 + Woodcock free flight,
// HeterogeneousMedium.cuh:576-678) and every later vertex (phase-function
// direction, Scattering.cuh:1039-1115, then free flight) until the path leaves
// the medium or is absorbed.  The walk is run twice over the same Philox
// streams: the first pass counts each path's vertices, an exclusive scan turns
// the counts into offsets, and the second pass writes the vertices compactly
// (16 bytes each: position and a packed word holding the material and the
// per-vertex phase draw).  The NEE kernel then reads them with no walk code.
#include <cuda_runtime.h>

#include <algorithm>

#include "pathwalk.h"
#include "gauss.cuh"

namespace sstmc {

namespace {

constexpr uint32_t kSlotVerts = kWalkSlotVerts;

__device__ __forceinline__ uint32_t u1_count_w(const DevScene& S, uint64_t seed, uint32_t wave)
{
    Stream ws;
    ws.init(seed, wave, 0u, kPurposeWave);
    int c = (int)ceilf(fm(ws.uniform(), (float)(S.P + 1u))) - 1;
    c = c < 0 ? 0 : (c > (int)S.P ? (int)S.P : c);
    return (uint32_t)c;
}

__device__ __forceinline__ uint32_t hash_v(const DevScene& S, uint32_t h, const V3& x, int m)
{
    h = hash_mix(h, __float_as_uint(x.x));
    h = hash_mix(h, __float_as_uint(x.y));
    if (S.dims == 3) h = hash_mix(h, __float_as_uint(x.z));
    return hash_mix(h, (uint32_t)m);
}

__device__ __forceinline__ float4 pack_vertex(const V3& x, int m, float xi)
{
    const uint32_t k = (uint32_t)(xi * 16777216.0f);  // xi = k * 2^-24 exactly
    return make_float4(x.x, x.y, x.z, __uint_as_float((k << 4) | (uint32_t)m));
}

// Flattened walk: a thread samples one vertex (or one first-vertex attempt)
// per iteration and takes a new path from a shared counter as soon as its
// path ends (warp-aggregated atomics), so the lanes of a warp stay busy until
// the whole pool is drawn.  The first two Philox blocks of each vertex are
// generated at the top of the iteration, where all lanes are converged.
// MODE kSlots: one pass that counts every path and writes its first
//   kSlotVerts vertices into a fixed slot and the rest into overflow blocks
//   of kSlotVerts vertices taken from a shared pool (compaction kernels then
//   pack both); a path that finds the pool empty is listed for kWrite;
// MODE kCount: count only;
// MODE kWrite: replay paths (all, or the W.list of long ones) and write their
//   vertices at their offsets.
constexpr int kCount = 0, kWrite = 1, kSlots = 2;
// resident walk blocks of 128 threads per SM (64 registers, no spills since
// the first vertices left the walk): the launch bound and the persistent
// grid's size
constexpr int kWalkBlocksPerSM = 8;

// GB: Gaussian-beam illumination (3D): the beam places the first vertex and
// samples the second direction (gauss.cuh)
template <int MODE, bool VMF, bool GB>
__global__ void __launch_bounds__(128, kWalkBlocksPerSM) walk_kernel(const __grid_constant__ DevScene S, const __grid_constant__ WalkParams W)
{
    constexpr bool WRITE = MODE == kWrite;
    constexpr bool COUNTS = MODE != kWrite;
    const uint32_t lane = threadIdx.x & 31u;
    const bool corr = S.correlation != 0;
    const uint32_t pool = (WRITE && W.list) ? W.list_n : W.paths;
    uint32_t q = 0, pid = 0, att = 0, b = 1, B = 0, h = 2166136261u;
    V3 prev{ 0.f, 0.f, 0.f }, cur{ 0.f, 0.f, 0.f };
    int mcur = 0;
    int beam = 0;   // GB: the beam of the path's first vertex
    float4* out = nullptr;
    uint32_t o0 = 0;   // vertex index stored at out[0]
    const DevSource* fsrc = &S.src[0];
    // next pool index for each active lane (one atomic per warp and call)
    auto fetch = [&]() -> uint32_t {
        const uint32_t mask = __activemask();
        const int leader = __ffs(mask) - 1;
        uint32_t base = 0;
        if ((int)lane == leader) base = atomicAdd(W.next, (uint32_t)__popc(mask));
        base = __shfl_sync(mask, base, leader);
        return base + (uint32_t)__popc(mask & ((1u << lane) - 1u));
    };
    // move to the next path that has work; false when the pool is drawn
    auto start = [&](uint32_t i) -> bool {
        for (;;) {
            if (i >= pool) return false;
            q = (WRITE && W.list) ? W.list[i] : i;
            if (!WRITE || W.counts[q] != 0) break;
            if (W.hash) W.hash[q] = 2166136261u;  // the count pass hit a limit: nothing to write
            i = fetch();
        }
        pid = W.first_path + q;
        const uint32_t slot = pid % S.P, wave = pid / S.P;
        fsrc = (!corr || slot < u1_count_w(S, W.seed, wave)) ? &S.src[0] : &S.src[2];
        att = 0; b = 1; B = 0; h = 2166136261u;
        if (WRITE) out = W.verts + W.offsets[q];
        if (MODE == kSlots) out = W.slots + (size_t)q * kSlotVerts;
        o0 = 0;
        return true;
    };
    auto finish = [&](bool ok) {
        if (!ok) { atomicExch(W.err, SSTMC_PATH_LIMIT); B = 0; }
        if (COUNTS) { W.counts[q] = B; W.misses[q] = att; }
        if (MODE != kCount && W.hash) W.hash[q] = h;
        if (MODE == kSlots && ok && out == nullptr) W.list[atomicAdd(W.list_count, 1u)] = q;   // replayed by the write pass
    };
    auto store = [&](uint32_t k, const V3& x, int m, float xi) {   // vertex k (0-based)
        if (WRITE) out[k] = pack_vertex(x, m, xi);
        if (MODE == kSlots) {
            if (k % kSlotVerts == 0 && k != 0 && out != nullptr) {   // slot or block full: take a block
                const uint32_t blk = atomicAdd(W.ovf_count, 1u);
                if (blk < W.ovf_cap) {
                    W.ovf_owner[blk] = make_uint2(q, k / kSlotVerts);
                    out = W.ovf + (size_t)blk * kSlotVerts;
                    o0 = k;
                } else {
                    out = nullptr;
                }
            }
            if (out != nullptr) out[k - o0] = pack_vertex(x, m, xi);
        }
        if (MODE != kCount && W.hash) h = hash_v(S, h, x, m);   // the debug trace's vertex hash
    };
    // non-beam walks: the path's first vertex from its record (first_vertex_kernel);
    // false when the first vertex hit a limit (the path then ends with no vertices)
    auto begin = [&]() -> bool {
        const float4 r0 = W.first[2 * (size_t)q], r1 = W.first[2 * (size_t)q + 1];
        const uint32_t w = __float_as_uint(r1.w);
        att = (w >> 4) & 0x7ffffffu;
        if (!(w >> 31)) return false;
        prev = V3{ r0.x, r0.y, r0.z };
        cur = V3{ r1.x, r1.y, r1.z };
        mcur = (int)(w & 15u);
        store(0, cur, mcur, r0.w);
        B = 1; b = 2;
        return true;
    };
    // the next path with work; false when the pool is drawn
    auto next_path = [&]() -> bool {
        for (;;) {
            if (!start(fetch())) return false;
            if constexpr (GB) {
                return true;
            } else {
                if (begin()) return true;
                finish(false);
            }
        }
    };
    if (!next_path()) return;
    for (;;) {
        Stream rs;
        rs.init(W.seed, pid, b, kPurposeWalk | (b == 1 ? att << 8 : 0u));
        rs.prime2();
        V3 o, d, xn;
        int mn = 0;
        bool ok;
        if constexpr (GB) {
            if (b == 1) {
                // the beam places x1; a point outside the medium is a miss
                gauss_first(S, *fsrc, rs, o, xn, beam);
                mn = inside(S, xn) ? material_at(S, xn) : 0;
                ok = true;
            } else {
                if (b == 2) {
                    // uniform with isotropic scattering, else from the beam's lobe pairs
                    d = S.iso_all ? random_direction(3, rs) : gauss_second_dir(S, *fsrc, beam, cur, rs);
                } else {
                    const V3 din = normalize32(S.dims, V3{ fsb(cur.x, prev.x), fsb(cur.y, prev.y), fsb(cur.z, prev.z) });
                    d = sample_direction<VMF>(S, mcur, din, rs);
                }
                o = cur;
                ok = woodcock(S, o, d, rs, xn, mn);
            }
        } else {
            // b >= 2: the first vertex came from its record
            const V3 din = normalize32(S.dims, V3{ fsb(cur.x, prev.x), fsb(cur.y, prev.y), fsb(cur.z, prev.z) });
            d = sample_direction<VMF>(S, mcur, din, rs);
            o = cur;
            ok = woodcock(S, o, d, rs, xn, mn);
        }
        bool done = !ok;
        if (ok) {
            if (GB && b == 1) {
                if (mn == 0) {
                    if (++att >= kMaxAttempts) { ok = false; done = true; }
                } else {
                    const float xi = corr ? 0.0f : rs.uniform();
                    store(0, xn, mn, xi);
                    B = 1; prev = o; cur = xn; mcur = mn; b = 2;
                }
            } else if (mn == 0) {
                done = true;
            } else if (b > kMaxVertices || (WRITE && b - 1 >= W.counts[q])) {
                ok = false; done = true;
            } else {
                const float xi = corr ? 0.0f : rs.uniform();
                store(b - 1, xn, mn, xi);
                B = b; prev = cur; cur = xn; mcur = mn; ++b;
            }
        }
        if (done) {
            finish(ok);
            if (!next_path()) return;
        }
    }
}

// The first vertex of every path of a chunk (non-beam sources): source
// sampling and free flight with the miss resampling of the walk's first
// iteration, over the same Philox streams (vertex 1, the attempt count in the
// purpose), so the walk continues from it at vertex 2 with identical results.
// Taking it out of the walk keeps the walk's lanes on the same code: inside
// the walk, a warp ran the source sampling and the flight from outside the
// medium in most of its iterations, for the few lanes whose paths had just
// started.  A thread takes one attempt per iteration and a new path from a
// warp-aggregated counter when its path has its first vertex, so a warp's
// time follows the mean number of attempts rather than its unluckiest lane's.
__global__ void __launch_bounds__(128) first_vertex_kernel(const __grid_constant__ DevScene S, const __grid_constant__ WalkParams W)
{
    const bool corr = S.correlation != 0;
    const uint32_t lane = threadIdx.x & 31u;
    auto fetch = [&]() -> uint32_t {
        const uint32_t mask = __activemask();
        const int leader = __ffs(mask) - 1;
        uint32_t base = 0;
        if ((int)lane == leader) base = atomicAdd(W.first_next, (uint32_t)__popc(mask));
        base = __shfl_sync(mask, base, leader);
        return base + (uint32_t)__popc(mask & ((1u << lane) - 1u));
    };
    uint32_t q = fetch();
    if (q >= W.paths) return;
    uint32_t pid = 0, att = 0;
    const DevSource* fsrc = &S.src[0];
    auto begin = [&]() {
        pid = W.first_path + q;
        const uint32_t slot = pid % S.P, wave = pid / S.P;
        fsrc = (!corr || slot < u1_count_w(S, W.seed, wave)) ? &S.src[0] : &S.src[2];
        att = 0;
    };
    begin();
    for (;;) {
        Stream rs;
        rs.init(W.seed, pid, 1u, kPurposeWalk | (att << 8));
        rs.prime2();
        V3 o, d, xn;
        int mn = 0;
        sample_source(S, *fsrc, rs, o, d);
        const bool flew = woodcock(S, o, d, rs, xn, mn);
        bool done = true, ok = false;
        float xi = 0.0f;
        if (flew && mn == 0) {
            done = ++att >= kMaxAttempts;   // a miss: another attempt, up to the limit
        } else if (flew) {
            xi = corr ? 0.0f : rs.uniform();
            ok = true;
        }
        if (done) {
            W.first[2 * (size_t)q] = make_float4(o.x, o.y, o.z, xi);
            W.first[2 * (size_t)q + 1] = make_float4(xn.x, xn.y, xn.z, __uint_as_float((ok ? 0x80000000u : 0u) | (att << 4) | (uint32_t)mn));
            q = fetch();
            if (q >= W.paths) return;
            begin();
        }
    }
}

// Packs the slots (first kSlotVerts vertices of every path) into the
// compact vertex array at the offsets, thread per slot entry.
__global__ void compact_kernel(const __grid_constant__ WalkParams W)
{
    const size_t total = (size_t)W.paths * kSlotVerts;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const uint32_t q = (uint32_t)(i / kSlotVerts), k = (uint32_t)(i % kSlotVerts);
        if (k < W.counts[q]) W.verts[W.offsets[q] + k] = W.slots[i];
    }
}

// Packs the overflow blocks (vertices kSlotVerts j .. of their owner path).
// A path whose walk found the pool empty is rewritten whole by the write pass.
__global__ void compact_overflow_kernel(const __grid_constant__ WalkParams W)
{
    const size_t total = (size_t)W.ovf_n * kSlotVerts;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const uint2 own = W.ovf_owner[i / kSlotVerts];
        const uint32_t v = own.y * kSlotVerts + (uint32_t)(i % kSlotVerts);
        if (v < W.counts[own.x]) W.verts[W.offsets[own.x] + v] = W.ovf[i];
    }
}

// Exclusive scan of counts[0, n) into offsets (three phases: per-block scan,
// scan of block totals, block offset add).  total[0] = sum.
constexpr int kScanBlock = 1024;

__global__ void scan_block_kernel(const uint32_t* counts, uint32_t* offsets, uint32_t* block_sums, uint32_t n)
{
    __shared__ uint32_t s[kScanBlock];
    const uint32_t i = blockIdx.x * kScanBlock + threadIdx.x;
    const uint32_t v = i < n ? counts[i] : 0u;
    s[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < kScanBlock; o <<= 1) {
        const uint32_t add = threadIdx.x >= (unsigned)o ? s[threadIdx.x - o] : 0u;
        __syncthreads();
        s[threadIdx.x] += add;
        __syncthreads();
    }
    if (i < n) offsets[i] = s[threadIdx.x] - v;
    if (threadIdx.x == kScanBlock - 1) block_sums[blockIdx.x] = s[threadIdx.x];
}

__global__ void scan_totals_kernel(uint32_t* block_sums, uint32_t nb, unsigned long long* total)
{
    __shared__ unsigned long long s[kScanBlock];
    unsigned long long run = 0;
    for (uint32_t base = 0; base < nb; base += kScanBlock) {
        const uint32_t i = base + threadIdx.x;
        const unsigned long long v = i < nb ? block_sums[i] : 0ull;
        s[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < kScanBlock; o <<= 1) {
            const unsigned long long add = threadIdx.x >= (unsigned)o ? s[threadIdx.x - o] : 0ull;
            __syncthreads();
            s[threadIdx.x] += add;
            __syncthreads();
        }
        if (i < nb) block_sums[i] = (uint32_t)(run + s[threadIdx.x] - v);
        const unsigned long long last = s[kScanBlock - 1];
        __syncthreads();
        run += last;
    }
    if (threadIdx.x == 0) *total = run;
}

__global__ void scan_add_kernel(uint32_t* offsets, const uint32_t* block_sums, uint32_t n)
{
    const uint32_t i = blockIdx.x * kScanBlock + threadIdx.x;
    if (i < n) offsets[i] += block_sums[blockIdx.x];
}

}  // namespace

static int walk_blocks(uint32_t paths)
{
    // about 4 paths per thread, at most one wave of resident blocks
    // (threads draw paths from the shared counter until the pool is empty)
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint32_t want = (paths + 4 * 128 - 1) / (4 * 128);
    const uint32_t cap = (uint32_t)sms * kWalkBlocksPerSM;
    return (int)std::max<uint32_t>(1, std::min(want, cap));
}

static int launch_scan(const WalkParams& W, cudaStream_t stream)
{
    const uint32_t nb = (W.paths + kScanBlock - 1) / kScanBlock;
    scan_block_kernel<<<nb, kScanBlock, 0, stream>>>(W.counts, W.offsets, W.block_sums, W.paths);
    scan_totals_kernel<<<1, kScanBlock, 0, stream>>>(W.block_sums, nb, W.total);
    scan_add_kernel<<<nb, kScanBlock, 0, stream>>>(W.offsets, W.block_sums, W.paths);
    return cudaGetLastError() == cudaSuccess ? SSTMC_NO_ERROR : SSTMC_KERNEL_ERROR;
}

// the scene has vMF materials in 3D (their sampler tables are uploaded)
static bool has_vmf(const DevScene& S) { return S.vmf_pf != nullptr; }

template <int MODE>
static void walk_launch(const DevScene& S, const WalkParams& W, int blocks, cudaStream_t stream)
{
    if (S.gauss && S.dims == 3) walk_kernel<MODE, true, true><<<blocks, 128, 0, stream>>>(S, W);
    else if (has_vmf(S)) walk_kernel<MODE, true, false><<<blocks, 128, 0, stream>>>(S, W);
    else walk_kernel<MODE, false, false><<<blocks, 128, 0, stream>>>(S, W);
}

int launch_walk_count(const DevScene& S, const WalkParams& W, cudaStream_t stream)
{
    if (cudaMemsetAsync(W.next, 0, 2 * sizeof(uint32_t), stream) != cudaSuccess) return SSTMC_DEVICE_ERROR;
    if (!(S.gauss && S.dims == 3)) {   // the beam walk places its own first vertices
        if (W.first == nullptr) return SSTMC_MISC_ERROR;
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (W.first_next == nullptr || cudaMemsetAsync(W.first_next, 0, sizeof(uint32_t), stream) != cudaSuccess) return SSTMC_DEVICE_ERROR;
        const uint32_t want = (W.paths + 4 * 128 - 1) / (4 * 128);   // about 4 paths per thread, drawn from the counter
        first_vertex_kernel<<<(int)std::max<uint32_t>(1, std::min(want, (uint32_t)sms * 8)), 128, 0, stream>>>(S, W);
    }
    if (W.slots) {
        if (cudaMemsetAsync(W.list_count, 0, sizeof(uint32_t), stream) != cudaSuccess
            || cudaMemsetAsync(W.ovf_count, 0, sizeof(uint32_t), stream) != cudaSuccess) return SSTMC_DEVICE_ERROR;
        walk_launch<kSlots>(S, W, walk_blocks(W.paths), stream);
    } else {
        walk_launch<kCount>(S, W, walk_blocks(W.paths), stream);
    }
    if (cudaGetLastError() != cudaSuccess) return SSTMC_KERNEL_ERROR_HetroMedium_heterogeneousSampleKernel;
    return launch_scan(W, stream);
}

int launch_walk_compact(const WalkParams& W, cudaStream_t stream)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const size_t total = (size_t)W.paths * kSlotVerts;
    const int blocks = (int)std::min<size_t>((total + 255) / 256, (size_t)sms * 16);
    compact_kernel<<<std::max(1, blocks), 256, 0, stream>>>(W);
    if (W.ovf_n) {
        const size_t ototal = (size_t)W.ovf_n * kSlotVerts;
        const int oblocks = (int)std::min<size_t>((ototal + 255) / 256, (size_t)sms * 16);
        compact_overflow_kernel<<<std::max(1, oblocks), 256, 0, stream>>>(W);
    }
    return cudaGetLastError() == cudaSuccess ? SSTMC_NO_ERROR : SSTMC_KERNEL_ERROR;
}

int launch_walk_write(const DevScene& S, const WalkParams& W, cudaStream_t stream)
{
    WalkParams Wn = W;
    Wn.next = W.next + 1;   // the write pass draws from the second counter (zeroed with the first)
    const uint32_t pool = W.list ? W.list_n : W.paths;
    if (pool == 0) return SSTMC_NO_ERROR;
    walk_launch<kWrite>(S, Wn, walk_blocks(pool), stream);
    return cudaGetLastError() == cudaSuccess ? SSTMC_NO_ERROR : SSTMC_KERNEL_ERROR_HetroMedium_heterogeneousSampleKernel;
}

// Default pool: one overflow block per 16 paths.  Paths longer than a slot
// are rare at a mean of 14 vertices per path (about 1 %); a chunk of long
// paths finds the pool short, and the engine grows it and walks the chunk
// again (the fixed-scratch render replays the overflowing paths in the write
// pass instead; api.cpp, trace_chunk).
uint32_t walk_overflow_blocks(uint32_t paths) { return paths / 16 + 64; }

size_t walk_slot_bytes_per_path()
{
    return kSlotVerts * sizeof(float4) + (kSlotVerts * sizeof(float4) + sizeof(uint2)) / 16 + 1 + sizeof(uint32_t)
         + 2 * sizeof(float4);   // the first-vertex record
}

}  // namespace sstmc
