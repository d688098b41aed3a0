// api.cpp -- C-ABI of include/sstmc.h: scene lifetime, render, debug traces.
//
// sstmc_render replaces the rendering loop of mexFunction
// (MatlabInterface.cu:1783-1801): per rendering, trace renderings' paths
// (fullIteration waves of batchSize paths, NextEventEstimation.cuh:1475),
// accumulate u, report iter = batchSize * fullIteration + missed first
// vertices (:1796), then seed + 1 for the next rendering (:1799-1800).
// Paths are processed in chunks of path ids sized to a device-memory budget;
// a path's random stream depends only on (seed, path id), so the chunking is
// invisible in the result.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "contract.h"
#include "scene.h"
#include "sstmc_internal.h"
#include "trace.h"
#include "viewsum.h"

namespace sstmc {

namespace {

int pow2ceil(int n)
{
    int p = 1;
    while (p < n) p <<= 1;
    return p;
}

size_t budget_bytes()
{
    const char* e = std::getenv("SSTMC_CHUNK_BYTES");
    if (e) { const long long v = std::atoll(e); if (v > 0) return (size_t)v; }
    // a quarter of the free device memory, at most 32 GiB
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) return (size_t)2 << 30;
    return std::min<size_t>((size_t)32 << 30, std::max<size_t>((size_t)256 << 20, fr / 4));
}

// The view vectors of the common cases come from the view-side kernel
// (viewsum.cu); SSTMC_VIEW_KERNEL=fused keeps them in the fused trace kernel.
bool use_view_kernel()
{
    const char* e = std::getenv("SSTMC_VIEW_KERNEL");
    return !(e && std::strcmp(e, "fused") == 0);
}

// The split-precision contraction runs on the tensor cores (gemm_tc.cu);
// SSTMC_CONTRACTION=simt selects the SIMT form (gemm_kernel) instead.
// vertices per segment of a long path in the general trace kernel
constexpr uint32_t kSegVerts = 256;

bool use_tensor_cores()
{
    const char* e = std::getenv("SSTMC_CONTRACTION");
    return !(e && std::strcmp(e, "simt") == 0);
}

}  // namespace

size_t Engine::bytes_per_path(const Scene& S)
{
    const size_t Nt = S.Nt, Nl = S.Nl, Nv = S.Nv;
    return 8 * Nt * (2 * Nl + 2 * Nv) + (S.correlation ? 8 * Nt * Nl : 0) + 4 * Nl + 12 + 1 + 12 * Nt + 16
         + ((S.cfg_copy.is_cbs && !S.correlation) ? 8 * Nt * (Nl + Nv) : 0)   // field CBS: the reversed path's rows
         + 4                                                                  // p2 (correlation CBS)
         + 4 + 1                                                              // single-scattering row, partition scratch
         + walk_slot_bytes_per_path();
}

// Freed chunk buffers stay cached in the device's stream-ordered pool (up
// to 96 GiB: three scenes' chunk buffers), so a scene created after another
// one was destroyed, or the next served request, reuses that memory instead
// of mapping it again.
static void keep_pool_memory(int device)
{
    static std::once_flag once[64];
    if (device < 0 || device >= 64) return;
    std::call_once(once[device], [device] {
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, device) != cudaSuccess) return;
        uint64_t keep = 0;
        cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        keep = std::max<uint64_t>(keep, (uint64_t)96 << 30);
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    });
}

int Engine::ensure(Scene& S, uint32_t paths)
{
    if (cap >= paths && a_ms) return SSTMC_NO_ERROR;
    keep_pool_memory(S.device);
    release();
    const size_t Nt = S.Nt, Nl = S.Nl, Nv = S.Nv;
    // stream-ordered: freeing never synchronises the device (requests of a
    // server run concurrently on other streams)
    auto alloc = [&](void** p, size_t bytes) {
        if (cudaMallocAsync(p, bytes ? bytes : 1, stream) != cudaSuccess) return false;
        return true;
    };
    const size_t rows = (S.cfg_copy.is_cbs && !S.correlation) ? 2 * (size_t)paths : paths;   // field CBS: direct rows, then the reversed path's
    bool ok = alloc((void**)&a_ms, rows * Nt * Nl * sizeof(float2)) && alloc((void**)&s_ms, rows * Nt * Nv * sizeof(float2))
           && alloc((void**)&a_ss, paths * Nt * Nl * sizeof(float2)) && alloc((void**)&b_ss, paths * Nt * Nv * sizeof(float2))
           && alloc((void**)&g2, S.correlation ? paths * Nt * Nl * sizeof(float2) : 8)
           && alloc((void**)&pl, paths * Nl * sizeof(float)) && alloc((void**)&x1, paths * 3 * sizeof(float))
           && alloc((void**)&x1t, S.correlation ? 8 : paths * Nt * 3 * sizeof(float))
           && alloc((void**)&m1, paths) && alloc((void**)&totals, 8 * sizeof(unsigned long long))
           && alloc((void**)&err, sizeof(int)) && alloc((void**)&V, Nt * Nv * Nl * sizeof(double2))
           && alloc((void**)&counts, paths * sizeof(uint32_t)) && alloc((void**)&misses, paths * sizeof(uint32_t))
           && alloc((void**)&offsets, paths * sizeof(uint32_t))
           && alloc((void**)&block_sums, ((paths + 1023) / 1024 + 1) * sizeof(uint32_t))
           && alloc((void**)&vtotal, 32)   // vertex total, the walk's two path counters, long-path and overflow-block counts, the NEE kernels' and the first-vertex kernel's path counters
           && alloc((void**)&slots, (size_t)paths * kWalkSlotVerts * sizeof(float4)) && alloc((void**)&longq, paths * sizeof(uint32_t))
           && alloc((void**)&first_v, (size_t)paths * 2 * sizeof(float4))
           && alloc((void**)&ovf, (size_t)std::max(walk_overflow_blocks(paths), ovf_want) * kWalkSlotVerts * sizeof(float4))
           && alloc((void**)&ovf_owner, (size_t)std::max(walk_overflow_blocks(paths), ovf_want) * sizeof(uint2))
           && alloc((void**)&p2v, paths * sizeof(float))
           && alloc((void**)&ss_row, paths * sizeof(uint32_t))
           && alloc((void**)&ss_hist, ((paths + 1023) / 1024) * kMat * sizeof(uint32_t))
           && alloc((void**)&ss_bucket, (kMat + 1) * sizeof(uint32_t));
    if (!ok) { release(); return SSTMC_ALLOCATION_ERROR; }
    ovf_blocks = std::max(walk_overflow_blocks(paths), ovf_want);
    cap = paths;
    return SSTMC_NO_ERROR;
}

void Engine::release()
{
    void* ps[] = { a_ms, s_ms, a_ss, b_ss, g2, pl, x1, x1t, m1, totals, err, V, W, counts, misses, offsets, block_sums, vtotal, verts,
                   slots, longq, first_v, ovf, ovf_owner, p2v, ss_row, ss_hist, ss_bucket, seg_list, seg_ctr };
    for (void* p : ps) if (p) cudaFreeAsync(p, stream);
    counts = misses = offsets = block_sums = nullptr; vtotal = nullptr; verts = nullptr; verts_cap = 0;
    slots = nullptr; longq = nullptr; first_v = nullptr; ovf = nullptr; ovf_owner = nullptr; p2v = nullptr;
    ss_row = ss_hist = ss_bucket = nullptr;
    seg_list = nullptr; seg_cap = 0; seg_ctr = nullptr;
    a_ms = s_ms = a_ss = b_ss = g2 = nullptr;
    pl = x1 = x1t = nullptr;
    m1 = nullptr; totals = nullptr; err = nullptr; V = nullptr; W = nullptr;
    cap = 0;
}

// Far-field x far-field single-scattering weight per (material, t, v, l):
// Scattering.cuh:1118-1188 (amplitudeKernel<2>) for the field sampler; for the
// correlation sampler the u1, u2 amplitudes and the temporal factor of
// SourceInterface.cuh:221-270.
int Engine::prepare_ss_tables(Scene& S)
{
    if (W) return SSTMC_NO_ERROR;
    const DevScene& D = S.dev;
    const int Nt = S.Nt, Nl = S.Nl, Nv = S.Nv;
    const size_t per = (size_t)Nt * Nv * Nl;
    std::vector<float> h(per * kMat, 0.0f);
    const Scene::HostSource& il = S.hsrc[0];
    const Scene::HostSource& vw = S.hsrc[1];
    const Scene::HostSource& il2 = S.correlation ? S.hsrc[2] : S.hsrc[0];
    const Scene::HostSource& vw2 = S.correlation ? S.hsrc[3] : S.hsrc[1];
    const double k2 = (2.0 * kPi / S.cfg_copy.lambda) * (2.0 * kPi / S.cfg_copy.lambda);
    auto amp = [&](int m, double c) -> double {
        if (D.scat_type[m] == SSTMC_SCATTERING_ISOTROPIC) return S.dims == 2 ? kIsoAmp2 : kIsoAmp3;
        if (D.scat_type[m] != SSTMC_SCATTERING_HENYEY_GREENSTEIN) return 0.0;
        const double g = S.g_d[m];
        const double gup = S.dims == 2 ? 2.0 * ((1.0 - g * g) / (4.0 * kPi)) : (1.0 - g * g) / (4.0 * kPi);
        const double dn = std::fma(-2.0 * g, c, 1.0 + g * g);
        return S.dims == 2 ? std::sqrt(gup / dn) : std::sqrt(gup / (dn * std::sqrt(dn)));
    };
    for (int m : S.materials_present) {
        const double Dm = S.D_d[m];
        for (int t = 0; t < Nt; ++t)
            for (int v = 0; v < Nv; ++v)
                for (int l = 0; l < Nl; ++l) {
                    double a1[3], a2[3], b1[3], b2[3];
                    for (int i = 0; i < 3; ++i) {
                        a1[i] = il.p[3 * l + i]; a2[i] = il2.p[3 * l + i];
                        b1[i] = vw.p[3 * v + i]; b2[i] = vw2.p[3 * v + i];
                    }
                    double w = amp(m, a1[0] * b1[0] + a1[1] * b1[1] + a1[2] * b1[2]);
                    if (S.correlation) {
                        w *= amp(m, a2[0] * b2[0] + a2[1] * b2[1] + a2[2] * b2[2]);
                        double q2 = 0;
                        for (int i = 0; i < 3; ++i) { const double qi = 0.5 * (a1[i] + a2[i] - b1[i] - b2[i]); q2 += qi * qi; }
                        w *= std::exp(-k2 * std::fabs(Dm * S.ticks[t]) * q2);
                    }
                    h[m * per + ((size_t)t * Nv + v) * Nl + l] = (float)w;
                }
    }
    if (cudaMallocAsync((void**)&W, h.size() * sizeof(float), stream) != cudaSuccess) { W = nullptr; return SSTMC_ALLOCATION_ERROR; }
    if (cudaMemcpyAsync(W, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice, stream) != cudaSuccess) return SSTMC_ALLOCATION_ERROR;
    if (cudaStreamSynchronize(stream) != cudaSuccess) return SSTMC_DEVICE_ERROR;   // h is freed on return
    return SSTMC_NO_ERROR;
}

// Lane split and chunks of the summed per-vertex vectors over Nx elements
// (views, or illuminations for the CBS reversed pass) and Nt ticks.
static void plan_elems(int Nt, int Nx, TraceParams& T, std::vector<std::pair<int, int>>* xchunks,
                       std::vector<std::pair<int, int>>* tchunks)
{
    const int vw = std::min(32, pow2ceil(Nx));
    const int tg = 32 / vw;
    int tpl = (Nt + tg - 1) / tg;
    if (tpl > kMaxSlots) tpl = kMaxSlots;
    const int tn = std::min(Nt, tpl * tg);
    const int vpl = std::max(1, kMaxSlots / tpl);
    const int vn = std::min(Nx, vpl * vw);
    T.vw = vw; T.tg = tg; T.tpl = tpl;
    T.slots = ((vn + vw - 1) / vw) * tpl;
    xchunks->clear(); tchunks->clear();
    for (int v = 0; v < Nx; v += vn) xchunks->push_back({ v, std::min(vn, Nx - v) });
    for (int t = 0; t < Nt; t += tn) tchunks->push_back({ t, std::min(tn, Nt - t) });
}

void Engine::plan(const Scene& S, TraceParams& T, std::vector<std::pair<int, int>>* vchunks, std::vector<std::pair<int, int>>* tchunks) const
{
    plan_elems(S.Nt, S.Nv, T, vchunks, tchunks);
    T.lw = std::min(32, pow2ceil(S.Nl)); T.lg = 32 / T.lw;
    T.vwa = T.vw; T.tga = T.tg;
}

int Engine::trace_chunk(Scene& S, uint64_t seed, uint32_t first, uint32_t n, PathDebug* dbg)
{
    // 1. random walk: single pass, scan, compaction (pathwalk.cu)
    WalkParams Wp;
    std::memset(&Wp, 0, sizeof(Wp));
    Wp.seed = seed; Wp.first_path = first; Wp.paths = n;
    Wp.counts = counts; Wp.misses = misses; Wp.offsets = offsets; Wp.block_sums = block_sums; Wp.total = vtotal;
    Wp.next = reinterpret_cast<uint32_t*>(vtotal + 1);
    Wp.err = err; Wp.hash = dbg ? dbg->hash : nullptr;
    // single pass: counts, the first 64 vertices of every path (slots) and
    // the rest in overflow blocks; paths that found the pool empty are
    // listed for a replay
    Wp.slots = slots; Wp.list = longq; Wp.list_count = reinterpret_cast<uint32_t*>(vtotal + 2);
    Wp.first = first_v;
    Wp.first_next = reinterpret_cast<uint32_t*>(vtotal) + 7;   // bytes 28..31 of the counter block
    Wp.ovf = ovf; Wp.ovf_owner = ovf_owner; Wp.ovf_count = Wp.list_count + 1; Wp.ovf_cap = ovf_blocks;
    int e = launch_walk_count(S.dev, Wp, stream);
    if (e) return e;
    // the first-vertex kernel (non-beam sources), the walk and the three scan kernels
    const int walk_launches = (S.dev.gauss && S.dims == 3) ? 4 : 5;
    launches += walk_launches;
    unsigned char hv[24];
    if (cudaMemcpyAsync(hv, vtotal, sizeof(hv), cudaMemcpyDeviceToHost, stream) != cudaSuccess) return SSTMC_DEVICE_ERROR;
    if (cudaStreamSynchronize(stream) != cudaSuccess) return SSTMC_KERNEL_ERROR;
    unsigned long long nverts = 0;
    uint32_t nlong = 0;
    std::memcpy(&nverts, hv, 8);
    std::memcpy(&nlong, hv + 16, 4);
    uint32_t novf = 0;
    std::memcpy(&novf, hv + 20, 4);
    if (novf > Wp.ovf_cap && !fixed) {
        // The overflow pool ran short.  Grow it to what the chunk can need (a
        // path of B > 64 vertices takes ceil(B / 64) - 1 blocks, at most
        // B / 64 + 1) and walk the chunk again: a path is a function of (seed,
        // path id), so the second pass repeats the first, and it costs less than
        // replaying the listed paths when many paths are long (a chunk of paths
        // of hundreds of vertices lists most of them).
        const uint64_t want = std::min<uint64_t>(nverts / kWalkSlotVerts + std::min<uint64_t>(n, nverts / (kWalkSlotVerts + 1)) + 64,
                                                 1u << 30);
        cudaFreeAsync(ovf, stream);
        cudaFreeAsync(ovf_owner, stream);
        ovf = nullptr; ovf_owner = nullptr; ovf_blocks = 0;
        if (cudaMallocAsync((void**)&ovf, (size_t)want * kWalkSlotVerts * sizeof(float4), stream) != cudaSuccess
            || cudaMallocAsync((void**)&ovf_owner, (size_t)want * sizeof(uint2), stream) != cudaSuccess)
            return SSTMC_ALLOCATION_ERROR;
        ovf_blocks = (uint32_t)want;
        ovf_want = std::max(ovf_want, (uint32_t)want);
        Wp.ovf = ovf; Wp.ovf_owner = ovf_owner; Wp.ovf_cap = ovf_blocks;
        e = launch_walk_count(S.dev, Wp, stream);
        if (e) return e;
        launches += walk_launches;
        if (cudaMemcpyAsync(hv, vtotal, sizeof(hv), cudaMemcpyDeviceToHost, stream) != cudaSuccess) return SSTMC_DEVICE_ERROR;
        if (cudaStreamSynchronize(stream) != cudaSuccess) return SSTMC_KERNEL_ERROR;
        std::memcpy(&nverts, hv, 8);
        std::memcpy(&nlong, hv + 16, 4);
        std::memcpy(&novf, hv + 20, 4);
    }
    Wp.ovf_n = std::min(novf, Wp.ovf_cap);
    if (nverts > verts_cap) {
        if (fixed) return SSTMC_SCRATCH_LIMIT;
        if (verts) cudaFreeAsync(verts, stream);
        verts = nullptr;
        const size_t cap = (size_t)(nverts * 5 / 4) + 1024;
        if (cudaMallocAsync((void**)&verts, cap * sizeof(float4), stream) != cudaSuccess) { verts_cap = 0; return SSTMC_ALLOCATION_ERROR; }
        verts_cap = cap;
    }
    Wp.verts = verts;
    e = launch_walk_compact(Wp, stream);
    if (e) return e;
    launches += Wp.ovf_n ? 2 : 1;
    if (nlong) {
        Wp.list_n = nlong;
        e = launch_walk_write(S.dev, Wp, stream);
        if (e) return e;
        launches++;
    }
    // The pool ran short (long paths: every path past its slot takes a block per
    // 64 vertices); this chunk was completed by the replay.  Grow the pool for the
    // next chunks and renders: a path of B vertices takes at most ceil(B / 64) - 1
    // blocks, so the chunk's vertex count / 64 plus the default share suffices.
    if (novf > Wp.ovf_cap && !fixed) {
        const uint64_t want = std::min<uint64_t>(nverts / kWalkSlotVerts + walk_overflow_blocks(n), 1u << 30);
        cudaFreeAsync(ovf, stream);
        cudaFreeAsync(ovf_owner, stream);
        ovf = nullptr; ovf_owner = nullptr; ovf_blocks = 0;
        if (cudaMallocAsync((void**)&ovf, (size_t)want * kWalkSlotVerts * sizeof(float4), stream) != cudaSuccess
            || cudaMallocAsync((void**)&ovf_owner, (size_t)want * sizeof(uint2), stream) != cudaSuccess)
            return SSTMC_ALLOCATION_ERROR;
        ovf_blocks = (uint32_t)want;
        ovf_want = std::max(ovf_want, (uint32_t)want);
    }
    // far-field x far-field single scattering on the tensor cores: group the
    // paths' single-scattering rows by first-vertex material, so each material's
    // GEMM reads only its own rows (contract_chunk)
    const bool farfar_tc = S.hsrc[0].type == SSTMC_SOURCE_FARFIELD && S.hsrc[1].type == SSTMC_SOURCE_FARFIELD && !S.dev.has_amp64;
    ss_bucketed = farfar_tc && ss_row && !dbg && !S.cfg_copy.is_cbs && use_tensor_cores() && S.precision == SSTMC_PRECISION_SPLIT
               && S.Nl % 2 == 0 && S.Nv % 2 == 0;
    if (ss_bucketed) {
        SsBucketParams Bp;
        std::memset(&Bp, 0, sizeof(Bp));
        Bp.verts = verts; Bp.counts = counts; Bp.offsets = offsets; Bp.n = n;
        Bp.hist = ss_hist; Bp.ss_row = ss_row; Bp.bucket = ss_bucket;
        e = launch_ss_buckets(Bp, stream);
        if (e) return e;
        launches += 3;
    }
    if (timing && ev[6]) cudaEventRecord(ev[6], stream);

    // 2. NEE vectors per path (trace.cu)
    TraceParams T;
    std::memset(&T, 0, sizeof(T));
    std::vector<std::pair<int, int>> vch, tch;
    plan(S, T, &vch, &tch);
    T.seed = seed; T.first_path = first; T.paths = n;
    T.verts = verts; T.counts = counts; T.offsets = offsets; T.misses = misses;
    T.a_ms = a_ms; T.s_ms = s_ms; T.a_ss = a_ss; T.b_ss = b_ss; T.g2 = g2; T.pl = pl;
    T.x1 = x1; T.x1t = S.correlation ? nullptr : x1t; T.m1 = m1; T.totals = totals; T.err = err;
    T.ss_row = ss_bucketed ? ss_row : nullptr;
    if (dbg) T.dda = dbg->dda;
    if (S.correlation && S.cfg_copy.is_cbs) T.p2 = p2v;   // for the CBS cross terms (contract_chunk)
    rows_real = false;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int threads = 128;
    const size_t smem = trace_smem_bytes(S.Nt, T.slots, threads);
    const int per_sm = occupancy_blocks(S.dev, threads, smem);
    const int blocks = std::max(1, std::min((int)((n + 3) / 4), sms * std::max(1, per_sm)));
    if (S.dev.gauss) {
        // Gaussian beams: every row of a path in one warp (gauss_trace_kernel)
        T.pass0 = 1; T.views = 1;
        T.v0 = 0; T.vn = S.Nv; T.t0 = 0; T.tn = S.Nt;
        e = launch_gauss_trace(S.dev, T, threads, stream);
        if (e) return e;
        launches++;
        return SSTMC_NO_ERROR;
    }
    bool moving_any = false;
    for (int m : S.materials_present) moving_any = moving_any || S.dev.moving[m] != 0;
    if (use_view_kernel() && !S.cfg_copy.is_cbs && view_kernel_covers(S.dev, &moving_any)) {
        // illumination side in the fused kernel (or illum_kernel), view side in viewsum.cu
        T.pass0 = 1; T.views = 0;
        T.v0 = 0; T.vn = S.Nv; T.t0 = 0; T.tn = S.Nt;
        // ss_fast_kernel reads tick 0 of the tick-invariant rows; the far-field x
        // far-field GEMM and the per-path debug trace read every tick
        const bool farfar = S.hsrc[0].type == SSTMC_SOURCE_FARFIELD && S.hsrc[1].type == SSTMC_SOURCE_FARFIELD;
        T.ss_all_ticks = (dbg || farfar) ? 1 : 0;
        T.work = reinterpret_cast<uint32_t*>(vtotal) + 6;   // bytes 24..27 of the counter block
        // correlation rows are real here: with the tensor-core GEMM they are stored as
        // floats (half the bytes); the debug trace reads the complex layout
        rows_real = S.correlation && illum_kernel_covers(S.dev) && use_tensor_cores() && !dbg
                 && S.precision == SSTMC_PRECISION_SPLIT && S.Nt % 2 == 0 && S.Nl % 2 == 0 && S.Nv % 2 == 0;
        T.real_rows = rows_real ? 1 : 0;
        if (illum_kernel_covers(S.dev)) e = launch_illum(S.dev, T, std::max(1, std::min((int)((n + 3) / 4), sms * 16)), threads, stream);
        else e = launch_trace(S.dev, T, blocks, threads, stream);
        if (e) return e;
        launches++;
        const int vmax = view_max_views(S.dev), tmax = view_max_ticks(S.dev);
        const int vblocks = std::max(1, (int)((n + 3) / 4));   // clamped to one resident wave by launch_view
        for (int v = 0; v < S.Nv; v += vmax)
            for (int t = 0; t < S.Nt; t += tmax) {
                T.v0 = v; T.vn = std::min(vmax, S.Nv - v); T.t0 = t; T.tn = std::min(tmax, S.Nt - t);
                e = launch_view(S.dev, T, vblocks, threads, stream);
                if (e) return e;
                launches++;
            }
        return SSTMC_NO_ERROR;
    }
    T.views = 1;
    // paths longer than kSegVerts + 1 vertices are summed in segments of
    // kSegVerts vertices by as many warps (one warp walking a path of thousands
    // of vertices would otherwise bound each launch); not in the static-scratch
    // render, which allocates nothing, nor for CBS's reversed pass
    const bool segmented = !S.cfg_copy.is_cbs && !fixed;
    if (segmented) {
        const size_t want = (size_t)(nverts / kSegVerts) + 1;
        if (want > seg_cap || !seg_ctr) {
            if (seg_list) cudaFreeAsync(seg_list, stream);
            seg_list = nullptr; seg_cap = 0;
            if (!seg_ctr && cudaMallocAsync((void**)&seg_ctr, 2 * sizeof(uint32_t), stream) != cudaSuccess) return SSTMC_ALLOCATION_ERROR;
            const size_t cap = want + want / 4 + 1024;
            if (cudaMallocAsync((void**)&seg_list, cap * sizeof(uint2), stream) != cudaSuccess) return SSTMC_ALLOCATION_ERROR;
            seg_cap = cap;
        }
        e = launch_seg_list(counts, n, kSegVerts, seg_list, (uint32_t)std::min<size_t>(seg_cap, 0xffffffffu), seg_ctr, stream);
        if (e) return e;
        launches++;
        T.seg = kSegVerts; T.seg_list = seg_list; T.seg_len = seg_ctr; T.seg_next = seg_ctr + 1;
    }
    bool first_pass = true;
    for (auto& vc : vch) {
        for (auto& tc : tch) {
            T.pass0 = first_pass ? 1 : 0;
            T.v0 = vc.first; T.vn = vc.second; T.t0 = tc.first; T.tn = tc.second;
            T.seg_mode = 0;
            e = launch_trace(S.dev, T, blocks, threads, stream);
            if (e) return e;
            launches++;
            if (segmented) {
                // the long paths' other segments, added to the rows just written
                TraceParams Sg = T;
                Sg.seg_mode = 1;
                Sg.pass0 = 0;
                if (cudaMemsetAsync(seg_ctr + 1, 0, sizeof(uint32_t), stream) != cudaSuccess) return SSTMC_DEVICE_ERROR;
                e = launch_trace(S.dev, Sg, blocks, threads, stream);
                if (e) return e;
                launches++;
            }
            first_pass = false;
        }
    }
    if (S.cfg_copy.is_cbs && !S.correlation) {
        // field CBS: the reversed path's rows (Gv0 of the views, GlSum of the
        // illuminations) into the second half of the row buffers, rows n .. 2n - 1,
        // so one contraction over 2n rows sums the direct and reversed products
        TraceParams R = T;
        R.cbs = 1; R.views = 1;
        R.a_ms = a_ms + (size_t)n * S.Nt * S.Nl;
        R.s_ms = s_ms + (size_t)n * S.Nt * S.Nv;
        std::vector<std::pair<int, int>> lch, tch2;
        plan_elems(S.Nt, S.Nl, R, &lch, &tch2);
        const size_t smem_r = trace_smem_bytes(S.Nt, R.slots, threads);
        const int per_r = occupancy_blocks(S.dev, threads, smem_r);
        const int blocks_r = std::max(1, std::min((int)((n + 3) / 4), sms * std::max(1, per_r)));
        bool first_r = true;
        for (auto& lc : lch)
            for (auto& tc : tch2) {
                R.pass0 = first_r ? 1 : 0;
                R.v0 = lc.first; R.vn = lc.second; R.t0 = tc.first; R.tn = tc.second;
                e = launch_trace(S.dev, R, blocks_r, threads, stream);
                if (e) return e;
                launches++;
                first_r = false;
            }
    }
    return SSTMC_NO_ERROR;
}

int Engine::contract_chunk(Scene& S, uint32_t n)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const bool compensated = S.precision == SSTMC_PRECISION_SPLIT;
    GemmParams G;
    std::memset(&G, 0, sizeof(G));
    // field CBS: 2n rows (direct, then reversed) and V += (direct + reversed) / sqrt(2);
    // correlation CBS: V += 0.5 (direct + the cross terms of cbs_corr_kernel)
    const bool cbs = S.cfg_copy.is_cbs != 0 && !S.correlation;
    const bool cbs_corr = S.cfg_copy.is_cbs != 0 && S.correlation;
    G.Nt = S.Nt; G.Nl = S.Nl; G.Nv = S.Nv; G.V = V; G.K = (int)(cbs ? 2 * n : n); G.compensated = compensated ? 1 : 0;
    G.scale = cbs ? std::sqrt(0.5) : (cbs_corr ? 0.5 : 1.0);
    const int tiles = ((S.Nl + 31) / 32) * ((S.Nv + 31) / 32) * S.Nt;
    const int ksplit = std::max(1, (4 * sms + tiles - 1) / tiles);
    int kchunk = (int)((G.K + ksplit - 1) / ksplit);
    kchunk = ((kchunk + 255) / 256) * 256;
    G.kchunk = kchunk;
    G.A = a_ms; G.B = s_ms;
    G.err = err;
    G.real = rows_real ? 1 : 0;
    const bool tc = use_tensor_cores() && gemm_tc_eligible(G);
    if (G.real && !tc) return SSTMC_MISC_ERROR;   // real rows are written only for the tensor-core form
    auto gemm = [&](const GemmParams& P) { return tc ? launch_gemm_tc(P, stream) : launch_gemm(P, stream); };
    int e = gemm(G);
    if (e) return e;
    launches++;
    if (timing) cudaEventRecord(ev[3], stream);
    // far-field x far-field: per-material weight tables on the tensor-core GEMM
    // (HG / isotropic amplitudes; tabular and vMF ones come from an FP64 angle in ss_kernel)
    const bool farfar = S.hsrc[0].type == SSTMC_SOURCE_FARFIELD && S.hsrc[1].type == SSTMC_SOURCE_FARFIELD && !S.dev.has_amp64;
    if (farfar) {
        e = prepare_ss_tables(S);
        if (e) return e;
        const size_t per = (size_t)S.Nt * S.Nv * S.Nl;
        G.A = a_ss; G.B = b_ss; G.mat = m1; G.real = 0; G.K = (int)n; G.scale = 1.0;
        if (ss_bucketed && !tc) return SSTMC_MISC_ERROR;   // grouped rows are written only for the tensor-core form
        if (ss_bucketed) {
            // rows grouped by material: one launch, each material's GEMM over its own rows
            G.mat = nullptr;
            G.bucket = ss_bucket;
            G.W = W;
            G.wstride = per;
            G.nmat = 0;
            for (int m : S.materials_present) G.mats[G.nmat++] = m;
            e = gemm(G);
            if (e) return e;
            launches++;
        } else {
            for (int m : S.materials_present) {
                G.mat_sel = m;
                G.W = W + (size_t)m * per;
                e = gemm(G);
                if (e) return e;
                launches++;
            }
        }
    } else {
        SsParams P;
        std::memset(&P, 0, sizeof(P));
        P.a = a_ss; P.b = b_ss; P.x1 = x1; P.x1t = x1t; P.m1 = m1; P.K = (int)n; P.V = V;
        P.compensated = compensated ? 1 : 0;
        const int stiles = ((S.Nl + 15) / 16) * ((S.Nv + 15) / 16) * ((S.Nt + 7) / 8);
        const int ks = std::max(1, (4 * sms + stiles - 1) / stiles);
        int kc = (int)((n + ks - 1) / ks);
        kc = ((kc + 255) / 256) * 256;
        P.kchunk = kc;
        e = launch_ss(S.dev, P, stream);
        if (e) return e;
        launches++;
    }
    if (cbs_corr) {
        CbsCorrParams C;
        std::memset(&C, 0, sizeof(C));
        C.verts = verts; C.counts = counts; C.offsets = offsets; C.p2 = p2v; C.V = V; C.K = (int)n;
        e = launch_cbs_corr(S.dev, C, stream);
        if (e) return e;
        launches++;
    }
    return SSTMC_NO_ERROR;
}

int Engine::render_one(Scene& S, uint64_t seed, double* u_out, double* iter_out, uint64_t limit)
{
    const uint64_t all = (uint64_t)S.P * S.full_iter;
    if (all > 0xffffffffull) return SSTMC_NOT_SUPPORTED;
    const uint64_t total = limit ? std::min(limit, all) : all;
    const size_t bud = budget ? budget : budget_bytes();
    uint64_t fit = std::max<uint64_t>(256, bud / bytes_per_path(S));
    if (tuned_chunk) fit = std::min<uint64_t>(fit, tuned_chunk);   // the autotuner's wavefront, within the budget
    uint32_t chunk = (uint32_t)std::min<uint64_t>(total, fit);
    chunk = std::max<uint32_t>(32, chunk);
    int e = ensure(S, chunk);
    if (e) return e;
    const size_t nout = (size_t)S.Nt * S.Nv * S.Nl;
    if (timing && init_events()) timing = false;
    launches = 0;
    if (cudaMemsetAsync(V, 0, nout * sizeof(double2), stream) != cudaSuccess) return SSTMC_DEVICE_ERROR;
    if (cudaMemsetAsync(totals, 0, 8 * sizeof(unsigned long long), stream) != cudaSuccess) return SSTMC_DEVICE_ERROR;
    if (cudaMemsetAsync(err, 0, sizeof(int), stream) != cudaSuccess) return SSTMC_DEVICE_ERROR;
    std::vector<float> t_trace, t_gemm, t_ss, t_walk;
    float t_all = 0.f;
    chunks = 0;
    if (timing) cudaEventRecord(ev[0], stream);
    for (uint64_t first = 0; first < total; first += chunk) {
        const uint32_t n = (uint32_t)std::min<uint64_t>(chunk, total - first);
        if (timing) cudaEventRecord(ev[1], stream);
        e = trace_chunk(S, seed, (uint32_t)first, n, nullptr);
        if (e) return e;
        if (timing) cudaEventRecord(ev[2], stream);
        e = contract_chunk(S, n);
        if (e) return e;
        chunks++;
        if (timing) {
            cudaEventRecord(ev[4], stream);
            cudaEventSynchronize(ev[4]);
            float a = 0, b = 0, c = 0, w = 0;
            cudaEventElapsedTime(&a, ev[1], ev[2]);
            cudaEventElapsedTime(&b, ev[2], ev[3]);
            cudaEventElapsedTime(&c, ev[3], ev[4]);
            cudaEventElapsedTime(&w, ev[1], ev[6]);
            t_trace.push_back(a); t_gemm.push_back(b); t_ss.push_back(c); t_walk.push_back(w);
        }
    }
    if (timing) {
        cudaEventRecord(ev[5], stream);
        cudaEventSynchronize(ev[5]);
        cudaEventElapsedTime(&t_all, ev[0], ev[5]);
        ms_trace = ms_gemm = ms_ss = ms_walk = 0;
        for (size_t i = 0; i < t_trace.size(); ++i) {
            ms_trace += t_trace[i]; ms_gemm += t_gemm[i]; ms_ss += t_ss[i]; ms_walk += t_walk[i];
        }
        ms_total = t_all;
    }
    unsigned long long tot[8];
    int herr = 0;
    if (cudaMemcpyAsync(tot, totals, sizeof(tot), cudaMemcpyDeviceToHost, stream) != cudaSuccess) return SSTMC_DEVICE_ERROR;
    if (cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, stream) != cudaSuccess) return SSTMC_DEVICE_ERROR;
    if (u_out && cudaMemcpyAsync(u_out, V, nout * sizeof(double2), cudaMemcpyDeviceToHost, stream) != cudaSuccess)
        return SSTMC_DEVICE_ERROR;
    if (cudaStreamSynchronize(stream) != cudaSuccess) return SSTMC_KERNEL_ERROR;
    if (herr) return herr;
    if (iter_out) *iter_out = (double)total + (double)tot[2];   // iter = batchSize * fullIteration + missed first vertices
    S.last_vertices = tot[0];
    S.last_dda = tot[1];
    S.last_paths = tot[3];
    S.last_contrib = tot[0] * (uint64_t)S.Nl * S.Nv * S.Nt;
    return SSTMC_NO_ERROR;
}

int Engine::init_events()
{
    if (ev[0]) return 0;
    for (auto& e : ev)
        if (cudaEventCreate(&e) != cudaSuccess) return 1;
    return 0;
}

void Engine::destroy_events()
{
    for (auto& e : ev) { if (e) cudaEventDestroy(e); e = nullptr; }
}

}  // namespace sstmc

using namespace sstmc;

struct sstmc_scene {
    Scene scene;
    Engine engine;
    std::mutex mu;
};

namespace sstmc {

// Every rendering of the scene's config (seed, seed + 1, ...), holding the
// scene's lock.  budget: device bytes for the chunk buffers (0: the default);
// release_after: return them to the stream-ordered pool afterwards (served
// requests, whose reservation ends with the request).
int32_t render_scene(sstmc_scene* s, uint64_t seed, double* u_out, double* iter_out, size_t budget, bool release_after,
                     uint64_t* contributions)
{
    std::lock_guard<std::mutex> lk(s->mu);
    if (cudaSetDevice(s->scene.device) != cudaSuccess) return SSTMC_DEVICE_ERROR;
    const size_t nout = (size_t)s->scene.Nt * s->scene.Nv * s->scene.Nl;
    if (budget && budget != s->engine.budget) s->engine.release();
    s->engine.budget = budget;
    uint64_t contrib = 0;
    int e = SSTMC_NO_ERROR;
    for (uint32_t r = 0; r < s->scene.renders && !e; ++r) {
        e = s->engine.render_one(s->scene, seed + r, u_out ? u_out + 2 * nout * r : nullptr, iter_out ? iter_out + r : nullptr);
        contrib += s->scene.last_contrib;
    }
    if (release_after) {
        s->engine.release();
        if (cudaStreamSynchronize(s->engine.stream) != cudaSuccess && !e) e = SSTMC_DEVICE_ERROR;
    }
    if (contributions) *contributions = contrib;
    return e;
}

// Device bytes a served render of the scene reserves with chunk buffers
// sized to at most cap bytes: the per-path rows of one chunk, its vertices
// (32 per path assumed) and the output accumulator.
size_t scene_request_bytes(const sstmc_scene* s, size_t cap)
{
    const Scene& S = s->scene;
    const uint64_t total = (uint64_t)S.P * S.full_iter;
    const size_t bpp = Engine::bytes_per_path(S) + 32 * sizeof(float4);
    const uint64_t chunk = std::min<uint64_t>(total, std::max<uint64_t>(256, cap / bpp));
    return (size_t)chunk * bpp + (size_t)S.Nt * S.Nv * S.Nl * 16 + ((size_t)1 << 20);
}

int scene_device(const sstmc_scene* s) { return s->scene.device; }

}  // namespace sstmc

extern "C" {

void sstmc_config_init(sstmc_config* cfg)
{
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->dims = 3;
    cfg->batch_size = 1024;
    cfg->full_iteration = 1;
    cfg->renderings_num = 1;
    cfg->lambda = 1.0;
    cfg->is_temporal_amplitude = 1;
    cfg->precision = SSTMC_PRECISION_SPLIT;
}

int32_t sstmc_scene_create(const sstmc_config* cfg, sstmc_scene** out)
{
    if (!cfg || !out) return SSTMC_INVALID_HANDLE;
    *out = nullptr;
    sstmc_scene* s = new (std::nothrow) sstmc_scene();
    if (!s) return SSTMC_ALLOCATION_ERROR;
    std::string why;
    int e = build_scene(cfg, &s->scene, &why);
    if (!e && cudaStreamCreateWithFlags(&s->engine.stream, cudaStreamNonBlocking) != cudaSuccess) e = SSTMC_DEVICE_ERROR;
    if (e) {
        set_last_error_text(why);
        delete s;
        return e;
    }
    *out = s;
    return SSTMC_NO_ERROR;
}

int32_t sstmc_scene_shape(const sstmc_scene* s, uint32_t* nl, uint32_t* nv, uint32_t* nt)
{
    if (!s) return SSTMC_INVALID_HANDLE;
    if (nl) *nl = (uint32_t)s->scene.Nl;
    if (nv) *nv = (uint32_t)s->scene.Nv;
    if (nt) *nt = (uint32_t)s->scene.Nt;
    return SSTMC_NO_ERROR;
}

int32_t sstmc_render(sstmc_scene* s, uint64_t seed, double* u_out, double* iter_out)
{
    return s ? render_scene(s, seed, u_out, iter_out, 0, false, nullptr) : SSTMC_INVALID_HANDLE;
}

int32_t sstmc_scene_autotune(sstmc_scene* s, uint32_t sample_paths, uint64_t* chunk_paths)
{
    if (!s) return SSTMC_INVALID_HANDLE;
    std::lock_guard<std::mutex> lk(s->mu);
    Scene& S = s->scene;
    Engine& E = s->engine;
    if (cudaSetDevice(S.device) != cudaSuccess) return SSTMC_DEVICE_ERROR;
    const uint64_t total = (uint64_t)S.P * S.full_iter;
    const uint64_t sample = std::min<uint64_t>(total, std::max<uint32_t>(sample_paths, 1u << 12));
    const uint64_t fit = std::max<uint64_t>(256, budget_bytes() / Engine::bytes_per_path(S));
    const bool timing = E.timing;
    E.timing = true;
    E.budget = 0;
    double best = 0.0;
    uint32_t best_chunk = 0;
    int e = SSTMC_NO_ERROR;
    // candidate wavefronts: powers of two from 2^12 paths up to the sample and the memory budget
    for (uint64_t c = 1u << 12; !e; c <<= 1) {
        const uint64_t chunk = std::min(std::min(c, sample), fit);
        E.release();
        E.tuned_chunk = (uint32_t)chunk;
        double ms = 0.0;
        for (int rep = 0; rep < 2 && !e; ++rep) {   // the first render at a size grows the pools
            e = E.render_one(S, 1, nullptr, nullptr, sample);
            ms = E.ms_total;
        }
        if (!e && ms > 0.0) {
            const double rate = (double)sample / ms;
            if (rate > 1.02 * best) { best = rate; best_chunk = (uint32_t)chunk; }
        }
        if (chunk >= sample || chunk >= fit) break;
    }
    E.release();
    E.timing = timing;
    E.tuned_chunk = e ? 0u : best_chunk;
    if (chunk_paths) *chunk_paths = E.tuned_chunk;
    return e;
}

int32_t sstmc_render_static(sstmc_scene* s, uint64_t seed, double* u_out, double* iter_out)
{
    if (!s) return SSTMC_INVALID_HANDLE;
    std::lock_guard<std::mutex> lk(s->mu);
    if (cudaSetDevice(s->scene.device) != cudaSuccess) return SSTMC_DEVICE_ERROR;
    return render_static(s->scene, s->engine.stream, seed, u_out, iter_out);
}

int32_t sstmc_last_stats(const sstmc_scene* s, uint64_t* contributions, uint64_t* dda_steps, uint64_t* vertices, uint64_t* paths)
{
    if (!s) return SSTMC_INVALID_HANDLE;
    if (contributions) *contributions = s->scene.last_contrib;
    if (dda_steps) *dda_steps = s->scene.last_dda;
    if (vertices) *vertices = s->scene.last_vertices;
    if (paths) *paths = s->scene.last_paths;
    return SSTMC_NO_ERROR;
}

int32_t sstmc_last_timing(const sstmc_scene* s, double* ms, uint64_t* launches)
{
    if (!s) return SSTMC_INVALID_HANDLE;
    if (ms) {
        ms[0] = s->engine.ms_total; ms[1] = s->engine.ms_trace;
        ms[2] = s->engine.ms_gemm; ms[3] = s->engine.ms_ss;
        ms[4] = s->engine.ms_walk; ms[5] = s->engine.ms_trace - s->engine.ms_walk;
    }
    if (launches) { launches[0] = s->engine.launches; launches[1] = s->engine.chunks; }
    return SSTMC_NO_ERROR;
}

int32_t sstmc_scene_destroy(sstmc_scene* s)
{
    if (!s) return SSTMC_INVALID_HANDLE;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        cudaSetDevice(s->scene.device);
        if (s->engine.stream) cudaStreamSynchronize(s->engine.stream);
        s->engine.release();
        s->engine.destroy_events();
        if (s->engine.stream) cudaStreamDestroy(s->engine.stream);
        s->engine.stream = nullptr;
    }
    delete s;
    return SSTMC_NO_ERROR;
}

int32_t sstmc_trace_paths(sstmc_scene* s, uint64_t seed, uint32_t first_path, uint32_t paths, sstmc_path_trace* out)
{
    if (!s || !out) return SSTMC_INVALID_HANDLE;
    if (paths == 0) return SSTMC_NO_ERROR;
    std::lock_guard<std::mutex> lk(s->mu);
    Scene& S = s->scene;
    Engine& E = s->engine;
    if (cudaSetDevice(S.device) != cudaSuccess) return SSTMC_DEVICE_ERROR;
    int e = E.ensure(S, paths);
    if (e) return e;
    PathDebug dbg;
    if (cudaMalloc((void**)&dbg.hash, paths * sizeof(uint32_t)) != cudaSuccess) return SSTMC_ALLOCATION_ERROR;
    if (cudaMalloc((void**)&dbg.dda, paths * sizeof(uint32_t)) != cudaSuccess) { cudaFree(dbg.hash); return SSTMC_ALLOCATION_ERROR; }
    cudaMemsetAsync(dbg.dda, 0, paths * sizeof(uint32_t), E.stream);
    cudaMemsetAsync(E.totals, 0, 8 * sizeof(unsigned long long), E.stream);
    cudaMemsetAsync(E.err, 0, sizeof(int), E.stream);
    e = E.trace_chunk(S, seed, first_path, paths, &dbg);
    int herr = 0;
    if (!e) {
        cudaMemcpyAsync(&herr, E.err, sizeof(int), cudaMemcpyDeviceToHost, E.stream);
        if (cudaStreamSynchronize(E.stream) != cudaSuccess) e = SSTMC_KERNEL_ERROR;
    }
    if (!e && herr) e = herr;
    if (!e) {
        const size_t Nt = S.Nt, Nl = S.Nl, Nv = S.Nv;
        if (out->misses) cudaMemcpy(out->misses, E.misses, paths * sizeof(int), cudaMemcpyDeviceToHost);
        if (out->vertices) cudaMemcpy(out->vertices, E.counts, paths * sizeof(int), cudaMemcpyDeviceToHost);
        if (out->vertex_hash) cudaMemcpy(out->vertex_hash, dbg.hash, paths * sizeof(uint32_t), cudaMemcpyDeviceToHost);
        if (out->dda_steps) cudaMemcpy(out->dda_steps, dbg.dda, paths * sizeof(uint32_t), cudaMemcpyDeviceToHost);
        if (out->x1) cudaMemcpy(out->x1, E.x1, paths * 3 * sizeof(float), cudaMemcpyDeviceToHost);
        if (out->m1) {
            std::vector<unsigned char> m(paths);
            cudaMemcpy(m.data(), E.m1, paths, cudaMemcpyDeviceToHost);
            for (uint32_t i = 0; i < paths; ++i) out->m1[i] = m[i];
        }
        auto copy_c = [&](double* dst, const float2* src, size_t n) {
            if (!dst) return;
            std::vector<float2> h(n);
            cudaMemcpy(h.data(), src, n * sizeof(float2), cudaMemcpyDeviceToHost);
            for (size_t i = 0; i < n; ++i) { dst[2 * i] = h[i].x; dst[2 * i + 1] = h[i].y; }
        };
        copy_c(out->a_ms, E.a_ms, paths * Nt * Nl);
        copy_c(out->s_ms, E.s_ms, paths * Nt * Nv);
        copy_c(out->a_ss, E.a_ss, paths * Nt * Nl);
        copy_c(out->b_ss, E.b_ss, paths * Nt * Nv);
    }
    cudaFree(dbg.hash); cudaFree(dbg.dda);
    return e;
}

}  // extern "C"
