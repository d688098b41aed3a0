// static_render.cu -- sstmc_render_static: the render of sstmc_render with every
// device buffer carved from one file-scope scratch array instead of cudaMalloc.
//
// The scratch (kStaticScratchBytes per device, part of this library's device
// image) holds, in order: the FP64 accumulator u, the render counters, the
// far-field x far-field single-scattering weight table with its FP64 ticks,
// then one chunk's per-path rows, and the walk's vertices in what is left.
// The chunk starts as large as half the free scratch allows and is halved
// whenever a chunk's vertices do not fit; a path's random streams depend only
// on (seed, path id), so the chunking does not change the result.
//
// What must start at zero, per rendering: u, the counters and the error
// word (cleared with cudaMemsetAsync on the scene's stream).  Everything else
// is written before it is read.
//
// The scratch is one array per device and per process: two calls that
// overlapped would race on it, so a per-device lock is held for the whole
// call.  The device address is looked up once per device with that device
// current (cudaGetSymbolAddress), on the first call for that device.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "sstmc_internal.h"

namespace sstmc {

namespace {

constexpr int kMaxDevices = 64;

__device__ __align__(256) static unsigned char g_scratch[kStaticScratchBytes];

std::mutex g_dev_mu[kMaxDevices];
unsigned char* g_dev_scratch[kMaxDevices] = { nullptr };

// Far-field x far-field single-scattering weight per (material, t, v, l), the
// same quantity as Engine::prepare_ss_tables computes on the host
// (Scattering.cuh:1118-1188 amplitudeKernel<2>; SourceInterface.cuh:221-270
// for the temporal factor of the correlation sampler).
struct SsTableParams {
    int dims, correlation, Nt, Nv, Nl;
    uint32_t present;            // bit m: material m occurs in the grid
    int scat[kMat];
    double g[kMat], D[kMat];
    double k2;
    const double* ticks;         // [Nt]
    const float *il, *vw, *il2, *vw2;
    float* W;                    // [kMat][Nt][Nv][Nl]
};

__device__ double ss_amp(const SsTableParams& P, int m, double c)
{
    if (P.scat[m] == SSTMC_SCATTERING_ISOTROPIC) return P.dims == 2 ? (double)kIsoAmp2 : (double)kIsoAmp3;
    if (P.scat[m] != SSTMC_SCATTERING_HENYEY_GREENSTEIN) return 0.0;
    const double g = P.g[m];
    const double gup = P.dims == 2 ? 2.0 * ((1.0 - g * g) / (4.0 * kPi)) : (1.0 - g * g) / (4.0 * kPi);
    const double dn = fma(-2.0 * g, c, 1.0 + g * g);
    return P.dims == 2 ? sqrt(gup / dn) : sqrt(gup / (dn * sqrt(dn)));
}

__global__ void ss_table_kernel(const __grid_constant__ SsTableParams P)
{
    const size_t per = (size_t)P.Nt * P.Nv * P.Nl;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < per; i += (size_t)gridDim.x * blockDim.x) {
        const int l = (int)(i % P.Nl);
        const int v = (int)((i / P.Nl) % P.Nv);
        const int t = (int)(i / ((size_t)P.Nl * P.Nv));
        double a1[3], a2[3], b1[3], b2[3];
        for (int k = 0; k < 3; ++k) {
            a1[k] = P.il[3 * l + k]; a2[k] = P.il2[3 * l + k];
            b1[k] = P.vw[3 * v + k]; b2[k] = P.vw2[3 * v + k];
        }
        double q2 = 0.0;
        for (int k = 0; k < 3; ++k) { const double qk = 0.5 * (a1[k] + a2[k] - b1[k] - b2[k]); q2 += qk * qk; }
        const double c1 = a1[0] * b1[0] + a1[1] * b1[1] + a1[2] * b1[2];
        const double c2 = a2[0] * b2[0] + a2[1] * b2[1] + a2[2] * b2[2];
        for (int m = 0; m < kMat; ++m) {
            if (!((P.present >> m) & 1u)) continue;
            double w = ss_amp(P, m, c1);
            if (P.correlation) {
                w *= ss_amp(P, m, c2);
                w *= exp(-P.k2 * fabs(P.D[m] * P.ticks[t]) * q2);
            }
            P.W[(size_t)m * per + i] = (float)w;
        }
    }
}

size_t up256(size_t b) { return (b + 255) & ~(size_t)255; }

// Byte layout of the scratch for a chunk of n paths.
struct Layout {
    size_t V, totals, err, vtotal, ticks, W, fixed_end;
    size_t a_ms, s_ms, a_ss, b_ss, g2, pl, x1, x1t, m1, counts, misses, offsets, block_sums, slots, longq, first, ovf, ovf_owner, p2v, rows_end;
    uint32_t ovf_blocks;
};

Layout layout(const Scene& S, bool farfar, uint32_t n)
{
    const size_t Nt = S.Nt, Nl = S.Nl, Nv = S.Nv;
    Layout L;
    size_t o = 0;
    auto take = [&](size_t bytes) { const size_t at = o; o += up256(bytes ? bytes : 1); return at; };
    L.V = take(Nt * Nv * Nl * sizeof(double2));
    L.totals = take(8 * sizeof(unsigned long long));
    L.err = take(sizeof(int));
    L.vtotal = take(32);   // vertex total, the walk's two path counters, long-path and overflow-block counts, the NEE kernels' path counter
    L.ticks = take(farfar ? Nt * sizeof(double) : 0);
    L.W = take(farfar ? (size_t)kMat * Nt * Nv * Nl * sizeof(float) : 0);
    L.fixed_end = o;
    const size_t rows = (S.cfg_copy.is_cbs && !S.correlation) ? 2 * (size_t)n : n;   // field CBS: direct rows, then the reversed path's
    L.a_ms = take(rows * Nt * Nl * sizeof(float2));
    L.s_ms = take(rows * Nt * Nv * sizeof(float2));
    L.a_ss = take(n * Nt * Nl * sizeof(float2));
    L.b_ss = take(n * Nt * Nv * sizeof(float2));
    L.g2 = take(S.correlation ? n * Nt * Nl * sizeof(float2) : 0);
    L.pl = take(n * Nl * sizeof(float));
    L.x1 = take(n * 3 * sizeof(float));
    L.x1t = take(S.correlation ? 0 : n * Nt * 3 * sizeof(float));
    L.m1 = take(n);
    L.counts = take(n * sizeof(uint32_t));
    L.misses = take(n * sizeof(uint32_t));
    L.offsets = take(n * sizeof(uint32_t));
    L.block_sums = take(((n + 1023) / 1024 + 1) * sizeof(uint32_t));
    L.slots = take((size_t)n * kWalkSlotVerts * sizeof(float4));
    L.longq = take(n * sizeof(uint32_t));
    L.first = take((size_t)n * 2 * sizeof(float4));
    L.ovf_blocks = walk_overflow_blocks(n);
    L.ovf = take((size_t)walk_overflow_blocks(n) * kWalkSlotVerts * sizeof(float4));
    L.ovf_owner = take((size_t)walk_overflow_blocks(n) * sizeof(uint2));
    L.p2v = take(n * sizeof(float));
    L.rows_end = o;
    return L;
}

void point_engine(Engine& E, unsigned char* base, const Layout& L)
{
    E.V = reinterpret_cast<double2*>(base + L.V);
    E.totals = reinterpret_cast<unsigned long long*>(base + L.totals);
    E.err = reinterpret_cast<int*>(base + L.err);
    E.vtotal = reinterpret_cast<unsigned long long*>(base + L.vtotal);
    E.a_ms = reinterpret_cast<float2*>(base + L.a_ms);
    E.s_ms = reinterpret_cast<float2*>(base + L.s_ms);
    E.a_ss = reinterpret_cast<float2*>(base + L.a_ss);
    E.b_ss = reinterpret_cast<float2*>(base + L.b_ss);
    E.g2 = reinterpret_cast<float2*>(base + L.g2);
    E.pl = reinterpret_cast<float*>(base + L.pl);
    E.x1 = reinterpret_cast<float*>(base + L.x1);
    E.x1t = reinterpret_cast<float*>(base + L.x1t);
    E.m1 = base + L.m1;
    E.counts = reinterpret_cast<uint32_t*>(base + L.counts);
    E.misses = reinterpret_cast<uint32_t*>(base + L.misses);
    E.offsets = reinterpret_cast<uint32_t*>(base + L.offsets);
    E.block_sums = reinterpret_cast<uint32_t*>(base + L.block_sums);
    E.slots = reinterpret_cast<float4*>(base + L.slots);
    E.longq = reinterpret_cast<uint32_t*>(base + L.longq);
    E.first_v = reinterpret_cast<float4*>(base + L.first);
    E.ovf = reinterpret_cast<float4*>(base + L.ovf);
    E.ovf_owner = reinterpret_cast<uint2*>(base + L.ovf_owner);
    E.ovf_blocks = L.ovf_blocks;   // fixed: a short pool leaves its paths to the replay
    E.p2v = reinterpret_cast<float*>(base + L.p2v);
    E.verts = reinterpret_cast<float4*>(base + L.rows_end);
    E.verts_cap = L.rows_end < kStaticScratchBytes ? (kStaticScratchBytes - L.rows_end) / sizeof(float4) : 0;
}

int scratch_limit(const std::string& what)
{
    set_last_error_text(what + " does not fit the " + std::to_string(kStaticScratchBytes >> 20)
                        + " MiB static scratch of sstmc_render_static: use sstmc_render");
    return SSTMC_SCRATCH_LIMIT;
}

// Look up the scratch's device address for the current device (once per device).
int scratch_base(int dev, unsigned char** out)
{
    if (!g_dev_scratch[dev]) {
        void* p = nullptr;
        const cudaError_t ce = cudaGetSymbolAddress(&p, g_scratch);
        if (ce != cudaSuccess || !p) {
            set_last_error_text(std::string("cudaGetSymbolAddress of the static scratch failed: ") + cudaGetErrorString(ce));
            return SSTMC_DEVICE_ERROR;
        }
        g_dev_scratch[dev] = static_cast<unsigned char*>(p);
    }
    *out = g_dev_scratch[dev];
    return SSTMC_NO_ERROR;
}

int render_one_static(Scene& S, Engine& E, unsigned char* base, bool farfar, uint64_t seed, double* u_out, double* iter_out)
{
    const uint64_t total = (uint64_t)S.P * S.full_iter;
    if (total > 0xffffffffull) return SSTMC_NOT_SUPPORTED;
    const Layout L1 = layout(S, farfar, 1);
    if (L1.rows_end + 64 * sizeof(float4) > kStaticScratchBytes) return scratch_limit("the scene's output and tables");
    // bytes per path of the chunk buffers: the slope between two chunk sizes (the
    // walk's overflow pool has a fixed part of 64 blocks that one path must not be
    // charged for); the first chunk takes half of the room after the fixed part,
    // the vertices the rest
    const size_t per_path = std::max<size_t>(1, (layout(S, farfar, 2048).rows_end - layout(S, farfar, 1024).rows_end) / 1024);
    const size_t room = kStaticScratchBytes - L1.fixed_end;
    uint32_t n = (uint32_t)std::min<uint64_t>(total, std::max<size_t>(1, room / 2 / per_path));
    const size_t nout = (size_t)S.Nt * S.Nv * S.Nl;
    point_engine(E, base, layout(S, farfar, n));
    E.launches = 0;
    if (cudaMemsetAsync(E.V, 0, nout * sizeof(double2), E.stream) != cudaSuccess) return SSTMC_DEVICE_ERROR;
    if (cudaMemsetAsync(E.totals, 0, 8 * sizeof(unsigned long long), E.stream) != cudaSuccess) return SSTMC_DEVICE_ERROR;
    if (cudaMemsetAsync(E.err, 0, sizeof(int), E.stream) != cudaSuccess) return SSTMC_DEVICE_ERROR;
    for (uint64_t first = 0; first < total;) {
        n = (uint32_t)std::min<uint64_t>(n, total - first);
        const Layout L = layout(S, farfar, n);
        if (L.rows_end > kStaticScratchBytes) { n = std::max<uint32_t>(1, n / 2); continue; }
        point_engine(E, base, L);
        int e = E.trace_chunk(S, seed, (uint32_t)first, n, nullptr);
        if (e == SSTMC_SCRATCH_LIMIT) {
            if (n == 1) return scratch_limit("one path's vertices");
            n /= 2;
            continue;
        }
        if (e) return e;
        e = E.contract_chunk(S, n);
        if (e) return e;
        first += n;
    }
    unsigned long long tot[8];
    int herr = 0;
    if (cudaMemcpyAsync(tot, E.totals, sizeof(tot), cudaMemcpyDeviceToHost, E.stream) != cudaSuccess) return SSTMC_DEVICE_ERROR;
    if (cudaMemcpyAsync(&herr, E.err, sizeof(int), cudaMemcpyDeviceToHost, E.stream) != cudaSuccess) return SSTMC_DEVICE_ERROR;
    if (u_out && cudaMemcpyAsync(u_out, E.V, nout * sizeof(double2), cudaMemcpyDeviceToHost, E.stream) != cudaSuccess)
        return SSTMC_DEVICE_ERROR;
    if (cudaStreamSynchronize(E.stream) != cudaSuccess) return SSTMC_KERNEL_ERROR;
    if (herr) return herr;
    if (iter_out) *iter_out = (double)total + (double)tot[2];
    S.last_vertices = tot[0];
    S.last_dda = tot[1];
    S.last_paths = tot[3];
    S.last_contrib = tot[0] * (uint64_t)S.Nl * S.Nv * S.Nt;
    return SSTMC_NO_ERROR;
}

int render_static_locked(Scene& S, cudaStream_t stream, uint64_t seed, double* u_out, double* iter_out)
{
    const int dev = S.device;
    unsigned char* base = nullptr;
    int e = scratch_base(dev, &base);
    if (e) return e;
    const bool farfar = S.hsrc[0].type == SSTMC_SOURCE_FARFIELD && S.hsrc[1].type == SSTMC_SOURCE_FARFIELD && !S.dev.has_amp64;
    Engine E;                  // buffers point into the scratch: never released
    E.stream = stream;
    E.timing = false;
    E.fixed = true;
    if (farfar) {
        const Layout L = layout(S, true, 1);
        if (L.rows_end > kStaticScratchBytes) return scratch_limit("the scene's output and tables");
        SsTableParams P;
        std::memset(&P, 0, sizeof(P));
        P.dims = S.dims; P.correlation = S.correlation ? 1 : 0; P.Nt = S.Nt; P.Nv = S.Nv; P.Nl = S.Nl;
        for (int m : S.materials_present) P.present |= 1u << m;
        for (int m = 0; m < kMat; ++m) { P.scat[m] = S.dev.scat_type[m]; P.g[m] = S.g_d[m]; P.D[m] = S.D_d[m]; }
        const double k = 2.0 * kPi / S.cfg_copy.lambda;
        P.k2 = k * k;
        double* ticks = reinterpret_cast<double*>(base + L.ticks);
        P.ticks = ticks;
        P.il = S.dev.src[0].p; P.vw = S.dev.src[1].p;
        P.il2 = S.correlation ? S.dev.src[2].p : S.dev.src[0].p;
        P.vw2 = S.correlation ? S.dev.src[3].p : S.dev.src[1].p;
        P.W = reinterpret_cast<float*>(base + L.W);
        if (cudaMemcpyAsync(ticks, S.ticks.data(), S.Nt * sizeof(double), cudaMemcpyHostToDevice, stream) != cudaSuccess)
            return SSTMC_DEVICE_ERROR;
        const size_t per = (size_t)S.Nt * S.Nv * S.Nl;
        const int blocks = (int)std::min<size_t>(1024, (per + 255) / 256);
        ss_table_kernel<<<blocks, 256, 0, stream>>>(P);
        if (cudaGetLastError() != cudaSuccess) return SSTMC_KERNEL_ERROR;
        E.W = P.W;
    }
    const size_t nout = (size_t)S.Nt * S.Nv * S.Nl;
    for (uint32_t r = 0; r < S.renders; ++r) {
        e = render_one_static(S, E, base, farfar, seed + r, u_out ? u_out + 2 * nout * r : nullptr,
                              iter_out ? iter_out + r : nullptr);
        if (e) return e;
    }
    return SSTMC_NO_ERROR;
}

}  // namespace

int render_static(Scene& S, cudaStream_t stream, uint64_t seed, double* u_out, double* iter_out)
{
    const int dev = S.device;
    if (dev < 0 || dev >= kMaxDevices) return SSTMC_DEVICE_ERROR;
    std::lock_guard<std::mutex> lk(g_dev_mu[dev]);
    const int e = render_static_locked(S, stream, seed, u_out, iter_out);
    // an error can leave copies and kernels queued on the stream that still use
    // the scratch: they end before the lock lets another call reuse it
    if (e) (void)cudaStreamSynchronize(stream);
    return e;
}

}  // namespace sstmc
