// refharness.cu -- runs the reference's own CUDA path (chabner/temporalSpecklesCode)
// without MATLAB: test and measurement infrastructure, never part of the library.
//
// It builds the reference's objects from a scene file in the order mexFunction
// builds them (MatlabInterface.cu:1677-1700): Simulation -> Scattering ->
// HeterogeneousMedium + setMaterial -> PointSource / FarField / GaussianBeam (illumination,
// view, and for the correlation sampler illumination2 / view2) ->
// TemporalSampler / TemporalCorrelationSampler + setMaterial ->
// NextEventEstimation, then renders `renderings` times with the seed
// incremented between renderings (:1783-1801), and writes per rendering u
// (Nl x Nv x Nt complex, Nl fastest), iter = batch * fullIteration +
// zeroContributionPaths (:1796) and the device time of the trace.
//
// Compiled against the reference's headers, staged (never committed) under
// oracle/_ref/src by oracle/stage_reference.sh, with oracle/refharness.mk:
// one binary per DIMS (the reference fixes DIMS at compile time).
//
// Scene file: whitespace-separated tokens, written by tests/refharness_lib.py:
//   batch B  full_iteration F  renderings R  seed S  lambda L
//   scattering n  then n x (kind g), kind 0 isotropic / 3 Henyey-Greenstein,
//                 or (4 k mu_1..mu_k c_1..c_k alpha_1..alpha_k) for a vMF mixture
//   axis a n v_0 .. v_{n-1}    (a = 0, 1, 2)
//   grid n m_0 .. m_{n-1}      (x fastest)
//   materials n  then n x (sigs siga)
//   source role type count xyz...   (role 0..3, type 1 point / 2 far field)
//   source role 3 count xyz... dir... aperture   (a Gaussian beam per focal point)
//   sampler type                    (0 temporal, 1 correlation)
//   ticks n t_0 .. t_{n-1}
//   motion n  then n x (D ux uy uz)
//   cbs c                           (optional: 1 renders with coherent backscattering)
//   end
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "Simulation.cuh"
#include "Implementation/Tracer/NextEventEstimation.cuh"
#include "Implementation/Scattering.cuh"
#include "Implementation/Medium/HeterogeneousMedium.cuh"
#include "Implementation/Sampler/TemporalSampler.cuh"
#include "Implementation/Sampler/TemporalSamplerCorrelation.cuh"
#include "Implementation/Source/PointSource.cuh"
#include "Implementation/Source/FarField.cuh"
#include "Implementation/Source/GaussianBeam.cuh"

namespace {

struct SceneFile {
    ub32 batch = 1024, full_iteration = 1, renderings = 1;
    ub64 seed = 0;
    double lambda = 1.0;
    std::vector<int> scat_kind;
    std::vector<double> scat_g;
    std::vector<std::vector<double>> vmf_mu, vmf_c, vmf_alpha;
    std::vector<double> axis[3];
    std::vector<ub32> grid;
    std::vector<double> sigs, siga;
    int src_type[4] = { 0, 0, 0, 0 };
    std::vector<double> src_xyz[4];
    std::vector<double> src_dir[4];
    double aperture[4] = { 0, 0, 0, 0 };
    int sampler = 0;
    std::vector<double> ticks;
    std::vector<double> D, U;
    int cbs = 0;
};

bool read_scene(const char* path, SceneFile* s)
{
    std::ifstream in(path);
    if (!in) return false;
    std::string key;
    while (in >> key) {
        if (key == "batch") in >> s->batch;
        else if (key == "full_iteration") in >> s->full_iteration;
        else if (key == "renderings") in >> s->renderings;
        else if (key == "seed") in >> s->seed;
        else if (key == "lambda") in >> s->lambda;
        else if (key == "scattering") {
            size_t n; in >> n;
            s->scat_kind.resize(n); s->scat_g.resize(n);
            s->vmf_mu.resize(n); s->vmf_c.resize(n); s->vmf_alpha.resize(n);
            for (size_t i = 0; i < n; ++i) {
                in >> s->scat_kind[i];
                if (s->scat_kind[i] != 4) { in >> s->scat_g[i]; continue; }
                size_t k; in >> k;
                for (auto* v : { &s->vmf_mu[i], &s->vmf_c[i], &s->vmf_alpha[i] }) {
                    v->resize(k);
                    for (auto& x : *v) in >> x;
                }
            }
        } else if (key == "axis") {
            int a; size_t n; in >> a >> n;
            s->axis[a].resize(n);
            for (auto& v : s->axis[a]) in >> v;
        } else if (key == "grid") {
            size_t n; in >> n;
            s->grid.resize(n);
            for (auto& v : s->grid) in >> v;
        } else if (key == "materials") {
            size_t n; in >> n;
            s->sigs.resize(n); s->siga.resize(n);
            for (size_t i = 0; i < n; ++i) in >> s->sigs[i] >> s->siga[i];
        } else if (key == "source") {
            int role, type; size_t n; in >> role >> type >> n;
            s->src_type[role] = type;
            s->src_xyz[role].resize(3 * n);
            for (auto& v : s->src_xyz[role]) in >> v;
            if (type == 3) {
                s->src_dir[role].resize(3 * n);
                for (auto& v : s->src_dir[role]) in >> v;
                in >> s->aperture[role];
            }
        } else if (key == "sampler") in >> s->sampler;
        else if (key == "ticks") {
            size_t n; in >> n;
            s->ticks.resize(n);
            for (auto& v : s->ticks) in >> v;
        } else if (key == "motion") {
            size_t n; in >> n;
            s->D.resize(n); s->U.resize(3 * n);
            for (size_t i = 0; i < n; ++i) in >> s->D[i] >> s->U[3 * i] >> s->U[3 * i + 1] >> s->U[3 * i + 2];
        } else if (key == "cbs") in >> s->cbs;
        else if (key == "end") return true;
        else { std::fprintf(stderr, "unknown key %s\n", key.c_str()); return false; }
        if (!in) return false;
    }
    return false;
}

#define CHECK(what) do { if (err != ErrorType::NO_ERROR) { std::fprintf(stderr, "%s failed: error %d\n", what, (int)err); return 3; } } while (0)

}  // namespace

int main(int argc, char** argv)
{
    if (argc != 3) { std::fprintf(stderr, "usage: %s <scene file> <output file>\n", argv[0]); return 2; }
    SceneFile sc;
    if (!read_scene(argv[1], &sc)) { std::fprintf(stderr, "cannot read scene %s\n", argv[1]); return 2; }
    ErrorType err = ErrorType::NO_ERROR;
    const float_type lambda = sc.lambda;
    Simulation* simulation = new Simulation(&err, sc.batch, &lambda, 1, 0);
    CHECK("Simulation");
    Scattering* scattering = new Scattering();
    for (size_t m = 0; m < sc.scat_kind.size(); ++m) {
        if (sc.scat_kind[m] == 4) {
            std::vector<float_type> mu(sc.vmf_mu[m].begin(), sc.vmf_mu[m].end()), c(sc.vmf_c[m].begin(), sc.vmf_c[m].end()),
                alpha(sc.vmf_alpha[m].begin(), sc.vmf_alpha[m].end());
            err = scattering->setVonMisesFisherScattering(mu.data(), c.data(), alpha.data(), (ub32)mu.size(), (ub32)m);
        } else {
            err = sc.scat_kind[m] == 3 ? scattering->setHenyeyGreensteinScattering(sc.scat_g[m], (ub32)m)
                                       : scattering->setIsotropicScattering((ub32)m);
        }
        CHECK("Scattering");
    }
    HeterogeneousMedium* medium = new HeterogeneousMedium(&err, sc.grid.data(), sc.axis[0].data(), (ub32)sc.axis[0].size(),
                                                          sc.axis[1].data(), (ub32)sc.axis[1].size()
#if DIMS==3
                                                          , sc.axis[2].data(), (ub32)sc.axis[2].size()
#endif
    );
    CHECK("HeterogeneousMedium");
    for (size_t m = 0; m < sc.sigs.size(); ++m) {
        MediumMaterial mat;
        mat.sigs = sc.sigs[m];
        mat.siga = sc.siga[m];
        err = medium->setMaterial(&mat, (ub32)m);
        CHECK("setMaterial");
    }
    const ConnectionType roles[4] = { ConnectionType::ConnectionTypeIllumination, ConnectionType::ConnectionTypeView,
                                      ConnectionType::ConnectionTypeIllumination2, ConnectionType::ConnectionTypeView2 };
    Source* src[4] = { nullptr, nullptr, nullptr, nullptr };
    for (int r = 0; r < 4; ++r) {
        if (!sc.src_type[r]) continue;
        const ub32 n = (ub32)(sc.src_xyz[r].size() / 3);
        std::vector<VectorType> v(n), dir(n);
        for (ub32 i = 0; i < n; ++i) {
#if DIMS==3
            v[i] = VectorType(sc.src_xyz[r][3 * i], sc.src_xyz[r][3 * i + 1], sc.src_xyz[r][3 * i + 2]);
            if (sc.src_type[r] == 3) dir[i] = VectorType(sc.src_dir[r][3 * i], sc.src_dir[r][3 * i + 1], sc.src_dir[r][3 * i + 2]);
#else
            v[i] = VectorType(sc.src_xyz[r][3 * i], sc.src_xyz[r][3 * i + 1]);
            if (sc.src_type[r] == 3) dir[i] = VectorType(sc.src_dir[r][3 * i], sc.src_dir[r][3 * i + 1]);
#endif
        }
        if (sc.src_type[r] == 3) src[r] = new GaussianBeam(&err, simulation, medium, scattering, v.data(), dir.data(), sc.aperture[r], n, roles[r]);
        else if (sc.src_type[r] == 1) src[r] = new PointSource(&err, simulation, medium, scattering, v.data(), n, false, roles[r]);
        else src[r] = new FarField(&err, simulation, medium, scattering, v.data(), n, roles[r]);
        CHECK("Source");
    }
    Sampler* sampler = nullptr;
    if (sc.sampler == 1) {
        TemporalCorrelationSampler* s = new TemporalCorrelationSampler(&err, src[0], src[2], src[1], src[3], simulation, medium,
                                                                       scattering, sc.ticks.data(), (ub32)sc.ticks.size());
        CHECK("TemporalCorrelationSampler");
        for (size_t m = 0; m < sc.D.size(); ++m) {
#if DIMS==3
            err = s->setMaterial(sc.D[m], VectorType(sc.U[3 * m], sc.U[3 * m + 1], sc.U[3 * m + 2]), (ub32)m);
#else
            err = s->setMaterial(sc.D[m], VectorType(sc.U[3 * m], sc.U[3 * m + 1]), (ub32)m);
#endif
            CHECK("sampler setMaterial");
        }
        sampler = s;
    } else {
        TemporalSampler* s = new TemporalSampler(&err, src[0], src[1], simulation, medium, scattering, sc.ticks.data(),
                                                 (ub32)sc.ticks.size(), true, false);
        CHECK("TemporalSampler");
        for (size_t m = 0; m < sc.D.size(); ++m) {
#if DIMS==3
            err = s->setMaterial(sc.D[m], VectorType(sc.U[3 * m], sc.U[3 * m + 1], sc.U[3 * m + 2]), (ub32)m);
#else
            err = s->setMaterial(sc.D[m], VectorType(sc.U[3 * m], sc.U[3 * m + 1]), (ub32)m);
#endif
            CHECK("sampler setMaterial");
        }
        sampler = s;
    }
    NextEventEstimationOptions options;
    options.fullIterationsNumber = sc.full_iteration;
    options.seed = sc.seed;
    options.isCBS = sc.cbs != 0;
    NextEventEstimation* tracer = new NextEventEstimation(&err, sampler, &options);
    CHECK("NextEventEstimation");
    const ub32 Nl = sampler->getIlluminationSize(), Nv = sampler->getViewSize(), Nt = sampler->getSamplerSize();
    std::vector<ComplexType> v((size_t)Nl * Nv * Nt);
    std::FILE* out = std::fopen(argv[2], "wb");
    if (!out) return 4;
    const double header[4] = { (double)Nl, (double)Nv, (double)Nt, (double)sc.renderings };
    std::fwrite(header, sizeof(double), 4, out);
    ub64 seed = sc.seed;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (ub32 r = 0; r < sc.renderings; ++r) {
        cudaDeviceSynchronize();
        cudaEventRecord(e0);
        err = tracer->trace(v.data());
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        CHECK("trace");
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        std::vector<double> buf(2 * v.size() + 2);
        for (size_t i = 0; i < v.size(); ++i) { buf[2 * i] = v[i].real(); buf[2 * i + 1] = v[i].imag(); }
        buf[2 * v.size()] = (double)((ub64)sc.batch * sc.full_iteration + tracer->getZeroContributionPaths());
        buf[2 * v.size() + 1] = (double)ms;
        std::fwrite(buf.data(), sizeof(double), buf.size(), out);
        seed++;
        tracer->updateSeed(seed);
    }
    std::fclose(out);
    delete tracer;
    delete simulation;
    delete scattering;
    delete medium;
    for (auto* s : src) delete s;
    delete sampler;
    return 0;
}
