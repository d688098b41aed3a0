// A C++ caller of the reference's object model (include/sstmc.hpp): builds one
// 3D scene object by object in mexFunction's order (MatlabInterface.cu:
// 1677-1700), renders two renderings with updateSeed between them as the MEX
// loop does (:1783-1801), and writes u, iter and the photons budget of each
// rendering to the file named by argv[1] as doubles.  tests/test_plugin_api.py
// builds the same scene as a config dict and compares.
#include <cstdio>
#include <vector>

#include "sstmc.hpp"

int main(int argc, char** argv)
{
    if (argc != 2) { std::fprintf(stderr, "usage: %s <output file>\n", argv[0]); return 2; }
    using namespace sstmc;
    ErrorType err = SSTMC_NO_ERROR;
    const ub32 batch = 64, fullIteration = 2, renderings = 2;
    ub64 seed = 5;
    const double lambda = 0.75;
    Simulation simulation(&err, batch, &lambda, 1, 0, 3);
    if (err) return 10;
    Scattering scattering;
    if (scattering.setIsotropicScattering(0) || scattering.setHenyeyGreensteinScattering(0.5, 1)
        || scattering.setHenyeyGreensteinScattering(0.7, 2)) return 11;
    // 4 x 3 x 2 cells over [-8, 8] x [-6, 6] x [0, 4], materials 1 and 2
    const double x[5] = { -8, -4, 0, 4, 8 }, y[4] = { -6, -2, 2, 6 }, z[3] = { 0, 2, 4 };
    std::vector<ub32> grid(4 * 3 * 2);
    for (ub32 k = 0; k < 2; ++k)
        for (ub32 j = 0; j < 3; ++j)
            for (ub32 i = 0; i < 4; ++i) grid[(k * 3 + j) * 4 + i] = 1 + (i + j + k) % 2;
    HeterogeneousMedium medium(&err, grid.data(), x, 5, y, 4, z, 3);
    if (err) return 12;
    const MediumMaterial mats[3] = { { 0.0, 0.0 }, { 0.5, 0.01 }, { 1.0, 0.02 } };
    for (ub32 m = 0; m < 3; ++m)
        if (medium.setMaterial(&mats[m], m)) return 13;
    const double il[9] = { -3, 1, -1, 0, 0, -1, 2.5, -1.5, -1 };
    const double vw[6] = { 0.6, 0, 0.8, 0, 0.6, 0.8 };
    PointSource illumination(&err, &simulation, &medium, &scattering, il, 3, false, ConnectionType::ConnectionTypeIllumination);
    if (err) return 14;
    FarField view(&err, &simulation, &medium, &scattering, vw, 2, ConnectionType::ConnectionTypeView);
    if (err) return 15;
    const double t[3] = { 0.0, 1.0, 2.5 };
    TemporalSampler sampler(&err, &illumination, &view, &simulation, &medium, &scattering, t, 3, true, false);
    if (err) return 16;
    const double U0[3] = { 0, 0, 0 }, U1[3] = { 0.01, 0, 0 }, U2[3] = { 0, 0.02, 0 };
    if (sampler.setMaterial(0.0, U0, 0) || sampler.setMaterial(2e-3, U1, 1) || sampler.setMaterial(5e-3, U2, 2)) return 17;
    const ub32 Nl = sampler.getIlluminationSize(), Nv = sampler.getViewSize(), Nt = sampler.getSamplerSize();
    if (Nl != 3 || Nv != 2 || Nt != 3 || sampler.isCorrelation()) return 18;
    NextEventEstimationOptions options{ false, fullIteration, seed };
    NextEventEstimation tracer(&err, &sampler, &options);
    if (err) { std::fprintf(stderr, "tracer: %s\n", sstmc_error_string(err)); return 19; }
    std::vector<double> out;
    std::vector<double> v(2 * (size_t)Nl * Nv * Nt);
    for (ub32 r = 0; r < renderings; ++r) {
        err = tracer.trace(v.data());
        if (err) { std::fprintf(stderr, "trace: %s\n", sstmc_error_string(err)); return 20; }
        out.insert(out.end(), v.begin(), v.end());
        out.push_back((double)((ub64)batch * fullIteration + tracer.getZeroContributionPaths()));
        out.push_back((double)tracer.getPhotonsBudget());
        seed++;
        tracer.updateSeed(seed);
    }
    std::FILE* f = std::fopen(argv[1], "wb");
    if (!f) return 21;
    const size_t w = std::fwrite(out.data(), sizeof(double), out.size(), f);
    std::fclose(f);
    return w == out.size() ? 0 : 22;
}
