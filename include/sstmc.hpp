/*
 * sstmc.hpp -- C++ host API with the reference's plugin classes, over the
 * C-ABI of sstmc.h.  Header only: every class owns one C handle.
 *
 * A C++ caller builds a render the way mexFunction does
 * (MatlabInterface.cu:1677-1801):
 *
 *   sstmc::ErrorType err;
 *   sstmc::Simulation simulation(&err, batchSize, lambda, 1, 0, 3);
 *   sstmc::Scattering scattering;
 *   scattering.setHenyeyGreensteinScattering(0.9, 0); ...
 *   sstmc::HeterogeneousMedium medium(&err, grid, x, nx, y, ny, z, nz);
 *   medium.setMaterial(&material, mNum); ...
 *   sstmc::PointSource illumination(&err, &simulation, &medium, &scattering,
 *       locations, n, false, sstmc::ConnectionType::ConnectionTypeIllumination);
 *   sstmc::TemporalSampler sampler(&err, &illumination, &view, &simulation,
 *       &medium, &scattering, t, tSize, true, false);
 *   sampler.setMaterial(D, U, mNum); ...
 *   sstmc::NextEventEstimation tracer(&err, &sampler, &options);
 *   for (r ...) { tracer.trace(v + r * Nl * Nv * Nt); tracer.updateSeed(++seed); }
 *
 * Class and method names, argument order and meaning follow the reference
 * (Simulation.cuh:179, Scattering.cuh:32-125, MediumInterface.cuh:39-135,
 * SourceInterface.cuh:10-179, SamplerInterface.cuh:11-176,
 * TracerInterface.cuh:9-50, NextEventEstimation.cuh:100-105); error codes are
 * the SSTMC_* values, which keep the reference's ErrorType numbers.  The
 * device work of the reference's per-method kernels is fused into the render
 * (the trace call); v is complex as interleaved (re, im) doubles.
 */
#ifndef SSTMC_HPP
#define SSTMC_HPP

#include <cstdint>

#include "sstmc.h"

namespace sstmc {

typedef int32_t ErrorType;
typedef uint32_t ub32;
typedef uint64_t ub64;

/* Simulation.cuh:80-86 */
enum class ConnectionType : int32_t {
    ConnectionTypeIllumination = SSTMC_CONNECTION_ILLUMINATION,
    ConnectionTypeView = SSTMC_CONNECTION_VIEW,
    ConnectionTypeIllumination2 = SSTMC_CONNECTION_ILLUMINATION2,
    ConnectionTypeView2 = SSTMC_CONNECTION_VIEW2,
};

/* MediumInterface.cuh: a material's scattering and absorption coefficients */
struct MediumMaterial {
    double sigs;
    double siga;
};

/* NextEventEstimation.cuh:100-105 */
struct NextEventEstimationOptions {
    bool isCBS;
    ub32 fullIterationsNumber;
    ub64 seed;
};

/* Simulation(err, batchNum, lambda, lambdaNum, gpuDeviceNumber): one
 * wavelength per simulation; dims 2 or 3 (the reference's DIMS). */
class Simulation {
public:
    Simulation(ErrorType* err, ub32 batchNum, const double* lambdaIn, ub32 lambdaNumIn, ub32 gpuDeviceNumber = 0,
               ub32 dims = 3, int32_t precision = SSTMC_PRECISION_SPLIT)
    {
        const ErrorType e = lambdaNumIn == 1 && lambdaIn
            ? sstmc_simulation_create(dims, batchNum, lambdaIn[0], (int32_t)gpuDeviceNumber, precision, &h_)
            : SSTMC_NOT_SUPPORTED;   // one wavelength per scene: render a lambda vector one wavelength at a time
        if (err) *err = e;
    }
    ~Simulation() { sstmc_simulation_destroy(h_); }
    Simulation(const Simulation&) = delete;
    Simulation& operator=(const Simulation&) = delete;
    const sstmc_simulation* handle() const { return h_; }

private:
    sstmc_simulation* h_ = nullptr;
};

/* Scattering.cuh:32-125 */
class Scattering {
public:
    Scattering() { sstmc_scattering_create(&h_); }
    ~Scattering() { sstmc_scattering_destroy(h_); }
    Scattering(const Scattering&) = delete;
    Scattering& operator=(const Scattering&) = delete;
    ErrorType setIsotropicScattering(ub32 materialNum) { return sstmc_scattering_set_isotropic(h_, materialNum); }
    ErrorType setHenyeyGreensteinScattering(double g, ub32 materialNum)
    {
        return sstmc_scattering_set_henyey_greenstein(h_, g, materialNum);
    }
    /* f: N complex amplitudes as (re, im) pairs */
    ErrorType setTabularScattering(const double* f, ub32 N, ub32 materialNum)
    {
        return sstmc_scattering_set_tabular(h_, f, N, materialNum);
    }
    ErrorType setVonMisesFisherScattering(const double* mixtureMu, const double* mixtureC, const double* mixtureAlpha,
                                          ub32 mixturesNum, ub32 materialNum)
    {
        return sstmc_scattering_set_von_mises_fisher(h_, mixtureMu, mixtureC, mixtureAlpha, mixturesNum, materialNum);
    }
    const sstmc_scattering* handle() const { return h_; }

private:
    sstmc_scattering* h_ = nullptr;
};

/* MediumInterface.cuh:39-135 */
class Medium {
public:
    virtual ~Medium() { sstmc_medium_destroy(h_); }
    Medium(const Medium&) = delete;
    Medium& operator=(const Medium&) = delete;
    ErrorType setMaterial(const MediumMaterial* material, ub32 materialNum)
    {
        return material ? sstmc_medium_set_material(h_, material->sigs, material->siga, materialNum) : SSTMC_INVALID_HANDLE;
    }
    const sstmc_medium* handle() const { return h_; }

protected:
    Medium() = default;
    sstmc_medium* h_ = nullptr;
};

/* HeterogeneousMedium(err, materialGrid, xAxis, xAxisSize, yAxis, yAxisSize
 * [, zAxis, zAxisSize]): grid x fastest, (nx-1)(ny-1)(nz-1) cells. */
class HeterogeneousMedium : public Medium {
public:
    HeterogeneousMedium(ErrorType* err, const ub32* materialGrid, const double* xAxis, ub32 xAxisSize, const double* yAxis,
                        ub32 yAxisSize, const double* zAxis = nullptr, ub32 zAxisSize = 0)
    {
        const ErrorType e = sstmc_medium_create_heterogeneous(materialGrid, xAxis, xAxisSize, yAxis, yAxisSize, zAxis, zAxisSize, &h_);
        if (err) *err = e;
    }
};

/* config.medium.type = 'Homogeneous': box and sigs */
class HomogeneousMedium : public Medium {
public:
    HomogeneousMedium(ErrorType* err, ub32 dims, const double boxMin[3], const double boxMax[3], double sigs)
    {
        const ErrorType e = sstmc_medium_create_homogeneous(dims, boxMin, boxMax, sigs, &h_);
        if (err) *err = e;
    }
};

/* SourceInterface.cuh:10-179 */
class Source {
public:
    virtual ~Source() { sstmc_source_destroy(h_); }
    Source(const Source&) = delete;
    Source& operator=(const Source&) = delete;
    ub32 getSourceSize() const
    {
        ub32 n = 0;
        sstmc_source_size(h_, &n);
        return n;
    }
    const sstmc_source* handle() const { return h_; }

protected:
    Source() = default;
    sstmc_source* h_ = nullptr;
};

/* PointSource(err, simulation, medium, scattering, locations (n x 3), n,
 * isAreaSource, connectionType) */
class PointSource : public Source {
public:
    PointSource(ErrorType* err, const Simulation* simulation, const Medium*, const Scattering*, const double* locations, ub32 n,
                bool isAreaSource, ConnectionType cn)
    {
        const ErrorType e = simulation
            ? sstmc_source_create_point(simulation->handle(), (int32_t)cn, locations, n, isAreaSource ? 1 : 0, &h_)
            : SSTMC_INVALID_HANDLE;
        if (err) *err = e;
    }
};

/* FarField(err, simulation, medium, scattering, directions (n x 3), n, connectionType) */
class FarField : public Source {
public:
    FarField(ErrorType* err, const Simulation* simulation, const Medium*, const Scattering*, const double* directions, ub32 n,
             ConnectionType cn)
    {
        const ErrorType e = simulation ? sstmc_source_create_far_field(simulation->handle(), (int32_t)cn, directions, n, &h_)
                                       : SSTMC_INVALID_HANDLE;
        if (err) *err = e;
    }
};

/* GaussianBeam(err, simulation, medium, scattering, focalPoints (n x 3),
 * focalDirections (n x 3), aperture, n, connectionType) */
class GaussianBeam : public Source {
public:
    GaussianBeam(ErrorType* err, const Simulation* simulation, const Medium*, const Scattering*, const double* focalPoints,
                 const double* focalDirections, double aperture, ub32 n, ConnectionType cn)
    {
        const ErrorType e = simulation
            ? sstmc_source_create_gaussian_beam(simulation->handle(), (int32_t)cn, focalPoints, focalDirections, n, aperture, &h_)
            : SSTMC_INVALID_HANDLE;
        if (err) *err = e;
    }
};

/* SamplerInterface.cuh:11-176 */
class Sampler {
public:
    virtual ~Sampler() { sstmc_sampler_destroy(h_); }
    Sampler(const Sampler&) = delete;
    Sampler& operator=(const Sampler&) = delete;
    /* D and U (3 doubles) of a material's scatterers */
    ErrorType setMaterial(double D, const double* U, ub32 materialNum) { return sstmc_sampler_set_material(h_, D, U, materialNum); }
    ub32 getIlluminationSize() const { ub32 n = 0; sstmc_sampler_shape(h_, &n, nullptr, nullptr); return n; }
    ub32 getViewSize() const { ub32 n = 0; sstmc_sampler_shape(h_, nullptr, &n, nullptr); return n; }
    ub32 getSamplerSize() const { ub32 n = 0; sstmc_sampler_shape(h_, nullptr, nullptr, &n); return n; }
    bool isCorrelation() const { int32_t c = 0; sstmc_sampler_is_correlation(h_, &c); return c != 0; }
    sstmc_sampler* handle() const { return h_; }

protected:
    Sampler() = default;
    sstmc_sampler* h_ = nullptr;
};

/* TemporalSampler(err, illuminationsHandle, viewsHandle, simulation, medium,
 * scattering, t, tSize, isTemporalAmplitude, isForcedInsideBin) */
class TemporalSampler : public Sampler {
public:
    TemporalSampler(ErrorType* err, const Source* illumination, const Source* view, const Simulation* simulation,
                    const Medium* medium, const Scattering* scattering, const double* t, ub32 tSize,
                    bool isTemporalAmplitude = true, bool isForcedInsideBin = false)
    {
        const ErrorType e = (illumination && view && simulation && medium && scattering)
            ? sstmc_sampler_create_temporal(simulation->handle(), medium->handle(), scattering->handle(), illumination->handle(),
                                            view->handle(), t, tSize, isTemporalAmplitude ? 1 : 0, isForcedInsideBin ? 1 : 0, &h_)
            : SSTMC_INVALID_HANDLE;
        if (err) *err = e;
    }
};

/* TemporalCorrelationSampler(err, illuminationsHandle, illuminationsHandle2,
 * viewsHandle, viewsHandle2, simulation, medium, scattering, t, tSize) */
class TemporalCorrelationSampler : public Sampler {
public:
    TemporalCorrelationSampler(ErrorType* err, const Source* illumination, const Source* illumination2, const Source* view,
                               const Source* view2, const Simulation* simulation, const Medium* medium,
                               const Scattering* scattering, const double* t, ub32 tSize)
    {
        const ErrorType e = (illumination && illumination2 && view && view2 && simulation && medium && scattering)
            ? sstmc_sampler_create_correlation(simulation->handle(), medium->handle(), scattering->handle(),
                                               illumination->handle(), illumination2->handle(), view->handle(), view2->handle(),
                                               t, tSize, &h_)
            : SSTMC_INVALID_HANDLE;
        if (err) *err = e;
    }
};

/* TracerInterface.cuh:9-50 */
class Tracer {
public:
    virtual ~Tracer() { sstmc_tracer_destroy(h_); }
    Tracer(const Tracer&) = delete;
    Tracer& operator=(const Tracer&) = delete;
    /* one rendering into v: 2 * Nl * Nv * Nt doubles (interleaved complex) */
    virtual ErrorType trace(double* v) { return sstmc_tracer_trace(h_, v); }
    ub64 getZeroContributionPaths() const { ub64 n = 0; sstmc_tracer_zero_contribution_paths(h_, &n); return n; }
    ub64 getPhotonsBudget() const { ub64 n = 0; sstmc_tracer_photons_budget(h_, &n); return n; }
    bool getCBS() const { int32_t c = 0; sstmc_tracer_is_cbs(h_, &c); return c != 0; }
    ErrorType updateSeed(ub64 seed) { return sstmc_tracer_update_seed(h_, seed); }
    sstmc_scene* scene() const { return sstmc_tracer_scene(h_); }

protected:
    Tracer() = default;
    sstmc_tracer* h_ = nullptr;
};

/* NextEventEstimation(err, samplerHandler, options) */
class NextEventEstimation : public Tracer {
public:
    NextEventEstimation(ErrorType* err, Sampler* sampler, const NextEventEstimationOptions* options)
    {
        const ErrorType e = (sampler && options)
            ? sstmc_tracer_create_nee(sampler->handle(), options->fullIterationsNumber, options->seed, options->isCBS ? 1 : 0, &h_)
            : SSTMC_INVALID_HANDLE;
        if (err) *err = e;
    }
};

}  // namespace sstmc

#endif /* SSTMC_HPP */
