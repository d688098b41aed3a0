/*
 * sstmc.h -- C-ABI of the GB300-native next-event-estimation (NEE) speckle
 * path tracer.  Plain C types only: pointers, sizes, integers and doubles.
 *
 * The boundary replaces the MATLAB MEX entry point of the reference
 *   [u, iter] = sstmc2D(config) / sstmc3D(config)
 *   (MatlabInterface.cu:1565-1825, mexFunction)
 * and the object model it builds (Simulation / Scattering / Medium / Source /
 * Sampler / Tracer, MatlabInterface.cu:1459-1563, 712-1457).  One
 * sstmc_config carries every field of the MATLAB config struct; one
 * sstmc_scene is the set of device-resident objects mexFunction constructs;
 * sstmc_render is one call of Tracer::trace per rendering
 * (NextEventEstimation.cuh:1461-1637).
 *
 * Output layout is the reference's: u is complex, Nl fastest, then Nv, then
 * Nt, then renderings (MatlabInterface.cu:1731-1738), stored here as
 * interleaved (re, im) doubles.  iter[r] = batchSize * fullIteration +
 * zeroContributionPaths (MatlabInterface.cu:1796).
 *
 * Error codes keep the numeric values of the reference's ErrorType enum
 * (Simulation.cuh:111-162) for every shared meaning; codes >= 100 are new.
 */
#ifndef SSTMC_H
#define SSTMC_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ */
/* Error codes: Simulation.cuh:111-162 (ErrorType)                      */
/* ------------------------------------------------------------------ */
#define SSTMC_NO_ERROR                 0
#define SSTMC_DEVICE_ERROR             1
#define SSTMC_ALLOCATION_ERROR         2
#define SSTMC_KERNEL_ERROR             3
#define SSTMC_CUBLAS_ERROR             4   /* reference: cuBLAS; here: contraction (GEMM) error */
#define SSTMC_NOT_SUPPORTED            5
#define SSTMC_MISC_ERROR               6
/* 7..47 are the reference's per-kernel KERNEL_ERROR_* codes; the ones this
 * build can raise keep their reference values: */
#define SSTMC_KERNEL_ERROR_HetroMedium_heterogeneousAttenuationKernel 44
#define SSTMC_KERNEL_ERROR_HetroMedium_heterogeneousSampleKernel      45
/* new in this build */
#define SSTMC_INVALID_CONFIG           100 /* the MEX layer raised a MATLAB error instead */
#define SSTMC_TIMEOUT                  101 /* a bounded wait or a bounded device loop ran out */
#define SSTMC_CANCELLED                102 /* a served request was cancelled */
#define SSTMC_INVALID_HANDLE           103
#define SSTMC_PATH_LIMIT               104 /* a path exceeded the vertex / retry limit */
#define SSTMC_SCRATCH_LIMIT            105 /* sstmc_render_static: the request does not fit its static scratch */

/* ------------------------------------------------------------------ */
/* Enumerations mirroring the reference's string / enum values          */
/* ------------------------------------------------------------------ */
/* ScatteringNS::ScatteringType (Scattering.cuh:17-23) */
#define SSTMC_SCATTERING_NOT_DEFINED      0
#define SSTMC_SCATTERING_ISOTROPIC        1
#define SSTMC_SCATTERING_TABULAR          2   /* table of the complex amplitude (tabular_n / tabular_f) */
#define SSTMC_SCATTERING_HENYEY_GREENSTEIN 3
#define SSTMC_SCATTERING_VMF_MIXTURE      4   /* von Mises-Fisher mixture (vmf_n / vmf_mu / vmf_c / vmf_alpha) */

/* config.medium.type (MatlabInterface.cu:896, 942) */
#define SSTMC_MEDIUM_HETEROGENEOUS 0
#define SSTMC_MEDIUM_HOMOGENEOUS   1   /* mapped to a single-cell heterogeneous grid */

/* config.<source>.type (MatlabInterface.cu:1101, 1137, 1161) */
#define SSTMC_SOURCE_NONE          0   /* absent illumination2 / view2 */
#define SSTMC_SOURCE_POINT         1
#define SSTMC_SOURCE_FARFIELD      2
#define SSTMC_SOURCE_GAUSSIANBEAM  3   /* focused beams: 3D field sampler, illumination and view both GaussianBeam */

/* config.sampler.type (MatlabInterface.cu:1238, 1295) */
#define SSTMC_SAMPLER_TEMPORAL              0
#define SSTMC_SAMPLER_TEMPORAL_CORRELATION  1

/* ConnectionType (Simulation.cuh:80-86): the role of a source. */
#define SSTMC_CONNECTION_ILLUMINATION  0
#define SSTMC_CONNECTION_VIEW          1
#define SSTMC_CONNECTION_ILLUMINATION2 2
#define SSTMC_CONNECTION_VIEW2         3

/* Contraction precision of the illumination x view accumulation. */
#define SSTMC_PRECISION_SPLIT  0  /* default: FP64 path length + phase reduction, 3xTF32 tensor-core contraction */
#define SSTMC_PRECISION_FP32   1  /* plain FP32 form: FP32 phase, FP32 SIMT contraction */

#define SSTMC_MATERIAL_NUM 10     /* Simulation.cuh:32 (MATERIAL_NUM) */

/* One source block of the config (illumination, view, illumination2, view2).
 * MatlabInterface.cu:1062-1215 (buildSource). */
typedef struct sstmc_source_cfg {
    int32_t type;            /* SSTMC_SOURCE_* */
    uint32_t count;          /* number of locations / directions / beams */
    const double* xyz;       /* count x 3 doubles (x, y, z); z ignored when dims == 2.  GaussianBeam: focal points */
    int32_t is_area_source;  /* PointSource isAreaSource (default 0) */
    /* GaussianBeam (MatlabInterface.cu:1161-1200): focalDirection per beam
     * (count x 3 doubles, used as given) and the scalar aperture; ignored by
     * the other types */
    const double* focal_direction;
    double aperture;
} sstmc_source_cfg;

/* The whole MATLAB config struct (README.md:74-373). */
typedef struct sstmc_config {
    uint32_t dims;                 /* 2 (sstmc2D) or 3 (sstmc3D) */

    /* config.simulation (MatlabInterface.cu:1459-1546, 1590-1671) */
    uint32_t batch_size;           /* default 1024 */
    uint32_t full_iteration;       /* default 1 */
    uint32_t renderings_num;       /* default 1 */
    double lambda;                 /* default 1; a single wavelength (Nw = 1) */
    uint64_t seed;
    int32_t device_number;         /* default 0 */

    /* config.scattering (MatlabInterface.cu:712-888); one entry per material
     * cell.  A single cell is duplicated into material 1 as the reference does
     * (MatlabInterface.cu:750-760, 878-881). */
    uint32_t scattering_num;       /* number of cells in scattering.type */
    const int32_t* scattering_type;  /* SSTMC_SCATTERING_*, [scattering_num] */
    const double* scattering_g;      /* HG anisotropy g, [scattering_num] (ignored for Isotropic) */

    /* config.medium (MatlabInterface.cu:890-1060) */
    int32_t medium_type;           /* SSTMC_MEDIUM_* */
    const double* x_axis; uint32_t x_axis_size;
    const double* y_axis; uint32_t y_axis_size;
    const double* z_axis; uint32_t z_axis_size;   /* 3D only */
    const uint32_t* material_grid; /* (nx-1)(ny-1)(nz-1) entries, x fastest */
    const double* sigs;            /* [material count] */
    const double* siga;            /* [material count] or NULL (zeros) */
    /* Homogeneous medium: box and scalars (used when medium_type == HOMOGENEOUS) */
    double box_min[3];
    double box_max[3];
    double homogeneous_sigs;

    /* config.illumination / view / illumination2 / view2 */
    sstmc_source_cfg illumination;
    sstmc_source_cfg view;
    sstmc_source_cfg illumination2;
    sstmc_source_cfg view2;

    /* config.sampler (MatlabInterface.cu:1217-1372) */
    int32_t sampler_type;          /* SSTMC_SAMPLER_* */
    const double* t; uint32_t t_num;
    const double* D;               /* [material count], non-negative */
    const double* U;               /* [material count x 3] (x, y, z) */
    int32_t is_temporal_amplitude; /* default 1 */
    int32_t is_forced_inside_bin;  /* default 0; field sampler: per vertex a tick drawn uniformly sits on the
                                      sampled point and ticks that leave its grid cell weigh 0 (ignored by the
                                      correlation sampler, TemporalSampler.cuh:439-534, 1637-1698) */

    /* config.tracer (MatlabInterface.cu:1374-1457) */
    int32_t is_cbs;                /* default 0; 1: coherent backscattering (field and correlation samplers; not with Gaussian beams) */

    /* build-specific */
    int32_t precision;             /* SSTMC_PRECISION_* */

    /* Tabular scattering (Scattering.cuh:191-482, MatlabInterface.cu:762-790):
     * the number of entries of each material's complex amplitude table (0 for
     * the other types) and the tables as (re, im) pairs, concatenated in
     * material order.  A table spans the scattering angle 0..pi (3D) or
     * 0..2pi (2D) in equal steps; it is normalised by its cross section at
     * scene creation. */
    const uint32_t* tabular_n;     /* [scattering_num] or NULL */
    const double* tabular_f;       /* [2 x sum(tabular_n)] or NULL */

    /* von Mises-Fisher mixture scattering (Scattering.cuh:613-884,
     * MatlabInterface.cu:827-868): per material the number of mixture
     * components (0 for the other types), and the components' mixtureMu,
     * mixtureC and mixtureAlpha concatenated in material order.  The
     * amplitude is sum_k alpha_k exp(mu_k cos(theta) + C_k) in 3D; in 2D the
     * reference scatters a vMF material isotropically.  With every material
     * isotropic (|g| < 1e-4, all |mu| <= 1e-4) point sources take the
     * isotropic amplitude and far-field sources the mixture's, as the
     * reference's sources do. */
    const uint32_t* vmf_n;         /* [scattering_num] or NULL */
    const double* vmf_mu;          /* [sum(vmf_n)] or NULL */
    const double* vmf_c;           /* [sum(vmf_n)] or NULL */
    const double* vmf_alpha;       /* [sum(vmf_n)] or NULL, each >= 0 */
} sstmc_config;

typedef struct sstmc_scene sstmc_scene;

/* Fill cfg with the reference's defaults (batchSize 1024, fullIteration 1,
 * renderingsNum 1, lambda 1, isTemporalAmplitude true, ...). */
void sstmc_config_init(sstmc_config* cfg);

/* Build the device-resident scene: replaces buildSimulation .. buildTracer
 * (MatlabInterface.cu:1677-1700).  The config arrays are copied; the caller
 * may free them after the call. */
int32_t sstmc_scene_create(const sstmc_config* cfg, sstmc_scene** out);

/* Nl, Nv, Nt of the scene (Sampler::getIlluminationSize/getViewSize/
 * getSamplerSize, SamplerInterface.cuh:147-151). */
int32_t sstmc_scene_shape(const sstmc_scene* scene, uint32_t* nl, uint32_t* nv, uint32_t* nt);

/* Render renderings_num fields / correlations: the loop of
 * MatlabInterface.cu:1783-1801 (trace, iter, seed++ per rendering).
 * u_out: 2 * Nl * Nv * Nt * renderings_num doubles (interleaved complex),
 * iter_out: renderings_num doubles (may be NULL).  seed overrides
 * cfg.seed for the first rendering.  Paths are traced in chunks whose device
 * buffers take at most min(32 GiB, a quarter of the free device memory), or
 * the bytes given by the environment variable SSTMC_CHUNK_BYTES; freed chunk
 * buffers stay in the device's stream-ordered memory pool (up to 96 GiB) for
 * the next scene or render. */
int32_t sstmc_render(sstmc_scene* scene, uint64_t seed, double* u_out, double* iter_out);

/* Wavefront autotuner.  No counterpart in the reference, whose wavefront is
 * batchSize paths.  Renders the scene's first sample_paths paths (at least
 * 4096) once per candidate wavefront -- paths traced per chunk of kernel
 * launches: powers of two from 4096 up to the sample and the device-memory
 * budget -- timing each with CUDA events after one untimed render at that
 * size, and keeps the fastest for the scene's later renders (sstmc_render and
 * served requests; a smaller reservation still bounds a served chunk).  The
 * result of a render does not depend on the wavefront beyond the order of
 * its FP32 windowed sums.  chunk_paths (may be NULL): the chosen wavefront.
 * Overwrites sstmc_last_stats / sstmc_last_timing. */
int32_t sstmc_scene_autotune(sstmc_scene* scene, uint32_t sample_paths, uint64_t* chunk_paths);

/* sstmc_render without device memory allocation.  No counterpart in the
 * reference: it is for callers that must not allocate device memory during a
 * render -- a host that owns a fixed device-memory budget (a serving process
 * whose admitted work must not fail later on an out-of-memory, or that must
 * not stall other streams on the implicit device synchronisation of
 * cudaFree), or a caller that has reserved all of the device for itself.
 * Same arguments, result and statistics as sstmc_render (within the FP64
 * accumulation-order tolerance); sstmc_last_timing is not updated.
 *
 * Every device buffer lives in one static scratch array of 64 MiB per device
 * that is part of this library's device image: no cudaMalloc, cudaFree or
 * allocating library routine is called.  The scratch holds the output
 * (16 * Nl * Nv * Nt bytes), the far-field weight table (40 * Nl * Nv * Nt
 * bytes when illumination and view are both far fields) and the per-path rows
 * of one chunk of paths; a request whose output and tables leave no room for
 * one path, or one of whose paths has more vertices than fit, returns
 * SSTMC_SCRATCH_LIMIT (sstmc_last_error_text says what did not fit).
 *
 * The scratch is shared by every scene on a device: overlapping calls would
 * race on it, so the library serialises sstmc_render_static calls per device
 * (a call waits for any other one on that device to return).  The call waits
 * on the host for each chunk of paths (it synchronises the scene's stream once
 * per chunk) and returns when the render is complete.  The first call on a
 * device looks up the scratch's device address (cudaGetSymbolAddress) with
 * that device current; make that first call before any stream capture.
 *
 * The 64 MiB array is part of the library's device image: every device on
 * which the library's module is loaded holds it until the process exits,
 * whether or not this entry point is ever called. */
int32_t sstmc_render_static(sstmc_scene* scene, uint64_t seed, double* u_out, double* iter_out);

/* ------------------------------------------------------------------ */
/* Serving: continuous batching of renders.  No counterpart in the      */
/* reference (one scene per MEX call, MatlabInterface.cu:1565-1825).    */
/* ------------------------------------------------------------------ */
typedef struct sstmc_server sstmc_server;

/* A request loop on `device` with `slots` worker threads.  A request
 * reserves the device memory of its chunk buffers (sized to at most
 * hbm_budget_bytes / slots); queued requests are admitted first-fit while
 * the reservations in flight stay within hbm_budget_bytes (0: half of the
 * free memory), and any request is admitted when nothing is in flight.
 * Requests on different scenes run concurrently on their scenes' streams;
 * requests on one scene run one after another. */
int32_t sstmc_server_create(int32_t device, uint64_t hbm_budget_bytes, uint32_t slots, sstmc_server** out);
/* Cancels queued requests, waits for the running ones, stops the loop. */
int32_t sstmc_server_destroy(sstmc_server* server);
/* Queue all renderings of `scene` starting at `seed` (sstmc_render's
 * semantics and output layout).  The scene and the output buffers must stay
 * valid until the ticket is done. */
int32_t sstmc_submit(sstmc_server* server, sstmc_scene* scene, uint64_t seed, double* u_out, double* iter_out,
                     uint64_t* ticket);
/* done = 1 once the request finished; status = its sstmc_render code. */
int32_t sstmc_poll(sstmc_server* server, uint64_t ticket, int32_t* done, int32_t* status);
/* Wait up to timeout_s seconds: SSTMC_TIMEOUT if the request is still open. */
int32_t sstmc_wait(sstmc_server* server, uint64_t ticket, double timeout_s, int32_t* status);
/* A queued request completes with SSTMC_CANCELLED; a running one finishes. */
int32_t sstmc_cancel(sstmc_server* server, uint64_t ticket);
/* Latency (submit to done) percentiles over the completed requests and
 * their contributions per second between the first start and the last end. */
int32_t sstmc_server_stats(sstmc_server* server, double* p50_ms, double* p99_ms, double* contributions_per_s,
                           uint64_t* completed);

/* Number of NEE path-contributions (sum over traced paths of vertices * Nl *
 * Nv * Nt) and of voxel DDA steps of the last sstmc_render call. */
int32_t sstmc_last_stats(const sstmc_scene* scene, uint64_t* contributions,
                         uint64_t* dda_steps, uint64_t* vertices, uint64_t* paths);

/* Device time of the last sstmc_render in milliseconds, measured with CUDA
 * events on the scene's stream: ms[0] whole render, ms[1] path tracing
 * (ms[4] + ms[5]), ms[2] multiple-scattering contraction, ms[3]
 * single-scattering contraction, ms[4] random walk (count, scan, write),
 * ms[5] NEE vectors; launches[0] = kernels launched, launches[1] = chunks
 * of paths.  ms: 6 doubles, launches: 2 integers.  No reference counterpart
 * (the reference's TIME_REC std::clock buckets,
 * NextEventEstimation.cuh:107-156). */
int32_t sstmc_last_timing(const sstmc_scene* scene, double* ms, uint64_t* launches);

int32_t sstmc_scene_destroy(sstmc_scene* scene);

/* Text of an error code (MatlabInterface.cu:24-272, getErrorMsg). */
const char* sstmc_error_string(int32_t code);

/* Detail text of the last failed sstmc_scene_create (config validation). */
const char* sstmc_last_error_text(void);

/* ------------------------------------------------------------------ */
/* The reference's object model, one object at a time (the plugin      */
/* setters).  mexFunction builds Simulation -> Scattering -> Medium ->  */
/* Sources -> Sampler -> Tracer (MatlabInterface.cu:1677-1700); these   */
/* handles are built in the same order and the tracer renders exactly   */
/* what the equivalent sstmc_config renders.  The caller creates every  */
/* object and destroys it in reverse order; a sampler borrows its       */
/* sources, medium and scattering, a tracer its sampler.  C++ callers:  */
/* include/sstmc.hpp wraps these handles in the reference's classes.    */
/* ------------------------------------------------------------------ */
typedef struct sstmc_simulation sstmc_simulation;
typedef struct sstmc_scattering sstmc_scattering;
typedef struct sstmc_medium sstmc_medium;
typedef struct sstmc_source sstmc_source;
typedef struct sstmc_sampler sstmc_sampler;
typedef struct sstmc_tracer sstmc_tracer;

/* Simulation(err, batchNum, lambda, 1, gpuDeviceNumber) (Simulation.cuh:179);
 * dims selects sstmc2D (2) or sstmc3D (3), which the reference fixes at
 * compile time; precision is SSTMC_PRECISION_*. */
int32_t sstmc_simulation_create(uint32_t dims, uint32_t batch_size, double lambda, int32_t device_number, int32_t precision,
                                sstmc_simulation** out);
int32_t sstmc_simulation_destroy(sstmc_simulation* sim);

/* Scattering() and its per-material setters (Scattering.cuh:32-125):
 * setIsotropicScattering(mat), setHenyeyGreensteinScattering(g, mat),
 * setTabularScattering(f, N, mat) with f as N (re, im) pairs,
 * setVonMisesFisherScattering(mu, c, alpha, mixtures, mat). */
int32_t sstmc_scattering_create(sstmc_scattering** out);
int32_t sstmc_scattering_set_isotropic(sstmc_scattering* s, uint32_t mat);
int32_t sstmc_scattering_set_henyey_greenstein(sstmc_scattering* s, double g, uint32_t mat);
int32_t sstmc_scattering_set_tabular(sstmc_scattering* s, const double* f, uint32_t n, uint32_t mat);
int32_t sstmc_scattering_set_von_mises_fisher(sstmc_scattering* s, const double* mu, const double* c, const double* alpha,
                                              uint32_t mixtures, uint32_t mat);
int32_t sstmc_scattering_destroy(sstmc_scattering* s);

/* HeterogeneousMedium(err, materialGrid, xAxis, nx, yAxis, ny[, zAxis, nz])
 * (HeterogeneousMedium.cuh, MatlabInterface.cu:998-1003; z NULL in 2D; grid
 * x fastest) and Medium::setMaterial(MediumMaterial{sigs, siga}, mat)
 * (MediumInterface.cuh:39-135).  The homogeneous medium is the box form of
 * config.medium (MatlabInterface.cu:896-945). */
int32_t sstmc_medium_create_heterogeneous(const uint32_t* grid, const double* x, uint32_t nx, const double* y, uint32_t ny,
                                          const double* z, uint32_t nz, sstmc_medium** out);
int32_t sstmc_medium_create_homogeneous(uint32_t dims, const double box_min[3], const double box_max[3], double sigs,
                                        sstmc_medium** out);
int32_t sstmc_medium_set_material(sstmc_medium* m, double sigs, double siga, uint32_t mat);
int32_t sstmc_medium_destroy(sstmc_medium* m);

/* PointSource(err, simulation, medium, scattering, locations, n, isAreaSource,
 * connectionType) and FarField(err, ..., directions, n, connectionType)
 * (PointSource.cuh, FarField.cuh; MatlabInterface.cu:1128, 1151).  xyz: n x 3
 * doubles; connection: SSTMC_CONNECTION_*.  getSourceSize: sstmc_source_size. */
int32_t sstmc_source_create_point(const sstmc_simulation* sim, int32_t connection, const double* xyz, uint32_t count,
                                  int32_t is_area_source, sstmc_source** out);
int32_t sstmc_source_create_far_field(const sstmc_simulation* sim, int32_t connection, const double* xyz, uint32_t count,
                                      sstmc_source** out);
/* GaussianBeam(err, simulation, medium, scattering, focalPoints, focalDirections,
 * aperture, beamsNum, connectionType) (GaussianBeam.cuh:62-64, MatlabInterface.cu:
 * 1193-1194): focal points and directions n x 3 doubles, one aperture. */
int32_t sstmc_source_create_gaussian_beam(const sstmc_simulation* sim, int32_t connection, const double* focal_points,
                                          const double* focal_directions, uint32_t count, double aperture, sstmc_source** out);
int32_t sstmc_source_size(const sstmc_source* s, uint32_t* count);
int32_t sstmc_source_destroy(sstmc_source* s);

/* TemporalSampler(err, illumination, view, simulation, medium, scattering, t,
 * tSize, isTemporalAmplitude, isForcedInsideBin) and
 * TemporalCorrelationSampler(err, illumination, illumination2, view, view2,
 * simulation, medium, scattering, t, tSize) (MatlabInterface.cu:1281, 1333),
 * setMaterial(D, U, mat) (:1299, :1350), getIlluminationSize / getViewSize /
 * getSamplerSize and isCorrelation (SamplerInterface.cuh:132-152). */
int32_t sstmc_sampler_create_temporal(const sstmc_simulation* sim, const sstmc_medium* medium, const sstmc_scattering* scattering,
                                      const sstmc_source* illumination, const sstmc_source* view, const double* t, uint32_t t_num,
                                      int32_t is_temporal_amplitude, int32_t is_forced_inside_bin, sstmc_sampler** out);
int32_t sstmc_sampler_create_correlation(const sstmc_simulation* sim, const sstmc_medium* medium, const sstmc_scattering* scattering,
                                         const sstmc_source* illumination, const sstmc_source* illumination2,
                                         const sstmc_source* view, const sstmc_source* view2, const double* t, uint32_t t_num,
                                         sstmc_sampler** out);
int32_t sstmc_sampler_set_material(sstmc_sampler* s, double D, const double U[3], uint32_t mat);
int32_t sstmc_sampler_shape(const sstmc_sampler* s, uint32_t* nl, uint32_t* nv, uint32_t* nt);
int32_t sstmc_sampler_is_correlation(const sstmc_sampler* s, int32_t* is_correlation);
/* The sstmc_config the objects describe (no counterpart: the MEX layer's
 * config struct in reverse).  Its arrays belong to the sampler and the
 * objects it borrows, valid until one of them changes or is destroyed. */
int32_t sstmc_sampler_config(sstmc_sampler* s, uint32_t full_iteration, uint64_t seed, int32_t is_cbs, sstmc_config* out);
int32_t sstmc_sampler_destroy(sstmc_sampler* s);

/* NextEventEstimation(err, sampler, {fullIterationsNumber, seed, isCBS})
 * (MatlabInterface.cu:1438): creates the device-resident scene.
 * trace(v): one rendering into v (2 * Nl * Nv * Nt doubles, the layout of
 * sstmc_render); updateSeed, getZeroContributionPaths (the missed first
 * vertices of the last trace), getPhotonsBudget (its scattering vertices,
 * the participating paths summed over path lengths), getCBS
 * (TracerInterface.cuh:9-50).  sstmc_tracer_scene gives the scene for
 * sstmc_last_stats / sstmc_last_timing. */
int32_t sstmc_tracer_create_nee(sstmc_sampler* sampler, uint32_t full_iteration, uint64_t seed, int32_t is_cbs,
                                sstmc_tracer** out);
int32_t sstmc_tracer_trace(sstmc_tracer* t, double* v);
int32_t sstmc_tracer_update_seed(sstmc_tracer* t, uint64_t seed);
int32_t sstmc_tracer_zero_contribution_paths(const sstmc_tracer* t, uint64_t* out);
int32_t sstmc_tracer_photons_budget(const sstmc_tracer* t, uint64_t* out);
int32_t sstmc_tracer_is_cbs(const sstmc_tracer* t, int32_t* out);
sstmc_scene* sstmc_tracer_scene(sstmc_tracer* t);
int32_t sstmc_tracer_destroy(sstmc_tracer* t);

/* ------------------------------------------------------------------ */
/* Per-path debug trace (parity tests): run one wave of `paths` paths  */
/* with path ids [first_path, first_path + paths) and copy the         */
/* per-path quantities to host arrays.  Any pointer may be NULL.        */
/* ------------------------------------------------------------------ */
typedef struct sstmc_path_trace {
    int32_t* misses;        /* [paths] missed first-vertex attempts */
    int32_t* vertices;      /* [paths] scattering vertices B */
    uint32_t* vertex_hash;  /* [paths] hash of vertex positions + materials */
    uint32_t* dda_steps;    /* [paths] voxel steps of all NEE rays */
    float* x1;              /* [paths x 3] first vertex */
    int32_t* m1;            /* [paths] first vertex material */
    double* a_ms;           /* [paths x Nt x Nl x 2] illumination vector of the multiple-scattering term */
    double* s_ms;           /* [paths x Nt x Nv x 2] summed view vector of the multiple-scattering term */
    double* a_ss;           /* [paths x Nt x Nl x 2] illumination vector of the single-scattering term */
    double* b_ss;           /* [paths x Nt x Nv x 2] view vector of the single-scattering term */
} sstmc_path_trace;

int32_t sstmc_trace_paths(sstmc_scene* scene, uint64_t seed, uint32_t first_path,
                          uint32_t paths, sstmc_path_trace* out);

#ifdef __cplusplus
}
#endif
#endif /* SSTMC_H */
