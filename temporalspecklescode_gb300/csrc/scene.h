// scene.h -- per-scene device descriptor and its host-side construction.
//
// The reference keeps every plugin's state in process-global __constant__
// symbols (MediumNS::mediumGpuData, HeterogeneousMediumNS::*, ScatteringNS::*,
// TemporalSamplerNS::*, Simulation.cuh:168-173), which allows one scene per
// process.  Here a scene is a plain descriptor (DevScene) passed to every
// kernel by value, pointing at device buffers the Scene owns, so any number
// of scenes can be resident at once.
#pragma once
#include <vector_types.h>   // float2

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/sstmc.h"

namespace sstmc {

constexpr int kMat = SSTMC_MATERIAL_NUM;
constexpr uint32_t kMaxAttempts = 1u << 20;
constexpr uint32_t kMaxVertices = 1u << 20;
constexpr uint32_t kMaxWoodcock = 1u << 22;
constexpr double kPi = 3.14159265358979323846;
constexpr float kIsoAmp2 = 0.398942280401432678f;
constexpr float kIsoAmp3 = 0.282094791773878143f;
constexpr float kIsoPdf2 = 0.159154943091895336f;
constexpr float kIsoPdf3 = 0.079577471545947668f;

// Source element tables.  FarField: p = unit direction and the sampling
// tables of FarField.cuh:71-127 (fillBuffers).  PointSource: p = location.
struct DevSource {
    int type, n, is_area, pad;
    const float* p;      // n*3
    const float* inv;    // n*3 inverse direction
    const float* tang;   // n*3 tangent point of the blocking circle
    const float* pt;     // n*3 perpendicular T
    const float* ps;     // n*3 perpendicular S (3D)
    const float* mint;
    const float* maxt;
    const float* mins;
    const float* maxs;
    const float* sprob;  // projected-box sampling probability q_l
    // GaussianBeam (GaussianBeam.cuh, 3D): p = focal points, gdir = beam
    // directions, ga = 1 / aperture^2, gnorm = the aperture normalisation.
    // Illumination only: the focal material of each beam, per beam (tmin, tmax,
    // dt, xy base 2 x 3), the distance-bin pdf / exclusive cdf of each lobe
    // [n][gM][kGaussBins] and the lobe pdf / exclusive cdf [n][gM].
    const float* gdir;
    double ga, gnorm;
    int gM;
    int gsame;           // every beam has the same direction
    const int* gfm;
    const double* gtab;
    const double* gpdf;
    const double* gicdf;
    const double* gapdf;
    const double* gaicdf;
};

// distance bins of a Gaussian beam's first-vertex table (zSamplesNum, GaussianBeam.cuh:62-64)
constexpr int kGaussBins = 1000;

struct DevScene {
    int dims, correlation, Nt, neg;
    int temporal_amp, iso_all, precision, sym;  // sym: illumination2 == illumination and view2 == view
    int single, grid_m0;          // single-cell medium and its material
    int all_static_corr;          // no material drifts (U == 0 everywhere)
    int ticks_geometric;          // |t_k| == (k + 1) |t_0| for every tick
    int forced_bin;               // field sampler isForcedInsideBin: per-vertex tick weights in {0, 1}
    uint32_t P;
    int n[3];
    const float* ax[3];
    const unsigned char* grid;
    int scat_type[kMat];
    float g[kMat], gup[kMat], sgup[kMat], gd1[kMat], gd2[kMat];
    float sigt[kMat], accept[kMat], survive[kMat];
    float inv_maxsigt;
    float bmin[3], bmax[3], center[3], radius[3], inv_radius[3];
    int moving[kMat];
    int static_corr[kMat];       // correlation: U == 0 (shifted positions coincide)
    float D[kMat];
    float U[kMat][3];
    const float* disp_scale;     // [kMat][Nt]
    const float* disp_u;         // [kMat][Nt][3]
    const float* ticks_f;        // [Nt] raw ticks (correlation)
    const float* abs_ticks;      // [Nt]
    double inv_lambda;
    float inv_lambda_f;
    float il_h, il_l;            // 1 / lambda as a float pair (hi + lo) for float-float phases
    float k2;                    // (2 pi / lambda)^2
    float iso_amp, iso_pdf;
    DevSource src[4];            // illumination, view, illumination2, view2
    // a tabular or vMF material is present: its amplitudes and pdfs are taken
    // from an FP64 cosine through the complex-amplitude route (amp64 / pdf64)
    int has_amp64;
    // tabular scattering (Scattering.cuh:191-482): per material its entries and
    // the offset of its rows in the concatenated tables
    int tab_n[kMat], tab_off[kMat];
    const float2* tab_f;         // amplitude normalised by the cross section
    const float* tab_pdf;        // evaluation pdf |f|^2 (x sin(theta) in 3D, as the reference)
    const float* tab_cos;        // cos(icdf): the sampler's scattering cosines
    // von Mises-Fisher mixtures in 3D (Scattering.cuh:613-884): per material its
    // component count and the offsets of its components and component pairs
    int vmf_n[kMat], vmf_off[kMat], vmf_poff[kMat];
    const double* vmf_mc;        // [components][2]: mu, C + log(alpha)
    const double* vmf_pd;        // [pairs][3]: kappa = mu1 + mu2, normalised weight, log normalisation
    const float* vmf_pf;         // [pairs][3]: exclusive cdf of the weights, kappa, exp(-2 |kappa|)
    // Gaussian beams: per material its vMF lobes (mu, C + log alpha) in gmix,
    // the mean view direction, k = 2 pi / lambda, sigs per material and the
    // box depth in z (the first-point probability's normalisation)
    int gauss;
    int gmix_n[kMat], gmix_off[kMat];
    const double* gmix;
    double gmean[3];
    double gk;
    double gsigs[kMat];
    double glz;
};

// Host-owned scene: normalised config, float tables and device buffers.
struct Scene {
    sstmc_config cfg_copy;       // scalars only: its pointers are not owned and not used after creation
    int dims = 0, M = 0, Nl = 0, Nv = 0, Nt = 0;
    uint32_t P = 0, full_iter = 1, renders = 1;
    uint64_t seed = 0;
    int device = 0;
    int precision = SSTMC_PRECISION_SPLIT;
    bool correlation = false;
    // host tables (also kept for the W tables and tests)
    struct HostSource {
        int type = 0, n = 0, is_area = 0;
        std::vector<float> p, inv, tang, pt, ps, mint, maxt, mins, maxs, sprob;
        std::vector<double> sprob_d;
        std::vector<float> gdir;
        double ga = 0.0, gnorm = 0.0;
        int gM = 0;
        std::vector<int> gfm;
        std::vector<double> gtab, gpdf, gicdf, gapdf, gaicdf;
    } hsrc[4];
    std::vector<double> gmix;    // Gaussian beams: vMF lobes (mu, C + log alpha) per material
    std::vector<float> ax[3];
    std::vector<unsigned char> grid;
    std::vector<float> disp_scale, disp_u, ticks_f, abs_ticks;
    std::vector<double> ticks;
    double g_d[kMat] = { 0 };    // HG g per material (double, for the weight tables)
    std::vector<float> tab_f, tab_pdf, tab_cos;   // tabular tables (device copies in dev.tab_*)
    std::vector<double> tab_f_d;                  // normalised amplitudes (re, im) in FP64 (weight tables)
    std::vector<double> vmf_mc, vmf_pd;           // vMF tables (device copies in dev.vmf_*)
    std::vector<float> vmf_pf;
    double D_d[kMat] = { 0 };    // Brownian D per material
    DevScene dev{};
    std::vector<void*> dev_allocs;
    // materials present in the grid
    std::vector<int> materials_present;
    // last render statistics
    uint64_t last_contrib = 0, last_dda = 0, last_vertices = 0, last_paths = 0;

    ~Scene();
};

// Build (validation + tables) and upload.  Returns an SSTMC_* code.
int build_scene(const sstmc_config* cfg, Scene* s, std::string* why);

}  // namespace sstmc
