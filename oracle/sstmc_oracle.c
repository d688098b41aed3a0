/*
 * sstmc_oracle.c -- TEST INFRASTRUCTURE: CPU oracle of the NEE speckle path
 * tracer (see sstmc_oracle.h).  Tests, smoke() and the bench's CPU baseline
 * are its only callers.
 *
 * Reference files restated here (paths inside chabner/temporalSpecklesCode):
 *   estimator / loop        Implementation/Tracer/NextEventEstimation.cuh:643-1637
 *   field sampler           Implementation/Sampler/TemporalSampler.cuh:139-937, 1324-1610
 *   correlation sampler     Implementation/Sampler/TemporalSamplerCorrelation.cuh:111-1087
 *   voxel medium            Implementation/Medium/HeterogeneousMedium.cuh:257-738
 *   medium box helpers      Interface/MediumInterface.cuh:138-222, 239-266
 *   far-field source        Implementation/Source/FarField.cuh:69-263, 439-599
 *   point source            Implementation/Source/PointSource.cuh:70-446
 *   temporal source terms   Interface/SourceInterface.cuh:184-354
 *   scattering (Iso, HG)    Implementation/Scattering.cuh:484-611, 891-1261
 *   vectors / directions    VectorType.cuh:155-362
 *   config semantics        MatlabInterface.cu:712-1457, 1565-1801
 *
 * Build: gcc -O2 -fPIC -shared -fopenmp -ffp-contract=off (oracle/Makefile).
 */
#include "sstmc_oracle.h"
#include "oracle_math.h"

#include <stdlib.h>
#include <stdio.h>
#include <math.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OM SSTMC_MATERIAL_NUM
#define O_PI 3.14159265358979323846
#define O_ISO_AMP2 0.398942280401432678
#define O_ISO_AMP3 0.282094791773878143
#define O_ISO_PDF2 0.159154943091895336
#define O_ISO_PDF3 0.079577471545947668
#define O_MAX_ATTEMPTS   (1u << 20)
#define O_MAX_VERTICES   (1u << 20)
#define O_MAX_WOODCOCK   (1u << 22)

typedef struct { float x, y, z; } f3;

/* ------------------------------------------------------------------ */
/* scene                                                              */
/* ------------------------------------------------------------------ */
typedef struct {
    int type, n, is_area;
    float* p;        /* n*3 point location or unit direction (float) */
    float* inv;      /* n*3 inverse direction (far field) */
    float* tang;     /* n*3 tangent point */
    float* pt;       /* n*3 perpendicular T */
    float* ps;       /* n*3 perpendicular S (3D) */
    float* mint; float* maxt; float* mins; float* maxs;
    double* sprob;   /* n: far-field projected-box sampling probability */
    /* Gaussian beam (GaussianBeam.cuh): p = focal points, gdir = beam directions */
    float* gdir;     /* n*3 */
    double ga;       /* beam concentration 1 / aperture^2 */
    double gnorm;    /* aperture normalisation vMFnormalizationLog(ga) */
    int gM;          /* illumination: table stride, the most lobes of a focal material */
    int* gfm;        /* illumination: material at each focal point */
    double* gtab;    /* illumination: per beam tmin, tmax, dt, xy base (2 x 3) */
    double* gpdf;    /* illumination: [n][gM][B] bin pdf */
    double* gicdf;   /* illumination: [n][gM][B] exclusive bin cdf */
    double* gapdf;   /* illumination: [n][gM] lobe pdf */
    double* gaicdf;  /* illumination: [n][gM] exclusive lobe cdf */
} o_src;

typedef struct {
    int dims, M;
    int scat_type[OM];
    float g_f[OM];
    /* tabular scattering: per material entries and offset into the tables */
    int tab_n[OM], tab_off[OM];
    double* tab_f;        /* normalised amplitude (re, im) */
    double* tab_pdf;      /* evaluation pdf */
    float* tab_cos;       /* cos(icdf) of the sampler */
    /* vMF mixtures (3D): per material components and offsets; components
     * (mu, C + log alpha); pairs (kappa, weight, log normalisation); the
     * sampler's pairs (exclusive cdf, kappa, exp(-2 |kappa|)) in FP32 */
    int vmf_n[OM], vmf_off[OM], vmf_poff[OM];
    double* vmf_mc;
    double* vmf_pd;
    float* vmf_pf;
    double gup[OM], gd1[OM], gd2[OM];
    int iso_all;
    /* medium */
    int n[3];             /* edges per axis (n[2] = 0 in 2D) */
    float* ax[3];
    double* axd[3];
    unsigned char* grid;
    float sigt_f[OM], inv_maxsigt_f, accept_f[OM], survive_f[OM];
    float bmin[3], bmax[3], center[3], radius[3], inv_radius[3];
    /* sources: 0 illumination, 1 view, 2 illumination2, 3 view2 */
    o_src src[4];
    int correlation;
    int cbs;              /* field sampler with coherent backscattering (reversed paths) */
    int Nt;
    double* ticks;        /* correlation: raw ticks; */
    float* ticks_f;
    /* field temporal: sorted ticks */
    int neg;
    float* disp_scale;    /* [OM][Nt] sqrt(2 dims D |dt|) */
    float* disp_u;        /* [OM][Nt][3] dt*U */
    int moving[OM];
    double D[OM];
    float U_f[OM][3];
    int temporal_amp;
    int forced_bin;       /* field sampler isForcedInsideBin */
    double lambda;
    unsigned P, full_iter;
    /* Gaussian beams: per material its vMF lobes (mu, C + log alpha), in 2D and 3D */
    int gauss;
    int gmix_n[OM], gmix_off[OM];
    double* gmix;
    double gmean[3];      /* mean view direction (normalised) */
    double sigs_d[OM];    /* scattering coefficient per material */
} o_scene;

static void o_free_scene(o_scene* S)
{
    for (int i = 0; i < 4; ++i) {
        o_src* s = &S->src[i];
        free(s->p); free(s->inv); free(s->tang); free(s->pt); free(s->ps);
        free(s->mint); free(s->maxt); free(s->mins); free(s->maxs); free(s->sprob);
        free(s->gdir); free(s->gfm); free(s->gtab); free(s->gpdf); free(s->gicdf); free(s->gapdf); free(s->gaicdf);
    }
    free(S->gmix);
    for (int a = 0; a < 3; ++a) { free(S->ax[a]); free(S->axd[a]); }
    free(S->grid); free(S->ticks); free(S->ticks_f); free(S->disp_scale); free(S->disp_u);
    free(S->tab_f); free(S->tab_pdf); free(S->tab_cos);
    free(S->vmf_mc); free(S->vmf_pd); free(S->vmf_pf);
}

/* Far-field tables: FarField.cuh:71-127 (fillBuffers) in double, stored as float. */
static int o_prep_farfield(o_src* s, const sstmc_source_cfg* c, int dims,
                           const double bmin[3], const double bmax[3])
{
    int n = (int)c->count;
    s->p = calloc((size_t)n * 3, sizeof(float)); s->inv = calloc((size_t)n * 3, sizeof(float));
    s->tang = calloc((size_t)n * 3, sizeof(float)); s->pt = calloc((size_t)n * 3, sizeof(float));
    s->ps = calloc((size_t)n * 3, sizeof(float));
    s->mint = calloc(n, sizeof(float)); s->maxt = calloc(n, sizeof(float));
    s->mins = calloc(n, sizeof(float)); s->maxs = calloc(n, sizeof(float));
    s->sprob = calloc(n, sizeof(double));
    if (!s->p || !s->inv || !s->tang || !s->pt || !s->ps || !s->mint || !s->maxt || !s->mins || !s->maxs || !s->sprob)
        return SSTMC_ALLOCATION_ERROR;
    double center[3], radius[3];
    for (int i = 0; i < 3; ++i) { center[i] = (bmax[i] + bmin[i]) * 0.5; radius[i] = (bmax[i] - bmin[i]) * 0.5; }
    double rc = radius[0] > radius[1] ? radius[0] : radius[1];
    if (dims == 3 && radius[2] > rc) rc = radius[2];
    rc = rc + 1e-12;
    for (int k = 0; k < n; ++k) {
        double v[3] = { c->xyz[3 * k], c->xyz[3 * k + 1], dims == 3 ? c->xyz[3 * k + 2] : 0.0 };
        double nrm = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        if (!(nrm > 0.0)) return SSTMC_INVALID_CONFIG;
        double inr = 1.0 / nrm;
        double d[3] = { v[0] * inr, v[1] * inr, v[2] * inr };
        double op[3] = { -d[0], -d[1], -d[2] };
        double tg[3], T[3], Sv[3] = { 0, 0, 0 };
        for (int i = 0; i < 3; ++i) tg[i] = center[i] + rc * op[i];
        if (dims == 3) {
            if (fabs(1.0 - fabs(op[2])) <= 1e-12) {
                T[0] = 1; T[1] = 0; T[2] = 0; Sv[0] = 0; Sv[1] = 1; Sv[2] = 0;
            } else {
                T[0] = -op[1]; T[1] = op[0]; T[2] = 0.0;
                double tn = 1.0 / sqrt(T[0] * T[0] + T[1] * T[1]);
                T[0] = T[0] * tn; T[1] = T[1] * tn;
                Sv[0] = T[1] * op[2] - T[2] * op[1];
                Sv[1] = T[2] * op[0] - T[0] * op[2];
                Sv[2] = T[0] * op[1] - T[1] * op[0];
            }
        } else {
            T[0] = -op[1]; T[1] = op[0]; T[2] = 0.0;
        }
        double mnT = 0, mxT = 0, mnS = 0, mxS = 0;
        int corners = dims == 3 ? 8 : 4;
        for (int q = 0; q < corners; ++q) {
            double cc[3] = { (q & 1) ? bmax[0] : bmin[0], (q & 2) ? bmax[1] : bmin[1],
                             dims == 3 ? ((q & 4) ? bmax[2] : bmin[2]) : 0.0 };
            double pT = (cc[0] - tg[0]) * T[0] + (cc[1] - tg[1]) * T[1] + (cc[2] - tg[2]) * T[2];
            double pS = (cc[0] - tg[0]) * Sv[0] + (cc[1] - tg[1]) * Sv[1] + (cc[2] - tg[2]) * Sv[2];
            if (q == 0 || pT < mnT) mnT = pT;
            if (q == 0 || pT > mxT) mxT = pT;
            if (q == 0 || pS < mnS) mnS = pS;
            if (q == 0 || pS > mxS) mxS = pS;
        }
        for (int i = 0; i < 3; ++i) {
            s->p[3 * k + i] = (float)d[i];
            s->inv[3 * k + i] = (float)(fabs(d[i]) < 1e-12 ? 1e12 : 1.0 / d[i]);
            s->tang[3 * k + i] = (float)tg[i];
            s->pt[3 * k + i] = (float)T[i];
            s->ps[3 * k + i] = (float)Sv[i];
        }
        s->mint[k] = (float)mnT; s->maxt[k] = (float)mxT;
        s->mins[k] = (float)mnS; s->maxs[k] = (float)mxS;
        s->sprob[k] = dims == 3 ? 1.0 / ((mxT - mnT) * (mxS - mnS)) : 1.0 / (mxT - mnT);
    }
    return SSTMC_NO_ERROR;
}

static double o_vmf_log_norm(double x);
static double o_vmf_log_norm2(double x);
static int o_prep_gauss(o_scene* S);

static int o_prep_source(o_src* s, const sstmc_source_cfg* c, int dims, const double bmin[3], const double bmax[3])
{
    memset(s, 0, sizeof(*s));
    s->type = c->type; s->n = (int)c->count; s->is_area = c->is_area_source ? 1 : 0;
    if (c->type == SSTMC_SOURCE_NONE) return SSTMC_NO_ERROR;
    if (c->count == 0 || c->xyz == NULL) return SSTMC_INVALID_CONFIG;
    if (c->type == SSTMC_SOURCE_FARFIELD) return o_prep_farfield(s, c, dims, bmin, bmax);
    if (c->type == SSTMC_SOURCE_GAUSSIANBEAM) {
        if (!c->focal_direction || !(c->aperture > 0.0) || !isfinite(c->aperture)) return SSTMC_INVALID_CONFIG;
        s->gdir = calloc((size_t)s->n * 3, sizeof(float));
        if (!s->gdir) return SSTMC_ALLOCATION_ERROR;
        for (int k = 0; k < 3 * s->n; ++k) s->gdir[k] = (float)c->focal_direction[k];
        for (int k = 0; k < s->n; ++k) {   /* a beam needs a direction */
            const float* d = s->gdir + 3 * k;
            if (!(d[0] != 0.0f || d[1] != 0.0f || d[2] != 0.0f) || !isfinite(d[0]) || !isfinite(d[1]) || !isfinite(d[2]))
                return SSTMC_INVALID_CONFIG;
        }
        /* GaussianBeam.cuh:1056-1068: ga = 1 / aperture^2, the aperture normalised */
        s->ga = 1.0 / (c->aperture * c->aperture);
        s->gnorm = dims == 3 ? o_vmf_log_norm(s->ga) : o_vmf_log_norm2(s->ga);
        if (dims == 2) for (int k = 0; k < s->n; ++k) s->gdir[3 * k + 2] = 0.0f;
    } else if (c->type != SSTMC_SOURCE_POINT) {
        return SSTMC_NOT_SUPPORTED;
    }
    s->p = calloc((size_t)s->n * 3, sizeof(float));
    if (!s->p) return SSTMC_ALLOCATION_ERROR;
    for (int k = 0; k < s->n; ++k) {
        s->p[3 * k] = (float)c->xyz[3 * k];
        s->p[3 * k + 1] = (float)c->xyz[3 * k + 1];
        s->p[3 * k + 2] = dims == 3 ? (float)c->xyz[3 * k + 2] : 0.0f;
    }
    return SSTMC_NO_ERROR;
}

/* Config normalisation and validation: MatlabInterface.cu:712-1372. */
/* Tables of one tabular material, Scattering.cuh:272-384 (setTabularScattering),
 * in FP64: sampling weights |f_i|^2 (x sin(theta_i) in 3D, theta_i = i pi / (N-1)),
 * their sum S, the cross section (S / N) 2 pi (x pi in 3D), the amplitude
 * scaled by sqrt(1 / cross section), the inverse cdf as the lower bound of
 * j / (N - 1) in the running sum of the normalised weights (angle = index x
 * pi / (N - 1), 2 pi / (N - 1) in 2D), the evaluation pdf |f_n|^2 (x sin(theta_i)
 * in 3D).  The sampler keeps cos(angle) in FP32. */
static int o_tabular(const double* f, uint32_t N, int dims, double* fn, double* pdf, float* cosv)
{
    double* raw = malloc(sizeof(double) * N);
    double* cdf = malloc(sizeof(double) * N);
    if (!raw || !cdf) { free(raw); free(cdf); return SSTMC_ALLOCATION_ERROR; }
    double sum = 0.0;
    for (uint32_t i = 0; i < N; ++i) {
        double a2 = f[2 * i] * f[2 * i] + f[2 * i + 1] * f[2 * i + 1];
        raw[i] = dims == 2 ? a2 : a2 * sin(((double)i / (double)(N - 1)) * O_PI);
        sum += raw[i];
    }
    double inv = 1.0 / sum, run = 0.0;
    for (uint32_t i = 0; i < N; ++i) { run += raw[i] * inv; cdf[i] = run; }
    double cross = (sum / (double)N) * 2.0 * O_PI * (dims == 3 ? O_PI : 1.0);
    double sc = sqrt(1.0 / cross);
    for (uint32_t i = 0; i < N; ++i) {
        fn[2 * i] = f[2 * i] * sc;
        fn[2 * i + 1] = f[2 * i + 1] * sc;
        double a2 = fn[2 * i] * fn[2 * i] + fn[2 * i + 1] * fn[2 * i + 1];
        pdf[i] = dims == 2 ? a2 : a2 * sin(((double)i / (double)(N - 1)) * O_PI);
    }
    double step = (dims == 2 ? 2.0 * O_PI : O_PI) / (double)(N - 1);
    for (uint32_t j = 0; j < N; ++j) {
        double th = (double)j / (double)(N - 1);
        uint32_t lo = 0, hi = N;   /* first index with cdf >= th */
        while (lo < hi) { uint32_t mid = lo + (hi - lo) / 2; if (cdf[mid] < th) lo = mid + 1; else hi = mid; }
        cosv[j] = (float)cos((double)lo * step);
    }
    free(raw); free(cdf);
    return 0;
}

/* vMFnormalizationLog in 3D, SpecialFunctions.cuh:187-203 (kappa below 1e-12,
 * negative ones included, takes the isotropic value). */
static double o_vmf_log_norm(double x)
{
    if (x < 1e-12) return -log(4.0 * O_PI);
    if (x < 5.0) return log(x) - log(4.0 * O_PI * sinh(x));
    return log(x) - log(2.0 * O_PI) - x;
}

/* Tables of one 3D vMF mixture, Scattering.cuh:636-774 (setVonMisesFisherScattering):
 * components (mu_k, C_k + log alpha_k); pairs j = k1 + N k2 with kappa = mu_k1 + mu_k2,
 * weight exp(C'_k1 + C'_k2 - logN(kappa)) normalised to sum 1; exclusive cdf. */
static void o_vmf_tables(const double* mu, const double* c, const double* alpha, uint32_t N,
                         double* mc, double* pd, float* pf)
{
    uint32_t P = N * N;
    for (uint32_t k = 0; k < N; ++k) { mc[2 * k] = mu[k]; mc[2 * k + 1] = c[k] + log(alpha[k]); }
    double sum = 0.0;
    for (uint32_t j = 0; j < P; ++j) {
        uint32_t k1 = j % N, k2 = j / N;
        double kap = mu[k1] + mu[k2];
        double ln = o_vmf_log_norm(kap);
        double w = exp(c[k1] + log(alpha[k1]) + c[k2] + log(alpha[k2]) - ln);
        pd[3 * j] = kap; pd[3 * j + 1] = w; pd[3 * j + 2] = ln;
        sum += w;
    }
    double cdf = 0.0;
    for (uint32_t j = 0; j < P; ++j) {
        double pj = pd[3 * j + 1] / sum;
        pd[3 * j + 1] = pj;
        pf[3 * j] = (float)cdf; pf[3 * j + 1] = (float)pd[3 * j]; pf[3 * j + 2] = (float)exp(-2.0 * fabs(pd[3 * j]));
        cdf += pj;
    }
}

static int o_build_scene(const sstmc_config* cfg, o_scene* S)
{
    memset(S, 0, sizeof(*S));
    if (cfg->dims != 2 && cfg->dims != 3) return SSTMC_INVALID_CONFIG;
    int dims = S->dims = (int)cfg->dims;
    if (cfg->batch_size == 0 || cfg->full_iteration == 0) return SSTMC_INVALID_CONFIG;
    if (!(cfg->lambda > 0)) return SSTMC_INVALID_CONFIG;
    S->P = cfg->batch_size; S->full_iter = cfg->full_iteration; S->lambda = cfg->lambda;

    /* scattering: a single cell is duplicated into material 1 */
    if (cfg->scattering_num == 0 || cfg->scattering_num > OM || !cfg->scattering_type) return SSTMC_INVALID_CONFIG;
    int M = (int)cfg->scattering_num;
    for (int m = 0; m < OM; ++m) S->scat_type[m] = SSTMC_SCATTERING_NOT_DEFINED;
    size_t tab_total = 0, tab_pos = 0, vmf_comp = 0, vmf_pairs = 0, vmf_pos = 0, vmf_cpos = 0, vmf_ppos = 0;
    for (int m = 0; m < M; ++m) {
        if (cfg->scattering_type[m] == SSTMC_SCATTERING_TABULAR) {
            if (!cfg->tabular_n || !cfg->tabular_f || cfg->tabular_n[m] < 2) return SSTMC_INVALID_CONFIG;
            tab_total += cfg->tabular_n[m];
        }
        if (cfg->scattering_type[m] == SSTMC_SCATTERING_VMF_MIXTURE) {
            if (!cfg->vmf_n || !cfg->vmf_mu || !cfg->vmf_c || !cfg->vmf_alpha || cfg->vmf_n[m] < 1) return SSTMC_INVALID_CONFIG;
            vmf_comp += cfg->vmf_n[m];
            vmf_pairs += (size_t)cfg->vmf_n[m] * cfg->vmf_n[m];
        }
    }
    if (vmf_comp) {
        S->gmix = malloc(sizeof(double) * 2 * vmf_comp);
        if (!S->gmix) return SSTMC_ALLOCATION_ERROR;
        S->vmf_mc = malloc(sizeof(double) * 2 * vmf_comp);
        S->vmf_pd = malloc(sizeof(double) * 3 * vmf_pairs);
        S->vmf_pf = malloc(sizeof(float) * 3 * vmf_pairs);
        if (!S->vmf_mc || !S->vmf_pd || !S->vmf_pf) return SSTMC_ALLOCATION_ERROR;
    }
    int iso_m[OM] = { 0 };
    if (tab_total) {
        S->tab_f = malloc(sizeof(double) * 2 * tab_total);
        S->tab_pdf = malloc(sizeof(double) * tab_total);
        S->tab_cos = malloc(sizeof(float) * tab_total);
        if (!S->tab_f || !S->tab_pdf || !S->tab_cos) return SSTMC_ALLOCATION_ERROR;
    }
    for (int m = 0; m < M; ++m) {
        int ty = cfg->scattering_type[m];
        double g = (ty == SSTMC_SCATTERING_HENYEY_GREENSTEIN && cfg->scattering_g) ? cfg->scattering_g[m] : 0.0;
        if (ty != SSTMC_SCATTERING_ISOTROPIC && ty != SSTMC_SCATTERING_HENYEY_GREENSTEIN && ty != SSTMC_SCATTERING_TABULAR
            && ty != SSTMC_SCATTERING_VMF_MIXTURE)
            return SSTMC_INVALID_CONFIG;
        if (ty == SSTMC_SCATTERING_HENYEY_GREENSTEIN && !(fabs(g) < 1.0)) return SSTMC_INVALID_CONFIG;
        int toff = 0, tn = 0;
        if (ty == SSTMC_SCATTERING_TABULAR) {
            tn = (int)cfg->tabular_n[m];
            toff = (int)tab_pos;
            int e = o_tabular(cfg->tabular_f + 2 * tab_pos, (uint32_t)tn, dims, S->tab_f + 2 * tab_pos, S->tab_pdf + tab_pos, S->tab_cos + tab_pos);
            if (e) return e;
            tab_pos += (size_t)tn;
        }
        /* isIsotropicScattering per material, Scattering.cuh:1484-1512 */
        int iso = ty == SSTMC_SCATTERING_ISOTROPIC || (ty == SSTMC_SCATTERING_HENYEY_GREENSTEIN && fabs(g) < 0.0001);
        int vn = 0, voff = 0, vpoff = 0, goff = 0;
        if (ty == SSTMC_SCATTERING_VMF_MIXTURE) {
            vn = (int)cfg->vmf_n[m];
            const double *mu = cfg->vmf_mu + vmf_pos, *cc = cfg->vmf_c + vmf_pos, *al = cfg->vmf_alpha + vmf_pos;
            /* the lobes the Gaussian-beam terms read: mixtureMu and mixtureC + log(alpha)
             * (Scattering.cuh:703-721), kept in 2D too */
            goff = (int)vmf_pos;
            for (int k = 0; k < vn; ++k) { S->gmix[2 * (vmf_pos + k)] = mu[k]; S->gmix[2 * (vmf_pos + k) + 1] = cc[k] + log(al[k]); }
            vmf_pos += (size_t)vn;
            double asum = 0.0;
            iso = 1;   /* every |mu| <= 1e-4, Scattering.cuh:744-751 */
            for (int k = 0; k < vn; ++k) {
                if (!isfinite(mu[k]) || !isfinite(cc[k]) || !isfinite(al[k]) || al[k] < 0.0) return SSTMC_INVALID_CONFIG;
                asum += al[k];
                if (fabs(mu[k]) > 0.0001) iso = 0;
            }
            if (!(asum > 0.0)) return SSTMC_INVALID_CONFIG;
            if (dims == 3) {   /* 2D: scattered isotropically (Scattering.cuh:899-905, 1093-1100) */
                voff = (int)vmf_cpos; vpoff = (int)vmf_ppos;
                o_vmf_tables(mu, cc, al, (uint32_t)vn, S->vmf_mc + 2 * vmf_cpos, S->vmf_pd + 3 * vmf_ppos, S->vmf_pf + 3 * vmf_ppos);
                vmf_cpos += (size_t)vn; vmf_ppos += (size_t)vn * vn;
            }
        }
        int targets[2] = { m, 1 };
        int nt = (M == 1) ? 2 : 1;
        for (int q = 0; q < nt; ++q) {
            int mm = targets[q];
            S->tab_n[mm] = tn;
            S->tab_off[mm] = toff;
            S->vmf_n[mm] = dims == 3 ? vn : 0;
            S->vmf_off[mm] = voff;
            S->vmf_poff[mm] = vpoff;
            S->gmix_n[mm] = vn;
            S->gmix_off[mm] = goff;
            iso_m[mm] = iso;
            S->scat_type[mm] = (ty == SSTMC_SCATTERING_VMF_MIXTURE && dims == 2) ? SSTMC_SCATTERING_ISOTROPIC : ty;
            S->g_f[mm] = (float)g;
            S->gup[mm] = dims == 2 ? 2.0 * ((1.0 - g * g) / (4.0 * O_PI)) : (1.0 - g * g) / (4.0 * O_PI);
            S->gd1[mm] = 1.0 + g * g;
            S->gd2[mm] = -2.0 * g;
        }
    }
    if (M == 1) M = 2;
    S->M = M;
    /* isIsotropicScattering over the defined materials, Scattering.cuh:1514-1528 */
    S->iso_all = 1;
    for (int m = 0; m < OM; ++m)
        if (S->scat_type[m] != SSTMC_SCATTERING_NOT_DEFINED && !iso_m[m]) S->iso_all = 0;

    /* medium */
    double bmin[3] = { 0, 0, 0 }, bmax[3] = { 0, 0, 0 };
    double sigs[OM] = { 0 }, siga[OM] = { 0 };
    if (cfg->medium_type == SSTMC_MEDIUM_HOMOGENEOUS) {
        if (M != 2) return SSTMC_INVALID_CONFIG;
        for (int a = 0; a < dims; ++a) {
            if (!(cfg->box_max[a] > cfg->box_min[a])) return SSTMC_INVALID_CONFIG;
            S->n[a] = 2;
            S->axd[a] = malloc(2 * sizeof(double)); S->ax[a] = malloc(2 * sizeof(float));
            S->ax[a][0] = (float)cfg->box_min[a]; S->ax[a][1] = (float)cfg->box_max[a];
        }
        S->grid = malloc(1); S->grid[0] = 1;
        sigs[1] = cfg->homogeneous_sigs;
    } else if (cfg->medium_type == SSTMC_MEDIUM_HETEROGENEOUS) {
        const double* axes[3] = { cfg->x_axis, cfg->y_axis, cfg->z_axis };
        uint32_t sizes[3] = { cfg->x_axis_size, cfg->y_axis_size, cfg->z_axis_size };
        size_t cells = 1;
        for (int a = 0; a < dims; ++a) {
            if (!axes[a] || sizes[a] < 2) return SSTMC_INVALID_CONFIG;
            S->n[a] = (int)sizes[a];
            S->axd[a] = malloc(sizes[a] * sizeof(double)); S->ax[a] = malloc(sizes[a] * sizeof(float));
            for (uint32_t i = 0; i < sizes[a]; ++i) {
                S->ax[a][i] = (float)axes[a][i];
                if (i > 0 && !(S->ax[a][i] > S->ax[a][i - 1])) return SSTMC_INVALID_CONFIG;
            }
            cells *= (size_t)(sizes[a] - 1);
        }
        if (!cfg->material_grid || !cfg->sigs) return SSTMC_INVALID_CONFIG;
        S->grid = malloc(cells);
        for (size_t i = 0; i < cells; ++i) {
            uint32_t m = cfg->material_grid[i];
            if (m == 0 || m >= (uint32_t)M) return SSTMC_INVALID_CONFIG; /* MatlabInterface.cu:979-991 */
            S->grid[i] = (unsigned char)m;
        }
        for (int m = 0; m < M; ++m) { sigs[m] = cfg->sigs[m]; siga[m] = cfg->siga ? cfg->siga[m] : 0.0; }
    } else {
        return SSTMC_NOT_SUPPORTED;
    }
    for (int m = 0; m < OM; ++m) S->sigs_d[m] = sigs[m];
    for (int a = 0; a < dims; ++a) for (int i = 0; i < S->n[a]; ++i) S->axd[a][i] = (double)S->ax[a][i];
    for (int a = 0; a < dims; ++a) {
        S->bmin[a] = S->ax[a][0]; S->bmax[a] = S->ax[a][S->n[a] - 1];
        bmin[a] = S->axd[a][0]; bmax[a] = S->axd[a][S->n[a] - 1];
        double c = (bmax[a] + bmin[a]) * 0.5, r = (bmax[a] - bmin[a]) * 0.5;
        S->center[a] = (float)c; S->radius[a] = (float)r;
        S->inv_radius[a] = fabsf(S->radius[a]) < 1e-12f ? 1e12f : 1.0f / S->radius[a];
    }
    float maxsigt = 0.0f;
    for (int m = 0; m < OM; ++m) {
        if (sigs[m] < 0 || siga[m] < 0) return SSTMC_INVALID_CONFIG;
        float ss = (float)sigs[m], sa = (float)siga[m];
        S->sigt_f[m] = ss + sa;
        S->survive_f[m] = S->sigt_f[m] > 0.0f ? ss / S->sigt_f[m] : 1.0f;
        if (S->sigt_f[m] > maxsigt) maxsigt = S->sigt_f[m];
    }
    if (!(maxsigt > 0.0f)) return SSTMC_INVALID_CONFIG;
    S->inv_maxsigt_f = 1.0f / maxsigt;
    for (int m = 0; m < OM; ++m) S->accept_f[m] = S->sigt_f[m] / maxsigt;

    /* sources */
    const sstmc_source_cfg* sc[4] = { &cfg->illumination, &cfg->view, &cfg->illumination2, &cfg->view2 };
    for (int i = 0; i < 4; ++i) {
        int e = o_prep_source(&S->src[i], sc[i], dims, bmin, bmax);
        if (e) return e;
    }
    if (S->src[0].type == SSTMC_SOURCE_NONE || S->src[1].type == SSTMC_SOURCE_NONE) return SSTMC_INVALID_CONFIG;
    S->gauss = S->src[0].type == SSTMC_SOURCE_GAUSSIANBEAM || S->src[1].type == SSTMC_SOURCE_GAUSSIANBEAM;

    /* sampler */
    if (!cfg->t || cfg->t_num == 0) return SSTMC_INVALID_CONFIG;
    S->correlation = cfg->sampler_type == SSTMC_SAMPLER_TEMPORAL_CORRELATION;
    S->cbs = cfg->is_cbs ? 1 : 0;
    /* isForcedInsideBin exists for the field sampler only (MatlabInterface.cu:1245-1282) */
    S->forced_bin = cfg->is_forced_inside_bin && !S->correlation;
    if (cfg->sampler_type != SSTMC_SAMPLER_TEMPORAL && !S->correlation) return SSTMC_INVALID_CONFIG;
    if (S->correlation) {
        if (S->src[2].type == SSTMC_SOURCE_NONE || S->src[3].type == SSTMC_SOURCE_NONE) return SSTMC_INVALID_CONFIG;
        if (S->src[2].n != S->src[0].n || S->src[3].n != S->src[1].n) return SSTMC_INVALID_CONFIG;
        if (S->src[2].type != S->src[0].type || S->src[3].type != S->src[1].type) return SSTMC_NOT_SUPPORTED;
    }
    S->temporal_amp = cfg->is_temporal_amplitude ? 1 : 0;
    int Nt = S->Nt = (int)cfg->t_num;
    S->ticks = malloc(Nt * sizeof(double)); S->ticks_f = malloc(Nt * sizeof(float));
    for (int t = 0; t < Nt; ++t) { S->ticks[t] = cfg->t[t]; S->ticks_f[t] = (float)cfg->t[t]; }
    for (int m = 0; m < OM; ++m) {
        S->D[m] = (m < M && cfg->D) ? cfg->D[m] : 0.0;
        if (S->D[m] < 0) return SSTMC_INVALID_CONFIG; /* MatlabInterface.cu:1278-1283 */
        for (int i = 0; i < 3; ++i) S->U_f[m][i] = (m < M && cfg->U && (i < dims)) ? (float)cfg->U[3 * m + i] : 0.0f;
    }
    if (S->gauss) {
        int e = o_prep_gauss(S);
        if (e) return e;
    }
    /* field sampler: ticks sorted around the mean, TemporalSampler.cuh:958-1150 */
    S->disp_scale = calloc((size_t)OM * Nt, sizeof(float));
    S->disp_u = calloc((size_t)OM * Nt * 3, sizeof(float));
    {
        double mean = 0;
        for (int t = 0; t < Nt; ++t) mean += S->ticks[t];
        mean = mean / Nt;
        int* used = calloc(Nt, sizeof(int));
        int* negl = malloc(Nt * sizeof(int));
        int* posl = malloc(Nt * sizeof(int));
        int nn = 0, np = 0;
        for (int t = 0; t < Nt; ++t) { if (S->ticks[t] - mean < 0) nn++; else np++; }
        for (int a = 0; a < nn; ++a) {
            int first = 1, idx = 0; double best = 0;
            for (int t = 0; t < Nt; ++t) if (!used[t] && S->ticks[t] - mean < 0) {
                if (first || mean - S->ticks[t] < best) { first = 0; best = mean - S->ticks[t]; idx = t; }
            }
            used[idx] = 1; negl[a] = idx;
        }
        for (int a = 0; a < np; ++a) {
            int first = 1, idx = 0; double best = 0;
            for (int t = 0; t < Nt; ++t) if (!used[t] && S->ticks[t] - mean >= 0) {
                if (first || S->ticks[t] - mean < best) { first = 0; best = S->ticks[t] - mean; idx = t; }
            }
            used[idx] = 1; posl[a] = idx;
        }
        S->neg = nn;
        double* dt = malloc(Nt * sizeof(double));
        int cn = 0, cp = 0, prev = -1;
        for (int j = 0; j < Nt; ++j) {
            int tick;
            if (j < nn) { tick = negl[cn]; if (cn == 0) prev = -1; cn++; }
            else { tick = posl[cp]; if (cp == 0) prev = -1; cp++; }
            dt[j] = prev < 0 ? S->ticks[tick] - mean : S->ticks[tick] - S->ticks[prev];
            prev = tick;
        }
        for (int m = 0; m < OM; ++m) {
            S->moving[m] = (S->D[m] != 0.0) || S->U_f[m][0] != 0.0f || S->U_f[m][1] != 0.0f || S->U_f[m][2] != 0.0f;
            for (int j = 0; j < Nt; ++j) {
                S->disp_scale[m * Nt + j] = (float)sqrt(2.0 * dims * S->D[m] * fabs(dt[j]));
                double U[3] = { m < M && cfg->U ? cfg->U[3 * m] : 0.0, m < M && cfg->U ? cfg->U[3 * m + 1] : 0.0,
                                (m < M && cfg->U && dims == 3) ? cfg->U[3 * m + 2] : 0.0 };
                for (int i = 0; i < 3; ++i) S->disp_u[(m * Nt + j) * 3 + i] = (float)(dt[j] * U[i]);
            }
        }
        free(dt); free(used); free(negl); free(posl);
    }
    return SSTMC_NO_ERROR;
}

/* ------------------------------------------------------------------ */
/* FP32 walk (decision path)                                          */
/* ------------------------------------------------------------------ */
static inline int o_inside(const o_scene* S, const float p[3])
{
    int in = p[0] >= S->bmin[0] && p[0] <= S->bmax[0] && p[1] >= S->bmin[1] && p[1] <= S->bmax[1];
    if (S->dims == 3) in = in && p[2] >= S->bmin[2] && p[2] <= S->bmax[2];
    return in;
}

/* Cell c with ax[c] <= x < ax[c+1]; clamped to [0, n-2]
 * (Simulation.cuh:325-367 binarySearchKernel, plus the clamp at the max edge). */
static inline int o_bin(const float* ax, int n, float x)
{
    int lo = 0, hi = n; /* count of ax[k] <= x in [lo, hi] */
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (ax[mid] <= x) lo = mid + 1; else hi = mid;
    }
    int c = lo - 1;
    if (c < 0) c = 0;
    if (c > n - 2) c = n - 2;
    return c;
}

static inline int o_cell(const o_scene* S, const float p[3])
{
    int ix = o_bin(S->ax[0], S->n[0], p[0]);
    int iy = o_bin(S->ax[1], S->n[1], p[1]);
    int idx = ix + iy * (S->n[0] - 1);
    if (S->dims == 3) idx += o_bin(S->ax[2], S->n[2], p[2]) * (S->n[0] - 1) * (S->n[1] - 1);
    return idx;
}

/* Does a ray from an outside point hit the box?  HeterogeneousMedium.cuh:269-383 (bdDistance). */
/* Whether the ray from p along d hits the box; *hit = distance to the face it
 * enters first (HeterogeneousMedium.cuh:269-383, bdDistance). */
static int o_points_toward(const o_scene* S, const float p[3], const float d[3], float* hit)
{
    int D = S->dims;
    float o[3], inv[3], dist[3];
    float mx = 0.0f;
    for (int i = 0; i < D; ++i) {
        o[i] = p[i] - S->center[i];
        float a = fabsf(o[i]) * S->inv_radius[i];
        if (i == 0 || a > mx) mx = a;
        inv[i] = fabsf(d[i]) < 1e-12f ? 1e12f : 1.0f / d[i];
    }
    float winding = mx <= 1.0f ? -1.0f : 1.0f;
    for (int i = 0; i < D; ++i) {
        float sg = d[i] < 0.0f ? 1.0f : -1.0f;
        dist[i] = inv[i] * (S->radius[i] * (winding * sg) - o[i]);
    }
    for (int i = 0; i < D; ++i) {
        if (!(dist[i] >= 0.0f)) continue;
        int ok = 1;
        for (int j = 0; j < D; ++j) {
            if (j == i) continue;
            if (!(fabsf(fmaf(d[j], dist[i], o[j])) < S->radius[j])) ok = 0;
        }
        if (ok) { if (hit) *hit = dist[i]; return 1; }
    }
    return 0;
}

static inline void o_normalize32(int dims, const float v[3], float out[3])
{
    float s = dims == 3 ? fmaf(v[0], v[0], fmaf(v[1], v[1], v[2] * v[2])) : fmaf(v[0], v[0], v[1] * v[1]);
    if (!(s > 0.0f)) {
        out[0] = 0.0f; out[1] = dims == 3 ? 0.0f : 1.0f; out[2] = dims == 3 ? 1.0f : 0.0f;
        return;
    }
    float inv = 1.0f / sqrtf(s);
    out[0] = v[0] * inv; out[1] = v[1] * inv; out[2] = dims == 3 ? v[2] * inv : 0.0f;
}

static inline void o_random_direction(int dims, o_stream* rs, float out[3])
{
    if (dims == 2) {
        float s, c;
        o_sincospif(2.0f * o_uniform(rs), &s, &c);
        out[0] = s; out[1] = c; out[2] = 0.0f;
    } else {
        float sp, cp;
        o_sincospif(2.0f * o_uniform(rs), &sp, &cp);
        float ct = fmaf(o_uniform(rs), 2.0f, -1.0f);
        float st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
        out[0] = st * cp; out[1] = st * sp; out[2] = ct;
    }
}

/* Scattering::newDirection: Scattering.cuh:1039-1115, VectorType.cuh:261-282. */
static void o_rotate(const o_scene* S, const float din[3], float c, o_stream* rs, float out[3]);

static void o_sample_direction(const o_scene* S, int m, const float din[3], o_stream* rs, float out[3])
{
    int ty = S->scat_type[m];
    if (ty != SSTMC_SCATTERING_HENYEY_GREENSTEIN && ty != SSTMC_SCATTERING_TABULAR && ty != SSTMC_SCATTERING_VMF_MIXTURE) {
        o_random_direction(S->dims, rs, out);
        return;
    }
    float g = S->g_f[m];
    float c;
    if (ty == SSTMC_SCATTERING_VMF_MIXTURE) {
        /* pair by the exclusive cdf (Scattering.cuh:1065-1077); the lobe's cosine
         * by the exact inverse cdf of exp(kappa w) on [-1, 1] (the reference's
         * Wood rejection loop, VectorType.cuh:169-203, samples the same density) */
        const float* pf = S->vmf_pf + 3 * S->vmf_poff[m];
        int P = S->vmf_n[m] * S->vmf_n[m];
        float u = o_uniform(rs);
        int j = 0;
        while (j + 1 < P && pf[3 * (j + 1)] <= u) ++j;
        float kap = pf[3 * j + 1], e2k = pf[3 * j + 2];
        float v = o_uniform(rs);
        float ak = fabsf(kap);
        if (ak < 1e-4f) {
            c = v * 2.0f - 1.0f;
        } else {
            float w = 1.0f + o_logf(v + (1.0f - v) * e2k) / ak;
            if (w < -1.0f) w = -1.0f;
            c = kap < 0.0f ? -w : w;
        }
    } else if (ty == SSTMC_SCATTERING_TABULAR) {
        /* Scattering.cuh:1030-1037: icdf entry round_num(xi N, N) (Simulation.cuh:287-298) */
        int N = S->tab_n[m];
        int k = (int)rintf(o_uniform(rs) * (float)N);
        k = k < 0 ? 0 : (k >= N ? N - 1 : k);
        c = S->tab_cos[S->tab_off[m] + k];
    } else if (fabsf(g) < 0.001f) {
        c = o_uniform(rs) * 2.0f - 1.0f;
    } else {
        float xi = o_uniform(rs);
        if (S->dims == 2) {
            float a = (1.0f - g) / (1.0f + g);
            float sp, cp;
            o_sincospif(xi, &sp, &cp);
            float s2 = sp * sp;
            float ac = a * cp;
            float ac2 = ac * ac;
            c = (s2 - ac2) / (s2 + ac2);
        } else {
            float gg = g * g;
            float s = (1.0f - gg) / fmaf(2.0f * g, xi, 1.0f - g);
            c = ((1.0f + gg) - s * s) / (2.0f * g);
        }
    }
    o_rotate(S, din, c, rs, out);
}

/* The direction at cosine c to din (VectorType.cuh:207-283, vector_rotation):
 * a side (2D) or an azimuth (3D) from the stream. */
static void o_rotate(const o_scene* S, const float din[3], float c, o_stream* rs, float out[3])
{
    float sa = (o_uniform(rs) < 0.5f ? -1.0f : 1.0f) * sqrtf(fmaxf(0.0f, 1.0f - c * c));
    if (S->dims == 2) {
        out[0] = din[0] * c - din[1] * sa;
        out[1] = din[0] * sa + din[1] * c;
        out[2] = 0.0f;
    } else {
        float sphi, cphi;
        o_sincospif(2.0f * o_uniform(rs), &sphi, &cphi);
        if (fabsf(din[2]) > 1.0f - 1e-6f) {
            out[0] = sa * cphi; out[1] = sa * sphi; out[2] = c * (signbit(din[2]) ? -1.0f : 1.0f);
        } else {
            float st = sqrtf(1.0f - din[2] * din[2]);
            float nx = (din[0] * din[2]) * cphi - din[1] * sphi;
            float ny = (din[1] * din[2]) * cphi + din[0] * sphi;
            out[0] = (sa * nx) / st + din[0] * c;
            out[1] = (sa * ny) / st + din[1] * c;
            out[2] = ((-sa) * cphi) * st + din[2] * c;
        }
    }
}

/* Woodcock free flight + absorption roulette: HeterogeneousMedium.cuh:576-678.
 * Returns 0 and writes the new vertex (material 0 = left the medium or absorbed). */
static int o_woodcock(const o_scene* S, const float o[3], const float d[3], o_stream* rs, float out[3], int* mat)
{
    float dist = 0.0f;
    float p[3] = { o[0], o[1], o[2] };
    int m = 0;
    unsigned steps = 0;
    const int from_inside = o_inside(S, o);
    for (;;) {
        if (++steps > O_MAX_WOODCOCK) return SSTMC_PATH_LIMIT;
        float u = o_uniform(rs);
        dist = dist + (-o_logf(u)) * S->inv_maxsigt_f;
        for (int i = 0; i < S->dims; ++i) p[i] = fmaf(dist, d[i], o[i]);
        if (!o_inside(S, p)) {
            /* still outside on a ray that enters the box: move on to the entry
             * face (flight lengths are memoryless, so the first point inside
             * keeps its distribution); a flight that started inside the
             * (convex) box ends at its first point outside */
            float te = 0.0f;
            if (from_inside || !o_points_toward(S, p, d, &te)) break;
            dist = dist + te;
        } else {
            m = S->grid[o_cell(S, p)];
            if (o_uniform(rs) <= S->accept_f[m]) break;
        }
    }
    out[0] = p[0]; out[1] = p[1]; out[2] = S->dims == 3 ? p[2] : 0.0f;
    if (o_inside(S, p)) {
        *mat = (o_uniform(rs) > S->survive_f[m]) ? 0 : m;
    } else {
        *mat = 0;
    }
    return 0;
}

/* First vertex source sampling: FarField.cuh:129-205, PointSource.cuh:72-90. */
static void o_sample_source(const o_scene* S, const o_src* src, o_stream* rs, float x0[3], float d0[3])
{
    int D = S->dims;
    int l = (int)ceilf(o_uniform(rs) * (float)src->n) - 1;
    if (l < 0) l = 0;
    if (l > src->n - 1) l = src->n - 1;
    if (src->type != SSTMC_SOURCE_FARFIELD) {   /* point sources, and 2D beams from their focal points */
        for (int i = 0; i < 3; ++i) x0[i] = src->p[3 * l + i];
        o_random_direction(D, rs, d0);
        return;
    }
    const float* dir = src->p + 3 * l;
    float st = src->mint[l] + o_uniform(rs) * (src->maxt[l] - src->mint[l]);
    float pt[3];
    for (int i = 0; i < 3; ++i) pt[i] = src->tang[3 * l + i] + st * src->pt[3 * l + i];
    if (D == 3) {
        float ss = src->mins[l] + o_uniform(rs) * (src->maxs[l] - src->mins[l]);
        for (int i = 0; i < 3; ++i) pt[i] = pt[i] + ss * src->ps[3 * l + i];
    }
    float sh[3], dist[3];
    for (int i = 0; i < D; ++i) {
        sh[i] = pt[i] - S->center[i];
        float sg = dir[i] < 0.0f ? 1.0f : -1.0f;
        dist[i] = src->inv[3 * l + i] * (S->radius[i] * sg - sh[i]);
    }
    float bd = 0.0f;
    for (int i = 0; i < D; ++i) {
        int ok = dist[i] >= 0.0f;
        for (int j = 0; j < D && ok; ++j) {
            if (j == i) continue;
            if (!(fabsf(fmaf(dir[j], dist[i], sh[j])) < S->radius[j])) ok = 0;
        }
        if (ok) { bd = dist[i]; break; }
    }
    float step = bd + 1e-12f;
    for (int i = 0; i < 3; ++i) { x0[i] = pt[i] + step * dir[i]; d0[i] = dir[i]; }
    if (D == 2) { x0[2] = 0.0f; d0[2] = 0.0f; }
}

/* FP32 parametric voxel traversal: the decision path of
 * HeterogeneousMedium.cuh:386-573; returns the number of voxel steps. */
static uint32_t o_dda32(const o_scene* S, const float o[3], const float d[3], float* tau)
{
    int D = S->dims;
    if (tau) *tau = 0.0f;
    if (!o_inside(S, o)) return 0;
    float inv[3], sg[3];
    int bin[3];
    for (int i = 0; i < D; ++i) {
        inv[i] = fabsf(d[i]) < 1e-12f ? (d[i] >= 0.0f ? 1e12f : -1e12f) : 1.0f / d[i];
        sg[i] = d[i] < 0.0f ? -1.0f : 1.0f;
        bin[i] = o_bin(S->ax[i], S->n[i], o[i]);
    }
    float t = 0.0f, acc = 0.0f;
    uint32_t steps = 0;
    for (;;) {
        float tn[3];
        for (int i = 0; i < D; ++i) {
            float face = S->ax[i][bin[i] + (sg[i] > 0.0f ? 1 : 0)];
            tn[i] = (face - o[i]) * inv[i];
        }
        int a;
        if (D == 2) a = tn[0] < tn[1] ? 0 : 1;
        else a = (tn[0] < tn[1] && tn[0] < tn[2]) ? 0 : (tn[1] < tn[2] ? 1 : 2);
        int idx = bin[0] + bin[1] * (S->n[0] - 1);
        if (D == 3) idx += bin[2] * (S->n[0] - 1) * (S->n[1] - 1);
        acc = fmaf(tn[a] - t, S->sigt_f[S->grid[idx]], acc);
        t = tn[a];
        steps++;
        if ((sg[a] < 0.0f && bin[a] == 0) || (sg[a] > 0.0f && bin[a] == S->n[a] - 2)) break;
        bin[a] += sg[a] > 0.0f ? 1 : -1;
    }
    if (tau) *tau = acc;
    return steps;
}

/* FP64 optical depth of the same ray (value path of the oracle). */
static double o_tau64(const o_scene* S, const double o[3], const double d[3])
{
    int D = S->dims;
    for (int i = 0; i < D; ++i) if (!(o[i] >= S->axd[i][0] && o[i] <= S->axd[i][S->n[i] - 1])) return 0.0;
    double inv[3]; int sg[3], bin[3];
    for (int i = 0; i < D; ++i) {
        inv[i] = fabs(d[i]) < 1e-12 ? (d[i] >= 0.0 ? 1e12 : -1e12) : 1.0 / d[i];
        sg[i] = d[i] < 0.0 ? -1 : 1;
        int lo = 0, hi = S->n[i];
        while (lo < hi) { int mid = (lo + hi) >> 1; if (S->axd[i][mid] <= o[i]) lo = mid + 1; else hi = mid; }
        int c = lo - 1; if (c < 0) c = 0; if (c > S->n[i] - 2) c = S->n[i] - 2;
        bin[i] = c;
    }
    double t = 0.0, acc = 0.0;
    for (int guard = 0; guard < (1 << 24); ++guard) {
        double tn[3];
        for (int i = 0; i < D; ++i) tn[i] = (S->axd[i][bin[i] + (sg[i] > 0 ? 1 : 0)] - o[i]) * inv[i];
        int a;
        if (D == 2) a = tn[0] < tn[1] ? 0 : 1;
        else a = (tn[0] < tn[1] && tn[0] < tn[2]) ? 0 : (tn[1] < tn[2] ? 1 : 2);
        int idx = bin[0] + bin[1] * (S->n[0] - 1);
        if (D == 3) idx += bin[2] * (S->n[0] - 1) * (S->n[1] - 1);
        double seg = tn[a] - t;
        if (seg > 0) acc += seg * (double)S->sigt_f[S->grid[idx]];
        if (tn[a] > t) t = tn[a];
        if ((sg[a] < 0 && bin[a] == 0) || (sg[a] > 0 && bin[a] == S->n[a] - 2)) break;
        bin[a] += sg[a];
    }
    return acc;
}

/* Tabular entry of a scattering cosine: round_num(safeAcos(c) (N - 1) / pi, N),
 * 2 pi in 2D (Scattering.cuh:907-917, Simulation.cuh:274-298; round half to even,
 * clamped to the table). */
static inline int o_tab_index(const o_scene* S, int m, double c)
{
    double th = c < -1.0 + 1e-12 ? O_PI : (c > 1.0 - 1e-12 ? 0.0 : acos(c));
    int N = S->tab_n[m];
    double x = th * (double)(N - 1) / (S->dims == 2 ? 2.0 * O_PI : O_PI);
    int n = (int)nearbyint(x);
    return n < 0 ? 0 : (n >= N ? N - 1 : n);
}

/* vMF mixture, 3D: amplitude sum_k exp(c mu_k + C'_k) (Scattering.cuh:933-946),
 * pdf sum_j w_j exp(c kappa_j + logN_j) (Scattering.cuh:997-1012) */
static inline double o_vmf_amp(const o_scene* S, int m, double c)
{
    const double* p = S->vmf_mc + 2 * S->vmf_off[m];
    double r = 0.0;
    for (int k = 0; k < S->vmf_n[m]; ++k) r += exp(fma(c, p[2 * k], p[2 * k + 1]));
    return r;
}

static inline double o_vmf_pdf(const o_scene* S, int m, double c)
{
    const double* p = S->vmf_pd + 3 * S->vmf_poff[m];
    int P = S->vmf_n[m] * S->vmf_n[m];
    double r = 0.0;
    for (int j = 0; j < P; ++j) r += p[3 * j + 1] * exp(fma(c, p[3 * j], p[3 * j + 2]));
    return r;
}

/* Scattering::amplitude / pdf device implementations, Scattering.cuh:895-1023 (FP64).
 * o_amp: the real amplitudes (Isotropic, HG); o_ampc below adds the tabular one. */
static inline double o_amp(const o_scene* S, int m, double c)
{
    int ty = S->scat_type[m];
    if (ty == SSTMC_SCATTERING_ISOTROPIC) return S->dims == 2 ? O_ISO_AMP2 : O_ISO_AMP3;
    if (ty == SSTMC_SCATTERING_HENYEY_GREENSTEIN) {
        double dn = fma(S->gd2[m], c, S->gd1[m]);
        return S->dims == 2 ? sqrt(S->gup[m] / dn) : sqrt(S->gup[m] / (dn * sqrt(dn)));
    }
    if (ty == SSTMC_SCATTERING_VMF_MIXTURE) return o_vmf_amp(S, m, c);
    return 0.0;
}

static inline double o_pdf(const o_scene* S, int m, double c)
{
    int ty = S->scat_type[m];
    if (ty == SSTMC_SCATTERING_ISOTROPIC) return S->dims == 2 ? O_ISO_PDF2 : O_ISO_PDF3;
    if (ty == SSTMC_SCATTERING_VMF_MIXTURE) return o_vmf_pdf(S, m, c);
    if (ty == SSTMC_SCATTERING_TABULAR) return S->tab_pdf[S->tab_off[m] + o_tab_index(S, m, c)];
    if (ty == SSTMC_SCATTERING_HENYEY_GREENSTEIN) {
        double dn = fma(S->gd2[m], c, S->gd1[m]);
        return S->dims == 2 ? S->gup[m] / dn : S->gup[m] / (dn * sqrt(dn));
    }
    return 0.0;
}

/* ------------------------------------------------------------------ */
/* FP64 NEE helpers                                                   */
/* ------------------------------------------------------------------ */
static inline void o_norm64(const double v[3], double out[3])
{
    double s = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    if (!(s > 0)) { out[0] = 0; out[1] = 0; out[2] = 1; return; }
    double r = 1.0 / sqrt(s);
    out[0] = v[0] * r; out[1] = v[1] * r; out[2] = v[2] * r;
}

static inline void o_dir64(const float a[3], const float b[3], double out[3]) /* normalize(b - a) */
{
    double v[3] = { (double)b[0] - a[0], (double)b[1] - a[1], (double)b[2] - a[2] };
    o_norm64(v, out);
}

static inline double o_dot(const double a[3], const double b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

static inline void o_cexp2pi(double ph, double* re, double* im)
{
    double f = ph - floor(ph);
    *re = cos(2.0 * O_PI * f); *im = sin(2.0 * O_PI * f);
}

typedef struct { double re, im; } oc;
static inline oc oc_mul(oc a, oc b) { oc r = { a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re }; return r; }
static inline oc oc_conj(oc a) { oc r = { a.re, -a.im }; return r; }
static inline oc oc_scale(oc a, double s) { oc r = { a.re * s, a.im * s }; return r; }

/* complex amplitude: the tabular table entry, else the real amplitude */
static inline oc o_ampc(const o_scene* S, int m, double c)
{
    if (S->scat_type[m] == SSTMC_SCATTERING_TABULAR) {
        int i = S->tab_off[m] + o_tab_index(S, m, c);
        oc r = { S->tab_f[2 * i], S->tab_f[2 * i + 1] };
        return r;
    }
    oc r = { o_amp(S, m, c), 0.0 };
    return r;
}

typedef struct { float x[3]; int valid; oc g; uint64_t steps; } o_gmemo;

/* Optical depth of one NEE ray from float point x along float dir df (FP32 steps
 * counted; FP64 value). */
static double o_ray(const o_scene* S, const float x[3], const float df[3], const double dd[3], uint64_t* steps)
{
    *steps += o_dda32(S, x, df, NULL);
    double xd[3] = { x[0], x[1], x[2] };
    return o_tau64(S, xd, dd);
}

/* First point probability term P_l(x): FarField.cuh:469-499, PointSource.cuh:92-115, 263-294. */
static double o_gauss_pfirst(const o_scene* S, const o_src* s, int l, const float x1[3], int m1);
static oc o_gauss_g(const o_scene* S, const o_src* s, int k, const float x[3], int role, uint64_t* steps);
static oc o_gauss_f(const o_scene* S, const o_src* s, int k, const float pa[3], const float pb[3], int m, int role);
static oc o_gauss_fs(const o_scene* S, const o_src* il, int l, const o_src* vw, int v, const float xf[3], int m);

static double o_pfirst(const o_scene* S, const o_src* s, int l, const float x[3], uint64_t* steps)
{
    /* 3D beams from their tables; 2D beams as point sources at their focal
     * points (GaussianBeam.cuh:1812-1832, probabilityPointNormalizeKernel :775-793) */
    if (s->type == SSTMC_SOURCE_GAUSSIANBEAM && S->dims == 3)
        return o_gauss_pfirst(S, s, l, x, o_inside(S, x) ? S->grid[o_cell(S, x)] : 0);
    if (s->type == SSTMC_SOURCE_FARFIELD) {
        float df[3] = { -s->p[3 * l], -s->p[3 * l + 1], -s->p[3 * l + 2] };
        double dd[3] = { df[0], df[1], df[2] };
        return exp(-o_ray(S, x, df, dd, steps)) * s->sprob[l];
    }
    const float* sp = s->p + 3 * l;
    float diff[3] = { sp[0] - x[0], sp[1] - x[1], sp[2] - x[2] };
    float df[3]; o_normalize32(S->dims, diff, df);
    double dd[3]; o_dir64(x, sp, dd);
    double T = exp(-o_ray(S, x, df, dd, steps));
    double v[3] = { (double)x[0] - sp[0], (double)x[1] - sp[1], (double)x[2] - sp[2] };
    double r = sqrt(o_dot(v, v));
    return S->dims == 3 ? T / (4.0 * O_PI * r * r) : T * (8.0 * O_PI) / r;
}

/* NEE vector g at x for source element k: FarField.cuh:223-263 (gDirectionKernel),
 * PointSource.cuh:117-172 (gPointKernel).  role: 0 illumination, 1 view. */
static oc o_g(const o_scene* S, const o_src* s, int k, const float x[3], int role, uint64_t* steps)
{
    oc g;
    if (s->type == SSTMC_SOURCE_GAUSSIANBEAM) return o_gauss_g(S, s, k, x, role, steps);
    if (s->type == SSTMC_SOURCE_FARFIELD) {
        const float* d = s->p + 3 * k;
        float sgn = role == 0 ? -1.0f : 1.0f;
        float df[3] = { sgn * d[0], sgn * d[1], sgn * d[2] };
        double dd[3] = { df[0], df[1], df[2] };
        double T = exp(-o_ray(S, x, df, dd, steps));
        double dx = (double)d[0] * x[0] + (double)d[1] * x[1] + (double)d[2] * x[2];
        double ph = (role == 0 ? 1.0 : -1.0) * dx / S->lambda;
        double a = sqrt(T);
        o_cexp2pi(ph, &g.re, &g.im);
        g.re *= a; g.im *= a;
        return g;
    }
    const float* sp = s->p + 3 * k;
    float diff[3] = { sp[0] - x[0], sp[1] - x[1], sp[2] - x[2] };
    float df[3]; o_normalize32(S->dims, diff, df);
    double dd[3]; o_dir64(x, sp, dd);
    double T = exp(-o_ray(S, x, df, dd, steps));
    double v[3] = { (double)x[0] - sp[0], (double)x[1] - sp[1], (double)x[2] - sp[2] };
    double r = sqrt(o_dot(v, v));
    double at = S->dims == 3 ? T * O_ISO_AMP3 / (r * r) : T / r;
    if (s->is_area) at *= (S->dims == 3 ? fabs(v[2]) : fabs(v[1])) / r;
    double a = sqrt(at);
    o_cexp2pi(r / S->lambda, &g.re, &g.im);
    g.re *= a; g.im *= a;
    return g;
}

/* Memoised o_g: the NEE vector is a pure function of (source slot, element,
 * position); a tick-invariant vertex reuses it and its DDA step count. */
static oc o_gm(const o_scene* S, o_gmemo* memo, const o_src* s, int k, const float x[3], int role, uint64_t* steps)
{
    o_gmemo* e = memo + k;
    if (e->valid && e->x[0] == x[0] && e->x[1] == x[1] && e->x[2] == x[2]) {
        *steps += e->steps;
        return e->g;
    }
    uint64_t st = 0;
    oc g = o_g(S, s, k, x, role, &st);
    e->x[0] = x[0]; e->x[1] = x[1]; e->x[2] = x[2]; e->valid = 1; e->g = g; e->steps = st;
    *steps += st;
    return g;
}

/* Incoming direction from source element k to scatterer x (illumination side):
 * far field d_k, point normalize(x - s_k).  For the view side the outgoing
 * direction toward the view: far d_k, point normalize(s_k - x). */
static void o_src_dir(const o_src* s, int k, const float x[3], int toward_source, double out[3])
{
    if (s->type == SSTMC_SOURCE_FARFIELD) {
        out[0] = s->p[3 * k]; out[1] = s->p[3 * k + 1]; out[2] = s->p[3 * k + 2];
        return;
    }
    if (toward_source) o_dir64(x, s->p + 3 * k, out);
    else o_dir64(s->p + 3 * k, x, out);
}

/* Source -> scatterer a -> point b amplitude (threePointFunction):
 * FarField.cuh:546-554, PointSource.cuh:317-345.  role 0 illumination, 1 view. */
static oc o_f3(const o_scene* S, const o_src* s, int k, const float a[3], const float b[3], int m, int role)
{
    if (s->type == SSTMC_SOURCE_GAUSSIANBEAM) return o_gauss_f(S, s, k, a, b, m, role);
    double ab[3]; o_dir64(a, b, ab);
    if (s->type == SSTMC_SOURCE_FARFIELD) {
        double d[3] = { s->p[3 * k], s->p[3 * k + 1], s->p[3 * k + 2] };
        double c = o_dot(d, ab);
        return o_ampc(S, m, role == 0 ? c : -c);
    }
    if (S->iso_all) { oc r = { S->dims == 2 ? O_ISO_AMP2 : O_ISO_AMP3, 0.0 }; return r; }
    double in[3]; o_dir64(s->p + 3 * k, a, in);
    return o_ampc(S, m, o_dot(in, ab));
}

/* Single-scattering amplitude illumination l -> x -> view v (threePointFunctionSingle):
 * FarField.cuh:556-599, PointSource.cuh:347-405. */
static oc o_fs(const o_scene* S, const o_src* il, int l, const o_src* vw, int v, const float x[3], int m)
{
    if (il->type == SSTMC_SOURCE_GAUSSIANBEAM) return o_gauss_fs(S, il, l, vw, v, x, m);
    if (il->type == SSTMC_SOURCE_POINT && S->iso_all) { oc r = { S->dims == 2 ? O_ISO_AMP2 : O_ISO_AMP3, 0.0 }; return r; }
    double in[3], out[3];
    if (il->type == SSTMC_SOURCE_FARFIELD) { in[0] = il->p[3 * l]; in[1] = il->p[3 * l + 1]; in[2] = il->p[3 * l + 2]; }
    else o_dir64(il->p + 3 * l, x, in);
    if (vw->type == SSTMC_SOURCE_FARFIELD) { out[0] = vw->p[3 * v]; out[1] = vw->p[3 * v + 1]; out[2] = vw->p[3 * v + 2]; }
    else o_dir64(x, vw->p + 3 * v, out);
    return o_ampc(S, m, o_dot(in, out));
}

/* ------------------------------------------------------------------ */
/* Gaussian beams (3D): Implementation/Source/GaussianBeam.cuh        */
/* ------------------------------------------------------------------ */
#define O_GB_BINS 1000   /* zSamplesNum, GaussianBeam.cuh:62-64 */

static inline oc oc_add(oc a, oc b) { oc r = { a.re + b.re, a.im + b.im }; return r; }
static inline oc oc_sub(oc a, oc b) { oc r = { a.re - b.re, a.im - b.im }; return r; }
static inline double oc_abs(oc a) { return sqrt(a.re * a.re + a.im * a.im); }
static inline oc oc_div(oc a, oc b)
{
    double d = b.re * b.re + b.im * b.im;
    oc r = { (a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d };
    return r;
}
static inline oc oc_exp(oc a)
{
    double e = exp(a.re);
    oc r = { e * cos(a.im), e * sin(a.im) };
    return r;
}
/* principal square root by the half-angle form of ComplexType.cuh:109-131:
 * s = sqrt((|re| + |z|) / 2); (s, im / 2s) for re >= 0, else (|im| / 2s, +-s) */
static inline oc oc_sqrt(oc a)
{
    oc r = { 0.0, 0.0 };
    if (a.re == 0.0 && a.im == 0.0) return r;
    double s = sqrt((fabs(a.re) + oc_abs(a)) * 0.5);
    if (a.re >= 0.0) { r.re = s; r.im = a.im / (2.0 * s); }
    else { r.re = fabs(a.im) / (2.0 * s); r.im = copysign(s, a.im); }
    return r;
}
/* 1 / sqrt(z) (ComplexType.cuh:133-146): the conjugate of the root over |root|^2 */
static inline oc oc_rsqrt(oc a)
{
    double s2 = (fabs(a.re) + oc_abs(a)) * 0.5;
    double mult = 1.0 / (s2 + (a.im * a.im) / (4.0 * s2));
    double s = sqrt(s2);
    oc r;
    if (a.re >= 0.0) { r.re = s * mult; r.im = -a.im * mult / (2.0 * s); }
    else { r.re = fabs(a.im) * mult / (2.0 * s); r.im = copysign(s * mult, -a.im); }
    return r;
}
/* e^(c + z) - e^(c - z), each exponential dropped when its real part is at or
 * below -10 (ComplexType.cuh:170-209, complex2timesSinh) */
static inline oc oc_2sinh(oc z, oc c)
{
    oc p = oc_add(c, z), n = oc_sub(c, z), r = { 0.0, 0.0 };
    if (p.re > -10.0) r = oc_add(r, oc_exp(p));
    if (n.re > -10.0) r = oc_sub(r, oc_exp(n));
    return r;
}
/* sum_i (a v_i + T_i)^2 over the three axes, a real, v real, T complex */
static inline oc o_gsumsq(double a, const double v[3], const oc T[3])
{
    oc r = { 0.0, 0.0 };
    for (int i = 0; i < 3; ++i) {
        double x = a * v[i] + T[i].re, y = T[i].im;
        r.re += x * x - y * y; r.im += 2.0 * x * y;
    }
    return r;
}
/* The beam's complex throughput ga d + i k (x - f) (GaussianBeam.cuh:530-532, 845-846) */
static inline void o_gthroughput(const o_src* s, int l, const double x[3], double k, oc T[3])
{
    for (int i = 0; i < 3; ++i) {
        T[i].re = (double)s->gdir[3 * l + i] * s->ga;
        T[i].im = k * (x[i] - (double)s->p[3 * l + i]);
    }
}

/* Complex modified Bessel function I0 (SpecialFunctions.cuh:42-178, besseli with
 * nu = 0): the power series sum_k ((z/2)^2)^k / (k!)^2 to k = 20 for |z| < 5
 * (the limit 3 + 2 sqrt(nu + 1)), else I0(z) = J0(iz) in the modulus-phase
 * asymptotic form of Abramowitz & Stegun 9.2.28-9.2.31 (y = iz, mu = 4 nu^2 = 0):
 * J0(y) = M cos(theta), M^2 = (2 / pi y) sum_k c_k prod_j (mu - (2j - 1)^2) / (2y)^(2k)
 * with c_k = (2k - 1)!! / (2k)!! up to k = 10, stopping once |(2y)^(2k)| or the
 * product exceeds 1e20, and theta = y - pi/4 + four terms in 1 / (4y).  I0(0) = 1
 * (the reference's form evaluates 0 log 0 there). */
static oc o_bessel_i0(oc z)
{
    double az = oc_abs(z);
    if (az == 0.0) { oc one = { 1.0, 0.0 }; return one; }
    if (az < 5.0) {
        oc h = { 0.5 * z.re, 0.5 * z.im };
        oc Y = { (h.re - h.im) * (h.re + h.im), 2.0 * h.re * h.im };
        oc Bk = { 1.0, 0.0 }, res = { 1.0, 0.0 };
        for (int k = 1; k <= 20; ++k) {
            double d = (double)k * (double)k;
            oc Zk = { Y.re / d, Y.im / d };
            Bk = oc_mul(Zk, Bk);
            res = oc_add(res, Bk);
        }
        return res;
    }
    const double mu = 0.0;
    oc y = { -z.im, z.re };                              /* i z */
    oc den = { 4.0 * y.re, 4.0 * y.im };
    oc den2 = oc_mul(den, den);
    oc th = { y.re - 0.25 * O_PI, y.im };
    const double tc[4] = { (mu - 1.0) / 2.0, (mu - 1.0) * (mu - 25.0) / 6.0,
                           (mu - 1.0) * (mu * mu - 114.0 * mu + 1073.0) / 5.0,
                           (mu - 1.0) * (5.0 * mu * mu * mu - 1535.0 * mu * mu + 54703.0 * mu - 375733.0) / 14.0 };
    for (int i = 0; i < 4; ++i) {
        oc one = { tc[i], 0.0 };
        th = oc_add(th, oc_div(one, den));
        den = oc_mul(den, den2);
    }
    oc ct = { cos(th.re) * cosh(th.im), -sin(th.re) * sinh(th.im) };
    oc M2 = { 1.0, 0.0 };
    oc t2 = { 2.0 * y.re, 2.0 * y.im };
    oc tq = oc_mul(t2, t2), tq1 = tq;
    double mm = mu - 1.0, ck = 1.0;
    for (int k = 1; k <= 10; ++k) {
        ck = ck * (2.0 * k - 1.0) / (2.0 * k);
        oc num = { ck * mm, 0.0 };
        M2 = oc_add(M2, oc_div(num, tq));
        tq = oc_mul(tq, tq1);
        mm *= mu - (2.0 * k + 1.0) * (2.0 * k + 1.0);
        if (oc_abs(tq) > 1e20 || mm > 1e20) break;
    }
    oc q = oc_div(M2, y);
    q.re *= 2.0 / O_PI; q.im *= 2.0 / O_PI;
    return oc_mul(oc_sqrt(q), ct);
}

static inline oc oc_log(oc a) { oc r = { log(oc_abs(a)), atan2(a.im, a.re) }; return r; }

/* vMFnormalizationLog in 2D (SpecialFunctions.cuh:187-203): -log(2 pi) - log I0(x) */
static double o_vmf_log_norm2(double x)
{
    oc z = { x, 0.0 };
    return -log(2.0 * O_PI) - log(oc_abs(o_bessel_i0(z)));
}

/* Lobe-pair proposal of the second direction for beam l at x1 (computeCdfBuffer,
 * GaussianBeam.cuh:489-621): per pair j = i1 + M i2 of the focal material's lobes
 * the summed real mean direction conv[j], log C[j] (1 / (4 pi) below kappa = 1e-4,
 * as the reference) and the normalised weight w[j]. */
static void o_gauss_pairs(const o_scene* S, const o_src* s, int l, const float x1[3], double* conv, double* logC, double* w)
{
    int fm = s->gfm[l], M = S->gmix_n[fm];
    const double* mix = S->gmix + 2 * S->gmix_off[fm];
    double k = 2.0 * O_PI / S->lambda;
    double x[3] = { x1[0], x1[1], x1[2] };
    oc T[3]; o_gthroughput(s, l, x, k, T);
    double lc[64], lv[64][3];   /* per lobe: c and the real mean (M <= 8) */
    for (int i = 0; i < M; ++i) {
        double mu = mix[2 * i];
        if (fabs(mu) < 1e-9) {
            double z0[3] = { 0, 0, 0 };
            oc C = oc_sqrt(o_gsumsq(0.0, z0, T));
            lc[i] = C.re - log(oc_abs(C)) + mix[2 * i + 1];
            lv[i][0] = lv[i][1] = lv[i][2] = 0.0;
        } else {
            oc g0 = oc_rsqrt(o_gsumsq(mu, S->gmean, T));
            g0.re *= mu; g0.im *= mu;
            double cv[3];
            for (int a = 0; a < 3; ++a) cv[a] = g0.re * T[a].re - g0.im * T[a].im;
            double r = 1.0 / sqrt(cv[0] * cv[0] + cv[1] * cv[1] + cv[2] * cv[2]);
            double wv[3] = { r * cv[0], r * cv[1], r * cv[2] };
            oc C = oc_sqrt(o_gsumsq(mu, wv, T));
            lc[i] = C.re - log(oc_abs(C)) + mix[2 * i + 1] - (wv[0] * cv[0] + wv[1] * cv[1] + wv[2] * cv[2]);
            lv[i][0] = cv[0]; lv[i][1] = cv[1]; lv[i][2] = cv[2];
        }
    }
    double sum = 0.0;
    for (int j = 0; j < M * M; ++j) {
        int i1 = j % M, i2 = j / M;
        double* cj = conv + 3 * j;
        for (int a = 0; a < 3; ++a) cj[a] = lv[i1][a] + lv[i2][a];
        double kap = sqrt(cj[0] * cj[0] + cj[1] * cj[1] + cj[2] * cj[2]);
        logC[j] = kap < 1e-4 ? 1.0 / (4.0 * O_PI) : o_vmf_log_norm(kap);
        w[j] = exp(lc[i1] + lc[i2] - logC[j] - 2.0 * s->ga);
        sum += w[j];
    }
    for (int j = 0; j < M * M; ++j) w[j] /= sum;
}

/* Largest i < n with cdf[i] <= u (cdf[0] = 0; Simulation.cuh:325-367 up to ties) */
static inline int o_cdf_pick(const double* cdf, int n, double u)
{
    int lo = 0, hi = n;
    while (hi - lo > 1) { int mid = (lo + hi) >> 1; if (cdf[mid] <= u) lo = mid; else hi = mid; }
    return lo;
}

/* Standard normal from two uniforms (Box-Muller, the cosine branch), in the
 * portable FP32 functions of the walk */
static inline float o_normal(o_stream* rs)
{
    float u1 = o_uniform(rs), u2 = o_uniform(rs);
    float r = sqrtf(-2.0f * o_logf(u1));
    float sn, cs;
    o_sincospif(2.0f * u2, &sn, &cs);
    return r * cs;
}

/* First vertex from a beam (sampleFirstBeam, GaussianBeam.cuh:357-418): a beam
 * uniformly, a lobe of the focal material by its cdf, a distance bin by the
 * lobe's cdf and a uniform offset in it, then a transverse Gaussian offset of
 * variance w^2(dz) = (ga + |mu|) / k^2 + dz^2 / ga in the beam's xy base.  The
 * previous point is one unit back along the beam.  Double arithmetic, the
 * vertex rounded to float. */
static void o_gauss_first(const o_scene* S, const o_src* s, o_stream* rs, float x0[3], float x1[3], int* beam)
{
    int n = s->n;
    int l = (int)ceilf(o_uniform(rs) * (float)n) - 1;
    if (l < 0) l = 0;
    if (l > n - 1) l = n - 1;
    *beam = l;
    int fm = s->gfm[l], M = S->gmix_n[fm];
    const double* mix = S->gmix + 2 * S->gmix_off[fm];
    const double* tb = s->gtab + 9 * l;
    int m = o_cdf_pick(s->gaicdf + (size_t)l * s->gM, M, (double)o_uniform(rs));
    int b = o_cdf_pick(s->gicdf + ((size_t)l * s->gM + m) * O_GB_BINS, O_GB_BINS, (double)o_uniform(rs));
    double uo = (double)o_uniform(rs);
    double d[3], f[3], z[3];
    for (int i = 0; i < 3; ++i) { d[i] = s->gdir[3 * l + i]; f[i] = s->p[3 * l + i]; }
    double t = tb[0] + (double)b * tb[2];
    double step = uo * tb[2];
    for (int i = 0; i < 3; ++i) z[i] = (f[i] + t * d[i]) + step * d[i];
    double k = 2.0 * O_PI / S->lambda;
    double dz = (z[0] - f[0]) * d[0] + (z[1] - f[1]) * d[1] + (z[2] - f[2]) * d[2];
    double wz = sqrt((s->ga + fabs(mix[2 * m])) / (k * k) + dz * dz / s->ga);
    double n1 = (double)o_normal(rs), n2 = (double)o_normal(rs);
    for (int i = 0; i < 3; ++i) {
        x1[i] = (float)(z[i] + wz * (n1 * tb[3 + i] + n2 * tb[6 + i]));
        x0[i] = x1[i] - s->gdir[3 * l + i];
    }
}

/* Projection distance of p on the line f + t d (MediumInterface.cuh:138-153) */
static inline double o_gproj(const double p[3], const double f[3], const double d[3])
{
    double o[3];
    for (int i = 0; i < 3; ++i)
        o[i] = d[i] * d[0] * (p[0] - f[0]) + d[i] * d[1] * (p[1] - f[1]) + d[i] * d[2] * (p[2] - f[2]);
    return o[0] * d[0] + o[1] * d[1] + o[2] * d[2];
}

/* P_l(x) of a beam (firstPointProbabilityKernel, GaussianBeam.cuh:420-487): the
 * bin pdf at x's axial offset times the transverse Gaussian, summed over the
 * focal material's lobes with their weights, over sigs(x) (box depth in z). */
static double o_gauss_pfirst(const o_scene* S, const o_src* s, int l, const float x1[3], int m1)
{
    int fm = s->gfm[l], M = S->gmix_n[fm];
    const double* mix = S->gmix + 2 * S->gmix_off[fm];
    const double* tb = s->gtab + 9 * l;
    double d[3], f[3], x[3];
    for (int i = 0; i < 3; ++i) { d[i] = s->gdir[3 * l + i]; f[i] = s->p[3 * l + i]; x[i] = x1[i]; }
    double dz = o_gproj(x, f, d);
    double dxy2 = 0.0;
    for (int i = 0; i < 3; ++i) { double e = f[i] + dz * d[i] - x[i]; dxy2 += e * e; }
    int zi;
    if (dz < tb[0]) zi = 0;
    else if (dz > tb[1]) zi = O_GB_BINS - 1;
    else { zi = (int)((dz - tb[0]) / tb[2]); if (zi < 0) zi = 0; if (zi > O_GB_BINS - 1) zi = O_GB_BINS - 1; }
    double k = 2.0 * O_PI / S->lambda;
    double pdf = 0.0;
    for (int m = 0; m < M; ++m) {
        double pz = s->gpdf[((size_t)l * s->gM + m) * O_GB_BINS + zi];
        double w2 = (s->ga + fabs(mix[2 * m])) / (k * k) + dz * dz / s->ga;
        double pxy = exp(-dxy2 / (2.0 * w2)) / ((2.0 * w2) * O_PI);
        pdf += s->gapdf[(size_t)l * s->gM + m] * pz * pxy;
    }
    return pdf / (S->sigs_d[m1] * ((double)S->bmax[2] - (double)S->bmin[2]));
}

/* Second direction at x1 for the path's beam (sampleCdfBuffer, GaussianBeam.cuh:
 * 636-690): a lobe pair by a running-sum scan whose step back after the loop is
 * kept, then a vMF direction about the pair's mean (the exact inverse cdf of the
 * cosine, as for vMF scattering) */
static void o_gauss_second_dir(const o_scene* S, const o_src* s, int l, const float x1[3], o_stream* rs, float out[3])
{
    int M = S->gmix_n[s->gfm[l]], P = M * M;
    double conv[3 * 64], logC[64], w[64];
    o_gauss_pairs(S, s, l, x1, conv, logC, w);
    float u = o_uniform(rs);
    double cdf = 0.0;
    int j;
    for (j = 0; j < P; ++j) {
        if ((double)u < cdf) break;
        cdf += w[j];
    }
    j--;
    const double* cj = conv + 3 * j;
    double kap = sqrt(cj[0] * cj[0] + cj[1] * cj[1] + cj[2] * cj[2]);
    float cen[3];
    if (kap < 1e-4) { cen[0] = 0.0f; cen[1] = 0.0f; cen[2] = 1.0f; }
    else for (int a = 0; a < 3; ++a) cen[a] = (float)(cj[a] / kap);
    float kf = (float)kap;
    float v = o_uniform(rs);
    float c;
    if (kf < 1e-4f) {
        c = v * 2.0f - 1.0f;
    } else {
        float e2k = (float)exp(-2.0 * (double)kf);
        c = 1.0f + o_logf(v + (1.0f - v) * e2k) / kf;
        if (c < -1.0f) c = -1.0f;
    }
    o_rotate(S, cen, c, rs, out);
}

/* p2 factor of beam l for the direction x1 -> x2 (sampleDirectionProbability,
 * GaussianBeam.cuh:693-753): sum_j w_j exp(conv_j . o + log C_j) */
static double o_gauss_pw(const o_scene* S, const o_src* s, int l, const float x1[3], const float x2[3])
{
    int P = S->gmix_n[s->gfm[l]] * S->gmix_n[s->gfm[l]];
    double conv[3 * 64], logC[64], w[64];
    o_gauss_pairs(S, s, l, x1, conv, logC, w);
    double o[3]; o_dir64(x1, x2, o);
    double r = 0.0;
    for (int j = 0; j < P; ++j) r += w[j] * exp(conv[3 * j] * o[0] + conv[3 * j + 1] * o[1] + conv[3 * j + 2] * o[2] + logC[j]);
    return r;
}

/* NEE vector of a beam: sqrt of the attenuation along the beam axis from x,
 * backward for an illumination, forward for a view (throughputFunction,
 * GaussianBeam.cuh:795-816, 1942-1965) */
static oc o_gauss_g(const o_scene* S, const o_src* s, int k, const float x[3], int role, uint64_t* steps)
{
    float sg = role == 0 ? -1.0f : 1.0f;
    float df[3] = { sg * s->gdir[3 * k], sg * s->gdir[3 * k + 1], sg * s->gdir[3 * k + 2] };
    double dd[3] = { df[0], df[1], df[2] };
    oc g = { sqrt(exp(-o_ray(S, x, df, dd, steps))), 0.0 };
    return g;
}

/* Beam -> scatterer pa -> pb amplitude (fGaussianBeam, GaussianBeam.cuh:818-892):
 * sum over pa's lobes of 2 sinh(sqrt(mu)) e^(log nu) / sqrt(mu), mu = sum (g w0 +
 * ga d + i k (pa - f))^2, w0 the path direction out of pa (illumination) or into
 * pa (view, with k negative), log nu = aperture normalisation + log 2 pi + C'. */
static oc o_gauss_f(const o_scene* S, const o_src* s, int k, const float pa[3], const float pb[3], int m, int role)
{
    oc acc = { 0.0, 0.0 };
    if (m <= 0) return acc;
    double w0[3];
    if (role == 0) o_dir64(pa, pb, w0);
    else o_dir64(pb, pa, w0);
    double kk = (role == 0 ? 2.0 : -2.0) * O_PI / S->lambda;
    double x[3] = { pa[0], pa[1], pa[2] };
    oc T[3]; o_gthroughput(s, k, x, kk, T);
    double tc = s->gnorm + log(2.0 * O_PI);
    const double* mix = S->gmix + 2 * S->gmix_off[m];
    for (int i = 0; i < S->gmix_n[m]; ++i) {
        oc lnu = { tc + mix[2 * i + 1], 0.0 };
        oc sm = oc_sqrt(o_gsumsq(mix[2 * i], w0, T));
        if (S->dims == 2) acc = oc_add(acc, oc_exp(oc_add(oc_log(o_bessel_i0(sm)), lnu)));
        else if (fabs(sm.re) < 0.0001 && fabs(sm.im) < 0.0001) acc.re += 2.0 * exp(lnu.re);
        else acc = oc_add(acc, oc_div(oc_2sinh(sm, lnu), sm));
    }
    return acc;
}

/* Illumination beam l -> x -> view beam v (fsGaussianBeam, GaussianBeam.cuh:894-999):
 * the lobe convolved with the illumination throughput, then integrated against the
 * view's. */
static oc o_gauss_fs(const o_scene* S, const o_src* il, int l, const o_src* vw, int v, const float xf[3], int m)
{
    oc acc = { 0.0, 0.0 };
    double k = 2.0 * O_PI / S->lambda;
    double x[3] = { xf[0], xf[1], xf[2] };
    oc aT[3], bT[3];
    o_gthroughput(il, l, x, k, aT);
    for (int i = 0; i < 3; ++i) {
        bT[i].re = (double)vw->gdir[3 * v + i] * vw->ga;
        bT[i].im = k * ((double)vw->p[3 * v + i] - x[i]);
    }
    double vd[3] = { vw->gdir[3 * v], vw->gdir[3 * v + 1], vw->gdir[3 * v + 2] };
    double tc = il->gnorm + vw->gnorm + 2.0 * log(2.0 * O_PI);
    const double* mix = S->gmix + 2 * S->gmix_off[m];
    double z0[3] = { 0, 0, 0 };
    for (int i = 0; i < S->gmix_n[m]; ++i) {
        double gs = mix[2 * i];
        oc lnu = { tc + mix[2 * i + 1], 0.0 };
        oc C, sm, c = { 0.0, 0.0 };
        if (fabs(gs) < 0.000001) {
            C = oc_sqrt(o_gsumsq(0.0, z0, aT));
            sm = oc_sqrt(o_gsumsq(0.0, z0, bT));
        } else {
            oc g0 = oc_rsqrt(o_gsumsq(gs, vd, aT));
            g0.re *= gs; g0.im *= gs;
            /* sqrt(sum (g0 aT + bT)^2), g0 complex */
            oc q = { 0.0, 0.0 };
            double wv[3];
            oc aw = { 0.0, 0.0 };
            for (int a = 0; a < 3; ++a) {
                oc e = oc_add(oc_mul(g0, aT[a]), bT[a]);
                q = oc_add(q, oc_mul(e, e));
                wv[a] = g0.re * aT[a].re - g0.im * aT[a].im;
            }
            sm = oc_sqrt(q);
            double ra = 1.0 / sqrt(wv[0] * wv[0] + wv[1] * wv[1] + wv[2] * wv[2]);
            C = oc_sqrt(o_gsumsq(gs * ra, wv, aT));
            for (int a = 0; a < 3; ++a) { aw.re += aT[a].re * wv[a]; aw.im += aT[a].im * wv[a]; }
            c = oc_mul(g0, aw);
            c.re *= -ra; c.im *= -ra;
        }
        oc cl = oc_add(c, lnu);
        if (S->dims == 2) {
            acc = oc_add(acc, oc_exp(oc_add(oc_add(oc_log(o_bessel_i0(C)), oc_log(o_bessel_i0(sm))), cl)));
            continue;
        }
        int sbig = fabs(sm.re) > 0.0001 || fabs(sm.im) > 0.0001;
        int cbig = fabs(C.re) > 0.0001 || fabs(C.im) > 0.0001;
        if (sbig && cbig) {
            acc = oc_add(acc, oc_div(oc_2sinh(oc_add(C, sm), cl), oc_mul(C, sm)));
        } else if (!sbig && !cbig) {
            oc e = oc_exp(cl);
            acc.re += 4.0 * e.re; acc.im += 4.0 * e.im;
        } else if (!sbig) {
            oc e = oc_div(oc_2sinh(C, cl), C);
            acc.re += 2.0 * e.re; acc.im += 2.0 * e.im;
        } else {
            oc e = oc_div(oc_2sinh(sm, lnu), sm);
            acc.re += 2.0 * e.re; acc.im += 2.0 * e.im;
        }
    }
    return acc;
}

/* Scene tables of the beams (GaussianBeam.cuh:1029-1228, 1284-1566): the
 * requirements, the mean view direction, and per illumination beam its focal
 * material, axial range over the box, xy base, the distance-bin pdf and cdf of
 * each lobe (attenuation at the bin point along the first beam's backward
 * direction, as the reference's attenuationDirection call with one direction
 * computes it, over w^2) and the lobe weights. */
static int o_prep_gauss(o_scene* S)
{
    o_src* il = &S->src[0];
    o_src* vw = &S->src[1];
    if (il->type != SSTMC_SOURCE_GAUSSIANBEAM || vw->type != SSTMC_SOURCE_GAUSSIANBEAM) return SSTMC_NOT_SUPPORTED;
    if (S->correlation || S->cbs) return SSTMC_NOT_SUPPORTED;
    for (int m = 0; m < OM; ++m)
        if (S->gmix_n[m] == 0 && S->scat_type[m] != SSTMC_SCATTERING_NOT_DEFINED) return SSTMC_NOT_SUPPORTED;
    if (S->dims == 2) return SSTMC_NO_ERROR;   /* 2D beams sample and weigh as point sources: no tables */
    double mv[3] = { 0, 0, 0 }, inv = 1.0 / vw->n;
    for (int v = 0; v < vw->n; ++v) for (int a = 0; a < 3; ++a) mv[a] = mv[a] + inv * (double)vw->gdir[3 * v + a];
    double r = sqrt(mv[0] * mv[0] + mv[1] * mv[1] + mv[2] * mv[2]);
    if (r < 0.0001) return SSTMC_NOT_SUPPORTED;   /* the reference draws a random direction here */
    for (int a = 0; a < 3; ++a) S->gmean[a] = mv[a] * (1.0 / r);
    int n = il->n, gM = 0;
    il->gfm = malloc(sizeof(int) * n);
    il->gtab = malloc(sizeof(double) * 9 * n);
    if (!il->gfm || !il->gtab) return SSTMC_ALLOCATION_ERROR;
    for (int l = 0; l < n; ++l) {
        const float* f = il->p + 3 * l;
        int fm = o_inside(S, f) ? S->grid[o_cell(S, f)] : 0;
        if (fm <= 0 || S->gmix_n[fm] < 1 || S->gmix_n[fm] > 8) return SSTMC_NOT_SUPPORTED;
        il->gfm[l] = fm;
        if (S->gmix_n[fm] > gM) gM = S->gmix_n[fm];
    }
    il->gM = gM;
    size_t nb = (size_t)n * gM * O_GB_BINS;
    il->gpdf = calloc(nb, sizeof(double)); il->gicdf = calloc(nb, sizeof(double));
    il->gapdf = calloc((size_t)n * gM, sizeof(double)); il->gaicdf = calloc((size_t)n * gM, sizeof(double));
    if (!il->gpdf || !il->gicdf || !il->gapdf || !il->gaicdf) return SSTMC_ALLOCATION_ERROR;
    double k = 2.0 * O_PI / S->lambda;
    double back0[3] = { -(double)il->gdir[0], -(double)il->gdir[1], -(double)il->gdir[2] };
    for (int l = 0; l < n; ++l) {
        double d[3], f[3];
        for (int i = 0; i < 3; ++i) { d[i] = il->gdir[3 * l + i]; f[i] = il->p[3 * l + i]; }
        double* tb = il->gtab + 9 * l;
        /* projectBoxToLine, MediumInterface.cuh:156-200 */
        double tmin = 0, tmax = 0;
        for (int c = 0; c < 8; ++c) {
            double cp[3] = { (c & 1) ? S->axd[0][S->n[0] - 1] : S->axd[0][0], (c & 2) ? S->axd[1][S->n[1] - 1] : S->axd[1][0],
                             (c & 4) ? S->axd[2][S->n[2] - 1] : S->axd[2][0] };
            double t = o_gproj(cp, f, d);
            if (c == 0 || t < tmin) tmin = t;
            if (c == 0 || t > tmax) tmax = t;
        }
        tb[0] = tmin; tb[1] = tmax; tb[2] = (tmax - tmin) / (double)O_GB_BINS;
        /* orthogonalBase, VectorType.cuh:293-314 */
        if (fabs(1.0 - fabs(d[2])) <= 1e-12) {
            tb[3] = 1; tb[4] = 0; tb[5] = 0; tb[6] = 0; tb[7] = 1; tb[8] = 0;
        } else {
            double b0[3] = { -d[1], d[0], 0.0 };
            double rb = sqrt(b0[0] * b0[0] + b0[1] * b0[1]);
            b0[0] /= rb; b0[1] /= rb;
            tb[3] = b0[0]; tb[4] = b0[1]; tb[5] = 0.0;
            tb[6] = b0[1] * d[2] - b0[2] * d[1];
            tb[7] = b0[2] * d[0] - b0[0] * d[2];
            tb[8] = b0[0] * d[1] - b0[1] * d[0];
        }
        int fm = il->gfm[l], M = S->gmix_n[fm];
        const double* mix = S->gmix + 2 * S->gmix_off[fm];
        for (int b = 0; b < O_GB_BINS; ++b) {
            double t = tmin + (double)b * tb[2];
            double z[3] = { f[0] + t * d[0], f[1] + t * d[1], f[2] + t * d[2] };
            double T = exp(-o_tau64(S, z, back0));
            double dz = (z[0] - f[0]) * d[0] + (z[1] - f[1]) * d[1] + (z[2] - f[2]) * d[2];
            for (int m = 0; m < M; ++m)
                il->gpdf[((size_t)l * gM + m) * O_GB_BINS + b] = T / ((il->ga + fabs(mix[2 * m])) / (k * k) + dz * dz / il->ga);
        }
        for (int m = 0; m < M; ++m) {
            double* pdf = il->gpdf + ((size_t)l * gM + m) * O_GB_BINS;
            double* cdf = il->gicdf + ((size_t)l * gM + m) * O_GB_BINS;
            double run = 0.0;
            for (int b = 0; b < O_GB_BINS; ++b) { cdf[b] = run; run += pdf[b]; }
            double tot = pdf[O_GB_BINS - 1] + cdf[O_GB_BINS - 1];
            for (int b = 0; b < O_GB_BINS; ++b) { pdf[b] *= (double)(O_GB_BINS - 1) / tot; cdf[b] /= tot; }
        }
        /* lobe weights, alphaPdfIcdfKernel (GaussianBeam.cuh:254-295) */
        double* ap = il->gapdf + (size_t)l * gM;
        double* ac = il->gaicdf + (size_t)l * gM;
        double asum = 0.0;
        for (int m = 0; m < M; ++m) {
            double kap = fabs(mix[2 * m]);
            double ln = kap < 1e-5 ? -log(4.0 * O_PI) : log(kap) - (kap > 10.0 ? log(2.0 * O_PI) * kap : log(4.0 * O_PI * sinh(kap)));
            ap[m] = exp(mix[2 * m + 1] + ln);
            asum += ap[m];
        }
        for (int m = 0; m < M; ++m) ap[m] /= asum;
        double run = 0.0;
        for (int m = 0; m < M; ++m) { ac[m] = run; run += ap[m]; }
    }
    return SSTMC_NO_ERROR;
}

/* ------------------------------------------------------------------ */
/* one path                                                           */
/* ------------------------------------------------------------------ */
typedef struct {
    int cap, B;
    float* x;     /* cap*3 */
    int* m;
    float* xi;
    float* xt;    /* cap*Nt*3 (field) */
    float* w;     /* cap*Nt tick weights (field, isForcedInsideBin) */
} o_verts;

static int o_verts_grow(o_verts* V, int Nt)
{
    int nc = V->cap ? V->cap * 2 : 64;
    float* x = realloc(V->x, (size_t)nc * 3 * sizeof(float));
    if (!x) return SSTMC_ALLOCATION_ERROR;
    V->x = x;
    int* m = realloc(V->m, (size_t)nc * sizeof(int));
    if (!m) return SSTMC_ALLOCATION_ERROR;
    V->m = m;
    float* xi = realloc(V->xi, (size_t)nc * sizeof(float));
    if (!xi) return SSTMC_ALLOCATION_ERROR;
    V->xi = xi;
    float* xt = realloc(V->xt, (size_t)nc * Nt * 3 * sizeof(float));
    if (!xt) return SSTMC_ALLOCATION_ERROR;
    V->xt = xt;
    float* w = realloc(V->w, (size_t)nc * Nt * sizeof(float));
    if (!w) return SSTMC_ALLOCATION_ERROR;
    V->w = w;
    V->cap = nc;
    return 0;
}

/* Cell along one axis as Simulation.cuh:325-367 returns it: ax[c] <= x < ax[c+1],
 * 0 below the first edge, n-1 at or beyond the last edge. */
static int o_edge_bin(const float* ax, int n, float x)
{
    int c = 0;
    while (c < n && ax[c] <= x) ++c;
    return c > 0 ? c - 1 : 0;
}

/* isSameBinKernel (HeterogeneousMedium.cuh:708-735) */
static int o_same_bin(const o_scene* S, const float x[3], const float p[3])
{
    if (!o_inside(S, p)) return 0;
    for (int a = 0; a < S->dims; ++a)
        if (o_edge_bin(S->ax[a], S->n[a], x[a]) != o_edge_bin(S->ax[a], S->n[a], p[a])) return 0;
    return 1;
}

/* isForcedInsideBin (TemporalSampler.cuh:439-534 getMaterialNumTemporal and
 * shiftRandomSampledIndex, :1637-1698 pathContribution): tick r = ceil(u Nt) - 1
 * drawn per vertex is moved onto the sampled point x (every tick shifted by
 * x - xt[r], read before any tick moves); ticks outside x's grid cell weigh 0,
 * with every tick beyond them on the same side of r (tick order). */
static int o_forced_inside_bin(const o_scene* S, uint64_t seed, uint32_t pid, uint32_t b, const float x[3],
                               float* xt, float* w)
{
    int Nt = S->Nt;
    o_stream rs;
    o_stream_init(&rs, seed, pid, b, O_PURPOSE_FORCED);
    uint64_t k = (uint64_t)(o_next_u32(&rs) >> 8) + 1u;   /* u = k 2^-24 */
    int r = (int)((k * (uint64_t)Nt - 1u) >> 24);
    float sh[3] = { x[0] - xt[3 * r], x[1] - xt[3 * r + 1], x[2] - xt[3 * r + 2] };
    int neg = -1, pos = Nt;
    for (int t = 0; t < Nt; ++t) {
        for (int i = 0; i < S->dims; ++i) xt[3 * t + i] = xt[3 * t + i] + sh[i];
        if (!o_same_bin(S, x, xt + 3 * t)) {
            if (t <= r) neg = t;
            else if (pos == Nt) pos = t;
        }
    }
    for (int t = 0; t < Nt; ++t) w[t] = (t > neg && t < pos) ? 1.0f : 0.0f;
    return r;
}

/* Per-tick positions of a vertex (field sampler): TemporalSampler.cuh:376-436, 540-647, 778-937. */
static int o_temporal_positions(const o_scene* S, uint64_t seed, uint32_t pid, uint32_t b, const float x[3], int m,
                                float* xt, float* w)
{
    int Nt = S->Nt;
    for (int t = 0; t < Nt; ++t) w[t] = 1.0f;
    if (!S->moving[m]) {
        for (int t = 0; t < Nt; ++t) { xt[3 * t] = x[0]; xt[3 * t + 1] = x[1]; xt[3 * t + 2] = x[2]; }
        return -1;
    }
    float cur[3] = { 0, 0, 0 };
    float buf[3];
    for (int j = 0; j < Nt; ++j) {
        float sc = S->disp_scale[m * Nt + j];
        const float* du = S->disp_u + (m * Nt + j) * 3;
        float disp[3] = { du[0], du[1], du[2] };
        if (sc != 0.0f) {
            o_stream ts;
            o_stream_init(&ts, seed, pid, b, O_PURPOSE_TEMPORAL | ((uint32_t)j << 8));
            float w[3];
            o_random_direction(S->dims, &ts, w);
            float u1 = o_uniform(&ts), u2 = o_uniform(&ts);
            float r = sqrtf(-2.0f * o_logf(u1));
            float s, c;
            o_sincospif(2.0f * u2, &s, &c);
            float dr = (r * c) * sc;
            for (int i = 0; i < S->dims; ++i) disp[i] = fmaf(dr, w[i], du[i]);
        }
        if (j == 0 || j == S->neg) { cur[0] = x[0]; cur[1] = x[1]; cur[2] = x[2]; }
        for (int i = 0; i < S->dims; ++i) cur[i] = cur[i] + disp[i];
        /* sorted index j -> output tick index */
        int t = j < S->neg ? S->neg - 1 - j : j;
        buf[0] = cur[0]; buf[1] = cur[1]; buf[2] = cur[2];
        xt[3 * t] = buf[0]; xt[3 * t + 1] = buf[1]; xt[3 * t + 2] = buf[2];
    }
    return S->forced_bin ? o_forced_inside_bin(S, seed, pid, b, x, xt, w) : -1;
}

/* Walk one path: vertices x_1..x_B.  Returns error code; misses counted. */
static int o_walk(const o_scene* S, uint64_t seed, uint32_t pid, int u1side, o_verts* V, int* misses)
{
    const o_src* first = (S->correlation && !u1side) ? &S->src[2] : &S->src[0];
    float x0[3], d0[3], x1[3];
    int m1 = 0;
    *misses = 0;
    V->B = 0;
    uint32_t att;
    o_stream rs;
    int beam = 0;
    const int gauss = first->type == SSTMC_SOURCE_GAUSSIANBEAM && S->dims == 3;
    for (att = 0; att < O_MAX_ATTEMPTS; ++att) {
        o_stream_init(&rs, seed, pid, 1u, O_PURPOSE_WALK | (att << 8));
        if (gauss) {
            /* the beam places x1 itself; a point outside the medium is a miss
             * (getMaterialInfo, GaussianBeam.cuh:1617-1618) */
            o_gauss_first(S, first, &rs, x0, x1, &beam);
            m1 = o_inside(S, x1) ? S->grid[o_cell(S, x1)] : 0;
        } else {
            o_sample_source(S, first, &rs, x0, d0);
            int e = o_woodcock(S, x0, d0, &rs, x1, &m1);
            if (e) return e;
        }
        if (m1 > 0) break;
        (*misses)++;
    }
    if (att == O_MAX_ATTEMPTS) return SSTMC_PATH_LIMIT;
    if (V->cap < 1 && o_verts_grow(V, S->Nt)) return SSTMC_ALLOCATION_ERROR;
    V->x[0] = x1[0]; V->x[1] = x1[1]; V->x[2] = x1[2]; V->m[0] = m1;
    V->xi[0] = S->correlation ? 0.0f : o_uniform(&rs);
    if (!S->correlation) o_temporal_positions(S, seed, pid, 1u, x1, m1, V->xt, V->w);
    V->B = 1;
    float prev[3] = { x0[0], x0[1], x0[2] };
    for (uint32_t b = 1; ; ++b) {
        if (b >= O_MAX_VERTICES) return SSTMC_PATH_LIMIT;
        const float* cur = V->x + 3 * (b - 1);
        int mb = V->m[b - 1];
        o_stream_init(&rs, seed, pid, b + 1, O_PURPOSE_WALK);
        float nd[3];
        if (gauss && b == 1) {
            /* the beam samples the second direction (GaussianBeam.cuh:1687-1780):
             * uniform with isotropic scattering, else from its lobe pairs */
            if (S->iso_all) o_random_direction(3, &rs, nd);
            else o_gauss_second_dir(S, first, beam, cur, &rs, nd);
        } else {
            float diff[3] = { cur[0] - prev[0], cur[1] - prev[1], cur[2] - prev[2] };
            float din[3]; o_normalize32(S->dims, diff, din);
            o_sample_direction(S, mb, din, &rs, nd);
        }
        float xn[3]; int mn = 0;
        int e = o_woodcock(S, cur, nd, &rs, xn, &mn);
        if (e) return e;
        if (mn == 0) break;
        if ((int)b >= V->cap && o_verts_grow(V, S->Nt)) return SSTMC_ALLOCATION_ERROR;
        cur = V->x + 3 * (b - 1);
        prev[0] = cur[0]; prev[1] = cur[1]; prev[2] = cur[2];
        V->x[3 * b] = xn[0]; V->x[3 * b + 1] = xn[1]; V->x[3 * b + 2] = xn[2];
        V->m[b] = mn;
        V->xi[b] = S->correlation ? 0.0f : o_uniform(&rs);
        if (!S->correlation)
            o_temporal_positions(S, seed, pid, b + 1, xn, mn, V->xt + (size_t)b * S->Nt * 3, V->w + (size_t)b * S->Nt);
        V->B = (int)b + 1;
    }
    return 0;
}

static uint32_t o_vertex_hash(const o_scene* S, const o_verts* V)
{
    uint32_t h = 2166136261u;
    for (int b = 0; b < V->B; ++b) {
        h = o_hash_mix(h, o_f2u(V->x[3 * b]));
        h = o_hash_mix(h, o_f2u(V->x[3 * b + 1]));
        if (S->dims == 3) h = o_hash_mix(h, o_f2u(V->x[3 * b + 2]));
        h = o_hash_mix(h, (uint32_t)V->m[b]);
    }
    return h;
}

/* correlation sampler shift x + h*U(m), h = -/+ tau/2 (TemporalSamplerCorrelation.cuh:229-255) */
static inline void o_shift(const o_scene* S, const float x[3], int m, float tau, float sign, float out[3])
{
    float h = tau * (0.5f * sign);
    out[0] = fmaf(h, S->U_f[m][0], x[0]);
    out[1] = fmaf(h, S->U_f[m][1], x[1]);
    out[2] = S->dims == 3 ? fmaf(h, S->U_f[m][2], x[2]) : 0.0f;
}

typedef struct {
    o_gmemo* memo[4];                 /* per source slot: last NEE vector of each element */
    oc *a_ms, *s_ms, *a_ss, *b_ss;   /* [Nt][Nl] / [Nt][Nv] */
    oc *ar_ms, *sr_ms;                /* CBS reversed path: GlSum [Nt][Nl], Gv0 [Nt][Nv] */
    oc *gl1, *gl2;                    /* [Nt][Nl] illumination NEE vectors at x1 */
    double* P1; double* P2;           /* [Nl] */
} o_work;

/* CBS of the correlation sampler (NextEventEstimation.cuh:1237-1378,
 * 1525-1600, SourceInterface.cuh:270-354): for every vertex x_b (b >= 2) the
 * cross terms of the direct and reversed paths,
 *   T2 = Gl_b(l) conj(u2Gv_b(v)) C2_l1v2(x_b) x conj(u2Gl0(l)) Gv0(v) C2_v1l2(x1)
 *   T3 = conj(u2Gl_b(l)) Gv_b(v) C3_v1l2(x_b) x Gl0(l) conj(u2Gv0(v)) C3_l1v2(x1)
 *   T4 = Gl_b(l) conj(u2Gl_b(l)) C4_l1l2(x_b) x Gv0(v) conj(u2Gv0(v)) C4_v1v2(x1)
 * each with the u1 path transfer exp(-k^2 |t| MT_b) (the path phase cancels),
 * added as 0.5 (T2 + T3 + T4) (the direct term T1 takes the same 0.5).  Gl0 /
 * Gv0 carry 1 / p2; G* at x_b are the NEE vector times the three-point
 * amplitude of the source attached there; C = exp(-k^2 |D t| |m|^2) with
 * m = (a + b) / 2 - (direction to the path's next point), a and b the
 * directions from the two ends' sources into the vertex (a view's is minus
 * its outgoing direction), the directions from the sampled (unshifted)
 * positions (TemporalSamplerCorrelation.cuh:316-342).  Rays traced here are
 * not counted in the DDA statistics. */
static void o_cbs_corr(const o_scene* S, const o_verts* V, oc* Vacc, double p2)
{
    int Nl = S->src[0].n, Nv = S->src[1].n, Nt = S->Nt, B = V->B;
    const o_src *il = &S->src[0], *vw = &S->src[1], *il2 = &S->src[2], *vw2 = &S->src[3];
    const float *x1 = V->x, *x2 = V->x + 3;
    int m1 = V->m[0], m2 = V->m[1];
    double k2 = (2.0 * O_PI / S->lambda) * (2.0 * O_PI / S->lambda);
    uint64_t dummy = 0;
    double d12[3]; o_dir64(x1, x2, d12);
    /* with drifting scatterers every vector is evaluated per tick: u1 NEE vectors
     * at x - U t/2, u2 ones at x + U t/2, and both three-point amplitudes at the
     * u1 positions (TemporalSamplerCorrelation.cuh:229-291, whose three-point copy
     * takes the minus sign for every connection); static scenes need one tick */
    int drift = 0;
    for (int m = 0; m < OM; ++m) if (S->U_f[m][0] != 0.0f || S->U_f[m][1] != 0.0f || S->U_f[m][2] != 0.0f) drift = 1;
    int Ne = drift ? Nt : 1;
    oc* G0l = malloc(sizeof(oc) * Nl * Ne); oc* U0l = malloc(sizeof(oc) * Nl * Ne);
    oc* G0v = malloc(sizeof(oc) * Nv * Ne); oc* U0v = malloc(sizeof(oc) * Nv * Ne);
    oc* Gl = malloc(sizeof(oc) * Nl * Ne); oc* U2l = malloc(sizeof(oc) * Nl * Ne);
    oc* Gv = malloc(sizeof(oc) * Nv * Ne); oc* U2v = malloc(sizeof(oc) * Nv * Ne);
    double* dl = malloc(sizeof(double) * 12 * (Nl + Nv));   /* directions at x1 and x_b */
    if (!G0l || !U0l || !G0v || !U0v || !Gl || !U2l || !Gv || !U2v || !dl) goto done;
    double *in1 = dl, *in2 = dl + 3 * Nl, *mo1 = dl + 6 * Nl, *mo2 = dl + 6 * Nl + 3 * Nv;
    double *in1b = dl + 6 * (Nl + Nv), *in2b = in1b + 3 * Nl, *mo1b = in1b + 6 * Nl, *mo2b = mo1b + 3 * Nv;
    for (int e = 0; e < Ne; ++e) {
        float tau = S->ticks_f[e];
        float g1[3], g2[3], fa[3], fb[3];
        o_shift(S, x1, m1, tau, -1.0f, g1); o_shift(S, x1, m1, tau, 1.0f, g2);
        o_shift(S, x1, m1, tau, -1.0f, fa); o_shift(S, x2, m2, tau, -1.0f, fb);
        for (int l = 0; l < Nl; ++l) {
            G0l[e * Nl + l] = oc_scale(oc_mul(o_g(S, il, l, g1, 0, &dummy), o_f3(S, il, l, fa, fb, m1, 0)), 1.0 / p2);
            U0l[e * Nl + l] = oc_mul(o_g(S, il2, l, g2, 0, &dummy), o_f3(S, il2, l, fa, fb, m1, 0));
        }
        for (int v = 0; v < Nv; ++v) {
            G0v[e * Nv + v] = oc_scale(oc_mul(o_g(S, vw, v, g1, 1, &dummy), o_f3(S, vw, v, fa, fb, m1, 1)), 1.0 / p2);
            U0v[e * Nv + v] = oc_mul(o_g(S, vw2, v, g2, 1, &dummy), o_f3(S, vw2, v, fa, fb, m1, 1));
        }
    }
    for (int l = 0; l < Nl; ++l) { o_src_dir(il, l, x1, 0, in1 + 3 * l); o_src_dir(il2, l, x1, 0, in2 + 3 * l); }
    for (int v = 0; v < Nv; ++v) {
        o_src_dir(vw, v, x1, 1, mo1 + 3 * v); o_src_dir(vw2, v, x1, 1, mo2 + 3 * v);
        for (int i = 0; i < 3; ++i) { mo1[3 * v + i] = -mo1[3 * v + i]; mo2[3 * v + i] = -mo2[3 * v + i]; }
    }
    double MT = 0;
    for (int b = 1; b < B; ++b) {
        const float* xb = V->x + 3 * b;
        const float* xa = V->x + 3 * (b - 1);
        int mb = V->m[b], ma = V->m[b - 1];
        if (b >= 2) {
            double u[3], w[3];
            o_dir64(V->x + 3 * (b - 2), xa, u); o_dir64(xa, xb, w);
            double q[3] = { u[0] - w[0], u[1] - w[1], u[2] - w[2] };
            MT += S->D[ma] * o_dot(q, q);
        }
        double back[3]; o_dir64(xb, xa, back);
        for (int e = 0; e < Ne; ++e) {
            float tau = S->ticks_f[e];
            float g1[3], g2[3], fa[3], fb[3];
            o_shift(S, xb, mb, tau, -1.0f, g1); o_shift(S, xb, mb, tau, 1.0f, g2);
            o_shift(S, xb, mb, tau, -1.0f, fa); o_shift(S, xa, ma, tau, -1.0f, fb);
            for (int l = 0; l < Nl; ++l) {
                Gl[e * Nl + l] = oc_mul(o_g(S, il, l, g1, 0, &dummy), o_f3(S, il, l, fa, fb, mb, 0));
                U2l[e * Nl + l] = oc_mul(o_g(S, il2, l, g2, 0, &dummy), o_f3(S, il2, l, fa, fb, mb, 0));
            }
            for (int v = 0; v < Nv; ++v) {
                Gv[e * Nv + v] = oc_mul(o_g(S, vw, v, g1, 1, &dummy), o_f3(S, vw, v, fa, fb, mb, 1));
                U2v[e * Nv + v] = oc_mul(o_g(S, vw2, v, g2, 1, &dummy), o_f3(S, vw2, v, fa, fb, mb, 1));
            }
        }
        for (int l = 0; l < Nl; ++l) { o_src_dir(il, l, xb, 0, in1b + 3 * l); o_src_dir(il2, l, xb, 0, in2b + 3 * l); }
        for (int v = 0; v < Nv; ++v) {
            o_src_dir(vw, v, xb, 1, mo1b + 3 * v); o_src_dir(vw2, v, xb, 1, mo2b + 3 * v);
            for (int i = 0; i < 3; ++i) { mo1b[3 * v + i] = -mo1b[3 * v + i]; mo2b[3 * v + i] = -mo2b[3 * v + i]; }
        }
        for (int t = 0; t < Nt; ++t) {
            int e = drift ? t : 0;
            double at = fabs(S->ticks[t]);
            double pt = exp(-k2 * at * MT);
            double dtD1 = k2 * fabs(S->D[m1] * S->ticks[t]), dtDb = k2 * fabs(S->D[mb] * S->ticks[t]);
            for (int v = 0; v < Nv; ++v)
                for (int l = 0; l < Nl; ++l) {
                    double q2b = 0, q21 = 0, q3b = 0, q31 = 0, q4b = 0, q41 = 0;
                    for (int i = 0; i < 3; ++i) {
                        double d;
                        d = 0.5 * (in1b[3 * l + i] + mo2b[3 * v + i]) - back[i]; q2b += d * d;
                        d = 0.5 * (mo1[3 * v + i] + in2[3 * l + i]) - d12[i]; q21 += d * d;
                        d = 0.5 * (mo1b[3 * v + i] + in2b[3 * l + i]) - back[i]; q3b += d * d;
                        d = 0.5 * (in1[3 * l + i] + mo2[3 * v + i]) - d12[i]; q31 += d * d;
                        d = 0.5 * (in1b[3 * l + i] + in2b[3 * l + i]) - back[i]; q4b += d * d;
                        d = 0.5 * (mo1[3 * v + i] + mo2[3 * v + i]) - d12[i]; q41 += d * d;
                    }
                    const oc gl = Gl[e * Nl + l], u2l = U2l[e * Nl + l], gv = Gv[e * Nv + v], u2v = U2v[e * Nv + v];
                    const oc g0l = G0l[e * Nl + l], u0l = U0l[e * Nl + l], g0v = G0v[e * Nv + v], u0v = U0v[e * Nv + v];
                    oc t2 = oc_mul(oc_mul(gl, oc_conj(u2v)), oc_mul(oc_conj(u0l), g0v));
                    oc t3 = oc_mul(oc_mul(oc_conj(u2l), gv), oc_mul(g0l, oc_conj(u0v)));
                    oc t4 = oc_mul(oc_mul(gl, oc_conj(u2l)), oc_mul(g0v, oc_conj(u0v)));
                    t2 = oc_scale(t2, exp(-dtDb * q2b - dtD1 * q21));
                    t3 = oc_scale(t3, exp(-dtDb * q3b - dtD1 * q31));
                    t4 = oc_scale(t4, exp(-dtDb * q4b - dtD1 * q41));
                    oc* dst = Vacc + ((size_t)t * Nv + v) * Nl + l;
                    dst->re += 0.5 * pt * (t2.re + t3.re + t4.re);
                    dst->im += 0.5 * pt * (t2.im + t3.im + t4.im);
                }
        }
    }
done:
    free(G0l); free(U0l); free(G0v); free(U0v); free(Gl); free(U2l); free(Gv); free(U2v); free(dl);
}

/* Evaluate the NEE vectors of one walked path and accumulate into V (if not NULL).
 * Field mode: NextEventEstimation.cuh:1016-1136 (single), 1138-1458 (multiple).
 * Correlation mode: the same, with TemporalSamplerCorrelation.cuh and
 * SourceInterface.cuh:220-354 temporal factors. */
static void o_nee(const o_scene* S, const o_verts* V, o_work* W, oc* Vacc, uint64_t* steps)
{
    int Nl = S->src[0].n, Nv = S->src[1].n, Nt = S->Nt, B = V->B, D = S->dims;
    const o_src *il = &S->src[0], *vw = &S->src[1], *il2 = &S->src[2], *vw2 = &S->src[3];
    const float* x1 = V->x;
    int m1 = V->m[0];
    double k2 = (2.0 * O_PI / S->lambda) * (2.0 * O_PI / S->lambda);
    memset(W->a_ms, 0, sizeof(oc) * Nt * Nl); memset(W->s_ms, 0, sizeof(oc) * Nt * Nv);
    memset(W->ar_ms, 0, sizeof(oc) * Nt * Nl); memset(W->sr_ms, 0, sizeof(oc) * Nt * Nv);

    if (!S->correlation) {
        double p1 = 0;
        for (int l = 0; l < Nl; ++l) { W->P1[l] = o_pfirst(S, il, l, x1, steps); p1 += W->P1[l]; }
        p1 = p1 / Nl;
        double sq1 = sqrt(p1);
        oc e1; o_cexp2pi((double)V->xi[0], &e1.re, &e1.im);
        for (int t = 0; t < Nt; ++t) {
            const float* x1t = V->xt + 3 * t;
            for (int l = 0; l < Nl; ++l) {
                W->gl1[t * Nl + l] = o_gm(S, W->memo[0], il, l, x1t, 0, steps);
                W->a_ss[t * Nl + l] = oc_scale(oc_mul(W->gl1[t * Nl + l], e1), V->w[t] / sq1);
            }
            for (int v = 0; v < Nv; ++v) W->b_ss[t * Nv + v] = o_gm(S, W->memo[1], vw, v, x1t, 1, steps);
        }
        if (Vacc) {
            for (int t = 0; t < Nt; ++t) {
                const float* pos = S->temporal_amp ? V->xt + 3 * t : x1;
                for (int v = 0; v < Nv; ++v) for (int l = 0; l < Nl; ++l) {
                    oc w = o_fs(S, il, l, vw, v, pos, m1);
                    oc c = oc_mul(oc_mul(W->a_ss[t * Nl + l], W->b_ss[t * Nv + v]), w);
                    oc* dst = Vacc + ((size_t)t * Nv + v) * Nl + l;
                    dst->re += c.re; dst->im += c.im;
                }
            }
        }
        if (B < 2) return;
        const float* x2 = V->x + 3;
        double x12[3]; o_dir64(x1, x2, x12);
        double p2 = 0;
        for (int l = 0; l < Nl; ++l) {
            if (il->type == SSTMC_SOURCE_GAUSSIANBEAM && D == 3) {
                /* a zero product is replaced by 1e20 (GaussianBeam.cuh:745-751) */
                double q = W->P1[l] * (S->iso_all ? O_ISO_PDF3 : o_gauss_pw(S, il, l, x1, x2));
                p2 += q == 0.0 ? 1e20 : q;
                continue;
            }
            double in[3]; o_src_dir(il, l, x1, 0, in);
            p2 += W->P1[l] * o_pdf(S, m1, o_dot(in, x12));
        }
        p2 = p2 / Nl;
        double sq2 = sqrt(p2);
        for (int t = 0; t < Nt; ++t) {
            const float* pa = S->temporal_amp ? V->xt + 3 * t : x1;
            const float* pb = S->temporal_amp ? V->xt + (size_t)Nt * 3 + 3 * t : x2;
            for (int l = 0; l < Nl; ++l)
                W->a_ms[t * Nl + l] = oc_scale(oc_mul(W->gl1[t * Nl + l], o_f3(S, il, l, pa, pb, m1, 0)), 1.0 / sq2);
            /* CBS: the reversed path starts at the view, v -> x1 -> x2 (Gv0,
             * NextEventEstimation.cuh:1533-1537 and :995-1004): the view's NEE vector at
             * x1 times its three-point amplitude with the view as the path's first end */
            if (S->cbs)
                for (int v = 0; v < Nv; ++v)
                    W->sr_ms[t * Nv + v] = oc_scale(oc_mul(W->b_ss[t * Nv + v], o_f3(S, vw, v, pa, pb, m1, 1)), 1.0 / sq2);
        }
        for (int t = 0; t < Nt; ++t) {
            double L = 0;
            for (int b = 1; b < B; ++b) {
                const float* xa = V->xt + ((size_t)(b - 1) * Nt + t) * 3;
                const float* xb = V->xt + ((size_t)b * Nt + t) * 3;
                double dv[3] = { (double)xb[0] - xa[0], (double)xb[1] - xa[1], (double)xb[2] - xa[2] };
                L += sqrt(o_dot(dv, dv));
                const float* pa = S->temporal_amp ? xb : V->x + 3 * b;
                const float* pb = S->temporal_amp ? xa : V->x + 3 * (b - 1);
                oc ph; o_cexp2pi(L / S->lambda + (double)V->xi[b], &ph.re, &ph.im);
                /* the tick weight of x_b multiplies its path contribution */
                ph = oc_scale(ph, V->w[(size_t)b * Nt + t]);
                for (int v = 0; v < Nv; ++v) {
                    oc g = o_gm(S, W->memo[1], vw, v, xb, 1, steps);
                    oc f = o_f3(S, vw, v, pa, pb, V->m[b], 1);
                    oc c = oc_mul(oc_mul(g, ph), f);
                    W->s_ms[t * Nv + v].re += c.re; W->s_ms[t * Nv + v].im += c.im;
                }
                /* CBS: the reversed path ends at the illumination, x_{b-1} -> x_b -> l
                 * (GlSum, NextEventEstimation.cuh:1573-1580, :1212-1235): the same path
                 * phase, the illumination's NEE vector and amplitude at x_b */
                if (S->cbs)
                    for (int l = 0; l < Nl; ++l) {
                        oc g = o_gm(S, W->memo[0], il, l, xb, 0, steps);
                        oc f = o_f3(S, il, l, pa, pb, V->m[b], 0);
                        oc c = oc_mul(oc_mul(g, ph), f);
                        W->ar_ms[t * Nl + l].re += c.re; W->ar_ms[t * Nl + l].im += c.im;
                    }
            }
        }
    } else {
        double p1 = 0;
        for (int l = 0; l < Nl; ++l) {
            double a = o_pfirst(S, il, l, x1, steps), b2 = o_pfirst(S, il2, l, x1, steps);
            W->P1[l] = 0.5 * (a + b2);
            p1 += W->P1[l];
        }
        p1 = p1 / Nl;
        for (int t = 0; t < Nt; ++t) {
            float tau = S->ticks_f[t];
            float xm[3], xp[3];
            o_shift(S, x1, m1, tau, -1.0f, xm); o_shift(S, x1, m1, tau, 1.0f, xp);
            for (int l = 0; l < Nl; ++l) {
                oc g1 = o_gm(S, W->memo[0], il, l, xm, 0, steps), g2 = o_gm(S, W->memo[2], il2, l, xp, 0, steps);
                W->gl1[t * Nl + l] = g1; W->gl2[t * Nl + l] = g2;
                W->a_ss[t * Nl + l] = oc_scale(oc_mul(g1, oc_conj(g2)), 1.0 / p1);
            }
            for (int v = 0; v < Nv; ++v) {
                oc g1 = o_gm(S, W->memo[1], vw, v, xm, 1, steps), g2 = o_gm(S, W->memo[3], vw2, v, xp, 1, steps);
                W->b_ss[t * Nv + v] = oc_mul(g1, oc_conj(g2));
            }
        }
        int scalarFs = il->type == SSTMC_SOURCE_POINT && vw->type == SSTMC_SOURCE_POINT && S->iso_all;
        if (Vacc) {
            for (int t = 0; t < Nt; ++t) {
                float xm[3]; o_shift(S, x1, m1, S->ticks_f[t], -1.0f, xm);
                double dtD = k2 * fabs(S->D[m1] * S->ticks[t]);
                for (int v = 0; v < Nv; ++v) {
                    double o1[3], o2[3];
                    o_src_dir(vw, v, x1, 1, o1); o_src_dir(vw2, v, x1, 1, o2);
                    for (int l = 0; l < Nl; ++l) {
                        oc w = { 0.0, 0.0 };
                        if (scalarFs) {
                            w.re = (D == 2 ? O_ISO_AMP2 : O_ISO_AMP3) * (D == 2 ? O_ISO_AMP2 : O_ISO_AMP3);
                        } else {
                            double in1[3], in2[3];
                            o_src_dir(il, l, x1, 0, in1); o_src_dir(il2, l, x1, 0, in2);
                            double q[3];
                            for (int i = 0; i < 3; ++i) q[i] = 0.5 * (in1[i] + in2[i] - o1[i] - o2[i]);
                            /* u1 amplitude x conj(u2 amplitude) (real unless tabular) */
                            w = oc_scale(oc_mul(o_fs(S, il, l, vw, v, xm, m1), oc_conj(o_fs(S, il2, l, vw2, v, xm, m1))),
                                         exp(-dtD * o_dot(q, q)));
                        }
                        oc c = oc_mul(oc_mul(W->a_ss[t * Nl + l], W->b_ss[t * Nv + v]), w);
                        oc* dst = Vacc + ((size_t)t * Nv + v) * Nl + l;
                        dst->re += c.re; dst->im += c.im;
                    }
                }
            }
        }
        if (B < 2) return;
        const float* x2 = V->x + 3;
        int m2 = V->m[1];
        double x12[3]; o_dir64(x1, x2, x12);
        double p2 = 0;
        for (int l = 0; l < Nl; ++l) {
            double in[3]; o_src_dir(il, l, x1, 0, in);
            p2 += W->P1[l] * o_pdf(S, m1, o_dot(in, x12));
        }
        p2 = p2 / Nl;
        for (int t = 0; t < Nt; ++t) {
            float tau = S->ticks_f[t];
            float pa[3], pb[3];
            o_shift(S, x1, m1, tau, -1.0f, pa); o_shift(S, x2, m2, tau, -1.0f, pb);
            double dtD = k2 * fabs(S->D[m1] * S->ticks[t]);
            for (int l = 0; l < Nl; ++l) {
                oc g1 = W->gl1[t * Nl + l], g2 = W->gl2[t * Nl + l];
                oc f1 = o_f3(S, il, l, pa, pb, m1, 0), f2 = o_f3(S, il2, l, pa, pb, m1, 0);
                double in1[3], in2[3], q[3];
                o_src_dir(il, l, x1, 0, in1); o_src_dir(il2, l, x1, 0, in2);
                for (int i = 0; i < 3; ++i) q[i] = 0.5 * (in1[i] + in2[i]) - x12[i];
                double c1 = exp(-dtD * o_dot(q, q));
                oc a = oc_mul(oc_scale(oc_mul(g1, f1), 1.0 / p2), oc_conj(oc_mul(g2, f2)));
                W->a_ms[t * Nl + l] = oc_scale(a, c1);
            }
        }
        double MT = 0;
        for (int b = 1; b < B; ++b) {
            const float* xb = V->x + 3 * b;
            const float* xa = V->x + 3 * (b - 1);
            int mb = V->m[b], ma = V->m[b - 1];
            if (b >= 2) {
                double u[3], w[3];
                o_dir64(V->x + 3 * (b - 2), xa, u); o_dir64(xa, xb, w);
                double q[3] = { u[0] - w[0], u[1] - w[1], u[2] - w[2] };
                MT += S->D[ma] * o_dot(q, q);
            }
            double back[3]; o_dir64(xb, xa, back);
            for (int t = 0; t < Nt; ++t) {
                float tau = S->ticks_f[t];
                float xm[3], xp[3], pa[3], pb[3];
                o_shift(S, xb, mb, tau, -1.0f, xm); o_shift(S, xb, mb, tau, 1.0f, xp);
                o_shift(S, xb, mb, tau, -1.0f, pa); o_shift(S, xa, ma, tau, -1.0f, pb);
                double pt = exp(-k2 * fabs(S->ticks[t]) * MT);
                double dtD = k2 * fabs(S->D[mb] * S->ticks[t]);
                for (int v = 0; v < Nv; ++v) {
                    oc g1 = o_gm(S, W->memo[1], vw, v, xm, 1, steps), g2 = o_gm(S, W->memo[3], vw2, v, xp, 1, steps);
                    oc f1 = o_f3(S, vw, v, pa, pb, mb, 1), f2 = o_f3(S, vw2, v, pa, pb, mb, 1);
                    double o1[3], o2[3], q[3];
                    o_src_dir(vw, v, xb, 1, o1); o_src_dir(vw2, v, xb, 1, o2);
                    for (int i = 0; i < 3; ++i) q[i] = 0.5 * (-o1[i] - o2[i]) - back[i];
                    double c1 = exp(-dtD * o_dot(q, q));
                    oc c = oc_mul(oc_scale(oc_mul(g1, f1), pt), oc_conj(oc_mul(g2, f2)));
                    c = oc_scale(c, c1);
                    W->s_ms[t * Nv + v].re += c.re; W->s_ms[t * Nv + v].im += c.im;
                }
            }
        }
        if (S->cbs && Vacc) o_cbs_corr(S, V, Vacc, p2);
    }
    if (Vacc) {
        /* CBS: field (direct + reversed) / sqrt(2), correlation 0.5 (the cross terms
         * are added by o_cbs_corr) (NextEventEstimation.cuh:1385-1391, :1448-1454) */
        const double sc = S->cbs ? (S->correlation ? 0.5 : sqrt(0.5)) : 1.0;
        for (int t = 0; t < Nt; ++t)
            for (int v = 0; v < Nv; ++v) {
                oc s = W->s_ms[t * Nv + v], sr = W->sr_ms[t * Nv + v];
                for (int l = 0; l < Nl; ++l) {
                    oc c = oc_mul(W->a_ms[t * Nl + l], s);
                    if (S->cbs && !S->correlation) {
                        oc r = oc_mul(W->ar_ms[t * Nl + l], sr);
                        c.re += r.re; c.im += r.im;
                    }
                    oc* dst = Vacc + ((size_t)t * Nv + v) * Nl + l;
                    dst->re += c.re * sc; dst->im += c.im * sc;
                }
            }
    }
}

static int o_work_alloc(const o_scene* S, o_work* W)
{
    int Nl = S->src[0].n, Nv = S->src[1].n, Nt = S->Nt;
    W->a_ms = calloc((size_t)Nt * Nl, sizeof(oc)); W->a_ss = calloc((size_t)Nt * Nl, sizeof(oc));
    W->s_ms = calloc((size_t)Nt * Nv, sizeof(oc)); W->b_ss = calloc((size_t)Nt * Nv, sizeof(oc));
    W->ar_ms = calloc((size_t)Nt * Nl, sizeof(oc)); W->sr_ms = calloc((size_t)Nt * Nv, sizeof(oc));
    if (!W->ar_ms || !W->sr_ms) return SSTMC_ALLOCATION_ERROR;
    for (int i = 0; i < 4; ++i) W->memo[i] = calloc(S->src[i].n > 0 ? (size_t)S->src[i].n : 1, sizeof(o_gmemo));
    for (int i = 0; i < 4; ++i) if (!W->memo[i]) return SSTMC_ALLOCATION_ERROR;
    W->gl1 = calloc((size_t)Nt * Nl, sizeof(oc)); W->gl2 = calloc((size_t)Nt * Nl, sizeof(oc));
    W->P1 = calloc(Nl, sizeof(double)); W->P2 = calloc(Nl, sizeof(double));
    return (W->a_ms && W->a_ss && W->s_ms && W->b_ss && W->gl1 && W->gl2 && W->P1 && W->P2) ? 0 : SSTMC_ALLOCATION_ERROR;
}

static void o_work_free(o_work* W)
{
    for (int i = 0; i < 4; ++i) free(W->memo[i]);
    free(W->a_ms); free(W->a_ss); free(W->s_ms); free(W->b_ss); free(W->gl1); free(W->gl2); free(W->P1); free(W->P2);
    free(W->ar_ms); free(W->sr_ms);
}

/* correlation u1/u2 split of a wave: TemporalSamplerCorrelation.cuh:369-372, 611-656 */
static uint32_t o_u1_count(const o_scene* S, uint64_t seed, uint32_t wave)
{
    o_stream ws;
    o_stream_init(&ws, seed, wave, 0u, O_PURPOSE_WAVE);
    int c = (int)ceilf(o_uniform(&ws) * (float)(S->P + 1u)) - 1;
    if (c < 0) c = 0;
    if (c > (int)S->P) c = (int)S->P;
    return (uint32_t)c;
}

/* ------------------------------------------------------------------ */
/* API                                                                */
/* ------------------------------------------------------------------ */
int32_t oracle_render(const sstmc_config* cfg, uint64_t seed, uint32_t first_wave,
                      uint32_t waves, int32_t threads, double* u_out, double* iter_out, uint64_t* stats)
{
    o_scene S;
    int err = o_build_scene(cfg, &S);
    if (err) { o_free_scene(&S); return err; }
    int Nl = S.src[0].n, Nv = S.src[1].n, Nt = S.Nt;
    size_t nout = (size_t)Nl * Nv * Nt;
#ifdef _OPENMP
    int nthr = threads > 0 ? threads : omp_get_max_threads();
#else
    int nthr = 1;
    (void)threads;
#endif
    oc* part = calloc(nout * (size_t)nthr, sizeof(oc));
    uint64_t* st = calloc((size_t)nthr * 5, sizeof(uint64_t));
    int* errs = calloc(nthr, sizeof(int));
    if (!part || !st || !errs) { free(part); free(st); free(errs); o_free_scene(&S); return SSTMC_ALLOCATION_ERROR; }
    uint64_t total = (uint64_t)waves * S.P;
#pragma omp parallel num_threads(nthr)
    {
#ifdef _OPENMP
        int tid = omp_get_thread_num();
#else
        int tid = 0;
#endif
        o_verts V; memset(&V, 0, sizeof(V));
        o_work W;
        int e = o_work_alloc(&S, &W);
        if (!e) e = o_verts_grow(&V, Nt);
        if (e) errs[tid] = e;
        oc* acc = part + nout * (size_t)tid;
        uint64_t* sst = st + 5 * tid;
#pragma omp for schedule(static)
        for (int64_t q = 0; q < (int64_t)total; ++q) {
            if (errs[tid]) continue;
            uint32_t wave = first_wave + (uint32_t)(q / S.P);
            uint32_t slot = (uint32_t)(q % S.P);
            uint32_t pid = wave * S.P + slot;
            int u1side = 1;
            if (S.correlation) u1side = slot < o_u1_count(&S, seed, wave);
            int misses = 0;
            int we = o_walk(&S, seed, pid, u1side, &V, &misses);
            if (we) { errs[tid] = we; continue; }
            uint64_t steps = 0;
            o_nee(&S, &V, &W, acc, &steps);
            sst[0] += (uint64_t)V.B * Nl * Nv * Nt;
            sst[1] += steps;
            sst[2] += (uint64_t)V.B;
            sst[3] += 1;
            sst[4] += (uint64_t)misses;
        }
        o_work_free(&W);
        free(V.x); free(V.m); free(V.xi); free(V.xt); free(V.w);
    }
    for (int t = 0; t < nthr; ++t) if (errs[t]) { err = errs[t]; break; }
    if (!err) {
        for (size_t i = 0; i < nout; ++i) {
            double re = 0, im = 0;
            for (int t = 0; t < nthr; ++t) { re += part[nout * t + i].re; im += part[nout * t + i].im; }
            u_out[2 * i] = re; u_out[2 * i + 1] = im;
        }
        uint64_t misses = 0, agg[4] = { 0, 0, 0, 0 };
        for (int t = 0; t < nthr; ++t) { for (int k = 0; k < 4; ++k) agg[k] += st[5 * t + k]; misses += st[5 * t + 4]; }
        if (iter_out) *iter_out = (double)total + (double)misses;
        if (stats) for (int k = 0; k < 4; ++k) stats[k] = agg[k];
    }
    free(part); free(st); free(errs);
    o_free_scene(&S);
    return err;
}

int32_t oracle_trace_paths(const sstmc_config* cfg, uint64_t seed, uint32_t first_path,
                           uint32_t paths, sstmc_path_trace* out)
{
    o_scene S;
    int err = o_build_scene(cfg, &S);
    if (err) { o_free_scene(&S); return err; }
    int Nl = S.src[0].n, Nv = S.src[1].n, Nt = S.Nt;
    o_verts V; memset(&V, 0, sizeof(V));
    o_work W;
    err = o_work_alloc(&S, &W);
    if (!err) err = o_verts_grow(&V, Nt);
    for (uint32_t i = 0; i < paths && !err; ++i) {
        uint32_t pid = first_path + i;
        uint32_t wave = pid / S.P, slot = pid % S.P;
        int u1side = 1;
        if (S.correlation) u1side = slot < o_u1_count(&S, seed, wave);
        int misses = 0;
        err = o_walk(&S, seed, pid, u1side, &V, &misses);
        if (err) break;
        uint64_t steps = 0;
        o_nee(&S, &V, &W, NULL, &steps);
        if (out->misses) out->misses[i] = misses;
        if (out->vertices) out->vertices[i] = V.B;
        if (out->vertex_hash) out->vertex_hash[i] = o_vertex_hash(&S, &V);
        if (out->dda_steps) out->dda_steps[i] = (uint32_t)steps;
        if (out->x1) for (int k = 0; k < 3; ++k) out->x1[3 * i + k] = V.x[k];
        if (out->m1) out->m1[i] = V.m[0];
        for (int t = 0; t < Nt; ++t) {
            for (int l = 0; l < Nl; ++l) {
                size_t o = (((size_t)i * Nt + t) * Nl + l) * 2;
                if (out->a_ms) { out->a_ms[o] = W.a_ms[t * Nl + l].re; out->a_ms[o + 1] = W.a_ms[t * Nl + l].im; }
                if (out->a_ss) { out->a_ss[o] = W.a_ss[t * Nl + l].re; out->a_ss[o + 1] = W.a_ss[t * Nl + l].im; }
            }
            for (int v = 0; v < Nv; ++v) {
                size_t o = (((size_t)i * Nt + t) * Nv + v) * 2;
                if (out->s_ms) { out->s_ms[o] = W.s_ms[t * Nv + v].re; out->s_ms[o + 1] = W.s_ms[t * Nv + v].im; }
                if (out->b_ss) { out->b_ss[o] = W.b_ss[t * Nv + v].re; out->b_ss[o + 1] = W.b_ss[t * Nv + v].im; }
            }
        }
    }
    o_work_free(&W);
    free(V.x); free(V.m); free(V.xi); free(V.xt); free(V.w);
    o_free_scene(&S);
    return err;
}

int32_t oracle_dda(const sstmc_config* cfg, const float* o, const float* d, double* tau32, double* tau64)
{
    o_scene S;
    int err = o_build_scene(cfg, &S);
    if (err) { o_free_scene(&S); return -err; }
    float o3[3] = { o[0], o[1], S.dims == 3 ? o[2] : 0.0f }, d3[3] = { d[0], d[1], S.dims == 3 ? d[2] : 0.0f };
    float t32 = 0;
    uint32_t steps = o_dda32(&S, o3, d3, &t32);
    double od[3] = { o3[0], o3[1], o3[2] }, dd[3] = { d3[0], d3[1], d3[2] };
    if (tau32) *tau32 = t32;
    if (tau64) *tau64 = o_tau64(&S, od, dd);
    o_free_scene(&S);
    return (int32_t)steps;
}

int32_t oracle_phase(const sstmc_config* cfg, int32_t m, double c, double* amp, double* pdf)
{
    o_scene S;
    int err = o_build_scene(cfg, &S);
    if (!err) {
        if (amp) *amp = o_ampc(&S, m, c).re;
        if (pdf) *pdf = o_pdf(&S, m, c);
    }
    o_free_scene(&S);
    return err;
}

int32_t oracle_amplitude(const sstmc_config* cfg, int32_t m, double c, double* re, double* im)
{
    o_scene S;
    int err = o_build_scene(cfg, &S);
    if (!err) {
        oc a = o_ampc(&S, m, c);
        if (re) *re = a.re;
        if (im) *im = a.im;
    }
    o_free_scene(&S);
    return err;
}

int32_t oracle_sample_cos(const sstmc_config* cfg, int32_t m, uint64_t seed, uint32_t n, float* out)
{
    o_scene S;
    int err = o_build_scene(cfg, &S);
    if (!err) {
        float din[3] = { 0.0f, S.dims == 2 ? 1.0f : 0.0f, S.dims == 3 ? 1.0f : 0.0f };
        for (uint32_t i = 0; i < n; ++i) {
            o_stream rs;
            o_stream_init(&rs, seed, i, 0u, O_PURPOSE_WALK);
            float nd[3];
            o_sample_direction(&S, m, din, &rs, nd);
            out[i] = S.dims == 2 ? nd[1] : nd[2];
        }
    }
    o_free_scene(&S);
    return err;
}

int32_t oracle_tick_positions(const sstmc_config* cfg, uint64_t seed, uint32_t pid, uint32_t b, const float* x,
                              int32_t m, float* xt, float* w, int32_t* r)
{
    o_scene S;
    int err = o_build_scene(cfg, &S);
    if (!err && (S.correlation || m < 0 || m >= OM)) err = SSTMC_INVALID_CONFIG;
    if (!err) {
        float xx[3] = { x[0], x[1], S.dims == 3 ? x[2] : 0.0f };
        *r = o_temporal_positions(&S, seed, pid, b, xx, m, xt, w);
    }
    o_free_scene(&S);
    return err;
}

float oracle_logf(float x) { return o_logf(x); }
void oracle_sincospif(float x, float* s, float* c) { o_sincospif(x, s, c); }
void oracle_philox(const uint32_t key[2], const uint32_t ctr[4], uint32_t out[4]) { o_philox(key, ctr, out); }

int32_t oracle_gauss_terms(const sstmc_config* cfg, int32_t l, int32_t v, const float* x1, int32_t m1,
                           const float* x2, double* out)
{
    o_scene S;
    int err = o_build_scene(cfg, &S);
    if (!err && !S.gauss) err = SSTMC_INVALID_CONFIG;
    if (!err && (l < 0 || l >= S.src[0].n || v < 0 || v >= S.src[1].n || m1 <= 0 || m1 >= OM)) err = SSTMC_INVALID_CONFIG;
    if (!err) {
        const o_src *il = &S.src[0], *vw = &S.src[1];
        uint64_t st = 0;
        out[0] = o_gauss_pfirst(&S, il, l, x1, m1);
        out[1] = S.iso_all ? O_ISO_PDF3 : o_gauss_pw(&S, il, l, x1, x2);
        oc f = o_gauss_f(&S, il, l, x1, x2, m1, 0);
        out[2] = f.re; out[3] = f.im;
        f = o_gauss_f(&S, vw, v, x1, x2, m1, 1);
        out[4] = f.re; out[5] = f.im;
        f = o_gauss_fs(&S, il, l, vw, v, x1, m1);
        out[6] = f.re; out[7] = f.im;
        out[8] = o_gauss_g(&S, il, l, x1, 0, &st).re;
        out[9] = o_gauss_g(&S, vw, v, x1, 1, &st).re;
    }
    o_free_scene(&S);
    return err;
}

int32_t oracle_gauss_sample(const sstmc_config* cfg, uint64_t seed, uint32_t n, const float* x1_fixed, int32_t beam_fixed,
                            float* xyz, int32_t* mat, int32_t* beam, float* dir)
{
    o_scene S;
    int err = o_build_scene(cfg, &S);
    if (!err && !S.gauss) err = SSTMC_INVALID_CONFIG;
    if (!err) {
        const o_src* il = &S.src[0];
        for (uint32_t i = 0; i < n; ++i) {
            o_stream rs;
            o_stream_init(&rs, seed, i, 1u, O_PURPOSE_WALK);
            float x0[3], x1[3], d[3];
            int b = 0;
            if (x1_fixed) {
                for (int a = 0; a < 3; ++a) x1[a] = x1_fixed[a];
                b = beam_fixed < 0 ? 0 : (beam_fixed >= il->n ? il->n - 1 : beam_fixed);
            } else {
                o_gauss_first(&S, il, &rs, x0, x1, &b);
            }
            int m = o_inside(&S, x1) ? S.grid[o_cell(&S, x1)] : 0;
            o_stream_init(&rs, seed, i, 2u, O_PURPOSE_WALK);
            if (S.iso_all) o_random_direction(3, &rs, d);
            else o_gauss_second_dir(&S, il, b, x1, &rs, d);
            for (int a = 0; a < 3; ++a) { xyz[3 * i + a] = x1[a]; dir[3 * i + a] = d[a]; }
            mat[i] = m; beam[i] = b;
        }
    }
    o_free_scene(&S);
    return err;
}

void oracle_bessel_i0(double re, double im, double* out_re, double* out_im)
{
    oc z = { re, im };
    oc r = o_bessel_i0(z);
    *out_re = r.re; *out_im = r.im;
}
