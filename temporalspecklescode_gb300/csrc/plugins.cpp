// plugins.cpp -- the reference's object model as C-ABI handles: Simulation,
// Scattering, Medium, Source, Sampler and Tracer, built one object at a time
// in the order mexFunction builds them (MatlabInterface.cu:1677-1700):
//
//   Simulation (batch, wavelength, device)          Simulation.cuh:179
//   Scattering + set{Isotropic,HenyeyGreenstein,
//     Tabular,VonMisesFisher}Scattering(.., mat)    Scattering.cuh:32-125
//   HeterogeneousMedium(grid, axes) + setMaterial   MediumInterface.cuh:39-135
//   FarField / PointSource(.., connection type)     SourceInterface.cuh:10-179
//   TemporalSampler / TemporalCorrelationSampler
//     + setMaterial(D, U, mat)                      SamplerInterface.cuh:11-176
//   NextEventEstimation(sampler, options): trace,
//     updateSeed, getZeroContributionPaths,
//     getPhotonsBudget, getCBS                      TracerInterface.cuh:9-50
//
// The objects hold host copies of what they were given.  Ownership follows the
// reference: the caller creates every object and destroys it in reverse order;
// a sampler borrows its sources, medium and scattering, and a tracer borrows
// its sampler.  The tracer assembles the objects into one sstmc_config and
// creates the device-resident scene from it (the same validation and tables
// as sstmc_scene_create), so an object-by-object build renders exactly what
// the equivalent config renders.  The per-method device work of the
// reference's plugins (attenuation, sampling, throughput, path contribution)
// is fused into the render's kernels.
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "sstmc_internal.h"

struct sstmc_simulation {
    uint32_t dims = 3, batch_size = 1024;
    double lambda = 1.0;
    int32_t device = 0, precision = SSTMC_PRECISION_SPLIT;
};

struct sstmc_scattering {
    // per material: type, g, tabular table (re, im), vMF components
    int32_t type[SSTMC_MATERIAL_NUM] = { 0 };
    double g[SSTMC_MATERIAL_NUM] = { 0 };
    std::vector<double> tab[SSTMC_MATERIAL_NUM];
    std::vector<double> mu[SSTMC_MATERIAL_NUM], c[SSTMC_MATERIAL_NUM], alpha[SSTMC_MATERIAL_NUM];
    uint32_t count = 0;   // highest material set + 1
};

struct sstmc_medium {
    int32_t type = SSTMC_MEDIUM_HETEROGENEOUS;
    uint32_t dims = 3;
    std::vector<double> ax[3];
    std::vector<uint32_t> grid;
    double box_min[3] = { 0 }, box_max[3] = { 0 }, homogeneous_sigs = 0;
    double sigs[SSTMC_MATERIAL_NUM] = { 0 }, siga[SSTMC_MATERIAL_NUM] = { 0 };
    uint32_t count = 0;   // highest material set + 1
};

struct sstmc_source {
    int32_t type = SSTMC_SOURCE_NONE, connection = SSTMC_CONNECTION_ILLUMINATION, is_area = 0;
    uint32_t dims = 3;
    std::vector<double> xyz;
    std::vector<double> dir;   // GaussianBeam: focal directions
    double aperture = 0.0;
};

struct sstmc_sampler {
    int32_t type = SSTMC_SAMPLER_TEMPORAL;
    const sstmc_simulation* sim = nullptr;
    const sstmc_medium* medium = nullptr;
    const sstmc_scattering* scattering = nullptr;
    const sstmc_source* src[4] = { nullptr, nullptr, nullptr, nullptr };   // illumination, view, illumination2, view2
    std::vector<double> t;
    double D[SSTMC_MATERIAL_NUM] = { 0 };
    double U[SSTMC_MATERIAL_NUM][3] = { { 0 } };
    uint32_t count = 0;   // highest material set + 1
    int32_t temporal_amplitude = 1, forced_inside_bin = 0;
    // storage of the last assembled config (sstmc_sampler_config)
    std::vector<int32_t> c_type;
    std::vector<double> c_g, c_D, c_U, c_sigs, c_siga, c_tab_f, c_vmf_mu, c_vmf_c, c_vmf_alpha;
    std::vector<uint32_t> c_tab_n, c_vmf_n;
};

struct sstmc_tracer {
    const sstmc_sampler* sampler = nullptr;
    sstmc_scene* scene = nullptr;
    uint64_t seed = 0;
    uint32_t full_iteration = 1;
    int32_t is_cbs = 0;
    uint64_t zero_contribution_paths = 0, photons_budget = 0;
};

namespace {

int32_t invalid(const std::string& why)
{
    sstmc::set_last_error_text(why);
    return SSTMC_INVALID_CONFIG;
}

bool finite_all(const double* p, size_t n)
{
    for (size_t i = 0; i < n; ++i)
        if (!std::isfinite(p[i])) return false;
    return true;
}

template <class T>
int32_t make(T** out)
{
    if (!out) return SSTMC_INVALID_HANDLE;
    *out = new (std::nothrow) T();
    return *out ? SSTMC_NO_ERROR : SSTMC_ALLOCATION_ERROR;
}

int32_t set_scattering(sstmc_scattering* s, uint32_t mat, int32_t type)
{
    if (!s) return SSTMC_INVALID_HANDLE;
    if (mat >= SSTMC_MATERIAL_NUM) return invalid("scattering material index out of range (0 .. 9)");
    s->type[mat] = type;
    s->g[mat] = 0.0;
    s->tab[mat].clear();
    s->mu[mat].clear(); s->c[mat].clear(); s->alpha[mat].clear();
    if (mat + 1 > s->count) s->count = mat + 1;
    return SSTMC_NO_ERROR;
}

int32_t make_source(int32_t type, int32_t connection, const double* xyz, uint32_t n, int32_t is_area, uint32_t dims,
                    sstmc_source** out)
{
    if (!out) return SSTMC_INVALID_HANDLE;
    *out = nullptr;
    if (connection < SSTMC_CONNECTION_ILLUMINATION || connection > SSTMC_CONNECTION_VIEW2)
        return invalid("unknown source connection type");
    if (dims != 2 && dims != 3) return invalid("source dims must be 2 or 3");
    if (!xyz || n == 0) return invalid("a source needs at least one location / direction");
    if (!finite_all(xyz, (size_t)3 * n)) return invalid("source locations / directions must be finite");
    int32_t e = make(out);
    if (e) return e;
    (*out)->type = type;
    (*out)->connection = connection;
    (*out)->is_area = is_area ? 1 : 0;
    (*out)->dims = dims;
    (*out)->xyz.assign(xyz, xyz + (size_t)3 * n);
    if (dims == 2)
        for (uint32_t i = 0; i < n; ++i) (*out)->xyz[3 * i + 2] = 0.0;
    return SSTMC_NO_ERROR;
}

void source_cfg(const sstmc_source* s, sstmc_source_cfg* c)
{
    std::memset(c, 0, sizeof(*c));
    if (!s) { c->type = SSTMC_SOURCE_NONE; return; }
    c->type = s->type;
    c->count = (uint32_t)(s->xyz.size() / 3);
    c->xyz = s->xyz.data();
    c->is_area_source = s->is_area;
    if (s->type == SSTMC_SOURCE_GAUSSIANBEAM) {
        c->focal_direction = s->dir.data();
        c->aperture = s->aperture;
    }
}

int32_t check_connection(const sstmc_source* s, int32_t want, const char* role)
{
    if (!s) return invalid(std::string("the sampler needs its ") + role + " source");
    if (s->connection != want) return invalid(std::string("source connection type does not match its role as ") + role);
    return SSTMC_NO_ERROR;
}

int32_t make_sampler(int32_t type, const sstmc_simulation* sim, const sstmc_medium* medium, const sstmc_scattering* scattering,
                     const sstmc_source* const src[4], const double* t, uint32_t t_num, sstmc_sampler** out)
{
    if (!out) return SSTMC_INVALID_HANDLE;
    *out = nullptr;
    if (!sim || !medium || !scattering) return SSTMC_INVALID_HANDLE;
    if (!t || t_num == 0) return invalid("sampler.t must have at least one element");
    if (!finite_all(t, t_num)) return invalid("sampler.t must be finite");
    static const char* roles[4] = { "illumination", "view", "illumination2", "view2" };
    const int want[4] = { SSTMC_CONNECTION_ILLUMINATION, SSTMC_CONNECTION_VIEW, SSTMC_CONNECTION_ILLUMINATION2, SSTMC_CONNECTION_VIEW2 };
    for (int i = 0; i < (type == SSTMC_SAMPLER_TEMPORAL_CORRELATION ? 4 : 2); ++i) {
        const int32_t e = check_connection(src[i], want[i], roles[i]);
        if (e) return e;
        if (src[i]->dims != sim->dims) return invalid(std::string("the ") + roles[i] + " source's dims differ from the simulation's");
    }
    if (medium->dims != sim->dims) return invalid("the medium's dims differ from the simulation's");
    int32_t e = make(out);
    if (e) return e;
    sstmc_sampler* s = *out;
    s->type = type;
    s->sim = sim; s->medium = medium; s->scattering = scattering;
    for (int i = 0; i < 4; ++i) s->src[i] = (type == SSTMC_SAMPLER_TEMPORAL_CORRELATION || i < 2) ? src[i] : nullptr;
    s->t.assign(t, t + t_num);
    return SSTMC_NO_ERROR;
}

}  // namespace

extern "C" {

int32_t sstmc_simulation_create(uint32_t dims, uint32_t batch_size, double lambda, int32_t device_number, int32_t precision,
                                sstmc_simulation** out)
{
    if (!out) return SSTMC_INVALID_HANDLE;
    *out = nullptr;
    if (dims != 2 && dims != 3) return invalid("dims must be 2 or 3");
    if (batch_size == 0) return invalid("batchSize must be positive");
    if (!(lambda > 0.0) || !std::isfinite(lambda)) return invalid("lambda must be positive and finite");
    if (precision != SSTMC_PRECISION_SPLIT && precision != SSTMC_PRECISION_FP32) return invalid("unknown precision");
    const int32_t e = make(out);
    if (e) return e;
    (*out)->dims = dims; (*out)->batch_size = batch_size; (*out)->lambda = lambda;
    (*out)->device = device_number; (*out)->precision = precision;
    return SSTMC_NO_ERROR;
}

int32_t sstmc_simulation_destroy(sstmc_simulation* s) { delete s; return SSTMC_NO_ERROR; }

int32_t sstmc_scattering_create(sstmc_scattering** out) { return make(out); }
int32_t sstmc_scattering_destroy(sstmc_scattering* s) { delete s; return SSTMC_NO_ERROR; }

int32_t sstmc_scattering_set_isotropic(sstmc_scattering* s, uint32_t mat)
{
    return set_scattering(s, mat, SSTMC_SCATTERING_ISOTROPIC);
}

int32_t sstmc_scattering_set_henyey_greenstein(sstmc_scattering* s, double g, uint32_t mat)
{
    if (!std::isfinite(g) || g <= -1.0 || g >= 1.0) return invalid("Henyey-Greenstein g must lie in (-1, 1)");
    const int32_t e = set_scattering(s, mat, SSTMC_SCATTERING_HENYEY_GREENSTEIN);
    if (!e) s->g[mat] = g;
    return e;
}

int32_t sstmc_scattering_set_tabular(sstmc_scattering* s, const double* f, uint32_t n, uint32_t mat)
{
    if (!f || n < 2) return invalid("a tabular amplitude function needs at least 2 entries");
    if (!finite_all(f, 2 * (size_t)n)) return invalid("tabular amplitudes must be finite");
    const int32_t e = set_scattering(s, mat, SSTMC_SCATTERING_TABULAR);
    if (!e) s->tab[mat].assign(f, f + 2 * (size_t)n);
    return e;
}

int32_t sstmc_scattering_set_von_mises_fisher(sstmc_scattering* s, const double* mu, const double* c, const double* alpha,
                                              uint32_t mixtures, uint32_t mat)
{
    if (!mu || !c || !alpha || mixtures == 0) return invalid("a vMF mixture needs at least one component");
    if (!finite_all(mu, mixtures) || !finite_all(c, mixtures) || !finite_all(alpha, mixtures))
        return invalid("vMF mixture parameters must be finite");
    bool any = false;
    for (uint32_t k = 0; k < mixtures; ++k) {
        if (alpha[k] < 0) return invalid("vMF mixtureAlpha must be non-negative");
        any = any || alpha[k] > 0;
    }
    if (!any) return invalid("vMF mixtureAlpha must not be all zero");
    const int32_t e = set_scattering(s, mat, SSTMC_SCATTERING_VMF_MIXTURE);
    if (e) return e;
    s->mu[mat].assign(mu, mu + mixtures);
    s->c[mat].assign(c, c + mixtures);
    s->alpha[mat].assign(alpha, alpha + mixtures);
    return SSTMC_NO_ERROR;
}

int32_t sstmc_medium_create_heterogeneous(const uint32_t* grid, const double* x, uint32_t nx, const double* y, uint32_t ny,
                                          const double* z, uint32_t nz, sstmc_medium** out)
{
    if (!out) return SSTMC_INVALID_HANDLE;
    *out = nullptr;
    if (!grid || !x || !y) return invalid("a heterogeneous medium needs its material grid and axes");
    if (nx < 2 || ny < 2 || (z && nz < 2)) return invalid("every medium axis needs at least 2 edges");
    if (!finite_all(x, nx) || !finite_all(y, ny) || (z && !finite_all(z, nz))) return invalid("medium axes must be finite");
    const int32_t e = make(out);
    if (e) return e;
    sstmc_medium* m = *out;
    m->type = SSTMC_MEDIUM_HETEROGENEOUS;
    m->dims = z ? 3 : 2;
    m->ax[0].assign(x, x + nx);
    m->ax[1].assign(y, y + ny);
    if (z) m->ax[2].assign(z, z + nz);
    const size_t cells = (size_t)(nx - 1) * (ny - 1) * (z ? nz - 1 : 1);
    m->grid.assign(grid, grid + cells);
    return SSTMC_NO_ERROR;
}

int32_t sstmc_medium_create_homogeneous(uint32_t dims, const double box_min[3], const double box_max[3], double sigs,
                                        sstmc_medium** out)
{
    if (!out) return SSTMC_INVALID_HANDLE;
    *out = nullptr;
    if (dims != 2 && dims != 3) return invalid("dims must be 2 or 3");
    if (!box_min || !box_max) return invalid("a homogeneous medium needs its box");
    const int32_t e = make(out);
    if (e) return e;
    sstmc_medium* m = *out;
    m->type = SSTMC_MEDIUM_HOMOGENEOUS;
    m->dims = dims;
    for (int i = 0; i < 3; ++i) { m->box_min[i] = box_min[i]; m->box_max[i] = box_max[i]; }
    m->homogeneous_sigs = sigs;
    return SSTMC_NO_ERROR;
}

int32_t sstmc_medium_set_material(sstmc_medium* m, double sigs, double siga, uint32_t mat)
{
    if (!m) return SSTMC_INVALID_HANDLE;
    if (mat >= SSTMC_MATERIAL_NUM) return invalid("medium material index out of range (0 .. 9)");
    if (!std::isfinite(sigs) || !std::isfinite(siga) || sigs < 0 || siga < 0)
        return invalid("sigs and siga must be finite and non-negative");
    m->sigs[mat] = sigs;
    m->siga[mat] = siga;
    if (mat + 1 > m->count) m->count = mat + 1;
    return SSTMC_NO_ERROR;
}

int32_t sstmc_medium_destroy(sstmc_medium* m) { delete m; return SSTMC_NO_ERROR; }

int32_t sstmc_source_create_point(const sstmc_simulation* sim, int32_t connection, const double* xyz, uint32_t count,
                                  int32_t is_area_source, sstmc_source** out)
{
    if (!sim) return SSTMC_INVALID_HANDLE;
    return make_source(SSTMC_SOURCE_POINT, connection, xyz, count, is_area_source, sim->dims, out);
}

int32_t sstmc_source_create_far_field(const sstmc_simulation* sim, int32_t connection, const double* xyz, uint32_t count,
                                      sstmc_source** out)
{
    if (!sim) return SSTMC_INVALID_HANDLE;
    return make_source(SSTMC_SOURCE_FARFIELD, connection, xyz, count, 0, sim->dims, out);
}

int32_t sstmc_source_create_gaussian_beam(const sstmc_simulation* sim, int32_t connection, const double* focal_points,
                                          const double* focal_directions, uint32_t count, double aperture, sstmc_source** out)
{
    if (!sim) return SSTMC_INVALID_HANDLE;
    if (!focal_directions || count == 0 || !finite_all(focal_directions, (size_t)3 * count))
        return invalid("a Gaussian beam needs a finite focal direction per focal point");
    if (!(aperture > 0.0) || !std::isfinite(aperture)) return invalid("the Gaussian-beam aperture must be positive");
    const int32_t e = make_source(SSTMC_SOURCE_GAUSSIANBEAM, connection, focal_points, count, 0, sim->dims, out);
    if (e) return e;
    (*out)->dir.assign(focal_directions, focal_directions + (size_t)3 * count);
    if (sim->dims == 2)
        for (uint32_t i = 0; i < count; ++i) (*out)->dir[3 * i + 2] = 0.0;
    (*out)->aperture = aperture;
    return SSTMC_NO_ERROR;
}

int32_t sstmc_source_size(const sstmc_source* s, uint32_t* count)
{
    if (!s || !count) return SSTMC_INVALID_HANDLE;
    *count = (uint32_t)(s->xyz.size() / 3);
    return SSTMC_NO_ERROR;
}

int32_t sstmc_source_destroy(sstmc_source* s) { delete s; return SSTMC_NO_ERROR; }

int32_t sstmc_sampler_create_temporal(const sstmc_simulation* sim, const sstmc_medium* medium, const sstmc_scattering* scattering,
                                      const sstmc_source* illumination, const sstmc_source* view, const double* t, uint32_t t_num,
                                      int32_t is_temporal_amplitude, int32_t is_forced_inside_bin, sstmc_sampler** out)
{
    const sstmc_source* src[4] = { illumination, view, nullptr, nullptr };
    const int32_t e = make_sampler(SSTMC_SAMPLER_TEMPORAL, sim, medium, scattering, src, t, t_num, out);
    if (e) return e;
    (*out)->temporal_amplitude = is_temporal_amplitude ? 1 : 0;
    (*out)->forced_inside_bin = is_forced_inside_bin ? 1 : 0;
    return SSTMC_NO_ERROR;
}

int32_t sstmc_sampler_create_correlation(const sstmc_simulation* sim, const sstmc_medium* medium, const sstmc_scattering* scattering,
                                         const sstmc_source* illumination, const sstmc_source* illumination2,
                                         const sstmc_source* view, const sstmc_source* view2, const double* t, uint32_t t_num,
                                         sstmc_sampler** out)
{
    const sstmc_source* src[4] = { illumination, view, illumination2, view2 };
    return make_sampler(SSTMC_SAMPLER_TEMPORAL_CORRELATION, sim, medium, scattering, src, t, t_num, out);
}

int32_t sstmc_sampler_set_material(sstmc_sampler* s, double D, const double U[3], uint32_t mat)
{
    if (!s) return SSTMC_INVALID_HANDLE;
    if (mat >= SSTMC_MATERIAL_NUM) return invalid("sampler material index out of range (0 .. 9)");
    if (!std::isfinite(D) || D < 0) return invalid("D values in temporal sampler must be non-negative");
    const double u0[3] = { 0.0, 0.0, 0.0 };
    const double* u = U ? U : u0;
    if (!finite_all(u, 3)) return invalid("U must be finite");
    s->D[mat] = D;
    for (int i = 0; i < 3; ++i) s->U[mat][i] = (i == 2 && s->sim && s->sim->dims == 2) ? 0.0 : u[i];
    if (mat + 1 > s->count) s->count = mat + 1;
    return SSTMC_NO_ERROR;
}

int32_t sstmc_sampler_shape(const sstmc_sampler* s, uint32_t* nl, uint32_t* nv, uint32_t* nt)
{
    if (!s) return SSTMC_INVALID_HANDLE;
    if (nl) *nl = (uint32_t)(s->src[0]->xyz.size() / 3);
    if (nv) *nv = (uint32_t)(s->src[1]->xyz.size() / 3);
    if (nt) *nt = (uint32_t)s->t.size();
    return SSTMC_NO_ERROR;
}

int32_t sstmc_sampler_is_correlation(const sstmc_sampler* s, int32_t* is_correlation)
{
    if (!s || !is_correlation) return SSTMC_INVALID_HANDLE;
    *is_correlation = s->type == SSTMC_SAMPLER_TEMPORAL_CORRELATION ? 1 : 0;
    return SSTMC_NO_ERROR;
}

int32_t sstmc_sampler_config(sstmc_sampler* s, uint32_t full_iteration, uint64_t seed, int32_t is_cbs, sstmc_config* out)
{
    if (!s || !out) return SSTMC_INVALID_HANDLE;
    const sstmc_simulation& sim = *s->sim;
    const sstmc_medium& med = *s->medium;
    const sstmc_scattering& sc = *s->scattering;
    if (sc.count == 0) return invalid("the scattering object has no material set");
    sstmc_config_init(out);
    out->dims = sim.dims;
    out->batch_size = sim.batch_size;
    out->full_iteration = full_iteration;
    out->renderings_num = 1;
    out->lambda = sim.lambda;
    out->seed = seed;
    out->device_number = sim.device;
    out->precision = sim.precision;
    // scattering: one cell per material, 0 .. count - 1 (an unset material is isotropic-free: type 0)
    const uint32_t n = sc.count;
    s->c_type.assign(sc.type, sc.type + n);
    s->c_g.assign(sc.g, sc.g + n);
    s->c_tab_n.assign(n, 0); s->c_vmf_n.assign(n, 0);
    s->c_tab_f.clear(); s->c_vmf_mu.clear(); s->c_vmf_c.clear(); s->c_vmf_alpha.clear();
    bool any_tab = false, any_vmf = false;
    for (uint32_t m = 0; m < n; ++m) {
        if (sc.type[m] == SSTMC_SCATTERING_NOT_DEFINED) return invalid("scattering material " + std::to_string(m) + " is not set");
        if (sc.type[m] == SSTMC_SCATTERING_TABULAR) {
            any_tab = true;
            s->c_tab_n[m] = (uint32_t)(sc.tab[m].size() / 2);
            s->c_tab_f.insert(s->c_tab_f.end(), sc.tab[m].begin(), sc.tab[m].end());
        }
        if (sc.type[m] == SSTMC_SCATTERING_VMF_MIXTURE) {
            any_vmf = true;
            s->c_vmf_n[m] = (uint32_t)sc.mu[m].size();
            s->c_vmf_mu.insert(s->c_vmf_mu.end(), sc.mu[m].begin(), sc.mu[m].end());
            s->c_vmf_c.insert(s->c_vmf_c.end(), sc.c[m].begin(), sc.c[m].end());
            s->c_vmf_alpha.insert(s->c_vmf_alpha.end(), sc.alpha[m].begin(), sc.alpha[m].end());
        }
    }
    out->scattering_num = n;
    out->scattering_type = s->c_type.data();
    out->scattering_g = s->c_g.data();
    if (any_tab) { out->tabular_n = s->c_tab_n.data(); out->tabular_f = s->c_tab_f.data(); }
    if (any_vmf) {
        out->vmf_n = s->c_vmf_n.data(); out->vmf_mu = s->c_vmf_mu.data();
        out->vmf_c = s->c_vmf_c.data(); out->vmf_alpha = s->c_vmf_alpha.data();
    }
    // one material cell is material 1 as well (MatlabInterface.cu:750-760)
    const uint32_t mat_num = n > 1 ? n : 2;
    out->medium_type = med.type;
    if (med.type == SSTMC_MEDIUM_HETEROGENEOUS) {
        if (med.count != mat_num) return invalid("medium materials set: " + std::to_string(med.count) + ", expected "
                                                 + std::to_string(mat_num) + " (one per scattering material)");
        out->x_axis = med.ax[0].data(); out->x_axis_size = (uint32_t)med.ax[0].size();
        out->y_axis = med.ax[1].data(); out->y_axis_size = (uint32_t)med.ax[1].size();
        if (sim.dims == 3) { out->z_axis = med.ax[2].data(); out->z_axis_size = (uint32_t)med.ax[2].size(); }
        out->material_grid = med.grid.data();
        s->c_sigs.assign(med.sigs, med.sigs + mat_num);
        s->c_siga.assign(med.siga, med.siga + mat_num);
        out->sigs = s->c_sigs.data();
        out->siga = s->c_siga.data();
    } else {
        for (int i = 0; i < 3; ++i) { out->box_min[i] = med.box_min[i]; out->box_max[i] = med.box_max[i]; }
        out->homogeneous_sigs = med.homogeneous_sigs;
    }
    source_cfg(s->src[0], &out->illumination);
    source_cfg(s->src[1], &out->view);
    source_cfg(s->src[2], &out->illumination2);
    source_cfg(s->src[3], &out->view2);
    out->sampler_type = s->type;
    out->t = s->t.data();
    out->t_num = (uint32_t)s->t.size();
    if (s->count > mat_num) return invalid("sampler materials set beyond the scattering materials");
    s->c_D.assign(s->D, s->D + mat_num);
    s->c_U.assign((size_t)3 * mat_num, 0.0);
    for (uint32_t m = 0; m < mat_num; ++m)
        for (int i = 0; i < 3; ++i) s->c_U[3 * m + i] = s->U[m][i];
    out->D = s->c_D.data();
    out->U = s->c_U.data();
    out->is_temporal_amplitude = s->temporal_amplitude;
    out->is_forced_inside_bin = s->forced_inside_bin;
    out->is_cbs = is_cbs ? 1 : 0;
    return SSTMC_NO_ERROR;
}

int32_t sstmc_sampler_destroy(sstmc_sampler* s) { delete s; return SSTMC_NO_ERROR; }

int32_t sstmc_tracer_create_nee(sstmc_sampler* sampler, uint32_t full_iteration, uint64_t seed, int32_t is_cbs,
                                sstmc_tracer** out)
{
    if (!out || !sampler) return SSTMC_INVALID_HANDLE;
    *out = nullptr;
    if (full_iteration == 0) return invalid("fullIteration must be positive");
    sstmc_config cfg;
    int32_t e = sstmc_sampler_config(sampler, full_iteration, seed, is_cbs, &cfg);
    if (e) return e;
    sstmc_scene* scene = nullptr;
    e = sstmc_scene_create(&cfg, &scene);
    if (e) return e;
    sstmc_tracer* t = new (std::nothrow) sstmc_tracer();
    if (!t) { sstmc_scene_destroy(scene); return SSTMC_ALLOCATION_ERROR; }
    t->sampler = sampler; t->scene = scene; t->seed = seed; t->full_iteration = full_iteration; t->is_cbs = is_cbs ? 1 : 0;
    *out = t;
    return SSTMC_NO_ERROR;
}

int32_t sstmc_tracer_trace(sstmc_tracer* t, double* v)
{
    if (!t || !v) return SSTMC_INVALID_HANDLE;
    double iter = 0.0;
    const int32_t e = sstmc_render(t->scene, t->seed, v, &iter);
    if (e) return e;
    uint64_t vertices = 0;
    sstmc_last_stats(t->scene, nullptr, nullptr, &vertices, nullptr);
    const uint64_t budget = (uint64_t)t->sampler->sim->batch_size * t->full_iteration;
    t->zero_contribution_paths = (uint64_t)iter - budget;
    t->photons_budget = vertices;
    return SSTMC_NO_ERROR;
}

int32_t sstmc_tracer_update_seed(sstmc_tracer* t, uint64_t seed)
{
    if (!t) return SSTMC_INVALID_HANDLE;
    t->seed = seed;
    return SSTMC_NO_ERROR;
}

int32_t sstmc_tracer_zero_contribution_paths(const sstmc_tracer* t, uint64_t* out)
{
    if (!t || !out) return SSTMC_INVALID_HANDLE;
    *out = t->zero_contribution_paths;
    return SSTMC_NO_ERROR;
}

int32_t sstmc_tracer_photons_budget(const sstmc_tracer* t, uint64_t* out)
{
    if (!t || !out) return SSTMC_INVALID_HANDLE;
    *out = t->photons_budget;
    return SSTMC_NO_ERROR;
}

int32_t sstmc_tracer_is_cbs(const sstmc_tracer* t, int32_t* out)
{
    if (!t || !out) return SSTMC_INVALID_HANDLE;
    *out = t->is_cbs;
    return SSTMC_NO_ERROR;
}

sstmc_scene* sstmc_tracer_scene(sstmc_tracer* t) { return t ? t->scene : nullptr; }

int32_t sstmc_tracer_destroy(sstmc_tracer* t)
{
    if (!t) return SSTMC_INVALID_HANDLE;
    const int32_t e = t->scene ? sstmc_scene_destroy(t->scene) : SSTMC_NO_ERROR;
    delete t;
    return e;
}

}  // extern "C"
