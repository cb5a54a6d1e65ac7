// params.cpp — derivation of the simulation constants and conversion to/from the reference's
// SimParams.  The derivation repeats the reference host block (src/sph/sph_run.cu:60-101)
// step for step in the same mixed double/float rounding, because the grid constants it
// produces (gridSize, grid minimum, grid dimensions) decide every cell hash bit for bit.
#include <cmath>
#include <cstring>

#include "sph_internal.h"

namespace {

constexpr double kPi = 3.141592654;  // the reference's PI (src/header/sph.cuh:4)

void fill_grid(sph_params* P, double pad, const float dmin[3], const float dmax[3]) {
    for (int c = 0; c < 3; c++) {
        P->grid_min[c] = (float)((double)dmin[c] - pad);
        P->grid_max[c] = (float)((double)dmax[c] + pad);
        float span = (P->grid_max[c] - P->grid_min[c]) / P->cell_size;  // float, as the reference
        P->grid_dim[c] = (int)std::ceil(span);
    }
    P->num_cells = P->grid_dim[0] * P->grid_dim[1] * P->grid_dim[2];
}

}  // namespace

namespace sph {

KParams make_kparams(const sph_params& p, int n) {
    KParams k{};
    k.n = n;
    k.gx = p.grid_dim[0];
    k.gy = p.grid_dim[1];
    k.gz = p.grid_dim[2];
    k.num_cells = p.num_cells;
    k.gz_local = p.grid_dim[2];
    k.gz_stride = p.grid_dim[2];
    k.inst_cells = 0;
    k.reach = 1;
    k.reach_cell = k.cell;
    k.threads = 128;
    k.ppt = 1;
    k.lanes = 1;
    k.list_win = 0;
    k.gmin_x = p.grid_min[0];
    k.gmin_y = p.grid_min[1];
    k.gmin_z = p.grid_min[2];
    k.cell = p.cell_size;
    k.inv_cell = 1.0 / (double)p.cell_size;
    k.h = p.h;
    k.inv_h = (float)(1.0 / (double)p.h);
    k.kh = p.kh;
    k.kh2 = p.kh * p.kh;
    k.kh2_list = k.kh2;
    k.eta2 = p.eta * p.eta;
    k.adh = p.adh;
    k.c_fr = (float)(-5.0 * (double)p.adh / ((double)p.h * (double)p.h));
    k.mass = p.mass;
    k.c_fr_mass = (float)(-5.0 * (double)p.adh / ((double)p.h * (double)p.h) * (double)p.mass);
    k.rho0 = p.rho0;
    k.cs = p.cs;
    k.g = p.gravity;
    k.half_dt = (float)((double)p.dt / 2.0);
    k.delta_h_cs = p.delta * p.h * p.cs;
    k.damper = p.rho0 * p.cs * p.h;
    k.visc = p.alpha * p.h * p.cs * p.rho0;
    k.eos = p.eos;
    k.tait_gamma = p.tait_gamma;
    k.tait_b = p.tait_b;
    k.inv_tait_b = p.tait_b != 0.f ? (float)(1.0 / (double)p.tait_b) : 0.f;
    k.inv_gamma = p.tait_gamma != 0.f ? (float)(1.0 / (double)p.tait_gamma) : 0.f;
    k.inv_cs2 = (float)(1.0 / ((double)p.cs * (double)p.cs));
    k.clamp_density = p.clamp_density;
    k.esc_min_x = p.escape_min[0];
    k.esc_min_y = p.escape_min[1];
    k.esc_min_z = p.escape_min[2];
    k.esc_max_x = p.escape_max[0];
    k.esc_max_y = p.escape_max[1];
    k.esc_max_z = p.escape_max[2];
    k.park_x = p.escape_park[0];
    k.park_y = p.escape_park[1];
    k.park_z = p.escape_park[2];
    k.park_inactive = p.park_inactive;
    k.inst_boxes = 0;
    return k;
}

template <>
KParams make_kparams_t<float>(const sph_params& p, int n) {
    return make_kparams(p, n);
}

// The same constants in double, from the same float parameters (the FP64 solver runs the
// parameters the FP32 solver runs, without rounding anything derived from them to float).
template <>
KParamsT<double> make_kparams_t<double>(const sph_params& p, int n) {
    KParamsT<double> k{};
    k.n = n;
    k.gx = p.grid_dim[0];
    k.gy = p.grid_dim[1];
    k.gz = p.grid_dim[2];
    k.num_cells = p.num_cells;
    k.gz_local = p.grid_dim[2];
    k.gz_stride = p.grid_dim[2];
    k.inst_cells = 0;
    k.reach = 1;
    k.reach_cell = k.cell;
    k.threads = 128;
    k.ppt = 1;
    k.lanes = 1;
    k.list_win = 0;
    k.gmin_x = p.grid_min[0];
    k.gmin_y = p.grid_min[1];
    k.gmin_z = p.grid_min[2];
    k.cell = p.cell_size;
    k.inv_cell = 1.0 / (double)p.cell_size;
    const double h = p.h, kh = p.kh, cs = p.cs, rho0 = p.rho0;
    k.h = h;
    k.inv_h = 1.0 / h;
    k.kh = kh;
    k.kh2 = kh * kh;
    k.kh2_list = k.kh2;
    k.eta2 = (double)p.eta * (double)p.eta;
    k.adh = p.adh;
    k.c_fr = -5.0 * (double)p.adh / (h * h);
    k.mass = p.mass;
    k.c_fr_mass = -5.0 * (double)p.adh / (h * h) * (double)p.mass;
    k.rho0 = rho0;
    k.cs = cs;
    k.g = p.gravity;
    k.half_dt = (double)p.dt / 2.0;
    k.delta_h_cs = (double)p.delta * h * cs;
    k.damper = rho0 * cs * h;
    k.visc = (double)p.alpha * h * cs * rho0;
    k.eos = p.eos;
    k.tait_gamma = p.tait_gamma;
    k.tait_b = p.tait_b;
    k.inv_tait_b = p.tait_b != 0.f ? 1.0 / (double)p.tait_b : 0.0;
    k.inv_gamma = p.tait_gamma != 0.f ? 1.0 / (double)p.tait_gamma : 0.0;
    k.inv_cs2 = 1.0 / (cs * cs);
    k.clamp_density = p.clamp_density;
    k.esc_min_x = p.escape_min[0];
    k.esc_min_y = p.escape_min[1];
    k.esc_min_z = p.escape_min[2];
    k.esc_max_x = p.escape_max[0];
    k.esc_max_y = p.escape_max[1];
    k.esc_max_z = p.escape_max[2];
    k.park_x = p.escape_park[0];
    k.park_y = p.escape_park[1];
    k.park_z = p.escape_park[2];
    k.park_inactive = p.park_inactive;
    k.inst_boxes = 0;
    return k;
}

}  // namespace sph

extern "C" int sph_params_derive(const sph_config* c, sph_params* P) {
    if (!c || !P || !(c->dx > 0.f) || !(c->h_factor > 0.0) || !(c->cs > 0.f) ||
        !(c->rho0 > 0.f) || c->num_particles < 0)
        return SPH_ERR_ARG;
    const double cell_factor = c->cell_factor > 0.0 ? c->cell_factor : 1.0;
    std::memset(P, 0, sizeof(*P));
    P->num_particles = c->num_particles;
    P->num_boundary = c->num_boundary;
    P->gravity = c->gravity;
    P->dx = c->dx;
    P->cs = c->cs;
    P->rho0 = c->rho0;
    // h = 1.5 * dx; kh = 2.0 * h; eta = 0.1 * h (src/sph/sph_run.cu:67-69)
    P->h = (float)(c->h_factor * (double)c->dx);
    P->kh = (float)(2.0 * (double)P->h);
    P->eta = (float)(0.1 * (double)P->h);
    P->delta = c->delta;
    P->alpha = c->alpha;
    P->cell_size = (float)(cell_factor * (double)P->kh);
    // particleMass = pow(particleR, 3) * restDensity; adh = 21/(16 PI h^3) (:73-74)
    P->mass = (float)(std::pow((double)c->dx, 3.0) * (double)c->rho0);
    P->adh = (float)(21.0 / (16.0 * kPi * (double)P->h * (double)P->h * (double)P->h));
    if (c->dt > 0.f) {
        P->dt = c->dt;
    } else {
        if (!(c->cfl > 0.f)) return SPH_ERR_ARG;
        P->dt = (float)((double)c->cfl * (double)P->h / (double)c->cs);
    }
    P->eos = c->eos;
    P->tait_gamma = c->tait_gamma > 0.f ? c->tait_gamma : 7.0f;
    P->tait_b = (float)((double)c->rho0 * (double)c->cs * (double)c->cs / (double)P->tait_gamma);
    P->clamp_density = c->clamp_density;
    fill_grid(P, c->pad, c->domain_min, c->domain_max);
    for (int k = 0; k < 3; k++) {
        P->escape_min[k] = c->escape_min[k];
        P->escape_max[k] = c->escape_max[k];
        P->escape_park[k] = c->escape_park[k];
    }
    if (P->num_cells <= 0 || P->grid_dim[0] <= 0 || P->grid_dim[1] <= 0 || P->grid_dim[2] <= 0)
        return SPH_ERR_ARG;
    return SPH_OK;
}

extern "C" int sph_params_reference(float dx, float vlx, float vly, float vlz, int np, int nb,
                                    sph_params* out) {
    // src/sph/sph_run.cu:11-16,60-101: rho0 1000, g -9.81, cs 25, dt 2e-4, h = 1.5 dx,
    // delta 0.2, afa 0.05, gridSize = kh, domain padded by 0.1 m, linear EOS, rho clamp.
    sph_config c;
    std::memset(&c, 0, sizeof(c));
    c.dx = dx;
    c.h_factor = 1.5;
    c.rho0 = 1000.0f;
    c.cs = 25.0f;
    c.gravity = -9.81f;
    c.delta = 0.2f;
    c.alpha = 0.05f;
    c.dt = 2e-4f;
    c.eos = SPH_EOS_LINEAR;
    c.tait_gamma = 7.0f;
    c.domain_max[0] = vlx;
    c.domain_max[1] = vly;
    c.domain_max[2] = vlz;
    c.pad = 0.1;
    c.cell_factor = 1.0;
    // escape box and parking point hard-coded at src/sph/sph_run.cu:437-447
    c.escape_max[0] = 3.23f;
    c.escape_max[1] = 1.0f;
    c.escape_max[2] = 1.0f;
    c.escape_park[1] = 0.5f;
    c.escape_park[2] = -0.08f;
    c.num_particles = np;
    c.num_boundary = nb;
    c.clamp_density = 1;
    return sph_params_derive(&c, out);
}

extern "C" int sph_params_from_reference(const sph_ref_simparams* r, sph_params* P) {
    if (!r || !P) return SPH_ERR_ARG;
    std::memset(P, 0, sizeof(*P));
    P->num_particles = r->numParticles;
    P->num_boundary = r->boundary_p_num;
    P->dt = r->timeStep;
    P->gravity = r->gravity;
    P->cell_size = r->gridSize;
    P->grid_min[0] = r->gridxmin;
    P->grid_min[1] = r->gridymin;
    P->grid_min[2] = r->gridzmin;
    P->grid_max[0] = r->gridxmax;
    P->grid_max[1] = r->gridymax;
    P->grid_max[2] = r->gridzmax;
    P->grid_dim[0] = r->gridxdim;
    P->grid_dim[1] = r->gridydim;
    P->grid_dim[2] = r->gridzdim;
    P->num_cells = r->numCells;
    P->dx = r->particleR;
    P->h = r->h;
    P->kh = r->kh;
    P->eta = r->eta;
    P->delta = r->delta;
    P->alpha = r->afa;
    P->adh = r->adh;
    P->mass = r->particleMass;
    P->rho0 = r->restDensity;
    P->cs = r->cs;
    P->eos = SPH_EOS_LINEAR;
    P->tait_gamma = 7.0f;
    P->tait_b = (float)((double)r->restDensity * (double)r->cs * (double)r->cs / 7.0);
    P->clamp_density = 1;
    P->escape_max[0] = 3.23f;
    P->escape_max[1] = 1.0f;
    P->escape_max[2] = 1.0f;
    P->escape_park[1] = 0.5f;
    P->escape_park[2] = -0.08f;
    if (P->num_cells <= 0 || !(P->cell_size > 0.f)) return SPH_ERR_ARG;
    return SPH_OK;
}

extern "C" int sph_params_to_reference(const sph_params* P, sph_ref_simparams* r) {
    if (!r || !P) return SPH_ERR_ARG;
    std::memset(r, 0, sizeof(*r));
    r->timeStep = P->dt;
    r->numParticles = P->num_particles;
    r->boundary_p_num = P->num_boundary;
    r->gravity = P->gravity;
    r->gridSize = P->cell_size;
    r->gridxmin = P->grid_min[0];
    r->gridymin = P->grid_min[1];
    r->gridzmin = P->grid_min[2];
    r->gridxmax = P->grid_max[0];
    r->gridymax = P->grid_max[1];
    r->gridzmax = P->grid_max[2];
    r->gridxdim = P->grid_dim[0];
    r->gridydim = P->grid_dim[1];
    r->gridzdim = P->grid_dim[2];
    r->numCells = P->num_cells;
    // hash_max as the reference sets it (src/sph/sph_run.cu:92)
    r->hash_max = P->grid_dim[0] * P->grid_dim[1] * P->grid_dim[2] +
                  P->grid_dim[0] * P->grid_dim[1] + P->grid_dim[0];
    r->hash_min = 0;
    r->pre_set_domain_x_min = P->grid_min[0];
    r->pre_set_domain_y_min = P->grid_min[1];
    r->pre_set_domain_z_min = P->grid_min[2];
    r->pre_set_domain_x_max = P->grid_max[0];
    r->pre_set_domain_y_max = P->grid_max[1];
    r->pre_set_domain_z_max = P->grid_max[2];
    r->particleR = P->dx;
    r->h = P->h;
    r->kh = P->kh;
    r->eta = P->eta;
    r->delta = P->delta;
    r->afa = P->alpha;
    r->particleMass = P->mass;
    r->restDensity = P->rho0;
    r->cs = P->cs;
    r->adh = P->adh;
    return SPH_OK;
}

extern "C" const char* sph_status_string(int s) {
    switch (s) {
        case SPH_OK: return "ok";
        case SPH_ERR_ARG: return "invalid argument";
        case SPH_ERR_CUDA: return "CUDA runtime error";
        case SPH_ERR_NOMEM: return "device allocation failed";
        case SPH_ERR_DEVICE: return "device error flag raised";
        case SPH_ERR_STATE: return "call out of order";
        case SPH_ERR_SCRATCH: return "scratch buffer too small";
        default: return "unknown status";
    }
}

extern "C" const char* sph_version(void) { return "tmp_sph_gb300 0.1 (sm_103a)"; }
