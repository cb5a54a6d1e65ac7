/*
 * sph_oracle.h — CPU oracle for the SPH hot path.  TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference solver's baseline version (`src/`) of ZZPHUB/tmp_sph:
 * cell hash, stable key/value sort, reorder with cell start/end, recover, the two neighbour
 * kernels and the midpoint predictor-corrector, plus the step loop that chains them.  Each
 * function cites the reference lines it follows.  Only tests, the smoke check and the
 * benchmark's CPU-baseline / reference legs may call it; the product never does.
 *
 * Two instantiations of the physics:
 *   *_f32 : float state with the reference's own double-literal promotions, compiled with
 *           -ffp-contract=off (IEEE float/double, no fused multiply-add).
 *   *_f64 : the same algorithm with every quantity in double; the accuracy oracle.
 *
 * Pinning: cell hash / sort / reorder outputs are compared bit-for-bit, and the physics
 * outputs within tolerance, against fixtures produced by running the reference's own
 * compiled kernels on a GB300 (tests/golden/, generator script beside them).
 */
#ifndef SPH_ORACLE_H
#define SPH_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Oracle parameters: the reference's SimParams quantities (src/header/data_struct.cuh:4-44)
 * plus the options the reference hard-codes (EOS form, escape box, density clamp). */
typedef struct or_params {
    int   num_particles, num_boundary;
    float dt, gravity, cell_size;
    float grid_min[3], grid_max[3];
    int   grid_dim[3], num_cells;
    float dx, h, kh, eta, delta, alpha, adh, mass, rho0, cs;
    int   eos;              /* 0 linear (reference), 1 Tait */
    float tait_gamma, tait_b;
    int   clamp_density;
    float escape_min[3], escape_max[3], escape_park[3];
    int   park_inactive;    /* 1: fluid outside the escape box is left out of the cell lists */
    int   reserved[7];
} or_params;

/* Derivation of the reference's host block, src/sph/sph_run.cu:60-101, for its hard-coded
 * constants (h = 1.5 dx, kh = 2h, eta = 0.1h, delta 0.2, alpha 0.05, cs 25, dt 2e-4,
 * rho0 1000, g -9.81, padding 0.1 m) and the escape box of src/sph/sph_run.cu:437. */
void or_params_reference(float dx, float vlx, float vly, float vlz, int np, int nb,
                         or_params* out);

/* Same derivation with the constants as inputs (h_factor, delta, alpha, cs, dt, cfl, eos). */
void or_params_general(float dx, double h_factor, float rho0, float cs, float gravity,
                       float delta, float alpha, float dt, float cfl, int eos,
                       float tait_gamma, const float dmin[3], const float dmax[3], double pad,
                       double cell_factor, int np, int nb, or_params* out);

/* Stable ascending sort of (hash, index) by signed hash — the order thrust::sort_by_key
 * produces for int keys (src/lib/mesh.cu:73-86; CUB's LSD radix sort is stable). */
void or_sort_particles(int* hash, int* index, int n);

/* Number of threads the OpenMP loops may use (0 = library default). Returns the value used. */
int or_set_threads(int nthreads);

/* Seeded dam-break generator (sph_oracle_gen.c): the layout of the product's sph_dam_break,
 * restated so the oracle side builds the benchmark workloads on its own. */
typedef struct or_dam_break {
    float dx;
    float tank[3], block[3];
    int wall_layers, has_obstacle;
    float obstacle_min[3], obstacle_max[3];
    float jitter;
    unsigned long long seed;
    int hydrostatic;
    float rho0, gravity, cs;
    int eos;
    float tait_gamma;
} or_dam_break;
/* Particles of a case (returned) and its fluid particles (*n_fluid). */
long or_dam_break_count(const or_dam_break* d, long* n_fluid);
/* Fill pos/vel [3n], rho, p [n], type [n] (walls, obstacle, water); 0 on success. */
int or_dam_break_generate(const or_dam_break* d, float* pos, float* vel, float* rho, float* p,
                          int* type, long n);

/* ---- float instantiation (reference arithmetic) ---- */
void or_calc_hash_f32(const or_params* P, const float* pos, int* hash, int* index, int n);
void or_reorder_f32(const or_params* P, const float* pos, const float* vel, const float* rho,
                    const float* p, const int* type, const int* zone, float* s_pos,
                    float* s_vel, float* s_rho, float* s_p, int* s_type, int* s_zone,
                    const int* hash, const int* index, int* cell_start, int* cell_end, int n);
void or_recover_f32(float* pos, float* vel, float* rho, float* p, int n, const int* index,
                    int* type, int* zone, const float* s_pos, const float* s_vel,
                    const float* s_rho, const float* s_p, const int* s_type, const int* s_zone);
void or_sph_ns_f32(const or_params* P, float* s_pos, float* s_vel, float* s_rho, float* s_p,
                   const int* s_type, float* rho_dt, float* vel_dt, const int* cell_start,
                   const int* cell_end, int n, const int* hash, float* dofv,
                   float* rhop_sum, float* w_sum);
void or_pc_prediction_f32(const or_params* P, float* s_pos, float* s_vel, float* s_rho,
                          float* s_p, const float* rho_dt, const float* vel_dt, const int* index,
                          float* pos_tmp, float* vel_tmp, float* rho_tmp, int n,
                          const int* s_type);
void or_pc_correction_f32(const or_params* P, float* s_pos, float* s_vel, float* s_rho,
                          float* s_p, const float* rho_dt, const float* vel_dt, const int* index,
                          const float* pos_tmp, const float* vel_tmp, const float* rho_tmp,
                          int n, const int* s_type);
/* nsteps of the src step loop (src/sph/sph_run.cu:285-336) on a state in original order,
 * updated in place.  Returns 0, or -1 if allocation failed. */
int or_run_f32(const or_params* P, float* pos, float* vel, float* rho, float* p, int* type,
               int n, int nsteps);

/* ---- double instantiation (accuracy oracle) ---- */
void or_calc_hash_f64(const or_params* P, const double* pos, int* hash, int* index, int n);
void or_reorder_f64(const or_params* P, const double* pos, const double* vel,
                    const double* rho, const double* p, const int* type, const int* zone,
                    double* s_pos, double* s_vel, double* s_rho, double* s_p, int* s_type,
                    int* s_zone, const int* hash, const int* index, int* cell_start,
                    int* cell_end, int n);
void or_recover_f64(double* pos, double* vel, double* rho, double* p, int n, const int* index,
                    int* type, int* zone, const double* s_pos, const double* s_vel,
                    const double* s_rho, const double* s_p, const int* s_type,
                    const int* s_zone);
void or_sph_ns_f64(const or_params* P, double* s_pos, double* s_vel, double* s_rho,
                   double* s_p, const int* s_type, double* rho_dt, double* vel_dt,
                   const int* cell_start, const int* cell_end, int n, const int* hash,
                   double* dofv, double* rhop_sum, double* w_sum);
void or_pc_prediction_f64(const or_params* P, double* s_pos, double* s_vel, double* s_rho,
                          double* s_p, const double* rho_dt, const double* vel_dt,
                          const int* index, double* pos_tmp, double* vel_tmp, double* rho_tmp,
                          int n, const int* s_type);
void or_pc_correction_f64(const or_params* P, double* s_pos, double* s_vel, double* s_rho,
                          double* s_p, const double* rho_dt, const double* vel_dt,
                          const int* index, const double* pos_tmp, const double* vel_tmp,
                          const double* rho_tmp, int n, const int* s_type);
int or_run_f64(const or_params* P, double* pos, double* vel, double* rho, double* p,
               int* type, int n, int nsteps);

#ifdef __cplusplus
}
#endif
#endif
