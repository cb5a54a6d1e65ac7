/*
 * sph_oracle.c — CPU oracle of the SPH hot path (see sph_oracle.h).  TEST INFRASTRUCTURE:
 * only tests, the smoke check and the benchmark's CPU legs use it.
 *
 * Build: gcc -O2 -std=c11 -fopenmp -ffp-contract=off -fPIC -shared (oracle/build_oracle.py).
 * -ffp-contract=off keeps every float and double operation separately rounded, so the
 * float instantiation evaluates exactly the expression the reference writes.
 */
#include "sph_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_PI 3.141592654 /* the reference's PI (src/header/sph.cuh:4) */

int or_set_threads(int nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
    return omp_get_max_threads();
#else
    (void)nthreads;
    return 1;
#endif
}

static void or_fill_grid(or_params* P, double pad, const float dmin[3], const float dmax[3])
{
    int c;
    for (c = 0; c < 3; c++) {
        float span;
        /* pre_set_domain_*_min = -0.1 and *_max = vl* + 0.1, stored as float
         * (src/sph/sph_run.cu:76-87) */
        P->grid_min[c] = (float)((double)dmin[c] - pad);
        P->grid_max[c] = (float)((double)dmax[c] + pad);
        /* gridxdim = (int)ceil((gridxmax - gridxmin) / gridSize) in float (:88-90) */
        span = (P->grid_max[c] - P->grid_min[c]) / P->cell_size;
        P->grid_dim[c] = (int)ceilf(span);
    }
    P->num_cells = P->grid_dim[0] * P->grid_dim[1] * P->grid_dim[2];
}

void or_params_general(float dx, double h_factor, float rho0, float cs, float gravity,
                       float delta, float alpha, float dt, float cfl, int eos,
                       float tait_gamma, const float dmin[3], const float dmax[3], double pad,
                       double cell_factor, int np, int nb, or_params* P)
{
    memset(P, 0, sizeof(*P));
    P->num_particles = np;
    P->num_boundary = nb;
    P->gravity = gravity;
    P->dx = dx;
    P->cs = cs;
    P->rho0 = rho0;
    /* h = 1.5 * dx; kh = 2.0 * h; eta = 0.1 * h (src/sph/sph_run.cu:67-69) */
    P->h = (float)(h_factor * (double)dx);
    P->kh = (float)(2.0 * (double)P->h);
    P->eta = (float)(0.1 * (double)P->h);
    P->delta = delta;
    P->alpha = alpha;
    P->cell_size = (float)(cell_factor * (double)P->kh);
    /* particleMass = pow(particleR, 3) * restDensity (:73) */
    P->mass = (float)(pow((double)dx, 3.0) * (double)rho0);
    /* adh = 21.0 / (16.0 * PI * h * h * h) (:74) */
    P->adh = (float)(21.0 / (16.0 * OR_PI * (double)P->h * (double)P->h * (double)P->h));
    P->dt = dt > 0 ? dt : (float)((double)cfl * (double)P->h / (double)cs);
    P->eos = eos;
    P->tait_gamma = tait_gamma;
    P->tait_b = (float)((double)rho0 * (double)cs * (double)cs / (double)(tait_gamma > 0 ? tait_gamma : 7.0f));
    P->clamp_density = 1;
    or_fill_grid(P, pad, dmin, dmax);
    {
        int c;
        for (c = 0; c < 3; c++) {
            P->escape_min[c] = dmin[c];
            P->escape_max[c] = dmax[c];
        }
        P->escape_park[0] = dmin[0];
        P->escape_park[1] = (float)(0.5 * ((double)dmin[1] + (double)dmax[1]));
        P->escape_park[2] = (float)((double)dmin[2] - 0.08);
    }
}

void or_params_reference(float dx, float vlx, float vly, float vlz, int np, int nb,
                         or_params* P)
{
    const float dmin[3] = {0.0f, 0.0f, 0.0f};
    const float dmax[3] = {vlx, vly, vlz};
    /* src/sph/sph_run.cu:12-16,60-101: rho0 1000, g -9.81, cs 25, dt 2e-4, delta 0.2,
     * afa 0.05, gridSize = kh, padding 0.1 */
    or_params_general(dx, 1.5, 1000.0f, 25.0f, -9.81f, 0.2f, 0.05f, 2e-4f, 0.0f, 0, 7.0f,
                      dmin, dmax, 0.1, 1.0, np, nb, P);
    /* escape box and parking point hard-coded at src/sph/sph_run.cu:437-447 */
    P->escape_min[0] = 0.0f; P->escape_max[0] = 3.23f;
    P->escape_min[1] = 0.0f; P->escape_max[1] = 1.0f;
    P->escape_min[2] = 0.0f; P->escape_max[2] = 1.0f;
    P->escape_park[0] = 0.0f; P->escape_park[1] = 0.5f; P->escape_park[2] = -0.08f;
}

/* Stable LSD radix sort of (hash, index) by signed 32-bit key: the sign bit is flipped so
 * the unsigned digit order equals the signed order; passes whose digit is the same for
 * every key are skipped (they would not move anything). */
void or_sort_particles(int* hash, int* index, int n)
{
    unsigned* k0;
    unsigned* k1;
    int* v1;
    int shift, i;
    if (n <= 1) return;
    k0 = (unsigned*)malloc((size_t)n * sizeof(unsigned));
    k1 = (unsigned*)malloc((size_t)n * sizeof(unsigned));
    v1 = (int*)malloc((size_t)n * sizeof(int));
    if (!k0 || !k1 || !v1) {
        free(k0); free(k1); free(v1);
        abort();
    }
    for (i = 0; i < n; i++) k0[i] = (unsigned)hash[i] ^ 0x80000000u;
    for (shift = 0; shift < 32; shift += 8) {
        size_t count[257];
        int d;
        memset(count, 0, sizeof(count));
        for (i = 0; i < n; i++) count[((k0[i] >> shift) & 0xffu) + 1]++;
        for (d = 0; d < 256; d++)
            if (count[d + 1] == (size_t)n) break;
        if (d < 256) continue; /* every key has this digit */
        for (d = 0; d < 256; d++) count[d + 1] += count[d];
        for (i = 0; i < n; i++) {
            size_t dst = count[(k0[i] >> shift) & 0xffu]++;
            k1[dst] = k0[i];
            v1[dst] = index[i];
        }
        memcpy(k0, k1, (size_t)n * sizeof(unsigned));
        memcpy(index, v1, (size_t)n * sizeof(int));
    }
    for (i = 0; i < n; i++) hash[i] = (int)(k0[i] ^ 0x80000000u);
    free(k0); free(k1); free(v1);
}

#define REAL float
#define OR_SUFFIX _f32
#include "sph_oracle_phys.inc"
#undef REAL
#undef OR_SUFFIX

#define REAL double
#define OR_SUFFIX _f64
#include "sph_oracle_phys.inc"
#undef REAL
#undef OR_SUFFIX
