/*
 * sph_oracle_gen.c — the seeded dam-break generator, restated on the oracle side.  TEST
 * INFRASTRUCTURE: it lets the benchmark's reference leg and the tests build the benchmark
 * workloads without loading the product library.
 *
 * The reference ships no input files (its ini_fluid, src/io/io.cu:6-111, reads seven text
 * files that are not in its tree), so the workloads are generated: a tank with `layers`
 * lattice layers of wall particles outside the floor and the four side walls (open top), an
 * optional rigid box obstacle on the lattice, and a water block at the x = 0, y = 0 corner,
 * every particle at (i + 1/2) dx on the lattice plus, optionally, a seeded uniform jitter of
 * +-jitter*dx per coordinate, hydrostatic pressure and the matching density in the water.
 * Output order: walls, obstacle, water.  The random stream is the 64-bit Mersenne twister
 * MT19937-64 (Matsumoto and Nishimura), written here from its published definition; each
 * jitter is 2u - 1 for the top 53 bits u of one draw.
 */
#include "sph_oracle.h"

#include <math.h>
#include <stdint.h>

/* ---- MT19937-64: degree 312, middle word 156, 31 lower bits in the twist ---- */
#define MT_N 312
#define MT_M 156
typedef struct {
    uint64_t s[MT_N];
    int i;
} or_mt64;

static void mt_seed(or_mt64* g, uint64_t seed)
{
    int i;
    g->s[0] = seed;
    for (i = 1; i < MT_N; i++)
        g->s[i] = 6364136223846793005ULL * (g->s[i - 1] ^ (g->s[i - 1] >> 62)) + (uint64_t)i;
    g->i = MT_N;
}

static uint64_t mt_next(or_mt64* g)
{
    const uint64_t upper = 0xFFFFFFFF80000000ULL, lower = 0x7FFFFFFFULL;
    const uint64_t matrix = 0xB5026F5AA96619E9ULL;
    uint64_t y;
    if (g->i >= MT_N) {
        int k;
        for (k = 0; k < MT_N; k++) {
            const uint64_t x = (g->s[k] & upper) | (g->s[(k + 1) % MT_N] & lower);
            g->s[k] = g->s[(k + MT_M) % MT_N] ^ (x >> 1) ^ ((x & 1ULL) ? matrix : 0ULL);
        }
        g->i = 0;
    }
    y = g->s[g->i++];
    y ^= (y >> 29) & 0x5555555555555555ULL;
    y ^= (y << 17) & 0x71D67FFFEDA60000ULL;
    y ^= (y << 37) & 0xFFF7EEE000000000ULL;
    y ^= y >> 43;
    return y;
}

static double mt_unit(or_mt64* g) { return (double)(mt_next(g) >> 11) * (1.0 / 9007199254740992.0); }

/* ---- lattice walk ---- */
static int lattice_count(float len, float dx) { return (int)floor((double)len / (double)dx + 0.5); }

static int in_box(double x, double y, double z, const float* lo, const float* hi)
{
    return x >= lo[0] && x <= hi[0] && y >= lo[1] && y <= hi[1] && z >= lo[2] && z <= hi[2];
}

typedef struct {
    const or_dam_break* d;
    float *pos, *vel, *rho, *p;
    int* type;
    long n, cap;
    or_mt64 rng;
    double amp, H, g, B, gamma;
} or_gen_state;

static void emit(or_gen_state* S, int kind, double x, double y, double z)
{
    const or_dam_break* d = S->d;
    double jx = 0.0, jy = 0.0, jz = 0.0, pr = 0.0, r = d->rho0;
    long i = S->n++;
    if (!S->pos) return; /* counting */
    if (i >= S->cap) return;
    if (S->amp > 0.0) {
        jx = (2.0 * mt_unit(&S->rng) - 1.0) * S->amp;
        jy = (2.0 * mt_unit(&S->rng) - 1.0) * S->amp;
        jz = (2.0 * mt_unit(&S->rng) - 1.0) * S->amp;
    }
    S->pos[3 * i] = (float)(x + jx);
    S->pos[3 * i + 1] = (float)(y + jy);
    S->pos[3 * i + 2] = (float)(z + jz);
    S->vel[3 * i] = S->vel[3 * i + 1] = S->vel[3 * i + 2] = 0.0f;
    S->type[i] = kind;
    if (kind == 1 && d->hydrostatic) {
        pr = (double)d->rho0 * S->g * (S->H - z);
        if (pr < 0.0) pr = 0.0;
        r = d->eos == 1 ? (double)d->rho0 * pow(pr / S->B + 1.0, 1.0 / S->gamma)
                        : (double)d->rho0 + pr / ((double)d->cs * (double)d->cs);
    }
    S->p[i] = (float)pr;
    S->rho[i] = (float)r;
}

static void walk(or_gen_state* S)
{
    const or_dam_break* d = S->d;
    const int ntx = lattice_count(d->tank[0], d->dx), nty = lattice_count(d->tank[1], d->dx),
              ntz = lattice_count(d->tank[2], d->dx);
    const int nbx = lattice_count(d->block[0], d->dx), nby = lattice_count(d->block[1], d->dx),
              nbz = lattice_count(d->block[2], d->dx);
    const int L = d->wall_layers;
    const double dx = d->dx;
    int i, j, k;
    for (k = -L; k < ntz; k++)
        for (j = -L; j < nty + L; j++)
            for (i = -L; i < ntx + L; i++) {
                if (i >= 0 && i < ntx && j >= 0 && j < nty && k >= 0) continue;
                emit(S, 0, (i + 0.5) * dx, (j + 0.5) * dx, (k + 0.5) * dx);
            }
    if (d->has_obstacle)
        for (k = 0; k < ntz; k++)
            for (j = 0; j < nty; j++)
                for (i = 0; i < ntx; i++) {
                    const double x = (i + 0.5) * dx, y = (j + 0.5) * dx, z = (k + 0.5) * dx;
                    if (in_box(x, y, z, d->obstacle_min, d->obstacle_max)) emit(S, 2, x, y, z);
                }
    for (k = 0; k < nbz; k++)
        for (j = 0; j < nby; j++)
            for (i = 0; i < nbx; i++) {
                const double x = (i + 0.5) * dx, y = (j + 0.5) * dx, z = (k + 0.5) * dx;
                if (d->has_obstacle && in_box(x, y, z, d->obstacle_min, d->obstacle_max)) continue;
                emit(S, 1, x, y, z);
            }
}

long or_dam_break_count(const or_dam_break* d, long* n_fluid)
{
    or_gen_state S = {0};
    const int nbx = lattice_count(d->block[0], d->dx), nby = lattice_count(d->block[1], d->dx),
              nbz = lattice_count(d->block[2], d->dx);
    const double dx = d->dx;
    long nf = 0;
    int i, j, k;
    S.d = d;
    walk(&S); /* no output arrays: counts every particle */
    for (k = 0; k < nbz; k++)
        for (j = 0; j < nby; j++)
            for (i = 0; i < nbx; i++) {
                const double x = (i + 0.5) * dx, y = (j + 0.5) * dx, z = (k + 0.5) * dx;
                if (d->has_obstacle && in_box(x, y, z, d->obstacle_min, d->obstacle_max)) continue;
                nf++;
            }
    if (n_fluid) *n_fluid = nf;
    return S.n;
}

int or_dam_break_generate(const or_dam_break* d, float* pos, float* vel, float* rho, float* p,
                          int* type, long n)
{
    or_gen_state S = {0};
    S.d = d;
    S.pos = pos;
    S.vel = vel;
    S.rho = rho;
    S.p = p;
    S.type = type;
    S.cap = n;
    mt_seed(&S.rng, d->seed);
    S.amp = (double)d->jitter * (double)d->dx;
    S.H = (double)lattice_count(d->block[2], d->dx) * (double)d->dx;
    S.g = fabs((double)d->gravity);
    S.gamma = d->tait_gamma > 0.f ? d->tait_gamma : 7.0;
    S.B = (double)d->rho0 * (double)d->cs * (double)d->cs / S.gamma;
    walk(&S);
    return S.n == n ? 0 : -1;
}
