// dam_break.cpp — initial conditions and the reference's text input format.
//
// The reference reads its initial state from seven whitespace text files in the working
// directory (ini_fluid, src/io/io.cu:6-111) that are not part of its source tree.  This file
// generates that state for the dam-break family of cases — tank with wall_layers lattice
// layers outside the floor and four side walls (open top), a water block at the x = 0, y = 0
// corner, an optional rigid box obstacle — and writes / reads the same seven files.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>
#include <string>

#include "sph_gb300.h"

namespace {

int lattice_count(float len, float dx) { return (int)std::floor((double)len / (double)dx + 0.5); }

bool in_box(double x, double y, double z, const float* lo, const float* hi) {
    return x >= lo[0] && x <= hi[0] && y >= lo[1] && y <= hi[1] && z >= lo[2] && z <= hi[2];
}

// Walks every particle in output order (boundary and rigid particles first, then fluid) and
// calls f(kind, lattice x, y, z).
template <class F>
void walk(const sph_dam_break& d, F&& f) {
    const int ntx = lattice_count(d.tank[0], d.dx), nty = lattice_count(d.tank[1], d.dx),
              ntz = lattice_count(d.tank[2], d.dx);
    const int nbx = lattice_count(d.block[0], d.dx), nby = lattice_count(d.block[1], d.dx),
              nbz = lattice_count(d.block[2], d.dx);
    const int L = d.wall_layers;
    const double dx = d.dx;
    for (int k = -L; k < ntz; k++)
        for (int j = -L; j < nty + L; j++)
            for (int i = -L; i < ntx + L; i++) {
                if (i >= 0 && i < ntx && j >= 0 && j < nty && k >= 0) continue;
                f(SPH_TYPE_WALL, (i + 0.5) * dx, (j + 0.5) * dx, (k + 0.5) * dx);
            }
    if (d.has_obstacle)
        for (int k = 0; k < ntz; k++)
            for (int j = 0; j < nty; j++)
                for (int i = 0; i < ntx; i++) {
                    double x = (i + 0.5) * dx, y = (j + 0.5) * dx, z = (k + 0.5) * dx;
                    if (in_box(x, y, z, d.obstacle_min, d.obstacle_max)) f(SPH_TYPE_RIGID, x, y, z);
                }
    for (int k = 0; k < nbz; k++)
        for (int j = 0; j < nby; j++)
            for (int i = 0; i < nbx; i++) {
                double x = (i + 0.5) * dx, y = (j + 0.5) * dx, z = (k + 0.5) * dx;
                if (d.has_obstacle && in_box(x, y, z, d.obstacle_min, d.obstacle_max)) continue;
                f(SPH_TYPE_FLUID, x, y, z);
            }
}

bool valid(const sph_dam_break* d) {
    return d && d->dx > 0.f && d->tank[0] > 0.f && d->tank[1] > 0.f && d->tank[2] > 0.f &&
           d->block[0] >= 0.f && d->block[1] >= 0.f && d->block[2] >= 0.f &&
           d->wall_layers >= 0 && d->jitter >= 0.f && d->jitter < 0.5f;
}

// Uniform double in [0, 1) from the top 53 bits of a 64-bit Mersenne-twister draw (identical
// on every platform, unlike std::uniform_real_distribution).
double unit(std::mt19937_64& g) { return (double)(g() >> 11) * (1.0 / 9007199254740992.0); }

}  // namespace

extern "C" int sph_dam_break_count(const sph_dam_break* d, int* n_fluid, int* n_boundary) {
    if (!valid(d)) return SPH_ERR_ARG;
    long long nf = 0, nb = 0;
    walk(*d, [&](int kind, double, double, double) {
        if (kind == SPH_TYPE_FLUID) nf++; else nb++;
    });
    if (nf + nb > 0x7fffffffLL) return SPH_ERR_ARG;
    if (n_fluid) *n_fluid = (int)nf;
    if (n_boundary) *n_boundary = (int)nb;
    return SPH_OK;
}

extern "C" int sph_dam_break_generate(const sph_dam_break* d, float* pos, float* vel, float* rho,
                                      float* p, int* type, int n) {
    int nf = 0, nb = 0;
    int st = sph_dam_break_count(d, &nf, &nb);
    if (st != SPH_OK) return st;
    if (n != nf + nb || !pos || !vel || !rho || !p || !type) return SPH_ERR_ARG;
    std::mt19937_64 rng(d->seed);
    const double amp = (double)d->jitter * (double)d->dx;
    const double H = (double)lattice_count(d->block[2], d->dx) * (double)d->dx;
    const double g = std::fabs((double)d->gravity);
    const double gamma = d->tait_gamma > 0.f ? d->tait_gamma : 7.0;
    const double B = (double)d->rho0 * (double)d->cs * (double)d->cs / gamma;
    long i = 0;
    walk(*d, [&](int kind, double x, double y, double z) {
        double jx = 0, jy = 0, jz = 0;
        if (amp > 0) {
            jx = (2.0 * unit(rng) - 1.0) * amp;
            jy = (2.0 * unit(rng) - 1.0) * amp;
            jz = (2.0 * unit(rng) - 1.0) * amp;
        }
        pos[3 * i] = (float)(x + jx);
        pos[3 * i + 1] = (float)(y + jy);
        pos[3 * i + 2] = (float)(z + jz);
        vel[3 * i] = vel[3 * i + 1] = vel[3 * i + 2] = 0.f;
        type[i] = kind;
        double pr = 0.0, r = d->rho0;
        if (kind == SPH_TYPE_FLUID && d->hydrostatic) {
            pr = (double)d->rho0 * g * (H - z);
            if (pr < 0) pr = 0;
            r = d->eos == SPH_EOS_TAIT ? (double)d->rho0 * std::pow(pr / B + 1.0, 1.0 / gamma)
                                       : (double)d->rho0 + pr / ((double)d->cs * (double)d->cs);
        }
        p[i] = (float)pr;
        rho[i] = (float)r;
        i++;
    });
    return SPH_OK;
}

namespace {

bool write_floats(const std::string& path, const float* v, long count, int per_line) {
    FILE* f = std::fopen(path.c_str(), "w");
    if (!f) return false;
    for (long i = 0; i < count; i++)
        std::fprintf(f, (i % per_line == per_line - 1) ? "%.9g\n" : "%.9g ", (double)v[i]);
    return std::fclose(f) == 0;
}

bool write_ints(const std::string& path, const int* v, long count) {
    FILE* f = std::fopen(path.c_str(), "w");
    if (!f) return false;
    for (long i = 0; i < count; i++) std::fprintf(f, "%d\n", v ? v[i] : 0);
    return std::fclose(f) == 0;
}

bool read_floats(const std::string& path, float* v, long count) {
    FILE* f = std::fopen(path.c_str(), "r");
    if (!f) return false;
    bool ok = true;
    for (long i = 0; i < count && ok; i++) {
        float x;
        ok = std::fscanf(f, "%f", &x) == 1;
        if (ok && v) v[i] = x;
    }
    std::fclose(f);
    return ok;
}

bool read_ints(const std::string& path, int* v, long count) {
    FILE* f = std::fopen(path.c_str(), "r");
    if (!f) return false;
    bool ok = true;
    for (long i = 0; i < count && ok; i++) {
        int x;
        ok = std::fscanf(f, "%d", &x) == 1;
        if (ok && v) v[i] = x;
    }
    std::fclose(f);
    return ok;
}

}  // namespace

extern "C" int sph_write_dat(const char* dir, const float* pos, const float* vel, const float* rho,
                             const float* p, const int* type, int n) {
    if (!dir || n < 0 || (n > 0 && (!pos || !vel || !rho || !p || !type))) return SPH_ERR_ARG;
    const std::string d = std::string(dir) + "/";
    const long n3 = 3L * n;
    float* zeros = new (std::nothrow) float[n3 > 0 ? n3 : 1]();
    if (!zeros) return SPH_ERR_NOMEM;
    bool ok = write_floats(d + "h_pos.dat", pos, n3, 3) && write_floats(d + "h_vel.dat", vel, n3, 3) &&
              write_floats(d + "h_ac.dat", zeros, n3, 3) && write_floats(d + "rhop.dat", rho, n, 1) &&
              write_floats(d + "p.dat", p, n, 1) && write_ints(d + "particle_type.dat", type, n) &&
              write_ints(d + "particle_zone.dat", nullptr, n);
    delete[] zeros;
    return ok ? SPH_OK : SPH_ERR_ARG;
}

extern "C" int sph_read_dat(const char* dir, float* pos, float* vel, float* ac, float* rho, float* p,
                            int* type, int* zone, int n) {
    if (!dir || n < 0) return SPH_ERR_ARG;
    const std::string d = std::string(dir) + "/";
    const long n3 = 3L * n;
    bool ok = read_floats(d + "h_pos.dat", pos, n3) && read_floats(d + "h_vel.dat", vel, n3) &&
              read_floats(d + "h_ac.dat", ac, n3) && read_floats(d + "rhop.dat", rho, n) &&
              read_floats(d + "p.dat", p, n) && read_ints(d + "particle_type.dat", type, n) &&
              read_ints(d + "particle_zone.dat", zone, n);
    return ok ? SPH_OK : SPH_ERR_ARG;
}
