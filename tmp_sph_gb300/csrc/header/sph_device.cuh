// sph_device.cuh — device-side building blocks shared by the cell-list, neighbour and
// integrator kernels: the per-launch constant block, cell coordinates/hash, the Wendland C2
// kernel in gradient-scalar form, the equation of state and the device error word.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "sph_gb300.h"

namespace sph {

// Constants every kernel reads, passed by value (they land in the kernel-parameter constant
// bank, which serves warp-uniform reads as fast as __constant__ memory and lets several
// contexts with different parameters run side by side).  Derived on the host from
// sph_params by make_kparams().
struct KParams {
    int n;
    int gx, gy, gz;      // grid dimensions
    int num_cells;
    float gmin_x, gmin_y, gmin_z;
    float cell;          // cell edge (gridSize)
    float h, inv_h, kh, kh2;
    float kh2_list;      // squared list cutoff (support radius + skin); kh2 without a skin
    float eta2;
    float adh;           // 21/(16 pi h^3)
    float c_fr;          // -5 adh / h^2: grad W = c_fr (1 - q/2)^3 r
    float mass, rho0, cs, g, half_dt;
    float delta_h_cs;    // delta h cs
    float damper;        // rho0 cs h
    float visc;          // alpha h cs rho0
    int eos;
    float tait_gamma, tait_b, inv_tait_b, inv_gamma;
    float inv_cs2;
    int clamp_density;
    float esc_min_x, esc_min_y, esc_min_z, esc_max_x, esc_max_y, esc_max_z;
    float park_x, park_y, park_z;
};

KParams make_kparams(const sph_params& p, int n);

// ---------------------------------------------------------------- cell math
// floorf((p - min) / gridSize) with explicitly IEEE-rounded subtract and divide, so the
// result is bit-identical to the reference's calcGridPos (src/lib/mesh.cu:6-17) whatever
// contraction flags the file is built with.
__device__ __forceinline__ int cell_coord(float p, float gmin, float cell) {
    return (int)floorf(__fdiv_rn(__fsub_rn(p, gmin), cell));
}

// Reference hash without clamping (src/lib/mesh.cu:20-23).
__device__ __forceinline__ int cell_hash_raw(const KParams& k, float x, float y, float z) {
    int cx = cell_coord(x, k.gmin_x, k.cell);
    int cy = cell_coord(y, k.gmin_y, k.cell);
    int cz = cell_coord(z, k.gmin_z, k.cell);
    return (cz * k.gx * k.gy) + (cy * k.gx) + cx;
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// Hash used by the resident solver: identical to the reference for in-grid positions; an
// out-of-grid or non-finite position is clamped into the grid and reported through `flag`.
__device__ __forceinline__ int cell_hash_clamped(const KParams& k, float x, float y, float z,
                                                 unsigned* flag) {
    if (!(isfinite(x) && isfinite(y) && isfinite(z))) {
        *flag |= SPH_FLAG_NONFINITE | SPH_FLAG_OUT_OF_GRID;
        x = isfinite(x) ? x : k.gmin_x;
        y = isfinite(y) ? y : k.gmin_y;
        z = isfinite(z) ? z : k.gmin_z;
    }
    int cx = cell_coord(x, k.gmin_x, k.cell);
    int cy = cell_coord(y, k.gmin_y, k.cell);
    int cz = cell_coord(z, k.gmin_z, k.cell);
    if ((unsigned)cx >= (unsigned)k.gx || (unsigned)cy >= (unsigned)k.gy ||
        (unsigned)cz >= (unsigned)k.gz) {
        *flag |= SPH_FLAG_OUT_OF_GRID;
        cx = clampi(cx, 0, k.gx - 1);
        cy = clampi(cy, 0, k.gy - 1);
        cz = clampi(cz, 0, k.gz - 1);
    }
    return (cz * k.gy + cy) * k.gx + cx;
}

// ---------------------------------------------------------------- equation of state
// Linear (the reference's only form, src/sph/sph_run.cu:467) or Tait.  The Tait form is
// evaluated as B expm1(gamma log1p((rho - rho0)/rho0)): accurate relative to p itself for the
// small density perturbations of weakly-compressible flow, where B((rho/rho0)^gamma - 1)
// would lose most of its float digits to cancellation.
__device__ __forceinline__ float eos_pressure(const KParams& k, float rho) {
    if (k.eos == SPH_EOS_TAIT)
        return k.tait_b * expm1f(k.tait_gamma * log1pf((rho - k.rho0) / k.rho0));
    return k.cs * k.cs * (rho - k.rho0);
}

// Inverse used for wall particles (src/equation/ns.cu:128 for the linear form).
__device__ __forceinline__ float eos_density(const KParams& k, float p) {
    if (k.eos == SPH_EOS_TAIT)
        return k.rho0 + k.rho0 * expm1f(k.inv_gamma * log1pf(p * k.inv_tait_b));
    return p / k.cs / k.cs + k.rho0;
}

__device__ __forceinline__ bool escaped(const KParams& k, float x, float y, float z) {
    return x > k.esc_max_x || x < k.esc_min_x || y > k.esc_max_y || y < k.esc_min_y ||
           z > k.esc_max_z || z < k.esc_min_z;
}

__device__ __forceinline__ bool is_fluid(float typef) { return typef == 1.0f; }

// Kernels of the cell-list rebuild take a gate word: NULL runs unconditionally, otherwise the
// kernel does nothing unless *gate is non-zero (decided on the device each half step, so one
// captured CUDA graph serves steps that rebuild and steps that reuse the neighbour list).
// Every thread of a block reads the same word, so a gated-off block returns as a whole.
__device__ __forceinline__ bool gated_off(const unsigned* gate) {
    return gate != nullptr && *gate == 0u;
}

// Fold a thread's flags into the device error word (flags are rare: one atomic per
// flagged thread, no warp-wide collective so it is safe under divergence).
__device__ __forceinline__ void raise_flags(unsigned* err, unsigned f) {
    if (f && err) atomicOr(err, f);
}

}  // namespace sph
