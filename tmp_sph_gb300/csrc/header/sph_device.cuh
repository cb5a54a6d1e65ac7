// sph_device.cuh — device-side building blocks shared by the cell-list, neighbour and
// integrator kernels: the per-launch constant block, cell coordinates/hash, the Wendland C2
// kernel in gradient-scalar form, the equation of state and the device error word.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "sph_gb300.h"

namespace sph {

// 32-byte-aligned vector of four doubles (the FP64 counterpart of float4).
struct __align__(32) dvec4 {
    double x, y, z, w;
};

template <class T> struct Vec4Of;
template <> struct Vec4Of<float> { using type = float4; };
template <> struct Vec4Of<double> { using type = dvec4; };
template <class T> using vec4_t = typename Vec4Of<T>::type;

template <class T>
__host__ __device__ __forceinline__ vec4_t<T> make4(T x, T y, T z, T w) {
    vec4_t<T> v;
    v.x = x;
    v.y = y;
    v.z = z;
    v.w = w;
    return v;
}

// Constants every kernel reads, passed by value (they land in the kernel-parameter constant
// bank, which serves warp-uniform reads as fast as __constant__ memory and lets several
// contexts with different parameters run side by side).  Derived on the host from
// sph_params by make_kparams<T>(): T = float for the FP32 and mixed-precision solvers (the
// float derivation the reference's kernels see), T = double for the FP64 solver (the same
// parameters, derived in double).
template <class T>
struct KParamsT {
    int n;
    int gx, gy, gz;      // grid dimensions
    int num_cells;
    // Batched instances are stacked along z every gz_stride cell layers: each gz_local cells
    // high, then at least `reach` empty layers (gz_stride is a multiple of reach, so the
    // anchor cells of mixed precision fall alike in every instance); the resident key of a
    // particle of instance b is b * inst_cells + its cell in its own grid.  A single simulation
    // has gz_local = gz and inst_cells = 0.
    int gz_local;
    int gz_stride;
    int inst_cells;
    // Cells walked on each side of a particle's cell: 1 (27 cells of at least the list cutoff),
    // 2 or 3 (cells of a half or a third of it: 125 or 343 cells, fewer candidates in all).
    // Mixed precision anchors a particle's offsets at the cell whose coordinates are its own
    // rounded down to multiples of `reach` (anchor_of), so two particles within the walk have
    // anchors at most one anchor step apart on each axis.
    int reach;
    // Launch shape of the neighbour kernels (host side): threads per block (multiple of 32, at
    // most 256) and particles per thread.
    int threads;
    int ppt;
    int lanes;   // lanes per particle in list pass 1 (1, or 2 .. 16: ns_groups.cu)
    int list_win;  // list entries interleaved in windows of eight (for lane groups; ns_pair.cuh)
    T gmin_x, gmin_y, gmin_z;
    T cell;              // cell edge (gridSize)
    T reach_cell;        // reach * cell, rounded once: one anchor step of mixed precision
    T inv_cell;          // 1 / cell (the FP64 and mixed solvers' hash scales by it)
    T h, inv_h, kh, kh2;
    T kh2_list;          // squared list cutoff (support radius + skin); kh2 without a skin
    T eta2;
    T adh;               // 21/(16 pi h^3)
    T c_fr;              // -5 adh / h^2: grad W = c_fr (1 - q/2)^3 r
    T c_fr_mass;         // c_fr * mass
    T mass, rho0, cs, g, half_dt;
    T delta_h_cs;        // delta h cs
    T damper;            // rho0 cs h
    T visc;              // alpha h cs rho0
    int eos;
    T tait_gamma, tait_b, inv_tait_b, inv_gamma;
    T inv_cs2;
    int clamp_density;
    T esc_min_x, esc_min_y, esc_min_z, esc_max_x, esc_max_y, esc_max_z;
    T park_x, park_y, park_z;
    // 1: a fluid particle outside the escape box takes key num_cells (sorted after every cell,
    // outside the neighbour search); 0: it is parked and stays in the search (reference)
    int park_inactive;
    // 1: batched instances keep a displacement box each and rebuild their lists on their own
    // decisions (IW_* words below); 0: one box and one decision for all particles
    int inst_boxes;
};
using KParams = KParamsT<float>;

KParams make_kparams(const sph_params& p, int n);
template <class T> KParamsT<T> make_kparams_t(const sph_params& p, int n);

// ---------------------------------------------------------------- cell math
// floorf((p - min) / gridSize) with explicitly IEEE-rounded subtract and divide, so the
// result is bit-identical to the reference's calcGridPos (src/lib/mesh.cu:6-17) whatever
// contraction flags the file is built with.
__device__ __forceinline__ int cell_coord(float p, float gmin, float cell) {
    return (int)floorf(__fdiv_rn(__fsub_rn(p, gmin), cell));
}
// Cell of a double position (FP64 and mixed-precision solvers, no reference counterpart):
// the offset from the grid origin in double, scaled by the reciprocal of the cell edge — in
// float for the mixed solver, whose constants are float — instead of a double division per
// axis (GB300's FP64 rate is a small fraction of FP32, and three divisions per particle and
// half step kept the FP64 pipe of the mixed predictor half busy).  Next to a cell face the
// scaled value can land in the neighbouring cell, by at most its rounding (about 1e-7 of the
// grid extent); every hash of a double position goes through this one function, so the keys
// stay consistent, and the neighbour search and the cell offsets absorb such a particle.
__device__ __forceinline__ int cell_coord_scaled(double p, double gmin, float inv_cell) {
    return (int)floorf((float)(p - gmin) * inv_cell);
}
__device__ __forceinline__ int cell_coord_scaled(double p, double gmin, double inv_cell) {
    return (int)floor((p - gmin) * inv_cell);
}

// Reference hash without clamping (src/lib/mesh.cu:20-23).
__device__ __forceinline__ int cell_hash_raw(const KParams& k, float x, float y, float z) {
    int cx = cell_coord(x, k.gmin_x, k.cell);
    int cy = cell_coord(y, k.gmin_y, k.cell);
    int cz = cell_coord(z, k.gmin_z, k.cell);
    return (cz * k.gx * k.gy) + (cy * k.gx) + cx;
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// Cell coordinates of a cell key (z-major: key = (z gy + y) gx + x).
__device__ __forceinline__ void cell_of_key(int gx, int gy, unsigned key, int& cx, int& cy,
                                            int& cz) {
    unsigned t = key / (unsigned)gx;
    cx = (int)(key - t * (unsigned)gx);
    cz = (int)(t / (unsigned)gy);
    cy = (int)(t - (unsigned)cz * (unsigned)gy);
}

// Anchor of a cell coordinate: rounded down to a multiple of the walk reach (the coordinate
// itself with reach 1).
__device__ __forceinline__ int anchor_of(int c, int reach) { return reach > 1 ? c - c % reach : c; }

// Origin of the anchor cell of a cell of the (float) grid, in double: the frame of the
// mixed-precision offsets.  `key` is a resident key; the origin is in the coordinates of the
// particle's own instance.
template <class KT>
__device__ __forceinline__ void cell_origin(const KParamsT<KT>& k, unsigned key, double& ox,
                                            double& oy, double& oz) {
    int cx, cy, cz;
    cell_of_key(k.gx, k.gy, key, cx, cy, cz);
    if (k.inst_cells) cz %= k.gz_stride;
    ox = (double)k.gmin_x + (double)anchor_of(cx, k.reach) * (double)k.cell;
    oy = (double)k.gmin_y + (double)anchor_of(cy, k.reach) * (double)k.cell;
    oz = (double)k.gmin_z + (double)anchor_of(cz, k.reach) * (double)k.cell;
}

// Position along one axis in units of the cell edge, measured from the grid origin: the
// expression whose floor is the cell coordinate (cell_coord for float positions,
// cell_coord_scaled for double ones), so both give the same cell.
__device__ __forceinline__ float cell_units(float p, float gmin, const KParamsT<float>& k) {
    return __fdiv_rn(__fsub_rn(p, gmin), k.cell);
}
__device__ __forceinline__ float cell_units(double p, float gmin, const KParamsT<float>& k) {
    return (float)(p - (double)gmin) * k.inv_cell;
}
__device__ __forceinline__ double cell_units(double p, double gmin, const KParamsT<double>& k) {
    return (p - gmin) * k.inv_cell;
}

__device__ __forceinline__ float floor_of(float v) { return floorf(v); }
__device__ __forceinline__ double floor_of(double v) { return floor(v); }

// Hash used by the resident solver: identical to the reference for in-grid positions; an
// out-of-grid or non-finite position is clamped into the grid (of one instance) and reported
// through `flag`.  KT is the constant block's real type, PT the position's (a mixed-precision
// solver hashes its double positions on the float grid, in double).
template <class KT, class PT>
__device__ __forceinline__ int cell_hash_clamped(const KParamsT<KT>& k, PT x, PT y, PT z,
                                                 unsigned* flag) {
    if (!(isfinite(x) && isfinite(y) && isfinite(z))) {
        *flag |= SPH_FLAG_NONFINITE | SPH_FLAG_OUT_OF_GRID;
        x = isfinite(x) ? x : (PT)k.gmin_x;
        y = isfinite(y) ? y : (PT)k.gmin_y;
        z = isfinite(z) ? z : (PT)k.gmin_z;
    }
    const auto ux = cell_units(x, k.gmin_x, k);
    const auto uy = cell_units(y, k.gmin_y, k);
    const auto uz = cell_units(z, k.gmin_z, k);
    const auto fx = floor_of(ux), fy = floor_of(uy), fz = floor_of(uz);
    int cx = (int)fx, cy = (int)fy, cz = (int)fz;
    if ((unsigned)cx >= (unsigned)k.gx || (unsigned)cy >= (unsigned)k.gy ||
        (unsigned)cz >= (unsigned)k.gz_local) {
        *flag |= SPH_FLAG_OUT_OF_GRID;
        cx = clampi(cx, 0, k.gx - 1);
        cy = clampi(cy, 0, k.gy - 1);
        cz = clampi(cz, 0, k.gz_local - 1);
    }
    return (cz * k.gy + cy) * k.gx + cx;
}

// Resident key of a particle of instance `inst` (0 for a single simulation).
template <class KT, class PT>
__device__ __forceinline__ unsigned resident_key(const KParamsT<KT>& k, int inst, PT x, PT y, PT z,
                                                 unsigned* flag) {
    return (unsigned)cell_hash_clamped(k, x, y, z, flag) + (unsigned)inst * (unsigned)k.inst_cells;
}

// ---------------------------------------------------------------- explicit rounding
// Arithmetic with its rounding spelled out.  The compiler fuses a product into a following add
// (fma contraction) where it sees fit, and an inlined expression can be fused one way in one
// kernel and another way in the next; the neighbour passes are written with these wherever a
// product meets a sum, so the list passes, the cell-walking passes and the batched runs get the
// same bits from the same pairs.
__device__ __forceinline__ float fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }

// ---------------------------------------------------------------- equation of state
__device__ __forceinline__ float dexpm1(float x) { return expm1f(x); }
__device__ __forceinline__ double dexpm1(double x) { return expm1(x); }
__device__ __forceinline__ float dlog1p(float x) { return log1pf(x); }
__device__ __forceinline__ double dlog1p(double x) { return log1p(x); }

// Pressure of the density perturbation drho = rho - rho0: linear (the reference's only form,
// src/sph/sph_run.cu:467) or Tait, evaluated as B expm1(gamma log1p(drho/rho0)) — accurate
// relative to p itself for the small perturbations of weakly-compressible flow, where
// B((rho/rho0)^gamma - 1) would lose most of its float digits to cancellation.
template <class T>
__device__ __forceinline__ T eos_pressure_d(const KParamsT<T>& k, T drho) {
    if (k.eos == SPH_EOS_TAIT) return k.tait_b * dexpm1(k.tait_gamma * dlog1p(drho / k.rho0));
    return k.cs * k.cs * drho;
}

template <class T>
__device__ __forceinline__ T eos_pressure(const KParamsT<T>& k, T rho) {
    return eos_pressure_d(k, rho - k.rho0);
}

// Inverse used for wall particles (src/equation/ns.cu:128 for the linear form).
template <class T>
__device__ __forceinline__ T eos_density(const KParamsT<T>& k, T p) {
    if (k.eos == SPH_EOS_TAIT)
        return fma_rn(k.rho0, dexpm1(k.inv_gamma * dlog1p(p * k.inv_tait_b)), k.rho0);
    return p / k.cs / k.cs + k.rho0;
}

template <class KT, class PT>
__device__ __forceinline__ bool escaped(const KParamsT<KT>& k, PT x, PT y, PT z) {
    return x > (PT)k.esc_max_x || x < (PT)k.esc_min_x || y > (PT)k.esc_max_y ||
           y < (PT)k.esc_min_y || z > (PT)k.esc_max_z || z < (PT)k.esc_min_z;
}

// Sort key of a resident slot: its cell, or, with park_inactive, num_cells for a fluid particle
// outside the escape box — past every cell's range, so it is nobody's candidate and walks no
// cells itself.
template <class KT, class PT>
__device__ __forceinline__ unsigned slot_key(const KParamsT<KT>& k, int inst, bool fluid, PT x,
                                             PT y, PT z, unsigned* flag) {
    if (k.park_inactive && fluid && escaped(k, x, y, z)) return (unsigned)k.num_cells;
    return resident_key(k, inst, x, y, z, flag);
}

template <class KT>
__device__ __forceinline__ bool inactive_key(const KParamsT<KT>& k, unsigned key) {
    return key >= (unsigned)k.num_cells;
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

// ---------------------------------------------------------------- list rebuild test
// The neighbour lists hold every pair closer than kh + s at the last build (s = skin kh).  A
// pair missing from them can only come within kh once the two particles' displacements since
// the build differ by more than s, and |d_i - d_j| <= |d_i - D| + |d_j - D| for any vector D.
// Taking D as the centre of the bounding box of all displacements, the lists stay complete
// while that box's half-diagonal is below s/2: a flow that carries many particles the same
// way (a surge) keeps its lists roughly twice as long as with the largest displacement
// itself.  The cell walk of a particle whose list overflowed uses the cells of the last build,
// which the same bound keeps within reach.
//
// The box is kept as order-preserving integer keys of its low and high corners in
// DISP_WORDS words of the rebuild block, each in its own 128-byte line so the atomics of
// different corners do not queue on one L2 slice.
constexpr int DISP_STRIDE = 32;  // words between corner words
constexpr int DISP_WORDS = 6 * DISP_STRIDE;

__device__ __forceinline__ unsigned ord_key(float f) {
    const unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord_value(unsigned key) {
    return __uint_as_float((key & 0x80000000u) ? (key & 0x7fffffffu) : ~key);
}

// Per-instance rebuild decisions (batched instances, KParams::inst_boxes): every instance keeps
// its own displacement box, list skin and rebuild decision, in IW_STRIDE words at
// iw + IW_STRIDE (b + 1) after a header of IW_STRIDE words.  An instance rebuilds when its own
// box says so, so it rebuilds in the same half steps, with the same skins, as it would alone.
constexpr int IW_STRIDE = 16;
constexpr int IW_ALL = 0;      // header: every instance rebuilds at the next decision
constexpr int IW_REBUILD = 0;  // the instance's lists are rebuilt in this half step
constexpr int IW_SKIN = 1;     // skin of its lists (float bits)
constexpr int IW_CUT2 = 2;     // squared list cutoff (float bits)
constexpr int IW_THR = 3;      // rebuild threshold on its box (float bits)
constexpr int IW_HS = 4;       // half steps since its last build
constexpr int IW_COUNT = 5;    // its rebuilds since the upload
constexpr int IW_HD2 = 6;      // squared half-diagonal of its last box (float bits)
constexpr int IW_BOX = 8;      // lo x, y, z, hi x, y, z
__device__ __forceinline__ unsigned* inst_words(unsigned* iw, int b) {
    return iw + IW_STRIDE * (b + 1);
}

// Lower (c < 3) or raise a corner word of a box to v, with an atomic only when v improves on
// the value already there.
__device__ __forceinline__ void fold_corner(unsigned* word, int c, unsigned v) {
    if (c < 3) {
        if (v < *(volatile unsigned*)word) atomicMin(word, v);
    } else {
        if (v > *(volatile unsigned*)word) atomicMax(word, v);
    }
}

// A thread's box of displacements (empty until the first add).
struct DispBox {
    unsigned lo[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu};
    unsigned hi[3] = {0u, 0u, 0u};
    int inst = -1;  // instance of the displacements added (per-instance boxes), -1: none yet
    // a displacement that is not a number counts as a huge one (the lists are rebuilt)
    __device__ __forceinline__ void add(float x, float y, float z) {
        const float v[3] = {x == x ? x : 3.0e38f, y == y ? y : 3.0e38f, z == z ? z : 3.0e38f};
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const unsigned kc = ord_key(v[c]);
            lo[c] = min(lo[c], kc);
            hi[c] = max(hi[c], kc);
        }
    }
    // The displacement of a particle of instance b: with per-instance boxes (iw != NULL) a
    // thread that moves on to another instance (particles per thread > 1) first folds what it
    // holds into the previous instance's box.
    __device__ __forceinline__ void add_at(unsigned* iw, int b, float x, float y, float z) {
        if (iw) {
            if (inst >= 0 && b != inst) {
                flush(iw);
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    lo[c] = 0xffffffffu;
                    hi[c] = 0u;
                }
            }
            inst = b;
        }
        add(x, y, z);
    }
    // This thread's box into its instance's words.
    __device__ __forceinline__ void flush(unsigned* iw) const {
        if (inst < 0) return;
        unsigned* w = inst_words(iw, inst) + IW_BOX;
#pragma unroll
        for (int c = 0; c < 3; c++) {
            fold_corner(w + c, c, lo[c]);
            fold_corner(w + 3 + c, 3 + c, hi[c]);
        }
    }
};

// Fold the boxes of a block into the rebuild words (lo x, y, z, hi x, y, z, DISP_STRIDE apart).
// Every thread of the block must call it (it synchronises); s_box holds 6 * (blockDim / 32)
// words.  A corner is only written when the block improves on the value already there.
__device__ __forceinline__ void reduce_disp_box(const DispBox& b, unsigned* disp,
                                                unsigned* s_box) {
    const int warps = (int)(blockDim.x >> 5), w = (int)(threadIdx.x >> 5);
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const unsigned l = __reduce_min_sync(0xffffffffu, b.lo[c]);
        const unsigned h = __reduce_max_sync(0xffffffffu, b.hi[c]);
        if ((threadIdx.x & 31) == 0) {
            s_box[c * warps + w] = l;
            s_box[(3 + c) * warps + w] = h;
        }
    }
    __syncthreads();
    if (threadIdx.x < 6 && disp) {
        const int c = (int)threadIdx.x;
        unsigned v = s_box[c * warps];
        for (int q = 1; q < warps; q++)
            v = c < 3 ? min(v, s_box[c * warps + q]) : max(v, s_box[c * warps + q]);
        fold_corner(disp + c * DISP_STRIDE, c, v);
    }
}

// The same with a box per instance (iw: the instance words).  The particles of a block are
// consecutive slots, so they belong to one instance or, next to an instance boundary, to a
// few: each warp whose lanes hold one instance folds its box with warp reductions, a warp that
// spans a boundary sends each lane's box on its own, and the first six threads fold the
// warps' boxes run by run of equal instances.  Every thread of the block must call it;
// s_box holds 6 * (blockDim / 32) words and s_inst blockDim / 32.
__device__ __forceinline__ void reduce_disp_box_inst(const DispBox& b, unsigned* iw,
                                                     unsigned* s_box, int* s_inst) {
    const int warps = (int)(blockDim.x >> 5), w = (int)(threadIdx.x >> 5);
    const int lead = __reduce_max_sync(0xffffffffu, b.inst);
    const bool uniform = __all_sync(0xffffffffu, b.inst < 0 || b.inst == lead);
    if (!uniform) b.flush(iw);
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const unsigned l = __reduce_min_sync(0xffffffffu, uniform ? b.lo[c] : 0xffffffffu);
        const unsigned h = __reduce_max_sync(0xffffffffu, uniform ? b.hi[c] : 0u);
        if ((threadIdx.x & 31) == 0) {
            s_box[c * warps + w] = l;
            s_box[(3 + c) * warps + w] = h;
        }
    }
    if ((threadIdx.x & 31) == 0) s_inst[w] = uniform ? lead : -1;
    __syncthreads();
    if (threadIdx.x < 6) {
        const int c = (int)threadIdx.x;
        int cur = -1;
        unsigned v = 0u;
        for (int q = 0; q < warps; q++) {
            const int bq = s_inst[q];
            if (bq < 0) continue;
            const unsigned u = s_box[c * warps + q];
            if (bq != cur) {
                if (cur >= 0) fold_corner(inst_words(iw, cur) + IW_BOX + c, c, v);
                cur = bq;
                v = u;
            } else {
                v = c < 3 ? min(v, u) : max(v, u);
            }
        }
        if (cur >= 0) fold_corner(inst_words(iw, cur) + IW_BOX + c, c, v);
    }
}

// Fold a block's displacement boxes: into the one box (disp) or, with KParams::inst_boxes,
// into the boxes of the instances (disp = the instance words).
template <class KP>
__device__ __forceinline__ void reduce_disp(const KP& k, const DispBox& b, unsigned* disp,
                                            unsigned* s_box, int* s_inst) {
    if (k.inst_boxes) reduce_disp_box_inst(b, disp, s_box, s_inst);
    else reduce_disp_box(b, disp, s_box);
}

}  // namespace sph
