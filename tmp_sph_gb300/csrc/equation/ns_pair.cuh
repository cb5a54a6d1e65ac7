// ns_pair.cuh — pair arithmetic and per-particle accumulators of the two neighbour passes,
// shared by the one-thread-per-particle kernels (ns.cu) and the lane-group kernels
// (ns_groups.cu).  Internal to those two translation units: everything is in an unnamed
// namespace, so each gets its own copy.  The kernel algebra and the record layout are
// described at the top of ns.cu.
#pragma once

#include <cuda_runtime.h>

#include "sph_internal.h"

namespace sph {

namespace {

// Block size of the neighbour kernels is a launch parameter (KParams::threads, a multiple of
// 32 up to NS_MAX_THREADS), as is the number of particles a thread handles (KParams::ppt); both
// are picked by the autotuner.  ppt > 1 runs the grid-stride instantiation (GS), which holds
// its loop state in registers (pass 2: 64 instead of 48), so ppt = 1 has its own.
constexpr int NS_MAX_THREADS = 256;
// Mixed precision: a list slot is j | code << CODE_SHIFT (j < 2^26), code the neighbour's
// anchor cell relative to i's (cell_code).
constexpr int CODE_SHIFT = 26;
constexpr unsigned IDX_MASK = (1u << CODE_SHIFT) - 1u;
__device__ __forceinline__ int slot_index(int e) { return (int)((unsigned)e & IDX_MASK); }
__device__ __forceinline__ unsigned slot_code(int e) { return (unsigned)e >> CODE_SHIFT; }
__device__ __forceinline__ int make_slot(int j, unsigned code) {
    return (int)((unsigned)j | (code << CODE_SHIFT));
}
// Code of a neighbour cell (xj, yj, zj) seen from cell (xi, yi, zi), both within one walk:
// the difference of their anchors (anchor_of) in anchor steps, each in {-1, 0, 1}, two bits
// per axis, (dz+1) << 4 | (dy+1) << 2 | (dx+1).
// One axis of it: 0, 1 or 2 as cell c lies before, in or after the anchor column starting at
// cell a (a = anchor_of of i's cell, c within the walk).
__device__ __forceinline__ unsigned anchor_step(int c, int a, int r) {
    return c < a ? 0u : (c < a + r ? 1u : 2u);
}
template <class KP>
__device__ __forceinline__ unsigned cell_code(const KP& k, int xi, int yi, int zi, int xj, int yj,
                                              int zj) {
    const int r = k.reach;
    return (anchor_step(zj, anchor_of(zi, r), r) << 4) |
           (anchor_step(yj, anchor_of(yi, r), r) << 2) | anchor_step(xj, anchor_of(xi, r), r);
}

// Column of particle i in the warp-interleaved list: slots 4g .. 4g+3 of i are the int4 at
// col + 32 * 4g (col = the warp's block + 4 * lane).  The 32 particles of a warp share one block
// of cap x 32 slots, so a warp reading slot group g of all its lanes touches four consecutive
// lines (512 bytes) with one 16-byte load per lane, and the build stores four slots at a time.
__device__ __forceinline__ size_t nbr_col(const NbrList& nl, int i) {
    return (size_t)(i >> 5) * ((size_t)nl.cap << 5) + ((size_t)(i & 31) << 2);
}

// Four list slots.  The slots stream past once per pass, so they are read without allocating
// in L1, which keeps L1 for the neighbour records (measured: passes 0.6% faster).
__device__ __forceinline__ int4 ld_slots(const int* p) {
    int4 v;
    asm("ld.global.nc.L1::no_allocate.v4.s32 {%0, %1, %2, %3}, [%4];"
        : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
        : "l"(p));
    return v;
}

// List windows.  A plain column keeps walk order (int4 chunk c holds entries 4c .. 4c+3), so
// the one-lane passes sum in the order a cell walk visits.  An interleaved column
// (KParams::list_win, set while a pass runs lane groups) is written in windows of eight
// entries, two chunks: chunk 2u holds entries 8u, 8u+2, 8u+4, 8u+6 and chunk 2u+1 the odd ones.
// Lane s of a group reads chunks s, s + G, ..., so the two lanes of every pair gather two
// consecutive entries — neighbouring records, mostly one line — at each step.  (Reading plain
// chunks that way had the lanes of a pair four entries apart: pass 1 at G = 2 took 0.86 ms
// against 0.79 with one lane and 0.76 interleaved; swapping entries between the lanes with
// shuffles cost more than it saved, 0.83.)  First entry of chunk c; its four entries are
// st = 2 (interleaved) or 1 (plain) apart.
template <bool WIN>
__device__ __forceinline__ int chunk_first(int c) {
    return WIN ? c + 6 * (c >> 1) : c << 2;
}

// one(slot) for the entries of a column (cnt <= cap of them) in chunks c0, c0 + dc, ... (the
// one-lane passes: c0 = 0, dc = 1; lane s of a group of G: c0 = s, dc = G), four to an int4,
// the next chunk loaded one chunk ahead (four record gathers in flight per thread).  Chunk
// firsts grow with c, so the first chunk past the count ends the column.
template <bool WIN, class F>
__device__ __forceinline__ void for_each_slot(const int* __restrict__ col, int cnt, int c0,
                                              int dc, F&& one) {
    constexpr int st = WIN ? 2 : 1;
    int c = c0, e = chunk_first<WIN>(c0);
    int4 q = e < cnt ? ld_slots(col + ((size_t)c << 7)) : make_int4(0, 0, 0, 0);
#pragma unroll 1
    while (e < cnt) {
        const int cn = c + dc, en = chunk_first<WIN>(cn);
        const int4 qn = en < cnt ? ld_slots(col + ((size_t)cn << 7)) : q;
        one(q.x);
        if (e + st < cnt) one(q.y);
        if (e + 2 * st < cnt) one(q.z);
        if (e + 3 * st < cnt) one(q.w);
        q = qn;
        c = cn;
        e = en;
    }
}

// Squared distance with an explicit rounding sequence, so the in-range test gives the same
// answer in the list build, in the walking passes and in the list passes.
__device__ __forceinline__ float dist2(float dx, float dy, float dz) {
    return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}
__device__ __forceinline__ double dist2(double dx, double dy, double dz) {
    return __fma_rn(dz, dz, __fma_rn(dy, dy, __dmul_rn(dx, dx)));
}
// Pair arithmetic: in FP32 the distance and the reciprocal of a pair come from the hardware's
// approximate instructions (sqrt.approx, rcp.approx: within about one ulp, instead of the
// correctly rounded sequences); FP64 keeps correctly rounded sqrt and division.  The .ftz
// forms flush subnormal inputs and results to zero, which no pair meets (the arguments are a
// density near rho0, r^2 + eta^2 >= eta^2, and r^2, which is 0 for coincident particles and
// otherwise many decades above the subnormal range), and so give the same value as the plain
// forms here; the plain forms wrap every approximation in a subnormal-scaling sequence, which
// cost pass 2 29% more instructions (0.728 against 0.641 ms at 4.96M particles).
__device__ __forceinline__ float pair_sqrt(float x) {
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ double pair_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float pair_rcp(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ double pair_rcp(double x) { return 1.0 / x; }
__device__ __forceinline__ float dabs(float x) { return fabsf(x); }
__device__ __forceinline__ double dabs(double x) { return fabs(x); }

// A neighbour sum: plain, or compensated (Neumaier) when COMP, with explicitly rounded
// arithmetic (no contraction folds the error terms away, and every kernel sums alike).
// add_prod(a, b) adds a b: one fused multiply-add into a plain sum, the rounded product into
// a compensated one.
template <class T, bool COMP>
struct Sum {
    T s = T(0), c = T(0);
    __device__ __forceinline__ void add(T v) {
        if constexpr (COMP) {
            const T t = add_rn(s, v);
            c = add_rn(c, dabs(s) >= dabs(v) ? add_rn(sub_rn(s, t), v) : add_rn(sub_rn(v, t), s));
            s = t;
        } else {
            s = add_rn(s, v);
        }
    }
    __device__ __forceinline__ void add_prod(T a, T b) {
        if constexpr (COMP) {
            add(mul_rn(a, b));
        } else {
            s = fma_rn(a, b, s);
        }
    }
    __device__ __forceinline__ T get() const {
        if constexpr (COMP) return add_rn(s, c);
        return s;
    }
};

// Visit the candidate slots of the (2 reach + 1)^3 cells around (cx, cy, cz) as contiguous
// ranges: run(j0, j1, code) for slots j0 .. j1 - 1.  Without CODES each x-strip is one range
// and code is 0; with CODES the strip is split into the runs of its cells that share an anchor
// column and code = cell_code of their cells seen from (cx, cy, cz).  Both visit the same
// slots in the same order.
// window(y, z, xa, xb) may narrow a strip to the cells [xa, xb] that can hold a particle in
// range, or return false to skip it (the list build); the passes take every candidate.
struct AllCells {
    __device__ __forceinline__ bool operator()(int, int, int&, int&) const { return true; }
};
template <bool CODES, class KP, class F, class W = AllCells>
__device__ __forceinline__ void for_each_run(const KP& k, const int* __restrict__ cs, int cx,
                                             int cy, int cz, F&& run, W window = W()) {
    const int r = k.reach;
    const int xl0 = cx > r - 1 ? cx - r : 0;
    const int xh0 = cx < k.gx - r ? cx + r : k.gx - 1;
    // anchors of i's cell (CODES): the walk spans at most the anchor columns before, at and
    // after them on each axis
    const int ax = CODES ? anchor_of(cx, r) : 0;
    const int ay = CODES ? anchor_of(cy, r) : 0;
    const int az = CODES ? anchor_of(cz, r) : 0;
#pragma unroll 1
    for (int dz = -r; dz <= r; dz++) {
        const int z = cz + dz;
        if ((unsigned)z >= (unsigned)k.gz) continue;
#pragma unroll 1
        for (int dy = -r; dy <= r; dy++) {
            const int y = cy + dy;
            if ((unsigned)y >= (unsigned)k.gy) continue;
            int xl = xl0, xh = xh0;
            if (!window(y, z, xl, xh)) continue;
            const int row = (z * k.gy + y) * k.gx;
            if constexpr (CODES) {
                // the strip in its (at most three) runs of cells that share an anchor column,
                // one code per run
                const unsigned cyz = (anchor_step(z, az, r) << 4) | (anchor_step(y, ay, r) << 2);
#pragma unroll 1
                for (unsigned sx = 0; sx < 3u; sx++) {
                    const int xa = max(xl, ax + ((int)sx - 1) * r);
                    const int xb = min(xh, ax + (int)sx * r - 1);
                    if (xa > xb) continue;
                    const int j0 = max(__ldg(cs + row + xa), 0);
                    const int j1 = min(__ldg(cs + row + xb + 1), k.n);  // bounds guard only
                    run(j0, j1, cyz | sx);
                }
            } else {
                const int j0 = max(__ldg(cs + row + xl), 0);
                const int j1 = min(__ldg(cs + row + xh + 1), k.n);  // bounds guard only
                run(j0, j1, 0u);
            }
        }
    }
}

// The list build's window: the cells of a strip that can hold a particle within the list
// cutoff of particle i.  u = i's position in cell units of its own instance's grid (cell c
// spans [c, c + 1)), zb the stacked index of that grid's first layer, rc2 the squared cutoff in
// cell units; a strip whose nearest point in y-z is beyond the cutoff is skipped, and the
// others keep the cells whose x range meets [u.x - w, u.x + w], w the half-chord of the cutoff
// sphere at that distance.  Widened by 2^-10 of rc2 and 1e-3 cells against rounding, so it
// only drops candidates the build's own distance test rejects: the lists, and the sums, are
// those of the full walk.
struct StripWindow {
    float ux, uy, uz, rc2;  // rc2 < 0: no window (i is not inside its cell: clamped)
    int zb;
    __device__ __forceinline__ bool operator()(int y, int z, int& xa, int& xb) const {
        if (rc2 < 0.f) return true;
        const float fy = (float)y, fz = (float)(z - zb);
        const float dy = fmaxf(0.f, fmaxf(fy - uy, uy - fy - 1.f));
        const float dz = fmaxf(0.f, fmaxf(fz - uz, uz - fz - 1.f));
        const float w2 = rc2 - dy * dy - dz * dz;
        if (w2 < 0.f) return false;
        const float w = pair_sqrt(w2) + 1e-3f;  // approximate root: ~1e-7 of w, inside 1e-3
        xa = max(xa, (int)floorf(ux - w));
        xb = min(xb, (int)floorf(ux + w));
        return xa <= xb;
    }
};

// The window of particle i (record position pi, cell (cx, cy, cz) of its resident key) for the
// squared cutoff cut2: positions in cell units of its instance's grid, from the absolute
// position or (cell codes) from its anchor and offsets.
template <class P>
__device__ __forceinline__ StripWindow strip_window(const KParamsT<typename P::T>& k,
                                                    const vec4_t<typename P::T>& pi, int cx,
                                                    int cy, int cz, typename P::T cut2) {
    StripWindow w;
    const int czl = k.inst_cells ? cz % k.gz_stride : cz;
    w.zb = cz - czl;
    if constexpr (P::kCodes) {
        const int r = k.reach;
        w.ux = (float)anchor_of(cx, r) + (float)(pi.x * k.inv_cell);
        w.uy = (float)anchor_of(cy, r) + (float)(pi.y * k.inv_cell);
        w.uz = (float)anchor_of(czl, r) + (float)(pi.z * k.inv_cell);
    } else {
        w.ux = (float)((pi.x - k.gmin_x) * k.inv_cell);
        w.uy = (float)((pi.y - k.gmin_y) * k.inv_cell);
        w.uz = (float)((pi.z - k.gmin_z) * k.inv_cell);
    }
    const bool inside = w.ux > (float)cx - 0.01f && w.ux < (float)cx + 1.01f &&
                        w.uy > (float)cy - 0.01f && w.uy < (float)cy + 1.01f &&
                        w.uz > (float)czl - 0.01f && w.uz < (float)czl + 1.01f;
    // on cells of the cutoff (reach 1) the sphere fills most of the 27 cells and the window
    // cost more than it saved (mixed precision's build +5%); it pays on the 343 cells of
    // reach 3 (FP32 build -7%, a step rebuilding every half step -2.5%)
    w.rc2 = inside && k.reach > 1 ? (float)(cut2 * k.inv_cell * k.inv_cell) * (1.f + 1.f / 1024.f)
                                  : -1.f;
    return w;
}

// Every candidate slot of that walk: f(j, code).
template <bool CODES, class KP, class F>
__device__ __forceinline__ void for_each_candidate(const KP& k, const int* __restrict__ cs,
                                                   int cx, int cy, int cz, F&& f) {
    for_each_run<CODES>(k, cs, cx, cy, cz, [&](int j0, int j1, unsigned code) {
#pragma unroll 4
        for (int j = j0; j < j1; j++) f(j, code);
    });
}

// The anchor steps of a mixed-precision cell code as floats: each 2-bit field f as f - 1,
// without an integer conversion (the float with bits 0x4B000000 | f is 2^23 + f).
__device__ __forceinline__ void code_steps(unsigned code, float& fx, float& fy, float& fz) {
    fx = __fsub_rn(__uint_as_float(0x4B000000u | (code & 3u)), 8388609.0f);
    fy = __fsub_rn(__uint_as_float(0x4B000000u | ((code >> 2) & 3u)), 8388609.0f);
    fz = __fsub_rn(__uint_as_float(0x4B000000u | (code >> 4)), 8388609.0f);
}

// One record (two vec4) in single 256-bit read-only loads: a neighbour gather touches one L1
// sector per 32 bytes with one request.  R is 32-byte aligned (cudaMalloc'd).
__device__ __forceinline__ void ld_rec(const float4* __restrict__ R, int j, float4& a,
                                       float4& b) {
    const float4* p = R + 2 * (size_t)j;
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p));
}
__device__ __forceinline__ void ld_rec(const dvec4* __restrict__ R, int j, dvec4& a, dvec4& b) {
    const dvec4* p = R + 2 * (size_t)j;
    asm("ld.global.nc.v4.f64 {%0, %1, %2, %3}, [%4];"
        : "=d"(a.x), "=d"(a.y), "=d"(a.z), "=d"(a.w)
        : "l"(p));
    asm("ld.global.nc.v4.f64 {%0, %1, %2, %3}, [%4];"
        : "=d"(b.x), "=d"(b.y), "=d"(b.z), "=d"(b.w)
        : "l"(p + 1));
}
__device__ __forceinline__ float4 ld_pos(const float4* __restrict__ X, size_t j) {
    return __ldg(X + j);
}
__device__ __forceinline__ dvec4 ld_pos(const dvec4* __restrict__ X, size_t j) {
    const dvec4* p = X + j;
    dvec4 a;
    asm("ld.global.nc.v4.f64 {%0, %1, %2, %3}, [%4];"
        : "=d"(a.x), "=d"(a.y), "=d"(a.z), "=d"(a.w)
        : "l"(p));
    return a;
}

// (ax - bx, ay - by) in one two-lane FP32 instruction (sub.rn.f32x2, sm_100 family), each lane
// rounded as __fsub_rn rounds it: the x and y components of a record sit in adjacent registers
// of its vector load, so the pair costs no moves.
__device__ __forceinline__ void sub2_rn(float ax, float ay, float bx, float by, float& dx,
                                        float& dy) {
    asm("{.reg .b64 ra, rb, rd;\n\t"
        "mov.b64 ra, {%2, %3};\n\t"
        "mov.b64 rb, {%4, %5};\n\t"
        "sub.rn.f32x2 rd, ra, rb;\n\t"
        "mov.b64 {%0, %1}, rd;}"
        : "=f"(dx), "=f"(dy)
        : "f"(ax), "f"(ay), "f"(bx), "f"(by));
}
__device__ __forceinline__ void sub2_rn(double ax, double ay, double bx, double by, double& dx,
                                        double& dy) {
    dx = sub_rn(ax, bx);
    dy = sub_rn(ay, by);
}

// Relative position r = x_i - x_j of a pair: from positions in the simulation's frame, or
// (cell codes) from the offsets from their anchor cells and j's anchor relative to i's
// (anchor steps of reach cells).
template <class P, class V>
__device__ __forceinline__ void rel_pos(const KParamsT<typename P::T>& k, const V& pi,
                                        const V& pj, unsigned code, typename P::T& dx,
                                        typename P::T& dy, typename P::T& dz) {
    using T = typename P::T;
    if constexpr (P::kCodes) {
        // one explicitly rounded difference and one fused multiply-add per axis, so every
        // caller (list, cell walk, list build) gets the same bits whatever the compiler hoists
        // the anchor steps of the code times one anchor step reach * cell
        float fx, fy, fz;
        code_steps(code, fx, fy, fz);
        float ox, oy;
        sub2_rn(pi.x, pi.y, pj.x, pj.y, ox, oy);
        dx = fma_rn(-fx, k.reach_cell, ox);
        dy = fma_rn(-fy, k.reach_cell, oy);
        dz = fma_rn(-fz, k.reach_cell, sub_rn(pi.z, pj.z));
    } else {
        (void)k;
        (void)code;
        sub2_rn(pi.x, pi.y, pj.x, pj.y, dx, dy);
        dz = sub_rn(pi.z, pj.z);
    }
}

// Walk the cells of particle i over the positions X[STRIDE * j] and call
// f(j, code, pj, dx, dy, dz, r2) for every j != i with r2 < cut2.  X is the dense
// (x, y, z, ±1) array (STRIDE 1) or a record array (STRIDE 2).
template <class P, int STRIDE, class F>
__device__ __forceinline__ void walk_pairs(const KParamsT<typename P::T>& k,
                                           const int* __restrict__ cs,
                                           const unsigned* __restrict__ keys,
                                           const vec4_t<typename P::T>* __restrict__ X, int i,
                                           const vec4_t<typename P::T>& pi, typename P::T cut2,
                                           F&& f) {
    using T = typename P::T;
    const unsigned key = keys[i];
    if (inactive_key(k, key)) return;  // outside the neighbour search (park_inactive)
    int cx, cy, cz;
    cell_of_key(k.gx, k.gy, key, cx, cy, cz);
    for_each_candidate<P::kCodes>(k, cs, cx, cy, cz, [&](int j, unsigned code) {
        const vec4_t<T> pj = ld_pos(X, (size_t)STRIDE * (size_t)j);
        T dx, dy, dz;
        rel_pos<P>(k, pi, pj, code, dx, dy, dz);
        const T r2 = dist2(dx, dy, dz);
        if (r2 < cut2 && j != i) f(j, code, pj, dx, dy, dz, r2);
    });
}


template <class T>
__device__ __forceinline__ bool fluid_rec(T signed_rho) { return signed_rho > T(0); }

// Position the list build records for the displacement test (offsets in mixed precision).
__device__ __forceinline__ float4 as_float4(const float4& v) { return v; }
__device__ __forceinline__ float4 as_float4(const dvec4& v) {
    return make_float4((float)v.x, (float)v.y, (float)v.z, (float)v.w);
}

// Pass 1: boundary pressure extrapolation (Adami-style, over fluid neighbours) for boundary
// particles; velocity divergence over fluid neighbours for fluid particles.  Writes the pass-2
// neighbour record and the particle's own (p', rho', dofv).
// (v_i - v_j) . r with explicit rounding: x, then y and z fused in.
template <class V, class T>
__device__ __forceinline__ T dot_rn(const V& vi, const V& vj, T dx, T dy, T dz) {
    T ux, uy;
    sub2_rn(vi.x, vi.y, vj.x, vj.y, ux, uy);
    return fma_rn(sub_rn(vi.z, vj.z), dz, fma_rn(uy, dy, mul_rn(ux, dx)));
}

// Pass-1 state of one particle: its own record and the three neighbour sums.
template <class P>
struct Pass1Acc {
    using T = typename P::T;
    using V = vec4_t<T>;
    V pi, vi;  // x, y, z, p / vx, vy, vz, ±rho
    bool fi;
    Sum<T, P::kComp> dofv, rs, ws;

    __device__ __forceinline__ void load(const V* __restrict__ R, int i) {
        pi = R[2 * (size_t)i];
        vi = R[2 * (size_t)i + 1];
        fi = fluid_rec(vi.w);
    }
    // One neighbour inside the support radius.
    __device__ __forceinline__ void pair(const KParamsT<T>& k, const V& aj, const V& vj, T dx,
                                         T dy, T dz, T r2) {
        if (!fluid_rec(vj.w)) return;
        const T rr = pair_sqrt(r2);
        const T q = mul_rn(rr, k.inv_h);
        const T t = fma_rn(T(-0.5), q, T(1));
        const T t2 = mul_rn(t, t);
        if (!fi) {
            const T w = mul_rn(mul_rn(mul_rn(k.adh, t2), t2), fma_rn(T(2), q, T(1)));
            rs.add_prod(fma_rn(mul_rn(vj.w, k.g), dz, aj.w), w);
            ws.add(w);
        } else {
            const T fr = mul_rn(mul_rn(k.c_fr, t2), t);
            const T vdotr = dot_rn(vi, vj, dx, dy, dz);
            dofv.add_prod(-mul_rn(fr, vdotr), mul_rn(k.mass, pair_rcp(vj.w)));
        }
    }
    template <bool WRITE_SUMS>
    __device__ __forceinline__ void finish(const KParamsT<T>& k, const Pass1OutT<T>& out,
                                           float* __restrict__ rhop_sum,
                                           float* __restrict__ w_sum, int i) {
        T p, rho;
        const T dv = dofv.get(), rsum = rs.get(), wsum = ws.get();
        if (fi) {
            p = pi.w;
            rho = vi.w;
        } else {
            p = dabs(wsum) > T(1.0e-8) ? rsum / wsum : T(0);
            if (p < T(0)) p = T(0);
            rho = eos_density(k, p);
        }
        const T qv = fi ? fma_rn(-k.damper, dv, p) : p;
        out.nrec[2 * (size_t)i] = make4<T>(pi.x, pi.y, pi.z, qv);
        out.nrec[2 * (size_t)i + 1] = make4<T>(vi.x, vi.y, vi.z, fi ? rho : -rho);
        out.self[i] = make4<T>(p, rho, dv, T(0));
        if constexpr (WRITE_SUMS) {
            rhop_sum[i] = (float)rsum;
            w_sum[i] = (float)wsum;
        }
    }
};


enum { MODE_RATES = 0, MODE_PRED = 1, MODE_CORR = 2 };

// Pass 2: continuity + delta density diffusion, momentum (pressure, acoustic damper,
// artificial viscosity, gravity); then either the rates are stored (MODE_RATES) or the
// midpoint predictor / corrector of src/sph/sph_run.cu:425-519 is applied and the updated
// particle written to `out` with its next cell hash.
//
// `out` may alias `in`: the update touches only particle i's own rows, and neighbours (also
// the positions of a cell walk) come from the pass-1 records.  Returns the squared distance
// of particle i from its position when the neighbour list was built (0 without a list).
// Pass-2 state of one particle: its pass-1 record, own side and the four neighbour sums.
template <class P, int MODE>
struct Pass2Acc {
    using T = typename P::T;
    using V = vec4_t<T>;
    V pi, vi;  // x, y, z, q / vx, vy, vz, ±rho
    T rhoi, presi, damp_i;
    bool fi, active;
    Sum<T, P::kComp> sd, sx, sy, sz;

    __device__ __forceinline__ void load(const KParamsT<T>& k, const Pass1OutT<T>& p1, int i,
                                         int wall_rates) {
        pi = p1.nrec[2 * (size_t)i];
        vi = p1.nrec[2 * (size_t)i + 1];
        const V si = p1.self[i];  // p_i, rho_i, dofv_i
        fi = fluid_rec(vi.w);
        rhoi = si.y;
        presi = si.x;
        damp_i = k.damper * si.z;
        active = fi || (MODE == MODE_RATES && wall_rates);
    }
    // One neighbour inside the support radius.  aj = (x, y, z, q), vj = (vx, vy, vz, ±rho).
    // rho_i - rho_j stays an exact difference of two close floats; writing the
    // density-diffusion term with the volume m / rho_j instead (rho_i V_j - m) cancels and lost
    // three digits of rho_dt.
    __device__ __forceinline__ void pair(const KParamsT<T>& k, const Pass1OutT<T>& p1, int j,
                                         const V& aj, const V& vj, T dx, T dy, T dz, T r2) {
        const bool fj = fluid_rec(vj.w);
        const T rhoj = dabs(vj.w);
        const T rr = pair_sqrt(r2);
        const T t = fma_rn(mul_rn(T(-0.5), k.inv_h), rr, T(1));
        // m / rho_j grad W / r in one factor: c_fr m t^3 / rho_j
        const T w = mul_rn(mul_rn(mul_rn(k.c_fr_mass, mul_rn(t, t)), t), pair_rcp(rhoj));
        const T vdotr = dot_rn(vi, vj, dx, dy, dz);
        const T inv_r2e = pair_rcp(add_rn(r2, k.eta2));
        const T diff = mul_rn(mul_rn(mul_rn(sub_rn(rhoi, rhoj), k.delta_h_cs), r2), inv_r2e);
        sd.add_prod(w, fma_rn(rhoi, vdotr, diff));
        T S;
        if (MODE != MODE_RATES || fi) {  // the integrating passes only visit fluid rows
            S = sub_rn(-presi, aj.w);
            if (fj) S = add_rn(S, fma_rn(mul_rn(k.visc, vdotr), inv_r2e, damp_i));
        } else {
            S = -add_rn(presi, __ldg(&p1.self[j].x));  // boundary rows (wall_rates): plain pressures
        }
        const T c = mul_rn(w, S);
        sx.add_prod(c, dx);
        sy.add_prod(c, dy);
        sz.add_prod(c, dz);
    }
};


// Rates, or the predictor / corrector update and the next key of particle i; adds its
// displacement from its list-build position to `box` (nothing without a list or for a particle
// outside the search; a huge one when it leaves or rejoins the search).
template <class P, int MODE>
__device__ __forceinline__ void pass2_finish(const KParamsT<typename P::T>& k, int i,
                                              const Pass2Acc<P, MODE>& acc,
                                              const ParticleSetT<typename P::T>& in,
                                              const unsigned* __restrict__ keys,
                                              const NbrList& nl, float* __restrict__ rho_dt,
                                              float* __restrict__ vel_dt, int wall_rates,
                                              const ParticleSetT<typename P::T>& out,
                                              unsigned* __restrict__ out_hash, unsigned* err,
                                              DispBox& box, unsigned* disp) {
    using T = typename P::T;
    using V = vec4_t<T>;
    // per-instance boxes: disp holds the instance words
    unsigned* const iw = k.inst_boxes ? disp : nullptr;
    const V& pi = acc.pi;
    const V& vi = acc.vi;
    const bool fi = acc.fi;
    const T rhoi = acc.rhoi, presi = acc.presi;
    T drho = T(0), ax = T(0), ay = T(0), az = T(0);
    if (acc.active) {
        drho = acc.sd.get();
        const T inv_rhoi = T(1) / rhoi;
        ax = mul_rn(acc.sx.get(), inv_rhoi);
        ay = mul_rn(acc.sy.get(), inv_rhoi);
        az = mul_rn(acc.sz.get(), inv_rhoi);
    }
    az = add_rn(az, k.g);

    if constexpr (MODE == MODE_RATES) {
        const bool have = fi || wall_rates;
        rho_dt[i] = have ? (float)drho : 0.f;
        vel_dt[3 * i] = have ? (float)ax : 0.f;
        vel_dt[3 * i + 1] = have ? (float)ay : 0.f;
        vel_dt[3 * i + 2] = have ? (float)az : 0.f;
        return;
    } else if constexpr (P::kMixed) {
        // FP64 position and density perturbation; FP32 velocity
        const dvec4 xm = in.xm[i];
        dvec4 nxm = xm, txm = xm;
        float4 nv, tv;
        float npres, nrho;
        const double hdt = (double)k.half_dt;
        if (fi) {
            // the escape test and the hash on the FP32 positions of the records when the passes
            // use them (fewer FP64 operations; every hash of such a particle is the FP32 one)
            if (P::kCodes ? escaped(k, xm.x, xm.y, xm.z) : escaped(k, pi.x, pi.y, pi.z)) {
                nxm = dvec4{(double)k.park_x, (double)k.park_y, (double)k.park_z, 0.0};
                nv = make_float4(0.f, 0.f, 0.f, 0.f);
                txm = nxm;
                tv = nv;
            } else if (MODE == MODE_PRED) {
                tv = make_float4(vi.x, vi.y, vi.z, 0.f);
                double d = fma_rn((double)drho, hdt, xm.w);
                if (k.clamp_density && d < 0.0) d = 0.0;
                nxm.x = fma_rn((double)vi.x, hdt, xm.x);
                nxm.y = fma_rn((double)vi.y, hdt, xm.y);
                nxm.z = fma_rn((double)vi.z, hdt, xm.z);
                nxm.w = d;
                nv = make_float4(fma_rn(ax, k.half_dt, vi.x), fma_rn(ay, k.half_dt, vi.y),
                                 fma_rn(az, k.half_dt, vi.z), 0.f);
            } else {
                txm = in.txm[i];
                tv = in.tvel[i];
                double ds = fma_rn((double)drho, hdt, txm.w);
                if (k.clamp_density && ds < 0.0) ds = 0.0;
                double d = fma_rn(2.0, ds, -txm.w);
                if (k.clamp_density && d < 0.0) d = 0.0;
                nxm.x = fma_rn(2.0, fma_rn((double)vi.x, hdt, txm.x), -txm.x);
                nxm.y = fma_rn(2.0, fma_rn((double)vi.y, hdt, txm.y), -txm.y);
                nxm.z = fma_rn(2.0, fma_rn((double)vi.z, hdt, txm.z), -txm.z);
                nxm.w = d;
                const float uxs = fma_rn(ax, k.half_dt, tv.x);
                const float uys = fma_rn(ay, k.half_dt, tv.y);
                const float uzs = fma_rn(az, k.half_dt, tv.z);
                nv = make_float4(fma_rn(2.f, uxs, -tv.x), fma_rn(2.f, uys, -tv.y),
                                 fma_rn(2.f, uzs, -tv.z), 0.f);
            }
            nrho = add_rn(k.rho0, (float)nxm.w);
            npres = eos_pressure_d(k, (float)nxm.w);
        } else {
            // boundary particles do not move; they keep the extrapolated pressure and density
            nv = make_float4(vi.x, vi.y, vi.z, 0.f);
            npres = presi;
            nrho = rhoi;
            tv = nv;
        }
        const float3 q = record_pos<P>(k, keys[i], nxm.x, nxm.y, nxm.z);
        const float px = q.x, py = q.y, pz = q.z;
        out.rec[2 * (size_t)i] = make_float4(px, py, pz, npres);
        out.rec[2 * (size_t)i + 1] = make_float4(nv.x, nv.y, nv.z, fi ? nrho : -nrho);
        if (out.xyz) out.xyz[i] = make_float4(px, py, pz, fi ? 1.f : -1.f);
        out.type[i] = in.type[i];
        out.id[i] = in.id[i];
        out.xm[i] = nxm;
        if (MODE == MODE_PRED) {
            out.txm[i] = txm;
            out.tvel[i] = tv;
        }
        // instance ids only move with the particles when instances are batched
        const int inst = k.inst_cells ? in.inst[i] : 0;
        if (k.inst_cells) out.inst[i] = inst;
        unsigned f = 0;
        const unsigned nk = P::kCodes ? slot_key(k, inst, fi, nxm.x, nxm.y, nxm.z, &f)
                                       : slot_key(k, inst, fi, px, py, pz, &f);
        out_hash[i] = nk;
        raise_flags(err, f);
        if (k.park_inactive) {
            // a particle that leaves (or rejoins) the neighbour search needs new lists; one
            // outside it is in no list, so its moves do not count
            const bool now = inactive_key(k, nk);
            if (now != inactive_key(k, keys[i])) {
                // every slot after it moves: with per-instance boxes all instances rebuild
                if (iw) atomicOr(iw + IW_ALL, 1u);
                box.add_at(iw, inst, 3.0e38f, 3.0e38f, 3.0e38f);
                box.add_at(iw, inst, -3.0e38f, -3.0e38f, -3.0e38f);
                return;
            }
            if (now) return;
        }
        if (!nl.xb) return;
        const float4 xb = nl.xb[i];
        box.add_at(iw, inst, px - xb.x, py - xb.y, pz - xb.z);
    } else {
        V np = pi, nv;
        T npres, nrho;
        V tp, tv;
        if (fi) {
            if (escaped(k, pi.x, pi.y, pi.z)) {
                np = make4<T>(k.park_x, k.park_y, k.park_z, T(0));
                nv = make4<T>(T(0), T(0), T(0), T(0));
                npres = T(0);
                nrho = k.rho0;
                tp = make4<T>(np.x, np.y, np.z, k.rho0);
                tv = make4<T>(T(0), T(0), T(0), T(0));
            } else if (MODE == MODE_PRED) {
                tp = make4<T>(pi.x, pi.y, pi.z, rhoi);
                tv = make4<T>(vi.x, vi.y, vi.z, T(0));
                T rho = fma_rn(drho, k.half_dt, rhoi);
                if (k.clamp_density && rho < k.rho0) rho = k.rho0;
                np.x = fma_rn(vi.x, k.half_dt, pi.x);
                np.y = fma_rn(vi.y, k.half_dt, pi.y);
                np.z = fma_rn(vi.z, k.half_dt, pi.z);
                nv = make4<T>(fma_rn(ax, k.half_dt, vi.x), fma_rn(ay, k.half_dt, vi.y),
                              fma_rn(az, k.half_dt, vi.z), T(0));
                nrho = rho;
                npres = eos_pressure(k, rho);
            } else {
                tp = in.tpos[i];
                tv = in.tvel[i];
                T rho = fma_rn(drho, k.half_dt, tp.w);
                if (k.clamp_density && rho < k.rho0) rho = k.rho0;
                const T xs = fma_rn(vi.x, k.half_dt, tp.x);
                const T ys = fma_rn(vi.y, k.half_dt, tp.y);
                const T zs = fma_rn(vi.z, k.half_dt, tp.z);
                const T uxs = fma_rn(ax, k.half_dt, tv.x);
                const T uys = fma_rn(ay, k.half_dt, tv.y);
                const T uzs = fma_rn(az, k.half_dt, tv.z);
                rho = fma_rn(T(2), rho, -tp.w);
                if (k.clamp_density && rho < k.rho0) rho = k.rho0;
                np.x = fma_rn(T(2), xs, -tp.x);
                np.y = fma_rn(T(2), ys, -tp.y);
                np.z = fma_rn(T(2), zs, -tp.z);
                nv = make4<T>(fma_rn(T(2), uxs, -tv.x), fma_rn(T(2), uys, -tv.y),
                              fma_rn(T(2), uzs, -tv.z), T(0));
                nrho = rho;
                npres = eos_pressure(k, rho);
            }
        } else {
            // boundary particles do not move; they keep the extrapolated pressure and density
            nv = make4<T>(vi.x, vi.y, vi.z, T(0));
            npres = presi;
            nrho = rhoi;
            tp = make4<T>(pi.x, pi.y, pi.z, rhoi);
            tv = make4<T>(vi.x, vi.y, vi.z, T(0));
        }
        out.rec[2 * (size_t)i] = make4<T>(np.x, np.y, np.z, npres);
        out.rec[2 * (size_t)i + 1] = make4<T>(nv.x, nv.y, nv.z, fi ? nrho : -nrho);
        if (out.xyz) out.xyz[i] = make4<T>(np.x, np.y, np.z, fi ? T(1) : T(-1));
        out.type[i] = in.type[i];
        out.id[i] = in.id[i];
        if (MODE == MODE_PRED) {
            out.tpos[i] = tp;
            out.tvel[i] = tv;
        }
        // instance ids only move with the particles when instances are batched
        const int inst = k.inst_cells ? in.inst[i] : 0;
        if (k.inst_cells) out.inst[i] = inst;
        unsigned f = 0;
        const unsigned nk = slot_key(k, inst, fi, np.x, np.y, np.z, &f);
        out_hash[i] = nk;
        raise_flags(err, f);
        if (k.park_inactive) {
            // a particle that leaves (or rejoins) the neighbour search needs new lists; one
            // outside it is in no list, so its moves do not count
            const bool now = inactive_key(k, nk);
            if (now != inactive_key(k, keys[i])) {
                // every slot after it moves: with per-instance boxes all instances rebuild
                if (iw) atomicOr(iw + IW_ALL, 1u);
                box.add_at(iw, inst, 3.0e38f, 3.0e38f, 3.0e38f);
                box.add_at(iw, inst, -3.0e38f, -3.0e38f, -3.0e38f);
                return;
            }
            if (now) return;
        }
        if (!nl.xb) return;
        const float4 xb = nl.xb[i];
        box.add_at(iw, inst, (float)(np.x - (T)xb.x), (float)(np.y - (T)xb.y),
                   (float)(np.z - (T)xb.z));
    }
}


}  // namespace

}  // namespace sph
