// ns.cu — the two neighbour passes of the weakly-compressible delta-SPH step.
//
// Reference counterparts: SPH_NS_simpleversion (src/equation/ns.cu:5-28) launching
// computeBoundary_Delta_acoustic_D (pass 1, src/equation/ns.cu:30-131) and
// computeGovering_equationD (pass 2, src/equation/ns.cu:134-249).
//
// Layout.  Particles are in cell-sorted order; each is one record of two vec4,
// rec[2i] = (x, y, z, p) and rec[2i+1] = (vx, vy, vz, ±rho) with the sign of rho marking a
// fluid (+) or boundary (-) particle, so everything a neighbour contributes to pass 1 is one
// aligned 32-byte sector in FP32.  Pass 1 writes the record pass 2 gathers, nrec[2i] =
// (x, y, z, q), nrec[2i+1] = (vx, vy, vz, ±rho'), where q = p' - rho0 cs h dofv: the
// acoustic-damper term of a fluid-fluid pair, rho0 cs h (dofv_i + dofv_j), splits into an i part
// and a j part, and the j part is folded into the neighbour's pressure (boundary particles
// have dofv = 0, so q = p').  It also writes self[i] = (p', rho', dofv, 0) for the particle's
// own side.
//
// Cells are walked as nine x-strips: the three cells (x-1 .. x+1) of one (y, z) row are
// consecutive in the sorted order, so each strip is one contiguous slot range
// [cell_start[row + x-1], cell_start[row + x+2]) — the dense cell_start array gives empty cells
// the start of the next non-empty one.
//
// Neighbour list.  About 15% of the ~475 candidates of a 27-cell walk lie inside the
// support radius, and the lanes of a warp (particles of two or three adjacent cells) almost
// always have at least one hit per candidate, so a pass that tests and evaluates in one loop
// pays the full pair body for every candidate.  k_nbr_build therefore walks the candidates
// once per list build and stores the hits of particle i, in walk order, in column i of its
// warp's slot block (nbr_col); both passes then iterate only true neighbours, in the same
// order, so the sums are the same as a walking pass.  The passes are limited by L1 data-stage
// wavefronts (each lane gathers a different record): interleaving the slots (in groups of four
// per lane) makes a warp's list read four lines per four steps instead of one line per lane
// and step.  A particle with more hits than
// the list capacity is marked and walks the cells itself (same order again).
//
// With a Verlet skin the list is built with the cutoff kh(1 + skin) (kh2_list) on cells that
// wide and kept while every particle stays within skin*kh/2 of its build position; both
// passes still test r < kh on the current positions, and k_nbr_build keeps the build
// positions (xb) that pass 2 measures each particle's displacement against.
//
// Precision.  Every kernel is instantiated for the three policies of sph_internal.h: FP32
// (records of float4), FP64 (records of two 32-byte double vectors) and mixed.  The mixed
// policy stores positions as FP32 offsets from the origin of the particle's cell at the last
// list build; a pair's relative position is (o_i - o_j) - (c_j - c_i) cell, exact to a few
// ulp of the cell size instead of a few ulp of the domain size, with c_j - c_i stored in the
// list slot (or known to the cell walk); its integrator advances FP64 positions and the FP64
// density perturbation rho - rho0.  A fourth policy adds compensated (Neumaier) accumulation
// of the density and force sums (measured on the 765,828-particle case: no accuracy gain over
// plain FP32 sums on relative positions, +14% time).
//
// Kernel algebra (same quantities as the reference, simplified): with r = x_i - x_j,
// q = |r|/h, t = 1 - q/2, the Wendland C2 gradient is grad W = c_fr t^3 r with
// c_fr = -5 adh / h^2, which is the reference's per-component expression
// adh(-2 t^3 (2q+1) + 2 t^4) r/(h|r|) after factoring.
#include <cuda_runtime.h>

#include "sph_internal.h"

namespace sph {

namespace {

// Block size of the neighbour kernels is a launch parameter (KParams::threads, a multiple of
// 32 up to NS_MAX_THREADS), as is the number of particles a thread handles (KParams::ppt); both
// are picked by the autotuner.  ppt > 1 runs the grid-stride instantiation (GS), which holds
// its loop state in registers (pass 2: 64 instead of 48), so ppt = 1 has its own.
constexpr int NS_MAX_THREADS = 256;
// Mixed precision: a list slot is j | code << CODE_SHIFT (j < 2^26).
constexpr int CODE_SHIFT = 26;
constexpr unsigned IDX_MASK = (1u << CODE_SHIFT) - 1u;

// Squared distance with an explicit rounding sequence, so the in-range test gives the same
// answer in the list build, in the walking passes and in the list passes.
__device__ __forceinline__ float dist2(float dx, float dy, float dz) {
    return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}
__device__ __forceinline__ double dist2(double dx, double dy, double dz) {
    return __fma_rn(dz, dz, __fma_rn(dy, dy, __dmul_rn(dx, dx)));
}
// Pair arithmetic: in FP32 the distance and the reciprocal of a pair come from the hardware's
// approximate instructions (sqrt.approx, rcp.approx: within about one ulp, one instruction each
// instead of the correctly rounded sequences); FP64 keeps correctly rounded sqrt and division.
__device__ __forceinline__ float pair_sqrt(float x) {
    float r;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ double pair_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float pair_rcp(float x) {
    float r;
    asm("rcp.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ double pair_rcp(double x) { return 1.0 / x; }
__device__ __forceinline__ float dabs(float x) { return fabsf(x); }
__device__ __forceinline__ double dabs(double x) { return fabs(x); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
[[maybe_unused]] __device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
[[maybe_unused]] __device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }

// A neighbour sum: plain, or compensated (Neumaier) when COMP.  The compensated form uses
// explicitly rounded adds so no contraction folds the error terms away.
template <class T, bool COMP>
struct Sum {
    T s = T(0), c = T(0);
    __device__ __forceinline__ void add(T v) {
        if constexpr (COMP) {
            const T t = add_rn(s, v);
            c = add_rn(c, dabs(s) >= dabs(v) ? add_rn(sub_rn(s, t), v) : add_rn(sub_rn(v, t), s));
            s = t;
        } else {
            s += v;
        }
    }
    __device__ __forceinline__ T get() const {
        if constexpr (COMP) return add_rn(s, c);
        return s;
    }
};

// Visit every candidate slot j of the 27 cells around (cx, cy, cz): f(j, code).  Without CODES
// each x-strip is one range and code is 0; with CODES the strip's three cells are visited one
// by one and code = (dz+1) << 4 | (dy+1) << 2 | (dx+1) is j's cell relative to (cx, cy, cz).
// Both visit the same slots in the same order.
template <bool CODES, class KP, class F>
__device__ __forceinline__ void for_each_candidate(const KP& k, const int* __restrict__ cs,
                                                   int cx, int cy, int cz, F&& f) {
    const int xl = cx > 0 ? cx - 1 : 0;
    const int xh = cx < k.gx - 1 ? cx + 1 : k.gx - 1;
#pragma unroll 1
    for (int dz = -1; dz <= 1; dz++) {
        const int z = cz + dz;
        if ((unsigned)z >= (unsigned)k.gz) continue;
#pragma unroll 1
        for (int dy = -1; dy <= 1; dy++) {
            const int y = cy + dy;
            if ((unsigned)y >= (unsigned)k.gy) continue;
            const int row = (z * k.gy + y) * k.gx;
            if constexpr (CODES) {
#pragma unroll 1
                for (int xc = xl; xc <= xh; xc++) {
                    const unsigned code =
                        (unsigned)(((dz + 1) << 4) | ((dy + 1) << 2) | (xc - cx + 1));
                    const int j0 = max(__ldg(cs + row + xc), 0);
                    const int j1 = min(__ldg(cs + row + xc + 1), k.n);  // bounds guard only
                    for (int j = j0; j < j1; j++) f(j, code);
                }
            } else {
                const int j0 = max(__ldg(cs + row + xl), 0);
                const int j1 = min(__ldg(cs + row + xh + 1), k.n);  // bounds guard only
#pragma unroll 4
                for (int j = j0; j < j1; j++) f(j, 0u);
            }
        }
    }
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

// Relative position r = x_i - x_j of a pair: from absolute positions, or (mixed precision)
// from cell-local offsets and j's cell relative to i's.
template <class P, class V>
__device__ __forceinline__ void rel_pos(const KParamsT<typename P::T>& k, const V& pi,
                                        const V& pj, unsigned code, typename P::T& dx,
                                        typename P::T& dy, typename P::T& dz) {
    using T = typename P::T;
    if constexpr (P::kMixed) {
        const int rz = (int)(code >> 4) - 1;
        const int ry = (int)((code >> 2) & 3u) - 1;
        const int rx = (int)(code & 3u) - 1;
        dx = (pi.x - pj.x) - (T)rx * k.cell;
        dy = (pi.y - pj.y) - (T)ry * k.cell;
        dz = (pi.z - pj.z) - (T)rz * k.cell;
    } else {
        (void)k;
        (void)code;
        dx = pi.x - pj.x;
        dy = pi.y - pj.y;
        dz = pi.z - pj.z;
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
    for_each_candidate<P::kMixed>(k, cs, cx, cy, cz, [&](int j, unsigned code) {
        const vec4_t<T> pj = ld_pos(X, (size_t)STRIDE * (size_t)j);
        T dx, dy, dz;
        rel_pos<P>(k, pi, pj, code, dx, dy, dz);
        const T r2 = dist2(dx, dy, dz);
        if (r2 < cut2 && j != i) f(j, code, pj, dx, dy, dz, r2);
    });
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

// Appends slots to a list column four at a time (one 16-byte store per four slots).
struct SlotWriter {
    int* __restrict__ col;
    int cap;
    int cnt = 0;
    int b0 = 0, b1 = 0, b2 = 0, b3 = 0;
    __device__ __forceinline__ void put(int v) {
        const int s = cnt & 3;
        b0 = s == 0 ? v : b0;
        b1 = s == 1 ? v : b1;
        b2 = s == 2 ? v : b2;
        b3 = s == 3 ? v : b3;
        cnt++;
        if (s == 3 && cnt <= cap)
            *reinterpret_cast<int4*>(col + ((size_t)(cnt - 4) << 5)) = make_int4(b0, b1, b2, b3);
    }
    // the last, partial group (its unused slots are never read: count bounds the readers)
    __device__ __forceinline__ void flush() {
        if ((cnt & 3) && cnt < cap)
            *reinterpret_cast<int4*>(col + ((size_t)(cnt & ~3) << 5)) = make_int4(b0, b1, b2, b3);
    }
};

// Neighbours of i (r2 < kh2) with their records R[2j], R[2j+1]: from the list (one record
// load per listed pair, the next slot loaded one pair ahead; pairs in the skin beyond the
// support radius are skipped), or by walking the cells over X[XSTRIDE * j] when i overflowed
// the list.  f(j, a, b, dx, dy, dz, r2).  (Skipping the gathers of slots in the skin with a
// pass-1 hit mask cost pass 2 more in instructions than it saved in sectors.)
template <class P, bool LIST, int XSTRIDE, class F>
__device__ __forceinline__ void visit_records(const KParamsT<typename P::T>& k,
                                              const int* __restrict__ cs,
                                              const unsigned* __restrict__ keys,
                                              const NbrList& nl,
                                              const vec4_t<typename P::T>* __restrict__ X,
                                              const vec4_t<typename P::T>* __restrict__ R, int i,
                                              const vec4_t<typename P::T>& pi, F&& f) {
    using T = typename P::T;
    using V = vec4_t<T>;
    if (LIST) {
        const int cnt = __ldg(nl.count + i);
        if (cnt <= nl.cap) {
            const int* __restrict__ col = nl.idx + nbr_col(nl, i);
            auto one = [&](int e) {
                const int j = P::kMixed ? (int)((unsigned)e & IDX_MASK) : e;
                V a, b;
                ld_rec(R, j, a, b);
                T dx, dy, dz;
                rel_pos<P>(k, pi, a, (unsigned)e >> CODE_SHIFT, dx, dy, dz);
                const T r2 = dist2(dx, dy, dz);
                if (r2 < k.kh2) f(j, a, b, dx, dy, dz, r2);
            };
            int4 q = cnt > 0 ? ld_slots(col) : make_int4(0, 0, 0, 0);
#pragma unroll 1
            for (int c = 0; c < cnt; c += 4) {
                // the next group is loaded one group ahead
                const int4 qn = c + 4 < cnt ? ld_slots(col + ((size_t)(c + 4) << 5)) : q;
                one(q.x);
                if (c + 1 < cnt) one(q.y);
                if (c + 2 < cnt) one(q.z);
                if (c + 3 < cnt) one(q.w);
                q = qn;
            }
            return;
        }
    }
    walk_pairs<P, XSTRIDE>(k, cs, keys, X, i, pi, k.kh2,
                           [&](int j, unsigned, const V&, T dx, T dy, T dz, T r2) {
        V a, b;
        ld_rec(R, j, a, b);
        f(j, a, b, dx, dy, dz, r2);
    });
}

template <class T>
__device__ __forceinline__ bool fluid_rec(T signed_rho) { return signed_rho > T(0); }

// Position the list build records for the displacement test (offsets in mixed precision).
__device__ __forceinline__ float4 as_float4(const float4& v) { return v; }
__device__ __forceinline__ float4 as_float4(const dvec4& v) {
    return make_float4((float)v.x, (float)v.y, (float)v.z, (float)v.w);
}

// Neighbour-list build: every boundary particle keeps its fluid neighbours (all that pass 1
// needs), every fluid particle all of them; with walls_all, boundary particles keep all.
// Slots are warp-interleaved (nbr_col): the passes read them coalesced, the build writes them
// scattered within its warp's block, which L2 merges before they reach HBM.
template <class P>
__device__ __forceinline__ void nbr_build_one(const KParamsT<typename P::T>& k,
                                              const vec4_t<typename P::T>* __restrict__ X,
                                              const unsigned* __restrict__ keys,
                                              const int* __restrict__ cs, const NbrList& nl,
                                              int walls_all, unsigned* err, int i) {
    using T = typename P::T;
    const vec4_t<T> pi = X[i];
    if (nl.xb) nl.xb[i] = as_float4(pi);
    const bool keep_all = fluid_rec(pi.w) || walls_all;
    SlotWriter w{nl.idx + nbr_col(nl, i), nl.cap};
    walk_pairs<P, 1>(k, cs, keys, X, i, pi, k.kh2_list,
                     [&](int j, unsigned code, const vec4_t<T>& pj, T, T, T, T) {
        if (keep_all || fluid_rec(pj.w))
            w.put(P::kMixed ? (int)((unsigned)j | (code << CODE_SHIFT)) : j);
    });
    w.flush();
    nl.count[i] = w.cnt;
    raise_flags(err, w.cnt > nl.cap ? SPH_FLAG_NEIGHBOR_OVERFLOW : 0u);
}

template <class P, bool GS>
__global__ void __launch_bounds__(NS_MAX_THREADS)
k_nbr_build(KParamsT<typename P::T> k, const vec4_t<typename P::T>* __restrict__ X,
            const unsigned* __restrict__ keys, const int* __restrict__ cs, NbrList nl,
            int walls_all, unsigned* err, const unsigned* gate) {
    if (gated_off(gate)) return;
    const int i0 = blockIdx.x * blockDim.x + threadIdx.x;
    if constexpr (GS) {
        for (int i = i0; i < k.n; i += gridDim.x * blockDim.x)
            nbr_build_one<P>(k, X, keys, cs, nl, walls_all, err, i);
    } else if (i0 < k.n) {
        nbr_build_one<P>(k, X, keys, cs, nl, walls_all, err, i0);
    }
}

// Pass 1: boundary pressure extrapolation (Adami-style, over fluid neighbours) for boundary
// particles; velocity divergence over fluid neighbours for fluid particles.  Writes the pass-2
// neighbour record and the particle's own (p', rho', dofv).
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
        const T q = rr * k.inv_h;
        const T t = T(1) - T(0.5) * q;
        const T t2 = t * t;
        if (!fi) {
            const T w = k.adh * t2 * t2 * (T(2) * q + T(1));
            rs.add((aj.w + vj.w * k.g * dz) * w);
            ws.add(w);
        } else {
            const T fr = k.c_fr * t2 * t;
            const T vdotr = (vi.x - vj.x) * dx + (vi.y - vj.y) * dy + (vi.z - vj.z) * dz;
            dofv.add(-(fr * vdotr * (k.mass * pair_rcp(vj.w))));
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
        const T qv = fi ? p - k.damper * dv : p;
        out.nrec[2 * (size_t)i] = make4<T>(pi.x, pi.y, pi.z, qv);
        out.nrec[2 * (size_t)i + 1] = make4<T>(vi.x, vi.y, vi.z, fi ? rho : -rho);
        out.self[i] = make4<T>(p, rho, dv, T(0));
        if constexpr (WRITE_SUMS) {
            rhop_sum[i] = (float)rsum;
            w_sum[i] = (float)wsum;
        }
    }
};

template <class P, bool WRITE_SUMS, bool LIST>
__device__ __forceinline__ void pass1_one(const KParamsT<typename P::T>& k,
                                          const ParticleSetT<typename P::T>& in,
                                          const unsigned* __restrict__ keys,
                                          const int* __restrict__ cs, const NbrList& nl,
                                          const Pass1OutT<typename P::T>& out,
                                          float* __restrict__ rhop_sum, float* __restrict__ w_sum,
                                          int i) {
    using T = typename P::T;
    using V = vec4_t<T>;
    Pass1Acc<P> acc;
    acc.load(in.rec, i);
    visit_records<P, LIST, 1>(k, cs, keys, nl, in.xyz, in.rec, i, acc.pi,
                              [&](int, const V& aj, const V& vj, T dx, T dy, T dz, T r2) {
        acc.pair(k, aj, vj, dx, dy, dz, r2);
    });
    acc.template finish<WRITE_SUMS>(k, out, rhop_sum, w_sum, i);
}

template <class P, bool WRITE_SUMS, bool LIST, bool GS>
__global__ void __launch_bounds__(NS_MAX_THREADS)
k_pass1(KParamsT<typename P::T> k, ParticleSetT<typename P::T> in,
        const unsigned* __restrict__ keys, const int* __restrict__ cs, NbrList nl,
        Pass1OutT<typename P::T> out, float* __restrict__ rhop_sum, float* __restrict__ w_sum) {
    const int i0 = blockIdx.x * blockDim.x + threadIdx.x;
    if constexpr (GS) {
        for (int i = i0; i < k.n; i += gridDim.x * blockDim.x)
            pass1_one<P, WRITE_SUMS, LIST>(k, in, keys, cs, nl, out, rhop_sum, w_sum, i);
    } else if (i0 < k.n) {
        pass1_one<P, WRITE_SUMS, LIST>(k, in, keys, cs, nl, out, rhop_sum, w_sum, i0);
    }
}

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
        const T q = rr * k.inv_h;
        const T t = T(1) - T(0.5) * q;
        const T fr = k.c_fr * t * t * t;
        const T vdotr = (vi.x - vj.x) * dx + (vi.y - vj.y) * dy + (vi.z - vj.z) * dz;
        const T volj = k.mass * pair_rcp(rhoj);
        const T inv_r2e = pair_rcp(r2 + k.eta2);
        sd.add(volj * fr * (rhoi * vdotr + (rhoi - rhoj) * k.delta_h_cs * r2 * inv_r2e));
        T S;
        if (fi) {
            S = -presi - aj.w;
            if (fj) S += damp_i + k.visc * vdotr * inv_r2e;
        } else {
            S = -(presi + __ldg(&p1.self[j].x));  // boundary rows (wall_rates): plain pressures
        }
        const T c = fr * S * volj;
        sx.add(c * dx);
        sy.add(c * dy);
        sz.add(c * dz);
    }
};

template <class P, int MODE>
__device__ __forceinline__ float pass2_finish(const KParamsT<typename P::T>& k, int i,
                                              const Pass2Acc<P, MODE>& acc,
                                              const ParticleSetT<typename P::T>& in,
                                              const unsigned* __restrict__ keys,
                                              const NbrList& nl, float* __restrict__ rho_dt,
                                              float* __restrict__ vel_dt, int wall_rates,
                                              const ParticleSetT<typename P::T>& out,
                                              unsigned* __restrict__ out_hash, unsigned* err);

template <class P, int MODE, bool LIST>
__device__ __forceinline__ float pass2_one(const KParamsT<typename P::T>& k, int i,
                                           const ParticleSetT<typename P::T>& in,
                                           const unsigned* __restrict__ keys,
                                           const int* __restrict__ cs, const NbrList& nl,
                                           const Pass1OutT<typename P::T>& p1,
                                           float* __restrict__ rho_dt, float* __restrict__ vel_dt,
                                           int wall_rates, const ParticleSetT<typename P::T>& out,
                                           unsigned* __restrict__ out_hash, unsigned* err) {
    using T = typename P::T;
    using V = vec4_t<T>;
    Pass2Acc<P, MODE> acc;
    acc.load(k, p1, i, wall_rates);
    if (acc.active)
        visit_records<P, LIST, 2>(k, cs, keys, nl, p1.nrec, p1.nrec, i, acc.pi,
                                  [&](int j, const V& aj, const V& vj, T dx, T dy, T dz, T r2) {
            acc.pair(k, p1, j, aj, vj, dx, dy, dz, r2);
        });
    return pass2_finish<P, MODE>(k, i, acc, in, keys, nl, rho_dt, vel_dt, wall_rates, out,
                                 out_hash, err);
}

// Rates, or the predictor / corrector update and the next key of particle i; returns its
// squared distance from its list-build position (0 without a list).
template <class P, int MODE>
__device__ __forceinline__ float pass2_finish(const KParamsT<typename P::T>& k, int i,
                                              const Pass2Acc<P, MODE>& acc,
                                              const ParticleSetT<typename P::T>& in,
                                              const unsigned* __restrict__ keys,
                                              const NbrList& nl, float* __restrict__ rho_dt,
                                              float* __restrict__ vel_dt, int wall_rates,
                                              const ParticleSetT<typename P::T>& out,
                                              unsigned* __restrict__ out_hash, unsigned* err) {
    using T = typename P::T;
    using V = vec4_t<T>;
    const V& pi = acc.pi;
    const V& vi = acc.vi;
    const bool fi = acc.fi;
    const T rhoi = acc.rhoi, presi = acc.presi;
    T drho = T(0), ax = T(0), ay = T(0), az = T(0);
    if (acc.active) {
        drho = acc.sd.get();
        const T inv_rhoi = T(1) / rhoi;
        ax = acc.sx.get() * inv_rhoi;
        ay = acc.sy.get() * inv_rhoi;
        az = acc.sz.get() * inv_rhoi;
    }
    az += k.g;

    if constexpr (MODE == MODE_RATES) {
        const bool have = fi || wall_rates;
        rho_dt[i] = have ? (float)drho : 0.f;
        vel_dt[3 * i] = have ? (float)ax : 0.f;
        vel_dt[3 * i + 1] = have ? (float)ay : 0.f;
        vel_dt[3 * i + 2] = have ? (float)az : 0.f;
        return 0.f;
    } else if constexpr (P::kMixed) {
        // FP64 position and density perturbation; FP32 velocity
        const dvec4 xm = in.xm[i];
        dvec4 nxm = xm, txm = xm;
        float4 nv, tv;
        float npres, nrho;
        const double hdt = (double)k.half_dt;
        if (fi) {
            if (escaped(k, xm.x, xm.y, xm.z)) {
                nxm = dvec4{(double)k.park_x, (double)k.park_y, (double)k.park_z, 0.0};
                nv = make_float4(0.f, 0.f, 0.f, 0.f);
                txm = nxm;
                tv = nv;
            } else if (MODE == MODE_PRED) {
                tv = make_float4(vi.x, vi.y, vi.z, 0.f);
                double d = xm.w + (double)drho * hdt;
                if (k.clamp_density && d < 0.0) d = 0.0;
                nxm.x = xm.x + (double)vi.x * hdt;
                nxm.y = xm.y + (double)vi.y * hdt;
                nxm.z = xm.z + (double)vi.z * hdt;
                nxm.w = d;
                nv = make_float4(vi.x + ax * k.half_dt, vi.y + ay * k.half_dt, vi.z + az * k.half_dt,
                                 0.f);
            } else {
                txm = in.txm[i];
                tv = in.tvel[i];
                double ds = txm.w + (double)drho * hdt;
                if (k.clamp_density && ds < 0.0) ds = 0.0;
                double d = 2.0 * ds - txm.w;
                if (k.clamp_density && d < 0.0) d = 0.0;
                nxm.x = 2.0 * (txm.x + (double)vi.x * hdt) - txm.x;
                nxm.y = 2.0 * (txm.y + (double)vi.y * hdt) - txm.y;
                nxm.z = 2.0 * (txm.z + (double)vi.z * hdt) - txm.z;
                nxm.w = d;
                const float uxs = tv.x + ax * k.half_dt;
                const float uys = tv.y + ay * k.half_dt;
                const float uzs = tv.z + az * k.half_dt;
                nv = make_float4(2.f * uxs - tv.x, 2.f * uys - tv.y, 2.f * uzs - tv.z, 0.f);
            }
            nrho = k.rho0 + (float)nxm.w;
            npres = eos_pressure_d(k, (float)nxm.w);
        } else {
            // boundary particles do not move; they keep the extrapolated pressure and density
            nv = make_float4(vi.x, vi.y, vi.z, 0.f);
            npres = presi;
            nrho = rhoi;
            tv = nv;
        }
        double ox, oy, oz;
        cell_origin(k, keys[i], ox, oy, oz);
        const float px = (float)(nxm.x - ox), py = (float)(nxm.y - oy), pz = (float)(nxm.z - oz);
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
        const unsigned nk = slot_key(k, inst, fi, nxm.x, nxm.y, nxm.z, &f);
        out_hash[i] = nk;
        raise_flags(err, f);
        if (k.park_inactive) {
            // a particle that leaves (or rejoins) the neighbour search needs new lists; one
            // outside it is in no list, so its moves do not count
            const bool now = inactive_key(k, nk);
            if (now != inactive_key(k, keys[i])) return 3.0e38f;
            if (now) return 0.f;
        }
        if (!fi || !nl.xb) return 0.f;
        const float4 xb = nl.xb[i];
        return dist2(px - xb.x, py - xb.y, pz - xb.z);
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
                T rho = rhoi + drho * k.half_dt;
                if (k.clamp_density && rho < k.rho0) rho = k.rho0;
                np.x = pi.x + vi.x * k.half_dt;
                np.y = pi.y + vi.y * k.half_dt;
                np.z = pi.z + vi.z * k.half_dt;
                nv = make4<T>(vi.x + ax * k.half_dt, vi.y + ay * k.half_dt, vi.z + az * k.half_dt,
                              T(0));
                nrho = rho;
                npres = eos_pressure(k, rho);
            } else {
                tp = in.tpos[i];
                tv = in.tvel[i];
                T rho = tp.w + drho * k.half_dt;
                if (k.clamp_density && rho < k.rho0) rho = k.rho0;
                const T xs = tp.x + vi.x * k.half_dt;
                const T ys = tp.y + vi.y * k.half_dt;
                const T zs = tp.z + vi.z * k.half_dt;
                const T uxs = tv.x + ax * k.half_dt;
                const T uys = tv.y + ay * k.half_dt;
                const T uzs = tv.z + az * k.half_dt;
                rho = T(2) * rho - tp.w;
                if (k.clamp_density && rho < k.rho0) rho = k.rho0;
                np.x = T(2) * xs - tp.x;
                np.y = T(2) * ys - tp.y;
                np.z = T(2) * zs - tp.z;
                nv = make4<T>(T(2) * uxs - tv.x, T(2) * uys - tv.y, T(2) * uzs - tv.z, T(0));
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
            if (now != inactive_key(k, keys[i])) return 3.0e38f;
            if (now) return 0.f;
        }
        if (!fi || !nl.xb) return 0.f;
        const float4 xb = nl.xb[i];
        return (float)dist2(np.x - (T)xb.x, np.y - (T)xb.y, np.z - (T)xb.z);
    }
}

template <class P, int MODE, bool LIST, bool GS>
__global__ void __launch_bounds__(NS_MAX_THREADS)
k_pass2(KParamsT<typename P::T> k, ParticleSetT<typename P::T> in,
        const unsigned* __restrict__ keys, const int* __restrict__ cs, NbrList nl,
        Pass1OutT<typename P::T> p1, float* __restrict__ rho_dt, float* __restrict__ vel_dt,
        int wall_rates, ParticleSetT<typename P::T> out, unsigned* __restrict__ out_hash,
        unsigned* err, unsigned* disp) {
    float d2 = 0.f;
    const int i0 = blockIdx.x * blockDim.x + threadIdx.x;
    if constexpr (GS) {
        for (int i = i0; i < k.n; i += gridDim.x * blockDim.x)
            d2 = fmaxf(d2, pass2_one<P, MODE, LIST>(k, i, in, keys, cs, nl, p1, rho_dt, vel_dt,
                                                    wall_rates, out, out_hash, err));
    } else if (i0 < k.n) {
        d2 = pass2_one<P, MODE, LIST>(k, i0, in, keys, cs, nl, p1, rho_dt, vel_dt, wall_rates,
                                      out, out_hash, err);
    }
    if (MODE == MODE_RATES || disp == nullptr) return;
    // block maximum of the squared displacement, one atomic per block (non-negative floats
    // order like their bit patterns); blockDim is a multiple of 32, every thread gets here
    __shared__ unsigned s_max[NS_MAX_THREADS / 32];
    const unsigned wmax = __reduce_max_sync(0xffffffffu, __float_as_uint(d2));
    if ((threadIdx.x & 31) == 0) s_max[threadIdx.x >> 5] = wmax;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned m = s_max[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) m = max(m, s_max[w]);
        if (m) atomicMax(disp, m);
    }
}

// The same kernel held to CAP registers (one particle per thread): the FP32 step kernel fits
// in 48 with an 8-byte stack frame, keeping ten 128-thread blocks resident per SM where the
// unconstrained 53 keeps nine; the mixed-precision one in 56 (nine blocks instead of eight).
template <class P, int MODE, bool LIST, bool GS, int CAP>
__global__ void __maxnreg__(CAP)
k_pass2_cap(KParamsT<typename P::T> k, ParticleSetT<typename P::T> in,
        const unsigned* __restrict__ keys, const int* __restrict__ cs, NbrList nl,
        Pass1OutT<typename P::T> p1, float* __restrict__ rho_dt, float* __restrict__ vel_dt,
        int wall_rates, ParticleSetT<typename P::T> out, unsigned* __restrict__ out_hash,
        unsigned* err, unsigned* disp) {
    float d2 = 0.f;
    const int i0 = blockIdx.x * blockDim.x + threadIdx.x;
    if constexpr (GS) {
        for (int i = i0; i < k.n; i += gridDim.x * blockDim.x)
            d2 = fmaxf(d2, pass2_one<P, MODE, LIST>(k, i, in, keys, cs, nl, p1, rho_dt, vel_dt,
                                                    wall_rates, out, out_hash, err));
    } else if (i0 < k.n) {
        d2 = pass2_one<P, MODE, LIST>(k, i0, in, keys, cs, nl, p1, rho_dt, vel_dt, wall_rates,
                                      out, out_hash, err);
    }
    if (MODE == MODE_RATES || disp == nullptr) return;
    // block maximum of the squared displacement, one atomic per block (non-negative floats
    // order like their bit patterns); blockDim is a multiple of 32, every thread gets here
    __shared__ unsigned s_max[NS_MAX_THREADS / 32];
    const unsigned wmax = __reduce_max_sync(0xffffffffu, __float_as_uint(d2));
    if ((threadIdx.x & 31) == 0) s_max[threadIdx.x >> 5] = wmax;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned m = s_max[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) m = max(m, s_max[w]);
        if (m) atomicMax(disp, m);
    }
}

// ---------------------------------------------------------------- particle pairs
// Pair mode (KParams::pairs, FP32 and FP64): a thread handles the two consecutive sorted
// particles 2c and 2c+1 (a "pair", usually in one cell) over the union of their neighbour
// lists, so each listed record is gathered once for both.  The passes are limited by those
// gathers (one L1 data-stage wavefront per distinct line a warp instruction touches), and the
// union of two consecutive particles' lists is about 1.38 times one list: 31% fewer gathers
// for up to twice the pair bodies per gather.  The list is indexed by pair (warp-interleaved
// over pairs); its slots hold every j within the list cutoff of either particle, in walk
// order; each particle tests r < kh (and j != itself) on every slot.  A pair whose union
// overflowed walks the cells for each of its two particles.

template <class P>
__device__ __forceinline__ void nbr_build_pair(const KParamsT<typename P::T>& k,
                                               const vec4_t<typename P::T>* __restrict__ X,
                                               const unsigned* __restrict__ keys,
                                               const int* __restrict__ cs, const NbrList& nl,
                                               int walls_all, unsigned* err, int c) {
    using T = typename P::T;
    using V = vec4_t<T>;
    const int i0 = 2 * c, i1 = 2 * c + 1;
    const V p0 = X[i0];
    const V p1 = i1 < k.n ? X[i1] : p0;
    if (nl.xb) {
        nl.xb[i0] = as_float4(p0);
        if (i1 < k.n) nl.xb[i1] = as_float4(p1);
    }
    // particles outside the neighbour search (park_inactive) sort last: take no candidates
    const bool has1 = i1 < k.n && !inactive_key(k, keys[i1]);
    if (inactive_key(k, keys[i0])) {
        nl.count[c] = 0;
        return;
    }
    const bool keep0 = fluid_rec(p0.w) || walls_all;
    const bool keep1 = has1 && (fluid_rec(p1.w) || walls_all);
    SlotWriter w{nl.idx + nbr_col(nl, c), nl.cap};
    auto visit = [&](int j) {
        const V pj = ld_pos(X, (size_t)j);
        const bool fj = fluid_rec(pj.w);
        bool in = dist2(p0.x - pj.x, p0.y - pj.y, p0.z - pj.z) < k.kh2_list && j != i0 &&
                  (keep0 || fj);
        if (has1)
            in = in || (dist2(p1.x - pj.x, p1.y - pj.y, p1.z - pj.z) < k.kh2_list && j != i1 &&
                        (keep1 || fj));
        if (in) w.put(j);
    };
    int x0, y0, z0;
    cell_of_key(k.gx, k.gy, keys[i0], x0, y0, z0);
    for_each_candidate<false>(k, cs, x0, y0, z0, [&](int j, unsigned) { visit(j); });
    if (has1 && keys[i1] != keys[i0]) {
        // the cells around the second particle's cell that the first walk did not cover
        int x1, y1, z1;
        cell_of_key(k.gx, k.gy, keys[i1], x1, y1, z1);
#pragma unroll 1
        for (int z = z1 - 1; z <= z1 + 1; z++) {
            if ((unsigned)z >= (unsigned)k.gz) continue;
#pragma unroll 1
            for (int y = y1 - 1; y <= y1 + 1; y++) {
                if ((unsigned)y >= (unsigned)k.gy) continue;
                const int row = (z * k.gy + y) * k.gx;
                const bool row_seen = abs(z - z0) <= 1 && abs(y - y0) <= 1;
#pragma unroll 1
                for (int x = max(x1 - 1, 0); x <= min(x1 + 1, k.gx - 1); x++) {
                    if (row_seen && abs(x - x0) <= 1) continue;
                    const int j0 = max(__ldg(cs + row + x), 0);
                    const int j1 = min(__ldg(cs + row + x + 1), k.n);  // bounds guard only
                    for (int j = j0; j < j1; j++) visit(j);
                }
            }
        }
    }
    w.flush();
    nl.count[c] = w.cnt;
    raise_flags(err, w.cnt > nl.cap ? SPH_FLAG_NEIGHBOR_OVERFLOW : 0u);
}

// Iterate a pair's union list: f(j, a, b) with the record of every slot.  Returns false (and
// calls nothing) when the union overflowed the list.
template <class P, class F>
__device__ __forceinline__ bool visit_union(const NbrList& nl,
                                            const vec4_t<typename P::T>* __restrict__ R, int c,
                                            F&& f) {
    using V = vec4_t<typename P::T>;
    const int cnt = __ldg(nl.count + c);
    if (cnt > nl.cap) return false;
    const int* __restrict__ col = nl.idx + nbr_col(nl, c);
    auto one = [&](int j) {
        V a, b;
        ld_rec(R, j, a, b);
        f(j, a, b);
    };
    int4 q = cnt > 0 ? ld_slots(col) : make_int4(0, 0, 0, 0);
#pragma unroll 1
    for (int e = 0; e < cnt; e += 4) {
        const int4 qn = e + 4 < cnt ? ld_slots(col + ((size_t)(e + 4) << 5)) : q;
        one(q.x);
        if (e + 1 < cnt) one(q.y);
        if (e + 2 < cnt) one(q.z);
        if (e + 3 < cnt) one(q.w);
        q = qn;
    }
    return true;
}

template <class P, bool WRITE_SUMS>
__device__ __forceinline__ void pass1_pair(const KParamsT<typename P::T>& k,
                                           const ParticleSetT<typename P::T>& in,
                                           const unsigned* __restrict__ keys,
                                           const int* __restrict__ cs, const NbrList& nl,
                                           const Pass1OutT<typename P::T>& out,
                                           float* __restrict__ rhop_sum,
                                           float* __restrict__ w_sum, int c) {
    using T = typename P::T;
    using V = vec4_t<T>;
    const int i0 = 2 * c, i1 = 2 * c + 1;
    const bool has1 = i1 < k.n;
    Pass1Acc<P> a0, a1;
    a0.load(in.rec, i0);
    if (has1) a1.load(in.rec, i1);
    // particles outside the neighbour search (park_inactive) take no pairs
    const bool use0 = !inactive_key(k, keys[i0]);
    const bool use1 = has1 && !inactive_key(k, keys[i1]);
    auto one = [&](Pass1Acc<P>& acc, int i, int j, const V& a, const V& b) {
        const T dx = acc.pi.x - a.x, dy = acc.pi.y - a.y, dz = acc.pi.z - a.z;
        const T r2 = dist2(dx, dy, dz);
        if (r2 < k.kh2 && j != i) acc.pair(k, a, b, dx, dy, dz, r2);
    };
    const bool listed = visit_union<P>(nl, in.rec, c, [&](int j, const V& a, const V& b) {
        if (use0) one(a0, i0, j, a, b);
        if (use1) one(a1, i1, j, a, b);
    });
    if (!listed) {
        visit_records<P, false, 1>(k, cs, keys, nl, in.xyz, in.rec, i0, a0.pi,
                                   [&](int, const V& aj, const V& vj, T dx, T dy, T dz, T r2) {
            a0.pair(k, aj, vj, dx, dy, dz, r2);
        });
        if (has1)
            visit_records<P, false, 1>(k, cs, keys, nl, in.xyz, in.rec, i1, a1.pi,
                                       [&](int, const V& aj, const V& vj, T dx, T dy, T dz,
                                           T r2) { a1.pair(k, aj, vj, dx, dy, dz, r2); });
    }
    a0.template finish<WRITE_SUMS>(k, out, rhop_sum, w_sum, i0);
    if (has1) a1.template finish<WRITE_SUMS>(k, out, rhop_sum, w_sum, i1);
}

template <class P, int MODE>
__device__ __forceinline__ float pass2_pair(const KParamsT<typename P::T>& k, int c,
                                            const ParticleSetT<typename P::T>& in,
                                            const unsigned* __restrict__ keys,
                                            const int* __restrict__ cs, const NbrList& nl,
                                            const Pass1OutT<typename P::T>& p1,
                                            float* __restrict__ rho_dt,
                                            float* __restrict__ vel_dt, int wall_rates,
                                            const ParticleSetT<typename P::T>& out,
                                            unsigned* __restrict__ out_hash, unsigned* err) {
    using T = typename P::T;
    using V = vec4_t<T>;
    const int i0 = 2 * c, i1 = 2 * c + 1;
    const bool has1 = i1 < k.n;
    Pass2Acc<P, MODE> a0, a1;
    a0.load(k, p1, i0, wall_rates);
    if (has1) a1.load(k, p1, i1, wall_rates);
    // particles outside the neighbour search (park_inactive) take no pairs
    a0.active = a0.active && !inactive_key(k, keys[i0]);
    const bool act1 = has1 && a1.active && !inactive_key(k, keys[i1]);
    if (a0.active || act1) {
        auto one = [&](Pass2Acc<P, MODE>& acc, int i, int j, const V& a, const V& b) {
            const T dx = acc.pi.x - a.x, dy = acc.pi.y - a.y, dz = acc.pi.z - a.z;
            const T r2 = dist2(dx, dy, dz);
            if (r2 < k.kh2 && j != i) acc.pair(k, p1, j, a, b, dx, dy, dz, r2);
        };
        const bool listed = visit_union<P>(nl, p1.nrec, c, [&](int j, const V& a, const V& b) {
            if (a0.active) one(a0, i0, j, a, b);
            if (act1) one(a1, i1, j, a, b);
        });
        if (!listed) {
            if (a0.active)
                visit_records<P, false, 2>(k, cs, keys, nl, p1.nrec, p1.nrec, i0, a0.pi,
                                           [&](int j, const V& aj, const V& vj, T dx, T dy, T dz,
                                               T r2) { a0.pair(k, p1, j, aj, vj, dx, dy, dz, r2); });
            if (act1)
                visit_records<P, false, 2>(k, cs, keys, nl, p1.nrec, p1.nrec, i1, a1.pi,
                                           [&](int j, const V& aj, const V& vj, T dx, T dy, T dz,
                                               T r2) { a1.pair(k, p1, j, aj, vj, dx, dy, dz, r2); });
        }
    }
    float d2 = pass2_finish<P, MODE>(k, i0, a0, in, keys, nl, rho_dt, vel_dt, wall_rates, out,
                                     out_hash, err);
    if (has1)
        d2 = fmaxf(d2, pass2_finish<P, MODE>(k, i1, a1, in, keys, nl, rho_dt, vel_dt, wall_rates,
                                             out, out_hash, err));
    return d2;
}

template <class P>
__global__ void __launch_bounds__(NS_MAX_THREADS)
k_nbr_build_pairs(KParamsT<typename P::T> k, const vec4_t<typename P::T>* __restrict__ X,
                  const unsigned* __restrict__ keys, const int* __restrict__ cs, NbrList nl,
                  int walls_all, unsigned* err, const unsigned* gate) {
    if (gated_off(gate)) return;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < (k.n + 1) / 2) nbr_build_pair<P>(k, X, keys, cs, nl, walls_all, err, c);
}

template <class P, bool WRITE_SUMS>
__global__ void __launch_bounds__(NS_MAX_THREADS)
k_pass1_pairs(KParamsT<typename P::T> k, ParticleSetT<typename P::T> in,
              const unsigned* __restrict__ keys, const int* __restrict__ cs, NbrList nl,
              Pass1OutT<typename P::T> out, float* __restrict__ rhop_sum,
              float* __restrict__ w_sum) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < (k.n + 1) / 2) pass1_pair<P, WRITE_SUMS>(k, in, keys, cs, nl, out, rhop_sum, w_sum, c);
}

template <class P, int MODE>
__global__ void __launch_bounds__(NS_MAX_THREADS)
k_pass2_pairs(KParamsT<typename P::T> k, ParticleSetT<typename P::T> in,
              const unsigned* __restrict__ keys, const int* __restrict__ cs, NbrList nl,
              Pass1OutT<typename P::T> p1, float* __restrict__ rho_dt,
              float* __restrict__ vel_dt, int wall_rates, ParticleSetT<typename P::T> out,
              unsigned* __restrict__ out_hash, unsigned* err, unsigned* disp) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    float d2 = 0.f;
    if (c < (k.n + 1) / 2)
        d2 = pass2_pair<P, MODE>(k, c, in, keys, cs, nl, p1, rho_dt, vel_dt, wall_rates, out,
                                 out_hash, err);
    if (MODE == MODE_RATES || disp == nullptr) return;
    __shared__ unsigned s_max[NS_MAX_THREADS / 32];
    const unsigned wmax = __reduce_max_sync(0xffffffffu, __float_as_uint(d2));
    if ((threadIdx.x & 31) == 0) s_max[threadIdx.x >> 5] = wmax;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned m = s_max[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) m = max(m, s_max[w]);
        if (m) atomicMax(disp, m);
    }
}

// Pair mode applies to the FP32 and FP64 policies (mixed-precision slots carry each
// neighbour's cell relative to one particle, which a pair of particles in two cells cannot
// share); the launchers below dispatch on KParams::pairs.
template <class KP>
inline dim3 pair_grid(const KP& k) {
    const long pairs = ((long)k.n + 1) / 2;
    return dim3((unsigned)((pairs + k.threads - 1) / k.threads > 0 ? (pairs + k.threads - 1) / k.threads : 1));
}

// Launch shape of a neighbour kernel: KParams::threads per block, KParams::ppt particles per
// thread.
template <class KP>
inline dim3 ns_grid(const KP& k) {
    const long per_block = (long)k.threads * (k.ppt > 0 ? k.ppt : 1);
    const long b = ((long)k.n + per_block - 1) / per_block;
    return dim3((unsigned)(b > 0 ? b : 1));
}

template <class P, bool LIST, bool GS>
void pass1_launch_gs(const KParamsT<typename P::T>& k, const ParticleSetT<typename P::T>& in,
                     const unsigned* keys, const int* cs, const NbrList& nl,
                     const Pass1OutT<typename P::T>& o, float* rhop_sum, float* w_sum,
                     cudaStream_t s) {
    const dim3 b = ns_grid(k);
    if constexpr (P::kId == SPH_PREC_FP32) {
        if (rhop_sum && w_sum) {
            k_pass1<P, true, LIST, GS><<<b, k.threads, 0, s>>>(k, in, keys, cs, nl, o, rhop_sum,
                                                               w_sum);
            return;
        }
    }
    k_pass1<P, false, LIST, GS><<<b, k.threads, 0, s>>>(k, in, keys, cs, nl, o, nullptr,
                                                        nullptr);
}

template <class P, bool LIST>
void pass1_launch(const KParamsT<typename P::T>& k, const ParticleSetT<typename P::T>& in,
                  const unsigned* keys, const int* cs, const NbrList& nl,
                  const Pass1OutT<typename P::T>& o, float* rhop_sum, float* w_sum,
                  cudaStream_t s) {
    if constexpr (LIST && !P::kMixed) {
        if (k.pairs) {
            if (rhop_sum && w_sum && P::kId == SPH_PREC_FP32)
                k_pass1_pairs<P, true><<<pair_grid(k), k.threads, 0, s>>>(k, in, keys, cs, nl, o,
                                                                           rhop_sum, w_sum);
            else
                k_pass1_pairs<P, false><<<pair_grid(k), k.threads, 0, s>>>(k, in, keys, cs, nl,
                                                                            o, nullptr, nullptr);
            return;
        }
    }
    if (k.ppt > 1)
        pass1_launch_gs<P, LIST, true>(k, in, keys, cs, nl, o, rhop_sum, w_sum, s);
    else
        pass1_launch_gs<P, LIST, false>(k, in, keys, cs, nl, o, rhop_sum, w_sum, s);
}

template <class P, int MODE, bool GS>
void pass2_launch_gs(const KParamsT<typename P::T>& k, const ParticleSetT<typename P::T>& in,
                     const unsigned* keys, const int* cs, const NbrList* nl,
                     const Pass1OutT<typename P::T>& p1, float* rho_dt, float* vel_dt,
                     int wall_rates, ParticleSetT<typename P::T> out, unsigned* out_hash,
                     unsigned* err, unsigned* disp, cudaStream_t s) {
    const dim3 b = ns_grid(k);
    if constexpr (MODE != MODE_RATES && !GS && (P::kId == SPH_PREC_FP32 || P::kMixed)) {
        constexpr int cap = P::kId == SPH_PREC_FP32 ? 48 : 56;
        if (nl) {
            k_pass2_cap<P, MODE, true, GS, cap><<<b, k.threads, 0, s>>>(
                k, in, keys, cs, *nl, p1, rho_dt, vel_dt, wall_rates, out, out_hash, err, disp);
            return;
        }
    }
    if (nl)
        k_pass2<P, MODE, true, GS><<<b, k.threads, 0, s>>>(k, in, keys, cs, *nl, p1, rho_dt,
                                                            vel_dt, wall_rates, out, out_hash,
                                                            err, disp);
    else
        k_pass2<P, MODE, false, GS><<<b, k.threads, 0, s>>>(k, in, keys, cs, NbrList{}, p1,
                                                             rho_dt, vel_dt, wall_rates, out,
                                                             out_hash, err, nullptr);
}

template <class P, int MODE>
void pass2_launch(const KParamsT<typename P::T>& k, const ParticleSetT<typename P::T>& in,
                  const unsigned* keys, const int* cs, const NbrList* nl,
                  const Pass1OutT<typename P::T>& p1, float* rho_dt, float* vel_dt,
                  int wall_rates, ParticleSetT<typename P::T> out, unsigned* out_hash,
                  unsigned* err, unsigned* disp, cudaStream_t s) {
    if constexpr (!P::kMixed) {
        if (nl && k.pairs) {
            k_pass2_pairs<P, MODE><<<pair_grid(k), k.threads, 0, s>>>(
                k, in, keys, cs, *nl, p1, rho_dt, vel_dt, wall_rates, out, out_hash, err, disp);
            return;
        }
    }
    if (k.ppt > 1)
        pass2_launch_gs<P, MODE, true>(k, in, keys, cs, nl, p1, rho_dt, vel_dt, wall_rates, out,
                                       out_hash, err, disp, s);
    else
        pass2_launch_gs<P, MODE, false>(k, in, keys, cs, nl, p1, rho_dt, vel_dt, wall_rates,
                                        out, out_hash, err, disp, s);
}

}  // namespace

int nbr_capacity_for(const sph_params& p, double skin, bool pairs) {
    // 1.5x the particles of a lattice inside the list sphere (of the union of two spheres, about
    // 1.4 times one, for a pair), rounded up to 16
    const double r = (double)p.kh * (1.0 + skin) / (double)p.dx;
    const double lattice = 4.18879020478639 * r * r * r * (pairs ? 1.4 : 1.0);
    int cap = (int)(1.5 * lattice) + 16;
    cap = (cap + 15) & ~15;
    return cap < 32 ? 32 : cap;
}

template <class P>
cudaError_t launch_nbr_build(const KParamsT<typename P::T>& k,
                             const ParticleSetT<typename P::T>& in, const unsigned* keys,
                             const int* cs, const NbrList& nl, int walls_all, unsigned* err,
                             cudaStream_t s, const unsigned* gate) {
    if (k.n <= 0) return cudaSuccess;
    if constexpr (!P::kMixed) {
        if (k.pairs) {
            k_nbr_build_pairs<P><<<pair_grid(k), k.threads, 0, s>>>(k, in.xyz, keys, cs, nl,
                                                                     walls_all, err, gate);
            return cudaGetLastError();
        }
    }
    if (k.ppt > 1)
        k_nbr_build<P, true><<<ns_grid(k), k.threads, 0, s>>>(k, in.xyz, keys, cs, nl, walls_all,
                                                              err, gate);
    else
        k_nbr_build<P, false><<<ns_grid(k), k.threads, 0, s>>>(k, in.xyz, keys, cs, nl,
                                                               walls_all, err, gate);
    return cudaGetLastError();
}

template <class P>
cudaError_t launch_pass1(const KParamsT<typename P::T>& k, const ParticleSetT<typename P::T>& in,
                         const unsigned* keys, const int* cs, const NbrList* nl,
                         const Pass1OutT<typename P::T>& out, float* rhop_sum, float* w_sum,
                         cudaStream_t s) {
    if (k.n <= 0) return cudaSuccess;
    if (nl)
        pass1_launch<P, true>(k, in, keys, cs, *nl, out, rhop_sum, w_sum, s);
    else
        pass1_launch<P, false>(k, in, keys, cs, NbrList{}, out, rhop_sum, w_sum, s);
    return cudaGetLastError();
}

cudaError_t launch_pass2_rates(const KParams& k, const ParticleSet& in, const unsigned* keys,
                               const int* cs, const NbrList* nl, const Pass1Out& p1,
                               float* rho_dt, float* vel_dt, int wall_rates, cudaStream_t s) {
    if (k.n <= 0) return cudaSuccess;
    pass2_launch<PrecF32, MODE_RATES>(k, in, keys, cs, nl, p1, rho_dt, vel_dt, wall_rates,
                                      ParticleSet{}, nullptr, nullptr, nullptr, s);
    return cudaGetLastError();
}

template <class P>
cudaError_t launch_pass2_step(const KParamsT<typename P::T>& k, HalfStep half,
                              const ParticleSetT<typename P::T>& in, const unsigned* keys,
                              const int* cs, const NbrList* nl,
                              const Pass1OutT<typename P::T>& p1,
                              ParticleSetT<typename P::T> out, unsigned* out_hash, unsigned* err,
                              unsigned* disp, cudaStream_t s) {
    if (k.n <= 0) return cudaSuccess;
    if (half == HALF_PREDICT)
        pass2_launch<P, MODE_PRED>(k, in, keys, cs, nl, p1, nullptr, nullptr, 0, out, out_hash,
                                   err, disp, s);
    else
        pass2_launch<P, MODE_CORR>(k, in, keys, cs, nl, p1, nullptr, nullptr, 0, out, out_hash,
                                   err, disp, s);
    return cudaGetLastError();
}

#define SPH_NS_INSTANTIATE(P)                                                                  \
    template cudaError_t launch_nbr_build<P>(const KParamsT<P::T>&, const ParticleSetT<P::T>&, \
                                             const unsigned*, const int*, const NbrList&, int, \
                                             unsigned*, cudaStream_t, const unsigned*);        \
    template cudaError_t launch_pass1<P>(const KParamsT<P::T>&, const ParticleSetT<P::T>&,     \
                                         const unsigned*, const int*, const NbrList*,          \
                                         const Pass1OutT<P::T>&, float*, float*, cudaStream_t);\
    template cudaError_t launch_pass2_step<P>(                                                 \
        const KParamsT<P::T>&, HalfStep, const ParticleSetT<P::T>&, const unsigned*,           \
        const int*, const NbrList*, const Pass1OutT<P::T>&, ParticleSetT<P::T>, unsigned*,    \
        unsigned*, unsigned*, cudaStream_t);
SPH_NS_INSTANTIATE(PrecF32)
SPH_NS_INSTANTIATE(PrecF64)
SPH_NS_INSTANTIATE(PrecMix)
SPH_NS_INSTANTIATE(PrecMixC)
#undef SPH_NS_INSTANTIATE

}  // namespace sph
