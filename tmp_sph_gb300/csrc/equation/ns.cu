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
// Cells are walked as x-strips: with cells at least as wide as the list cutoff the 27 cells
// around a particle's cell are nine strips of three cells (x-1 .. x+1) of one (y, z) row,
// consecutive in the sorted order, so each strip is one contiguous slot range
// [cell_start[row + x-1], cell_start[row + x+2]) — the dense cell_start array gives empty cells
// the start of the next non-empty one.  With cells of a half or a third of the cutoff
// (KParams::reach 2 or 3) the walk covers 25 strips of five cells or 49 strips of seven.
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
// With a Verlet skin the list is built with the cutoff kh(1 + s) (NbrList::cut2, else
// kh2_list) on cells kh(1 + skin) wide, s <= skin, and kept while the displacements since the
// build stay within the bound the solver's rebuild test checks; both passes still test r < kh
// on the current positions, and k_nbr_build keeps the build positions (xb) that pass 2
// measures each particle's displacement against.
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

#include <type_traits>

#include "ns_pair.cuh"
#include "sph_internal.h"

namespace sph {

namespace {
// Appends slots to a list column.  Plain: four slots at a time (one 16-byte store per four),
// the group being filled staged in the thread's 16 bytes of shared memory — one store per slot
// at a computed address, where keeping it in registers took a select per register per slot,
// and the walk's divergent hit path runs for nearly every candidate a warp tests (build −6%).
// Interleaved: the window of eight staged the same way (the thread's eight slots NS_MAX_THREADS
// words apart, so a warp's stores hit 32 banks) and stored as two int4.  Shared memory of a
// block: SlotWriter<WIN>::kStage int4 per thread.
template <bool WIN>
struct SlotWriter;

template <>
struct SlotWriter<false> {
    static constexpr int kStage = 1;
    int* __restrict__ col;
    int cap;
    int* buf;  // the thread's four staging slots (shared memory, 16-byte aligned)
    int cnt = 0;
    __device__ __forceinline__ SlotWriter(int* c, int cp, int4* stage)
        : col(c), cap(cp), buf(reinterpret_cast<int*>(stage + threadIdx.x)) {}
    __device__ __forceinline__ void put(int v) {
        buf[cnt & 3] = v;
        cnt++;
        if ((cnt & 3) == 0 && cnt <= cap)
            *reinterpret_cast<int4*>(col + ((size_t)(cnt - 4) << 5)) =
                *reinterpret_cast<const int4*>(buf);
    }
    // the last, partial group (its unused slots are never read: count bounds the readers)
    __device__ __forceinline__ void flush() {
        if ((cnt & 3) && cnt < cap)
            *reinterpret_cast<int4*>(col + ((size_t)(cnt & ~3) << 5)) =
                *reinterpret_cast<const int4*>(buf);
    }
};

template <>
struct SlotWriter<true> {
    static constexpr int kStage = 2;
    int* __restrict__ col;
    int cap;
    int* buf;  // the thread's eight staging slots, buf[p * NS_MAX_THREADS] (shared memory)
    int cnt = 0;
    __device__ __forceinline__ SlotWriter(int* c, int cp, int4* stage)
        : col(c), cap(cp), buf(reinterpret_cast<int*>(stage) + threadIdx.x) {}
    // entry e of a window goes to chunk e mod 2, component e / 2
    __device__ __forceinline__ void put(int v) {
        const int e = cnt & 7;
        buf[(((e & 1) << 2) | (e >> 1)) * NS_MAX_THREADS] = v;
        cnt++;
        if ((cnt & 7) == 0 && cnt <= cap) store(cnt - 8, 2);
    }
    // the last, partial window: its chunks that hold entries (chunk a holds entry a first);
    // cap is a multiple of 16, so the window fits
    __device__ __forceinline__ void flush() {
        const int r = cnt & 7;
        if (r && cnt < cap) store(cnt & ~7, r > 1 ? 2 : 1);
    }
    __device__ __forceinline__ void store(int e0, int chunks) {
        for (int a = 0; a < chunks; a++) {
            const int* w = buf + 4 * a * NS_MAX_THREADS;
            *reinterpret_cast<int4*>(col + ((size_t)(e0 + 4 * a) << 5)) =
                make_int4(w[0], w[NS_MAX_THREADS], w[2 * NS_MAX_THREADS], w[3 * NS_MAX_THREADS]);
        }
    }
};

// List modes of the one-lane passes (template LIST): no list (cell walks), a list of plain
// windows, or one of interleaved windows (KParams::list_win).  The mode is a template
// parameter: a runtime choice between the two loops cost pass 2 1%.
enum { LIST_NONE = 0, LIST_PLAIN = 1, LIST_WIN = 2 };

// Neighbours of i (r2 < kh2) with their records R[2j], R[2j+1]: from the list (one record
// load per listed pair, the next slot loaded one pair ahead; pairs in the skin beyond the
// support radius are skipped), or by walking the cells over X[XSTRIDE * j] when i overflowed
// the list.  f(j, a, b, dx, dy, dz, r2).  (Skipping the gathers of slots in the skin with a
// pass-1 hit mask cost pass 2 more in instructions than it saved in sectors.)
template <class P, int LIST, int XSTRIDE, class F>
__device__ __forceinline__ void visit_records(const KParamsT<typename P::T>& k,
                                              const int* __restrict__ cs,
                                              const unsigned* __restrict__ keys,
                                              const NbrList& nl,
                                              const vec4_t<typename P::T>* __restrict__ X,
                                              const vec4_t<typename P::T>* __restrict__ R, int i,
                                              const vec4_t<typename P::T>& pi, F&& f) {
    using T = typename P::T;
    using V = vec4_t<T>;
    if constexpr (LIST != LIST_NONE) {
        const int cnt = __ldg(nl.count + i);
        if (cnt <= nl.cap) {
            auto one = [&](int e) {
                const int j = P::kCodes ? slot_index(e) : e;
                V a, b;
                ld_rec(R, j, a, b);
                T dx, dy, dz;
                rel_pos<P>(k, pi, a, P::kCodes ? slot_code(e) : 0u, dx, dy, dz);
                const T r2 = dist2(dx, dy, dz);
                if (r2 < k.kh2) f(j, a, b, dx, dy, dz, r2);
            };
            for_each_slot<LIST == LIST_WIN>(nl.idx + nbr_col(nl, i), cnt, 0, 1, one);
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

// Neighbour-list build: every boundary particle keeps its fluid neighbours (all that pass 1
// needs), every fluid particle all of them; with walls_all, boundary particles keep all.
// Slots are warp-interleaved (nbr_col): the passes read them coalesced, the build writes them
// scattered within its warp's block, which L2 merges before they reach HBM.
template <class P, bool WIN>
__device__ __forceinline__ void nbr_build_one(const KParamsT<typename P::T>& k,
                                              const vec4_t<typename P::T>* __restrict__ X,
                                              const unsigned* __restrict__ keys,
                                              const int* __restrict__ cs, const NbrList& nl,
                                              int walls_all, unsigned* err, int4* stage, int i) {
    using T = typename P::T;
    T cut2 = nl.cut2 ? (T)__ldg(nl.cut2) : k.kh2_list;
    if (nl.iw) {
        // per-instance decisions: the particles of the instances that rebuild, each at its
        // instance's list cutoff; the others keep their lists
        const unsigned* w = nl.iw + IW_STRIDE * (__ldg(nl.inst + i) + 1);
        if (!w[IW_REBUILD]) return;
        cut2 = (T)__uint_as_float(w[IW_CUT2]);
    }
    const vec4_t<T> pi = X[i];
    if (nl.xb) nl.xb[i] = as_float4(pi);
    const bool keep_all = fluid_rec(pi.w) || walls_all;
    if (!keep_all && nl.fluid_cells && !inactive_key(k, keys[i])) {
        // a boundary particle with no fluid in the cells it walks has an empty list
        int cx, cy, cz;
        cell_of_key(k.gx, k.gy, keys[i], cx, cy, cz);
        bool any = false;
        const int r = k.reach;
        for (int z = max(cz - r, 0); z <= min(cz + r, k.gz - 1); z++)
            for (int y = max(cy - r, 0); y <= min(cy + r, k.gy - 1); y++) {
                const int row = (z * k.gy + y) * k.gx;
                for (int x = max(cx - r, 0); x <= min(cx + r, k.gx - 1); x++)
                    any = any || __ldg(nl.fluid_cells + row + x) != 0;
            }
        if (!any) {
            nl.count[i] = 0;
            return;
        }
    }
    SlotWriter<WIN> w(nl.idx + nbr_col(nl, i), nl.cap, stage);
    if constexpr (P::kCodes) {
        // i's offsets moved into each run's anchor frame once per run instead of decoding the
        // code for every candidate.  That rounds differently from the passes' decode, so the
        // cutoff is widened by 2^-16: every pair the passes would put inside it is listed, and
        // the passes test r < kh with their own decode, so they still evaluate exactly the
        // pairs of a cell walk.
        const unsigned key = keys[i];
        if (!inactive_key(k, key)) {
            int cx, cy, cz;
            cell_of_key(k.gx, k.gy, key, cx, cy, cz);
            const T cut2w = cut2 * (T(1) + T(1.0 / 65536.0));
            const StripWindow win = strip_window<P>(k, pi, cx, cy, cz, cut2w);
            for_each_run<true>(k, cs, cx, cy, cz, [&](int j0, int j1, unsigned code) {
                float fx, fy, fz;
                code_steps(code, fx, fy, fz);
                const float sx = fma_rn(-fx, k.reach_cell, pi.x);
                const float sy = fma_rn(-fy, k.reach_cell, pi.y);
                const float sz = fma_rn(-fz, k.reach_cell, pi.z);
#pragma unroll 4
                for (int j = j0; j < j1; j++) {
                    const vec4_t<T> pj = ld_pos(X, (size_t)j);
                    const T r2 = dist2(sub_rn(sx, pj.x), sub_rn(sy, pj.y), sub_rn(sz, pj.z));
                    if (r2 < cut2w && j != i && (keep_all || fluid_rec(pj.w)))
                        w.put(make_slot(j, code));
                }
            }, win);
        }
    } else {
        // the cell walk of walk_pairs, narrowed to the cells the cutoff sphere reaches (the
        // same slots pass the distance test, in the same order)
        const unsigned key = keys[i];
        if (!inactive_key(k, key)) {
            int cx, cy, cz;
            cell_of_key(k.gx, k.gy, key, cx, cy, cz);
            const StripWindow win = strip_window<P>(k, pi, cx, cy, cz, cut2);
            for_each_run<false>(k, cs, cx, cy, cz, [&](int j0, int j1, unsigned) {
#pragma unroll 4
                for (int j = j0; j < j1; j++) {
                    const vec4_t<T> pj = ld_pos(X, (size_t)j);
                    T dx, dy, dz;
                    rel_pos<P>(k, pi, pj, 0u, dx, dy, dz);
                    const T r2 = dist2(dx, dy, dz);
                    if (r2 < cut2 && j != i && (keep_all || fluid_rec(pj.w))) w.put(j);
                }
            }, win);
        }
    }
    w.flush();
    nl.count[i] = w.cnt;
    raise_flags(err, w.cnt > nl.cap ? SPH_FLAG_NEIGHBOR_OVERFLOW : 0u);
}

template <class P, bool GS, bool WIN>
__global__ void __launch_bounds__(NS_MAX_THREADS)
k_nbr_build(KParamsT<typename P::T> k, const vec4_t<typename P::T>* __restrict__ X,
            const unsigned* __restrict__ keys, const int* __restrict__ cs, NbrList nl,
            int walls_all, unsigned* err, const unsigned* gate) {
    __shared__ int4 s_stage[SlotWriter<WIN>::kStage * NS_MAX_THREADS];
    if (gated_off(gate)) return;
    int4* stage = s_stage;
    const int i0 = blockIdx.x * blockDim.x + threadIdx.x;
    if constexpr (GS) {
        for (int i = i0; i < k.n; i += gridDim.x * blockDim.x)
            nbr_build_one<P, WIN>(k, X, keys, cs, nl, walls_all, err, stage, i);
    } else if (i0 < k.n) {
        nbr_build_one<P, WIN>(k, X, keys, cs, nl, walls_all, err, stage, i0);
    }
}

template <class P, bool WRITE_SUMS, int LIST>
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

template <class P, bool WRITE_SUMS, int LIST, bool GS>
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
template <class P, int MODE, int LIST>
__device__ __forceinline__ void pass2_one(const KParamsT<typename P::T>& k, int i,
                                          const ParticleSetT<typename P::T>& in,
                                          const unsigned* __restrict__ keys,
                                          const int* __restrict__ cs, const NbrList& nl,
                                          const Pass1OutT<typename P::T>& p1,
                                          float* __restrict__ rho_dt, float* __restrict__ vel_dt,
                                          int wall_rates, const ParticleSetT<typename P::T>& out,
                                          unsigned* __restrict__ out_hash, unsigned* err,
                                          DispBox& box, unsigned* disp) {
    using T = typename P::T;
    using V = vec4_t<T>;
    Pass2Acc<P, MODE> acc;
    acc.load(k, p1, i, wall_rates);
    if (acc.active)
        visit_records<P, LIST, 2>(k, cs, keys, nl, p1.nrec, p1.nrec, i, acc.pi,
                                  [&](int j, const V& aj, const V& vj, T dx, T dy, T dz, T r2) {
            acc.pair(k, p1, j, aj, vj, dx, dy, dz, r2);
        });
    pass2_finish<P, MODE>(k, i, acc, in, keys, nl, rho_dt, vel_dt, wall_rates, out, out_hash,
                          err, box, disp);
}


template <class P, int MODE, int LIST, bool GS>
__global__ void __launch_bounds__(NS_MAX_THREADS)
k_pass2(KParamsT<typename P::T> k, ParticleSetT<typename P::T> in,
        const unsigned* __restrict__ keys, const int* __restrict__ cs, NbrList nl,
        Pass1OutT<typename P::T> p1, float* __restrict__ rho_dt, float* __restrict__ vel_dt,
        int wall_rates, ParticleSetT<typename P::T> out, unsigned* __restrict__ out_hash,
        unsigned* err, unsigned* disp) {
    DispBox box;
    const int i0 = blockIdx.x * blockDim.x + threadIdx.x;
    if constexpr (GS) {
        for (int i = i0; i < k.n; i += gridDim.x * blockDim.x)
            pass2_one<P, MODE, LIST>(k, i, in, keys, cs, nl, p1, rho_dt, vel_dt, wall_rates, out,
                                     out_hash, err, box, disp);
    } else if (i0 < k.n) {
        pass2_one<P, MODE, LIST>(k, i0, in, keys, cs, nl, p1, rho_dt, vel_dt, wall_rates, out,
                                 out_hash, err, box, disp);
    }
    if (MODE == MODE_RATES || disp == nullptr) return;
    // the block's displacement box; blockDim is a multiple of 32, every thread gets here
    __shared__ unsigned s_box[6 * (NS_MAX_THREADS / 32)];
    __shared__ int s_inst[NS_MAX_THREADS / 32];
    reduce_disp(k, box, disp, s_box, s_inst);
}

// The same kernel held to CAP registers (one particle per thread).  The FP32 step kernel (and
// the one of mixed precision on FP32 positions) runs in 40: six 256-thread blocks per SM
// instead of the five of its spill-free 48, for 40 bytes of spill
// (0.610 against 0.634 ms at 4.96M particles; before the pair approximations were taken in
// their flush-to-zero forms, with more instructions per pair to hide the gathers, the two
// measured the same).  The mixed-precision kernel on cell-local offsets runs in 56 (nine
// 128-thread blocks instead of eight).
template <class P, int MODE, int LIST, bool GS, int CAP>
__global__ void __maxnreg__(CAP)
k_pass2_cap(KParamsT<typename P::T> k, ParticleSetT<typename P::T> in,
        const unsigned* __restrict__ keys, const int* __restrict__ cs, NbrList nl,
        Pass1OutT<typename P::T> p1, float* __restrict__ rho_dt, float* __restrict__ vel_dt,
        int wall_rates, ParticleSetT<typename P::T> out, unsigned* __restrict__ out_hash,
        unsigned* err, unsigned* disp) {
    DispBox box;
    const int i0 = blockIdx.x * blockDim.x + threadIdx.x;
    if constexpr (GS) {
        for (int i = i0; i < k.n; i += gridDim.x * blockDim.x)
            pass2_one<P, MODE, LIST>(k, i, in, keys, cs, nl, p1, rho_dt, vel_dt, wall_rates, out,
                                     out_hash, err, box, disp);
    } else if (i0 < k.n) {
        pass2_one<P, MODE, LIST>(k, i0, in, keys, cs, nl, p1, rho_dt, vel_dt, wall_rates, out,
                                 out_hash, err, box, disp);
    }
    if (MODE == MODE_RATES || disp == nullptr) return;
    // the block's displacement box; blockDim is a multiple of 32, every thread gets here
    __shared__ unsigned s_box[6 * (NS_MAX_THREADS / 32)];
    __shared__ int s_inst[NS_MAX_THREADS / 32];
    reduce_disp(k, box, disp, s_box, s_inst);
}

// Launch shape of a neighbour kernel: KParams::threads per block, KParams::ppt particles per
// thread.
template <class KP>
inline dim3 ns_grid(const KP& k) {
    const long per_block = (long)k.threads * (k.ppt > 0 ? k.ppt : 1);
    const long b = ((long)k.n + per_block - 1) / per_block;
    return dim3((unsigned)(b > 0 ? b : 1));
}

template <class P, int LIST, bool GS>
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

template <class P, int LIST>
void pass1_launch(const KParamsT<typename P::T>& k, const ParticleSetT<typename P::T>& in,
                  const unsigned* keys, const int* cs, const NbrList& nl,
                  const Pass1OutT<typename P::T>& o, float* rhop_sum, float* w_sum,
                  cudaStream_t s) {
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
    if (!nl) {
        k_pass2<P, MODE, LIST_NONE, GS><<<b, k.threads, 0, s>>>(k, in, keys, cs, NbrList{}, p1,
                                                                 rho_dt, vel_dt, wall_rates, out,
                                                                 out_hash, err, nullptr);
        return;
    }
    auto with_list = [&](auto mode) {
        constexpr int L = decltype(mode)::value;
        if constexpr (MODE != MODE_RATES && !GS && (P::kId == SPH_PREC_FP32 || P::kMixed)) {
            constexpr int cap = P::kCodes ? 56 : 40;
            k_pass2_cap<P, MODE, L, GS, cap><<<b, k.threads, 0, s>>>(
                k, in, keys, cs, *nl, p1, rho_dt, vel_dt, wall_rates, out, out_hash, err, disp);
        } else {
            k_pass2<P, MODE, L, GS><<<b, k.threads, 0, s>>>(k, in, keys, cs, *nl, p1, rho_dt,
                                                             vel_dt, wall_rates, out, out_hash,
                                                             err, disp);
        }
    };
    // the rates (sph_ns) run on the drop-in's own list, which has plain windows
    if constexpr (MODE != MODE_RATES) {
        if (k.list_win) {
            with_list(std::integral_constant<int, LIST_WIN>{});
            return;
        }
    }
    with_list(std::integral_constant<int, LIST_PLAIN>{});
}

template <class P, int MODE>
void pass2_launch(const KParamsT<typename P::T>& k, const ParticleSetT<typename P::T>& in,
                  const unsigned* keys, const int* cs, const NbrList* nl,
                  const Pass1OutT<typename P::T>& p1, float* rho_dt, float* vel_dt,
                  int wall_rates, ParticleSetT<typename P::T> out, unsigned* out_hash,
                  unsigned* err, unsigned* disp, cudaStream_t s) {
    if (k.ppt > 1)
        pass2_launch_gs<P, MODE, true>(k, in, keys, cs, nl, p1, rho_dt, vel_dt, wall_rates, out,
                                       out_hash, err, disp, s);
    else
        pass2_launch_gs<P, MODE, false>(k, in, keys, cs, nl, p1, rho_dt, vel_dt, wall_rates,
                                        out, out_hash, err, disp, s);
}

}  // namespace

int nbr_capacity_for(const sph_params& p, double skin) {
    // 1.5x the particles of a lattice inside the list sphere, rounded up to 16
    const double r = (double)p.kh * (1.0 + skin) / (double)p.dx;
    const double lattice = 4.18879020478639 * r * r * r;
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
    const dim3 g = ns_grid(k);
    if (k.ppt > 1) {
        if (k.list_win)
            k_nbr_build<P, true, true><<<g, k.threads, 0, s>>>(k, in.xyz, keys, cs, nl,
                                                                walls_all, err, gate);
        else
            k_nbr_build<P, true, false><<<g, k.threads, 0, s>>>(k, in.xyz, keys, cs, nl,
                                                                 walls_all, err, gate);
    } else {
        if (k.list_win)
            k_nbr_build<P, false, true><<<g, k.threads, 0, s>>>(k, in.xyz, keys, cs, nl,
                                                                 walls_all, err, gate);
        else
            k_nbr_build<P, false, false><<<g, k.threads, 0, s>>>(k, in.xyz, keys, cs, nl,
                                                                  walls_all, err, gate);
    }
    return cudaGetLastError();
}

template <class P>
cudaError_t launch_pass1(const KParamsT<typename P::T>& k, const ParticleSetT<typename P::T>& in,
                         const unsigned* keys, const int* cs, const NbrList* nl,
                         const Pass1OutT<typename P::T>& out, float* rhop_sum, float* w_sum,
                         cudaStream_t s) {
    if (k.n <= 0) return cudaSuccess;
    if (nl && k.lanes > 1 && !rhop_sum && !w_sum)
        return launch_pass1_groups<P>(k, in, keys, cs, *nl, out, s);
    if (nl && k.list_win)
        pass1_launch<P, LIST_WIN>(k, in, keys, cs, *nl, out, rhop_sum, w_sum, s);
    else if (nl)
        pass1_launch<P, LIST_PLAIN>(k, in, keys, cs, *nl, out, rhop_sum, w_sum, s);
    else
        pass1_launch<P, LIST_NONE>(k, in, keys, cs, NbrList{}, out, rhop_sum, w_sum, s);
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
SPH_NS_INSTANTIATE(PrecMixA)
#undef SPH_NS_INSTANTIATE

}  // namespace sph
