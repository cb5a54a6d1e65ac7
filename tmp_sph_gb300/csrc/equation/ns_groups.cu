// ns_groups.cu — the neighbour kernels with a group of G lanes per particle (G = 2, 4, 8, 16).
//
// Same passes as ns.cu (reference: computeBoundary_Delta_acoustic_D and
// computeGovering_equationD, src/equation/ns.cu:30-249), same list contents, different
// assignment of work to lanes.  With one thread per particle every lane of a warp gathers a
// different neighbour record, and a warp-level gather touches about twenty distinct 128-byte
// lines: the passes are limited by L1 data-stage wavefronts.  With G lanes per particle, lane s
// of particle i handles its list entries s, s + G, s + 2G, ...: the G records a group gathers
// in one step are consecutive entries of one list — runs of nearby slots of a few cell strips —
// and the 32/G particles of a warp are neighbours in the sorted order with largely the same
// lists.  A model of the 765,828-particle case on the host counts 0.70 distinct lines per
// gathered pair with one lane per particle and 0.34 with eight.
//
// Sums.  Each lane accumulates its share of the pairs; a group reduces them with xor shuffles
// in a fixed tree, so results are deterministic and independent of the launch shape, but not
// bit-equal to one lane per particle (the sums associate differently).
//
// List layout.  The 32/G particles a warp handles together share a block of cap * 32/G slots
// in which each lane's entries come four to an int4 (gslot): a warp reads four entries of
// every lane with one 16-byte load per lane.  The build walks the cells with the whole group, G candidates per step,
// and compacts the hits with a ballot, so the list holds the same entries in the same (walk)
// order as the one-lane build.
//
// Blocks.  A block of T threads owns T consecutive particles and visits them in G rounds of T/G
// particles (one group each), parking the reduced sums in shared memory; then every thread
// finishes one particle (pass 1: the record pass 2 gathers; pass 2: the predictor or
// corrector, the next key and the displacement), so the per-particle epilogue runs on all
// lanes rather than on one lane per group.
#include <cuda_runtime.h>

#include "ns_pair.cuh"
#include "sph_internal.h"

namespace sph {

namespace {

constexpr unsigned FULL_MASK = 0xffffffffu;

template <int G>
__device__ __forceinline__ int sub_lane() {
    return (int)(threadIdx.x & (unsigned)(G - 1));
}

// This group's bits of a warp ballot, in sub-lane order.
template <int G>
__device__ __forceinline__ unsigned group_bits(unsigned ballot) {
    if constexpr (G == 32) {
        return ballot;
    } else {
        return (ballot >> ((threadIdx.x & 31u) & ~(unsigned)(G - 1))) & ((1u << G) - 1u);
    }
}

// Entry c of particle i in the group layout.  The 32/G particles a warp handles together
// share a block of cap * 32/G slots; lane L = (i mod 32/G) G + c mod G of the warp holds
// entries c = s, s + G, s + 2G, ... of its particle, and its entries 4m .. 4m+3 (in that
// order) are one int4 at block + 128 m + 4 L: a warp reads four entries of every lane with
// one 16-byte load per lane, as the one-lane layout does.
template <int G>
__device__ __forceinline__ size_t gslot(const NbrList& nl, int i, int c) {
    constexpr unsigned PPW = 32 / G;
    const unsigned ui = (unsigned)i, uc = (unsigned)c;
    const unsigned lane = (ui % PPW) * G + uc % G, t = uc / G;
    return (size_t)(ui / PPW) * ((size_t)nl.cap * PPW) + (size_t)(t >> 2) * 128u +
           (size_t)(lane * 4u + (t & 3u));
}

// Four list slots, read past L1 (the slots stream through once per pass).
__device__ __forceinline__ int4 ld_slots4(const int* p) {
    int4 v;
    asm("ld.global.nc.L1::no_allocate.v4.s32 {%0, %1, %2, %3}, [%4];"
        : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
        : "l"(p));
    return v;
}

// Sum a Sum<> over the G lanes of the group (all lanes of the warp take part).
template <int G, class T, bool COMP>
__device__ __forceinline__ void reduce_group(Sum<T, COMP>& a) {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) {
        if constexpr (COMP) {
            const T os = __shfl_xor_sync(FULL_MASK, a.s, o);
            const T oc = __shfl_xor_sync(FULL_MASK, a.c, o);
            a.add(os);
            a.c = add_rn(a.c, oc);
        } else {
            a.s += __shfl_xor_sync(FULL_MASK, a.s, o);
        }
    }
}

template <class T, bool COMP>
__device__ __forceinline__ Sum<T, COMP> sum_of(T v) {
    Sum<T, COMP> s;
    s.s = v;
    return s;
}

// The nine x-strips of particle i's cells: strip t is rows (dz, dy) = (t/3 - 1, t%3 - 1), slots
// [j0, j1); with cell codes, b1 and b2 are the first slots of its second and third cells.
struct Strip {
    int j0 = 0, j1 = 0, xl = 0, b1 = 0, b2 = 0;
};

template <bool CODES, class KP>
__device__ __forceinline__ Strip strip_of(const KP& k, const int* __restrict__ cs, int cx,
                                          int cy, int cz, int t) {
    Strip st;
    const int z = cz + t / 3 - 1, y = cy + t % 3 - 1;
    if ((unsigned)z >= (unsigned)k.gz || (unsigned)y >= (unsigned)k.gy) return st;
    const int row = (z * k.gy + y) * k.gx;
    st.xl = cx > 0 ? cx - 1 : 0;
    const int xh = cx < k.gx - 1 ? cx + 1 : k.gx - 1;
    st.j0 = max(__ldg(cs + row + st.xl), 0);
    st.j1 = min(__ldg(cs + row + xh + 1), k.n);  // bounds guard only
    if constexpr (CODES) {
        st.b1 = st.xl + 1 <= xh ? __ldg(cs + row + st.xl + 1) : st.j1;
        st.b2 = st.xl + 2 <= xh ? __ldg(cs + row + st.xl + 2) : st.j1;
    }
    return st;
}

// Cell code of slot j of strip t (its cell relative to (cx, ., .)), as the one-lane walk
// stores it.
__device__ __forceinline__ unsigned strip_code(const Strip& st, int t, int cx, int j) {
    const int xc = st.xl + (j >= st.b1) + (j >= st.b2);
    return (unsigned)(((t / 3) << 4) | ((t % 3) << 2) | (xc - cx + 1));
}

// ---------------------------------------------------------------- list build
template <class P, int G>
__device__ __forceinline__ void build_group(const KParamsT<typename P::T>& k,
                                            const vec4_t<typename P::T>* __restrict__ X,
                                            const unsigned* __restrict__ keys,
                                            const int* __restrict__ cs, const NbrList& nl,
                                            int walls_all, unsigned* err, int i) {
    using T = typename P::T;
    using V = vec4_t<T>;
    const int s = sub_lane<G>();
    const bool valid = i < k.n;
    const V pi = valid ? X[i] : make4<T>(T(0), T(0), T(0), T(0));
    const unsigned key = valid ? keys[i] : (unsigned)k.num_cells;
    // particles outside the neighbour search (park_inactive) take no candidates
    const bool live = valid && !inactive_key(k, key);
    if (valid && s == 0 && nl.xb) nl.xb[i] = as_float4(pi);
    const bool keep_all = fluid_rec(pi.w) || walls_all;
    int cx = 0, cy = 0, cz = 0;
    if (live) cell_of_key(k.gx, k.gy, key, cx, cy, cz);
    const T cut2 = nl.cut2 ? (T)__ldg(nl.cut2) : k.kh2_list;
    int cnt = 0;
#pragma unroll 1
    for (int t = 0; t < 9; t++) {
        const Strip st = live ? strip_of<P::kMixed>(k, cs, cx, cy, cz, t) : Strip{};
        // every lane of the warp runs the loop while any group has candidates left
#pragma unroll 1
        for (int jb = st.j0; __any_sync(FULL_MASK, jb < st.j1); jb += G) {
            const int j = jb + s;
            bool hit = false;
            unsigned code = 0;
            if (j < st.j1) {
                const V pj = ld_pos(X, (size_t)j);
                if constexpr (P::kMixed) code = strip_code(st, t, cx, j);
                T dx, dy, dz;
                rel_pos<P>(k, pi, pj, code, dx, dy, dz);
                hit = dist2(dx, dy, dz) < cut2 && j != i && (keep_all || fluid_rec(pj.w));
            }
            const unsigned m = group_bits<G>(__ballot_sync(FULL_MASK, hit));
            if (hit) {
                const int c = cnt + __popc(m & ((1u << s) - 1u));
                if (c < nl.cap)
                    nl.idx[gslot<G>(nl, i, c)] =
                        P::kMixed ? (int)((unsigned)j | (code << CODE_SHIFT)) : j;
            }
            cnt += __popc(m);
        }
    }
    if (valid && s == 0) {
        nl.count[i] = cnt;
        raise_flags(err, cnt > nl.cap ? SPH_FLAG_NEIGHBOR_OVERFLOW : 0u);
    }
}

// A block of T threads builds the lists of T particles in G rounds of T/G groups.
template <class P, int G>
__global__ void __launch_bounds__(NS_MAX_THREADS)
k_nbr_build_g(KParamsT<typename P::T> k, const vec4_t<typename P::T>* __restrict__ X,
              const unsigned* __restrict__ keys, const int* __restrict__ cs, NbrList nl,
              int walls_all, unsigned* err, const unsigned* gate) {
    if (gated_off(gate)) return;
    const int nt = (int)blockDim.x, base = (int)blockIdx.x * nt;
#pragma unroll 1
    for (int r = 0; r < G; r++)
        build_group<P, G>(k, X, keys, cs, nl, walls_all, err,
                          base + r * (nt / G) + (int)threadIdx.x / G);
}

// ---------------------------------------------------------------- neighbour visits
// The group's share of particle i's neighbours (r2 < kh2) with their records: from the list,
// lane s taking entries s, s + G, ... two at a time; or, when i overflowed the list, by walking
// the cells over X[XSTRIDE * j], G candidates per step.  f(j, a, b, dx, dy, dz, r2).
template <class P, int G, int XSTRIDE, class F>
__device__ __forceinline__ void visit_group(const KParamsT<typename P::T>& k,
                                            const int* __restrict__ cs,
                                            const unsigned* __restrict__ keys,
                                            const NbrList& nl,
                                            const vec4_t<typename P::T>* __restrict__ X,
                                            const vec4_t<typename P::T>* __restrict__ R, int i,
                                            const vec4_t<typename P::T>& pi, F&& f) {
    using T = typename P::T;
    using V = vec4_t<T>;
    const int s = sub_lane<G>();
    const int cnt = __ldg(nl.count + i);
    if (cnt <= nl.cap) {
        auto one = [&](int e) {
            const int j = P::kMixed ? (int)((unsigned)e & IDX_MASK) : e;
            V a, b;
            ld_rec(R, j, a, b);
            T dx, dy, dz;
            rel_pos<P>(k, pi, a, (unsigned)e >> CODE_SHIFT, dx, dy, dz);
            const T r2 = dist2(dx, dy, dz);
            if (r2 < k.kh2) f(j, a, b, dx, dy, dz, r2);
        };
        // this lane's entries s, s + G, ...: n of them, four per int4, the next int4 loaded
        // one group ahead (four record gathers in flight per lane)
        const int n = cnt > s ? (cnt - s + G - 1) / G : 0;
        const int* __restrict__ col = nl.idx + gslot<G>(nl, i, s);
        int4 q = n > 0 ? ld_slots4(col) : make_int4(0, 0, 0, 0);
#pragma unroll 1
        for (int t = 0; t < n; t += 4) {
            const int4 qn = t + 4 < n ? ld_slots4(col + ((size_t)(t + 4) << 5)) : q;
            one(q.x);
            if (t + 1 < n) one(q.y);
            if (t + 2 < n) one(q.z);
            if (t + 3 < n) one(q.w);
            q = qn;
        }
        return;
    }
    const unsigned key = keys[i];
    if (inactive_key(k, key)) return;
    int cx, cy, cz;
    cell_of_key(k.gx, k.gy, key, cx, cy, cz);
#pragma unroll 1
    for (int t = 0; t < 9; t++) {
        const Strip st = strip_of<P::kMixed>(k, cs, cx, cy, cz, t);
#pragma unroll 1
        for (int j = st.j0 + s; j < st.j1; j += G) {
            const V pj = ld_pos(X, (size_t)XSTRIDE * (size_t)j);
            const unsigned code = P::kMixed ? strip_code(st, t, cx, j) : 0u;
            T dx, dy, dz;
            rel_pos<P>(k, pi, pj, code, dx, dy, dz);
            const T r2 = dist2(dx, dy, dz);
            if (r2 < k.kh2 && j != i) {
                V a, b;
                ld_rec(R, j, a, b);
                f(j, a, b, dx, dy, dz, r2);
            }
        }
    }
}

// ---------------------------------------------------------------- pass 1
template <class P, int G>
__global__ void __launch_bounds__(NS_MAX_THREADS)
k_pass1_g(KParamsT<typename P::T> k, ParticleSetT<typename P::T> in,
          const unsigned* __restrict__ keys, const int* __restrict__ cs, NbrList nl,
          Pass1OutT<typename P::T> out) {
    using T = typename P::T;
    using V = vec4_t<T>;
    __shared__ T s_sum[3][NS_MAX_THREADS];
    const int nt = (int)blockDim.x, base = (int)blockIdx.x * nt, s = sub_lane<G>();
#pragma unroll 1
    for (int r = 0; r < G; r++) {
        const int loc = r * (nt / G) + (int)threadIdx.x / G;
        const int i = base + loc;
        Pass1Acc<P> acc;
        if (i < k.n) {
            acc.load(in.rec, i);
            visit_group<P, G, 1>(k, cs, keys, nl, in.xyz, in.rec, i, acc.pi,
                                 [&](int, const V& aj, const V& vj, T dx, T dy, T dz, T r2) {
                acc.pair(k, aj, vj, dx, dy, dz, r2);
            });
        }
        reduce_group<G>(acc.dofv);
        reduce_group<G>(acc.rs);
        reduce_group<G>(acc.ws);
        if (s == 0) {
            s_sum[0][loc] = acc.dofv.get();
            s_sum[1][loc] = acc.rs.get();
            s_sum[2][loc] = acc.ws.get();
        }
    }
    __syncthreads();
    const int i = base + (int)threadIdx.x;
    if (i < k.n) {
        Pass1Acc<P> acc;
        acc.load(in.rec, i);
        acc.dofv = sum_of<T, P::kComp>(s_sum[0][threadIdx.x]);
        acc.rs = sum_of<T, P::kComp>(s_sum[1][threadIdx.x]);
        acc.ws = sum_of<T, P::kComp>(s_sum[2][threadIdx.x]);
        acc.template finish<false>(k, out, nullptr, nullptr, i);
    }
}

// ---------------------------------------------------------------- pass 2 (predictor / corrector)
template <class P, int MODE, int G>
__global__ void __launch_bounds__(NS_MAX_THREADS)
k_pass2_g(KParamsT<typename P::T> k, ParticleSetT<typename P::T> in,
          const unsigned* __restrict__ keys, const int* __restrict__ cs, NbrList nl,
          Pass1OutT<typename P::T> p1, ParticleSetT<typename P::T> out,
          unsigned* __restrict__ out_hash, unsigned* err, unsigned* disp) {
    using T = typename P::T;
    using V = vec4_t<T>;
    __shared__ T s_sum[4][NS_MAX_THREADS];
    __shared__ unsigned s_box[6 * (NS_MAX_THREADS / 32)];
    const int nt = (int)blockDim.x, base = (int)blockIdx.x * nt, s = sub_lane<G>();
#pragma unroll 1
    for (int r = 0; r < G; r++) {
        const int loc = r * (nt / G) + (int)threadIdx.x / G;
        const int i = base + loc;
        Pass2Acc<P, MODE> acc;
        if (i < k.n) {
            acc.load(k, p1, i, 0);
            if (acc.active)
                visit_group<P, G, 2>(k, cs, keys, nl, p1.nrec, p1.nrec, i, acc.pi,
                                     [&](int j, const V& aj, const V& vj, T dx, T dy, T dz,
                                         T r2) { acc.pair(k, p1, j, aj, vj, dx, dy, dz, r2); });
        }
        reduce_group<G>(acc.sd);
        reduce_group<G>(acc.sx);
        reduce_group<G>(acc.sy);
        reduce_group<G>(acc.sz);
        if (s == 0) {
            s_sum[0][loc] = acc.sd.get();
            s_sum[1][loc] = acc.sx.get();
            s_sum[2][loc] = acc.sy.get();
            s_sum[3][loc] = acc.sz.get();
        }
    }
    __syncthreads();
    const int i = base + (int)threadIdx.x;
    DispBox box;
    if (i < k.n) {
        Pass2Acc<P, MODE> acc;
        acc.load(k, p1, i, 0);
        acc.sd = sum_of<T, P::kComp>(s_sum[0][threadIdx.x]);
        acc.sx = sum_of<T, P::kComp>(s_sum[1][threadIdx.x]);
        acc.sy = sum_of<T, P::kComp>(s_sum[2][threadIdx.x]);
        acc.sz = sum_of<T, P::kComp>(s_sum[3][threadIdx.x]);
        pass2_finish<P, MODE>(k, i, acc, in, keys, nl, nullptr, nullptr, 0, out, out_hash, err,
                              box);
    }
    // the block's displacement box; blockDim is a multiple of 32, every thread gets here
    reduce_disp_box(box, disp, s_box);
}

inline int group_blocks(int n, int threads) { return (n + threads - 1) / threads; }

template <int G>
struct Lanes {
    static constexpr int value = G;
};

// Calls f(Lanes<G>{}) for the group size `lanes`.
template <class F>
cudaError_t with_group(int lanes, F&& f) {
    switch (lanes) {
        case 2: return f(Lanes<2>{});
        case 4: return f(Lanes<4>{});
        case 8: return f(Lanes<8>{});
        case 16: return f(Lanes<16>{});
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace

template <class P>
cudaError_t launch_nbr_build_groups(const KParamsT<typename P::T>& k,
                                    const ParticleSetT<typename P::T>& in, const unsigned* keys,
                                    const int* cs, const NbrList& nl, int walls_all,
                                    unsigned* err, cudaStream_t s, const unsigned* gate) {
    if (k.n <= 0) return cudaSuccess;
    // the layout needs whole steps of G entries and whole warps per block
    if (nl.cap % (4 * k.lanes) != 0 || k.threads % 32 != 0) return cudaErrorInvalidValue;
    return with_group(k.lanes, [&](auto tag) {
        constexpr int G = decltype(tag)::value;
        k_nbr_build_g<P, G><<<group_blocks(k.n, k.threads), k.threads, 0, s>>>(
            k, in.xyz, keys, cs, nl, walls_all, err, gate);
        return cudaGetLastError();
    });
}

template <class P>
cudaError_t launch_pass1_groups(const KParamsT<typename P::T>& k,
                                const ParticleSetT<typename P::T>& in, const unsigned* keys,
                                const int* cs, const NbrList& nl,
                                const Pass1OutT<typename P::T>& out, cudaStream_t s) {
    if (k.n <= 0) return cudaSuccess;
    // the layout needs whole steps of G entries and whole warps per block
    if (nl.cap % (4 * k.lanes) != 0 || k.threads % 32 != 0) return cudaErrorInvalidValue;
    return with_group(k.lanes, [&](auto tag) {
        constexpr int G = decltype(tag)::value;
        k_pass1_g<P, G><<<group_blocks(k.n, k.threads), k.threads, 0, s>>>(k, in, keys, cs, nl,
                                                                         out);
        return cudaGetLastError();
    });
}

template <class P>
cudaError_t launch_pass2_groups(const KParamsT<typename P::T>& k, HalfStep half,
                                const ParticleSetT<typename P::T>& in, const unsigned* keys,
                                const int* cs, const NbrList& nl,
                                const Pass1OutT<typename P::T>& p1,
                                ParticleSetT<typename P::T> out, unsigned* out_hash,
                                unsigned* err, unsigned* disp, cudaStream_t s) {
    if (k.n <= 0) return cudaSuccess;
    // the layout needs whole steps of G entries and whole warps per block
    if (nl.cap % (4 * k.lanes) != 0 || k.threads % 32 != 0) return cudaErrorInvalidValue;
    return with_group(k.lanes, [&](auto tag) {
        constexpr int G = decltype(tag)::value;
        const int blocks = group_blocks(k.n, k.threads);
        if (half == HALF_PREDICT)
            k_pass2_g<P, MODE_PRED, G><<<blocks, k.threads, 0, s>>>(k, in, keys, cs, nl, p1, out,
                                                                    out_hash, err, disp);
        else
            k_pass2_g<P, MODE_CORR, G><<<blocks, k.threads, 0, s>>>(k, in, keys, cs, nl, p1, out,
                                                                    out_hash, err, disp);
        return cudaGetLastError();
    });
}

#define SPH_NS_GROUPS_INSTANTIATE(P)                                                          \
    template cudaError_t launch_nbr_build_groups<P>(                                          \
        const KParamsT<P::T>&, const ParticleSetT<P::T>&, const unsigned*, const int*,        \
        const NbrList&, int, unsigned*, cudaStream_t, const unsigned*);                       \
    template cudaError_t launch_pass1_groups<P>(const KParamsT<P::T>&,                        \
                                                const ParticleSetT<P::T>&, const unsigned*,   \
                                                const int*, const NbrList&,                   \
                                                const Pass1OutT<P::T>&, cudaStream_t);        \
    template cudaError_t launch_pass2_groups<P>(                                              \
        const KParamsT<P::T>&, HalfStep, const ParticleSetT<P::T>&, const unsigned*,          \
        const int*, const NbrList&, const Pass1OutT<P::T>&, ParticleSetT<P::T>, unsigned*,   \
        unsigned*, unsigned*, cudaStream_t);
SPH_NS_GROUPS_INSTANTIATE(PrecF32)
SPH_NS_GROUPS_INSTANTIATE(PrecF64)
SPH_NS_GROUPS_INSTANTIATE(PrecMix)
SPH_NS_GROUPS_INSTANTIATE(PrecMixC)
#undef SPH_NS_GROUPS_INSTANTIATE

}  // namespace sph
