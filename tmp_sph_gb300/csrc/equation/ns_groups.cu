// ns_groups.cu — neighbour pass 1 with a group of G lanes per particle (G = 2, 4, 8, 16).
//
// Same passes as ns.cu (reference: computeBoundary_Delta_acoustic_D and
// computeGovering_equationD, src/equation/ns.cu:30-249), same list contents, different
// assignment of work to lanes.  With one thread per particle every lane of a warp gathers a
// different neighbour record, and a warp-level gather touches about twenty distinct 128-byte
// lines: the passes are limited by L1 data-stage wavefronts.  With G lanes per particle each
// pair of lanes of a group gathers two consecutive entries of one list in one step —
// neighbouring records, mostly one line — and a warp runs its loop for the longest list of
// 32/G particles rather than of 32.  Measured on the 4.96M-particle dam break: pass 1 at G = 2
// 0.756 ms against 0.793 with one lane (the resident default in FP32 with a list skin).  Pass 2
// runs one lane per particle: with groups it was slower at every G measured (0.849 ms at G = 2
// against 0.814: its larger per-pair body on half the particles per warp, and more sums to
// reduce), so that variant was removed.
//
// Sums.  Each lane accumulates its share of the pairs; a group reduces them with xor shuffles
// in a fixed tree, so results are deterministic and independent of the launch shape, but not
// bit-equal to one lane per particle (the sums associate differently).
//
// List layout.  The groups read the one-lane list with interleaved windows (ns_pair.cuh):
// lane s of a group takes int4 chunks s, s + G, s + 2G, ... of its particle's column, so at
// every step each pair of lanes gathers two consecutive entries.  With G = 2 the 16 particles
// of a warp read 16 consecutive int4s of each of two chunk rows — four whole lines per request,
// as the one-lane passes do.  The list build is the one-lane build with another slot order, and
// each pass picks its own G.
//
// Blocks.  A block of T threads owns T consecutive particles and visits them in G rounds of T/G
// particles (one group each), parking the reduced sums in shared memory; then every thread
// finishes one particle (the record pass 2 gathers), so the per-particle epilogue runs on all
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

// ---------------------------------------------------------------- neighbour visits
// The group's share of particle i's neighbours (r2 < kh2) with their records: from the list,
// lane s taking chunks s, s + G, ... of four entries; or, when i overflowed the list, by walking
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
            const int j = P::kCodes ? slot_index(e) : e;
            V a, b;
            ld_rec(R, j, a, b);
            T dx, dy, dz;
            rel_pos<P>(k, pi, a, P::kCodes ? slot_code(e) : 0u, dx, dy, dz);
            const T r2 = dist2(dx, dy, dz);
            if (r2 < k.kh2) f(j, a, b, dx, dy, dz, r2);
        };
        // this lane's chunks s, s + G, ... (each pair of lanes gathers two consecutive entries
        // per step)
        if (k.list_win)
            for_each_slot<true>(nl.idx + nbr_col(nl, i), cnt, s, G, one);
        else
            for_each_slot<false>(nl.idx + nbr_col(nl, i), cnt, s, G, one);
        return;
    }
    // the cells one by one (each a contiguous slot range), G candidates per step
    const unsigned key = keys[i];
    if (inactive_key(k, key)) return;
    int cx, cy, cz;
    cell_of_key(k.gx, k.gy, key, cx, cy, cz);
    const int r = k.reach;
    const int xl = cx > r - 1 ? cx - r : 0;
    const int xh = cx < k.gx - r ? cx + r : k.gx - 1;
#pragma unroll 1
    for (int dz = -r; dz <= r; dz++) {
        const int z = cz + dz;
        if ((unsigned)z >= (unsigned)k.gz) continue;
#pragma unroll 1
        for (int dy = -r; dy <= r; dy++) {
            const int y = cy + dy;
            if ((unsigned)y >= (unsigned)k.gy) continue;
            const int row = (z * k.gy + y) * k.gx;
#pragma unroll 1
            for (int xc = xl; xc <= xh; xc++) {
                const unsigned code = P::kCodes ? cell_code(k, cx, cy, cz, xc, y, z) : 0u;
                const int j0 = max(__ldg(cs + row + xc), 0);
                const int j1 = min(__ldg(cs + row + xc + 1), k.n);  // bounds guard only
#pragma unroll 1
                for (int j = j0 + s; j < j1; j += G) {
                    const V pj = ld_pos(X, (size_t)XSTRIDE * (size_t)j);
                    T dx, dy2, dz2;
                    rel_pos<P>(k, pi, pj, code, dx, dy2, dz2);
                    const T r2 = dist2(dx, dy2, dz2);
                    if (r2 < k.kh2 && j != i) {
                        V a, b;
                        ld_rec(R, j, a, b);
                        f(j, a, b, dx, dy2, dz2, r2);
                    }
                }
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
cudaError_t launch_pass1_groups(const KParamsT<typename P::T>& k,
                                const ParticleSetT<typename P::T>& in, const unsigned* keys,
                                const int* cs, const NbrList& nl,
                                const Pass1OutT<typename P::T>& out, cudaStream_t s) {
    if (k.n <= 0) return cudaSuccess;
    // whole warps per block (each block's rounds split its warps into groups)
    if (k.threads % 32 != 0) return cudaErrorInvalidValue;
    return with_group(k.lanes, [&](auto tag) {
        constexpr int G = decltype(tag)::value;
        k_pass1_g<P, G><<<group_blocks(k.n, k.threads), k.threads, 0, s>>>(k, in, keys, cs, nl,
                                                                         out);
        return cudaGetLastError();
    });
}

#define SPH_NS_GROUPS_INSTANTIATE(P)                                                          \
    template cudaError_t launch_pass1_groups<P>(const KParamsT<P::T>&,                        \
                                                const ParticleSetT<P::T>&, const unsigned*,   \
                                                const int*, const NbrList&,                   \
                                                const Pass1OutT<P::T>&, cudaStream_t);
SPH_NS_GROUPS_INSTANTIATE(PrecF32)
SPH_NS_GROUPS_INSTANTIATE(PrecF64)
SPH_NS_GROUPS_INSTANTIATE(PrecMix)
SPH_NS_GROUPS_INSTANTIATE(PrecMixC)
SPH_NS_GROUPS_INSTANTIATE(PrecMixA)
#undef SPH_NS_GROUPS_INSTANTIATE

}  // namespace sph
