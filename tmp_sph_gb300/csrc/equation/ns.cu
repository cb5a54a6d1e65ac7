// ns.cu — the two neighbour passes of the weakly-compressible delta-SPH step.
//
// Reference counterparts: SPH_NS_simpleversion (src/equation/ns.cu:5-28) launching
// computeBoundary_Delta_acoustic_D (pass 1, src/equation/ns.cu:30-131) and
// computeGovering_equationD (pass 2, src/equation/ns.cu:134-249).
//
// Layout.  Particles are in cell-sorted order; each is one 32-byte record of two float4,
// rec[2i] = (x, y, z, p) and rec[2i+1] = (vx, vy, vz, ±rho) with the sign of rho marking a
// fluid (+) or boundary (-) particle, so everything a neighbour contributes to pass 1 is one
// aligned 32-byte sector.  Pass 1 writes the record pass 2 gathers, nrec[2i] = (x, y, z, q),
// nrec[2i+1] = (vx, vy, vz, ±rho'), where q = p' - rho0 cs h dofv: the acoustic-damper term of a
// fluid-fluid pair, rho0 cs h (dofv_i + dofv_j), splits into an i part and a j part, and the j
// part is folded into the neighbour's pressure (boundary particles have dofv = 0, so q = p').
// It also writes self[i] = (p', rho', dofv, 0) for the particle's own side.
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
// wavefronts (each lane gathers a different record): interleaving the slots makes a warp's
// list read one line per step instead of one line per lane.  A particle with more hits than
// the list capacity is marked and walks the cells itself (same order again).
//
// With a Verlet skin the list is built with the cutoff kh(1 + skin) (kh2_list) on cells that
// wide and kept while every particle stays within skin*kh/2 of its build position; both
// passes still test r < kh on the current positions, and k_nbr_build keeps the build
// positions (xb) that pass 2 measures each particle's displacement against.
//
// Kernel algebra (same quantities as the reference, simplified): with r = x_i - x_j,
// q = |r|/h, t = 1 - q/2, the Wendland C2 gradient is grad W = c_fr t^3 r with
// c_fr = -5 adh / h^2, which is the reference's per-component expression
// adh(-2 t^3 (2q+1) + 2 t^4) r/(h|r|) after factoring.
#include <cuda_runtime.h>

#include "sph_internal.h"

namespace sph {

namespace {

constexpr int NS_THREADS = 128;

__device__ __forceinline__ void cell_of_key(const KParams& k, unsigned key, int& cx, int& cy,
                                            int& cz) {
    unsigned t = key / (unsigned)k.gx;
    cx = (int)(key - t * (unsigned)k.gx);
    cz = (int)(t / (unsigned)k.gy);
    cy = (int)(t - (unsigned)cz * (unsigned)k.gy);
}

// Squared distance with an explicit rounding sequence, so the in-range test gives the same
// answer in the list build, in the walking passes and in the list passes.
__device__ __forceinline__ float dist2(float dx, float dy, float dz) {
    return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}

// Visit every candidate slot j of the 27 cells around (cx, cy, cz), strip by strip.
template <class F>
__device__ __forceinline__ void for_each_candidate(const KParams& k, const int* __restrict__ cs,
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
            const int j0 = max(__ldg(cs + row + xl), 0);
            const int j1 = min(__ldg(cs + row + xh + 1), k.n);  // bounds guard only
#pragma unroll 4
            for (int j = j0; j < j1; j++) f(j);
        }
    }
}

// One 32-byte record (two float4) in a single 256-bit read-only load: a neighbour gather
// touches one L1 sector with one request.  R is 32-byte aligned (cudaMalloc'd, two float4 per
// particle).
__device__ __forceinline__ void ld_rec(const float4* __restrict__ R, int j, float4& a,
                                       float4& b) {
    const float4* p = R + 2 * (size_t)j;
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p));
}

// Walk the cells of particle i over the positions X[STRIDE * j] and call
// f(j, pj, dx, dy, dz, r2) for every j != i with r2 < cut2.  X is the dense (x, y, z, ±1) array
// (STRIDE 1) or a record array (STRIDE 2).
template <int STRIDE, class F>
__device__ __forceinline__ void walk_pairs(const KParams& k, const int* __restrict__ cs,
                                           const unsigned* __restrict__ keys,
                                           const float4* __restrict__ X, int i, const float4& pi,
                                           float cut2, F&& f) {
    int cx, cy, cz;
    cell_of_key(k, keys[i], cx, cy, cz);
    for_each_candidate(k, cs, cx, cy, cz, [&](int j) {
        const float4 pj = __ldg(X + (size_t)STRIDE * (size_t)j);
        const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
        const float r2 = dist2(dx, dy, dz);
        if (r2 < cut2 && j != i) f(j, pj, dx, dy, dz, r2);
    });
}

// Column of particle i in the warp-interleaved list: entry c of i is col[32 c].  The 32
// particles of a warp share one block of cap x 32 slots, so a warp reading entry c of all its
// lanes touches one 128-byte line.
__device__ __forceinline__ size_t nbr_col(const NbrList& nl, int i) {
    return (size_t)(i >> 5) * ((size_t)nl.cap << 5) + (size_t)(i & 31);
}

// Neighbours of i (r2 < kh2) with their records R[2j], R[2j+1]: from the list (one 256-bit
// record load per listed pair, the next slot loaded one pair ahead; pairs in the skin beyond
// the support radius are skipped), or by walking the cells over X[XSTRIDE * j] when i
// overflowed the list.  f(j, a, b, dx, dy, dz, r2).  (Skipping the gathers of slots in the skin
// with a pass-1 hit mask cost pass 2 more in instructions than it saved in sectors.)
template <bool LIST, int XSTRIDE, class F>
__device__ __forceinline__ void visit_records(const KParams& k, const int* __restrict__ cs,
                                              const unsigned* __restrict__ keys,
                                              const NbrList& nl, const float4* __restrict__ X,
                                              const float4* __restrict__ R, int i,
                                              const float4& pi, F&& f) {
    if (LIST) {
        const int cnt = __ldg(nl.count + i);
        if (cnt <= nl.cap) {
            const int* __restrict__ col = nl.idx + nbr_col(nl, i);
            int j = cnt > 0 ? __ldg(col) : 0;
#pragma unroll 1
            for (int c = 0; c < cnt; c++) {
                const int jn = c + 1 < cnt ? __ldg(col + ((size_t)(c + 1) << 5)) : 0;
                float4 a, b;
                ld_rec(R, j, a, b);
                const float dx = pi.x - a.x, dy = pi.y - a.y, dz = pi.z - a.z;
                const float r2 = dist2(dx, dy, dz);
                if (r2 < k.kh2) f(j, a, b, dx, dy, dz, r2);
                j = jn;
            }
            return;
        }
    }
    walk_pairs<XSTRIDE>(k, cs, keys, X, i, pi, k.kh2,
                        [&](int j, const float4&, float dx, float dy, float dz, float r2) {
        float4 a, b;
        ld_rec(R, j, a, b);
        f(j, a, b, dx, dy, dz, r2);
    });
}

__device__ __forceinline__ bool fluid_rec(float signed_rho) { return signed_rho > 0.f; }

// Neighbour-list build: every boundary particle keeps its fluid neighbours (all that pass 1
// needs), every fluid particle all of them; with walls_all, boundary particles keep all.
// Slots are warp-interleaved (nbr_col): the passes read them coalesced, the build writes them
// scattered within its warp's block, which L2 merges before they reach HBM.
__global__ void __launch_bounds__(NS_THREADS)
k_nbr_build(KParams k, const float4* __restrict__ X, const unsigned* __restrict__ keys,
            const int* __restrict__ cs, NbrList nl, int walls_all, unsigned* err,
            const unsigned* gate) {
    if (gated_off(gate)) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.n) return;
    const float4 pi = X[i];
    if (nl.xb) nl.xb[i] = pi;
    const bool keep_all = fluid_rec(pi.w) || walls_all;
    int cnt = 0;
    int* __restrict__ col = nl.idx + nbr_col(nl, i);
    const int cap = nl.cap;
    walk_pairs<1>(k, cs, keys, X, i, pi, k.kh2_list,
                  [&](int j, const float4& pj, float, float, float, float) {
        if (keep_all || fluid_rec(pj.w)) {
            if (cnt < cap) col[(size_t)cnt << 5] = j;
            cnt++;
        }
    });
    nl.count[i] = cnt;
    raise_flags(err, cnt > cap ? SPH_FLAG_NEIGHBOR_OVERFLOW : 0u);
}

// Pass 1: boundary pressure extrapolation (Adami-style, over fluid neighbours) for boundary
// particles; velocity divergence over fluid neighbours for fluid particles.  Writes the pass-2
// neighbour record and the particle's own (p', rho', dofv).
template <bool WRITE_SUMS, bool LIST>
__global__ void __launch_bounds__(NS_THREADS)
k_pass1(KParams k, ParticleSet in, const unsigned* __restrict__ keys,
        const int* __restrict__ cs, NbrList nl, Pass1Out out, float* __restrict__ rhop_sum,
        float* __restrict__ w_sum) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.n) return;
    const float4* __restrict__ R = in.rec;
    const float4 pi = R[2 * (size_t)i];      // x, y, z, p
    const float4 vi = R[2 * (size_t)i + 1];  // vx, vy, vz, ±rho
    const bool fi = fluid_rec(vi.w);
    float dofv = 0.f, rs = 0.f, ws = 0.f;
    visit_records<LIST, 1>(k, cs, keys, nl, in.xyz, R, i, pi,
                        [&](int, const float4& aj, const float4& vj, float dx, float dy, float dz,
                            float r2) {
        if (!fluid_rec(vj.w)) return;
        const float rr = sqrtf(r2);
        const float q = rr * k.inv_h;
        const float t = 1.f - 0.5f * q;
        const float t2 = t * t;
        if (!fi) {
            const float w = k.adh * t2 * t2 * (2.f * q + 1.f);
            rs += (aj.w + vj.w * k.g * dz) * w;
            ws += w;
        } else {
            const float fr = k.c_fr * t2 * t;
            const float vdotr = (vi.x - vj.x) * dx + (vi.y - vj.y) * dy + (vi.z - vj.z) * dz;
            dofv -= fr * vdotr * (k.mass / vj.w);
        }
    });
    float p, rho;
    if (fi) {
        p = pi.w;
        rho = vi.w;
    } else {
        p = fabsf(ws) > 1.0e-8f ? rs / ws : 0.f;
        if (p < 0.f) p = 0.f;
        rho = eos_density(k, p);
    }
    const float qv = fi ? p - k.damper * dofv : p;
    out.nrec[2 * (size_t)i] = make_float4(pi.x, pi.y, pi.z, qv);
    out.nrec[2 * (size_t)i + 1] = make_float4(vi.x, vi.y, vi.z, fi ? rho : -rho);
    out.self[i] = make_float4(p, rho, dofv, 0.f);
    if (WRITE_SUMS) {
        rhop_sum[i] = rs;
        w_sum[i] = ws;
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
template <int MODE, bool LIST>
__device__ __forceinline__ float pass2_one(const KParams& k, int i, const ParticleSet& in,
                                           const unsigned* __restrict__ keys,
                                           const int* __restrict__ cs, const NbrList& nl,
                                           const Pass1Out& p1, float* __restrict__ rho_dt,
                                           float* __restrict__ vel_dt, int wall_rates,
                                           const ParticleSet& out,
                                           unsigned* __restrict__ out_hash, unsigned* err) {
    const float4* __restrict__ NR = p1.nrec;
    const float4 pi = NR[2 * (size_t)i];
    const float4 vi = NR[2 * (size_t)i + 1];
    const float4 si = p1.self[i];  // p_i, rho_i, dofv_i
    const bool fi = fluid_rec(vi.w);
    const float rhoi = si.y, presi = si.x, dofvi = si.z;
    float drho = 0.f, ax = 0.f, ay = 0.f, az = 0.f;
    if (fi || (MODE == MODE_RATES && wall_rates)) {
        const float damp_i = k.damper * dofvi;
        // aj = (x, y, z, q), vj = (vx, vy, vz, ±rho) of the neighbour
        visit_records<LIST, 2>(k, cs, keys, nl, NR, NR, i, pi,
                            [&](int j, const float4& aj, const float4& vj, float dx, float dy,
                                float dz, float r2) {
            const bool fj = fluid_rec(vj.w);
            const float rhoj = fabsf(vj.w);
            const float rr = sqrtf(r2);
            const float q = rr * k.inv_h;
            const float t = 1.f - 0.5f * q;
            const float fr = k.c_fr * t * t * t;
            const float vdotr = (vi.x - vj.x) * dx + (vi.y - vj.y) * dy + (vi.z - vj.z) * dz;
            const float m_rhoj = k.mass / rhoj;
            const float inv_r2e = 1.f / (r2 + k.eta2);
            drho += m_rhoj * fr * (rhoi * vdotr + (rhoi - rhoj) * k.delta_h_cs * r2 * inv_r2e);
            float S;
            if (fi) {
                S = -presi - aj.w;
                if (fj) S += damp_i + k.visc * vdotr * inv_r2e;
            } else {
                S = -(presi + __ldg(&p1.self[j].x));  // boundary rows (wall_rates): plain pressures
            }
            const float c = fr * S * m_rhoj;
            ax += c * dx;
            ay += c * dy;
            az += c * dz;
        });
        const float inv_rhoi = 1.f / rhoi;
        ax *= inv_rhoi;
        ay *= inv_rhoi;
        az *= inv_rhoi;
    }
    az += k.g;

    if (MODE == MODE_RATES) {
        const bool have = fi || wall_rates;
        rho_dt[i] = have ? drho : 0.f;
        vel_dt[3 * i] = have ? ax : 0.f;
        vel_dt[3 * i + 1] = have ? ay : 0.f;
        vel_dt[3 * i + 2] = have ? az : 0.f;
        return 0.f;
    }

    float4 np = pi, nv;
    float npres, nrho;
    float4 tp, tv;
    if (fi) {
        if (escaped(k, pi.x, pi.y, pi.z)) {
            np = make_float4(k.park_x, k.park_y, k.park_z, 0.f);
            nv = make_float4(0.f, 0.f, 0.f, 0.f);
            npres = 0.f;
            nrho = k.rho0;
            tp = make_float4(np.x, np.y, np.z, k.rho0);
            tv = make_float4(0.f, 0.f, 0.f, 0.f);
        } else if (MODE == MODE_PRED) {
            tp = make_float4(pi.x, pi.y, pi.z, rhoi);
            tv = make_float4(vi.x, vi.y, vi.z, 0.f);
            float rho = rhoi + drho * k.half_dt;
            if (k.clamp_density && rho < k.rho0) rho = k.rho0;
            np.x = pi.x + vi.x * k.half_dt;
            np.y = pi.y + vi.y * k.half_dt;
            np.z = pi.z + vi.z * k.half_dt;
            nv = make_float4(vi.x + ax * k.half_dt, vi.y + ay * k.half_dt, vi.z + az * k.half_dt, 0.f);
            nrho = rho;
            npres = eos_pressure(k, rho);
        } else {
            tp = in.tpos[i];
            tv = in.tvel[i];
            float rho = tp.w + drho * k.half_dt;
            if (k.clamp_density && rho < k.rho0) rho = k.rho0;
            const float xs = tp.x + vi.x * k.half_dt;
            const float ys = tp.y + vi.y * k.half_dt;
            const float zs = tp.z + vi.z * k.half_dt;
            const float uxs = tv.x + ax * k.half_dt;
            const float uys = tv.y + ay * k.half_dt;
            const float uzs = tv.z + az * k.half_dt;
            rho = 2.f * rho - tp.w;
            if (k.clamp_density && rho < k.rho0) rho = k.rho0;
            np.x = 2.f * xs - tp.x;
            np.y = 2.f * ys - tp.y;
            np.z = 2.f * zs - tp.z;
            nv = make_float4(2.f * uxs - tv.x, 2.f * uys - tv.y, 2.f * uzs - tv.z, 0.f);
            nrho = rho;
            npres = eos_pressure(k, rho);
        }
    } else {
        // boundary particles do not move; they keep the extrapolated pressure and density
        nv = make_float4(vi.x, vi.y, vi.z, 0.f);
        npres = presi;
        nrho = rhoi;
        tp = make_float4(pi.x, pi.y, pi.z, rhoi);
        tv = make_float4(vi.x, vi.y, vi.z, 0.f);
    }
    out.rec[2 * (size_t)i] = make_float4(np.x, np.y, np.z, npres);
    out.rec[2 * (size_t)i + 1] = make_float4(nv.x, nv.y, nv.z, fi ? nrho : -nrho);
    if (out.xyz) out.xyz[i] = make_float4(np.x, np.y, np.z, fi ? 1.f : -1.f);
    out.type[i] = in.type[i];
    out.id[i] = in.id[i];
    if (MODE == MODE_PRED) {
        out.tpos[i] = tp;
        out.tvel[i] = tv;
    }
    unsigned f = 0;
    out_hash[i] = (unsigned)cell_hash_clamped(k, np.x, np.y, np.z, &f);
    raise_flags(err, f);
    if (!fi || !nl.xb) return 0.f;
    const float4 xb = nl.xb[i];
    return dist2(np.x - xb.x, np.y - xb.y, np.z - xb.z);
}

template <int MODE, bool LIST>
__global__ void __launch_bounds__(NS_THREADS)
k_pass2(KParams k, ParticleSet in, const unsigned* __restrict__ keys,
        const int* __restrict__ cs, NbrList nl, Pass1Out p1, float* __restrict__ rho_dt,
        float* __restrict__ vel_dt, int wall_rates, ParticleSet out,
        unsigned* __restrict__ out_hash, unsigned* err, unsigned* disp) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float d2 = 0.f;
    if (i < k.n)
        d2 = pass2_one<MODE, LIST>(k, i, in, keys, cs, nl, p1, rho_dt, vel_dt, wall_rates, out,
                                   out_hash, err);
    if (MODE == MODE_RATES || disp == nullptr) return;
    // block maximum of the squared displacement, one atomic per block (non-negative floats
    // order like their bit patterns)
    __shared__ unsigned s_max[NS_THREADS / 32];
    const unsigned wmax = __reduce_max_sync(0xffffffffu, __float_as_uint(d2));
    if ((threadIdx.x & 31) == 0) s_max[threadIdx.x >> 5] = wmax;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned m = s_max[0];
#pragma unroll
        for (int w = 1; w < NS_THREADS / 32; w++) m = max(m, s_max[w]);
        if (m) atomicMax(disp, m);
    }
}

inline int blocks_for(long n, int t) { return (int)((n + t - 1) / t); }

template <bool LIST>
void pass1_launch(const KParams& k, const ParticleSet& in, const unsigned* keys, const int* cs,
                  const NbrList& nl, const Pass1Out& o, float* rhop_sum, float* w_sum,
                  cudaStream_t s) {
    const int b = blocks_for(k.n, NS_THREADS);
    if (rhop_sum && w_sum)
        k_pass1<true, LIST><<<b, NS_THREADS, 0, s>>>(k, in, keys, cs, nl, o, rhop_sum, w_sum);
    else
        k_pass1<false, LIST><<<b, NS_THREADS, 0, s>>>(k, in, keys, cs, nl, o, nullptr, nullptr);
}

template <int MODE>
void pass2_launch(const KParams& k, const ParticleSet& in, const unsigned* keys, const int* cs,
                  const NbrList* nl, const Pass1Out& p1, float* rho_dt, float* vel_dt,
                  int wall_rates, ParticleSet out, unsigned* out_hash, unsigned* err,
                  unsigned* disp, cudaStream_t s) {
    const int b = blocks_for(k.n, NS_THREADS);
    if (nl)
        k_pass2<MODE, true><<<b, NS_THREADS, 0, s>>>(k, in, keys, cs, *nl, p1, rho_dt, vel_dt,
                                                      wall_rates, out, out_hash, err, disp);
    else
        k_pass2<MODE, false><<<b, NS_THREADS, 0, s>>>(k, in, keys, cs, NbrList{}, p1, rho_dt,
                                                       vel_dt, wall_rates, out, out_hash, err,
                                                       nullptr);
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

cudaError_t launch_nbr_build(const KParams& k, const ParticleSet& in, const unsigned* keys,
                             const int* cs, const NbrList& nl, int walls_all, unsigned* err,
                             cudaStream_t s, const unsigned* gate) {
    if (k.n <= 0) return cudaSuccess;
    k_nbr_build<<<blocks_for(k.n, NS_THREADS), NS_THREADS, 0, s>>>(k, in.xyz, keys, cs, nl,
                                                                   walls_all, err, gate);
    return cudaGetLastError();
}

cudaError_t launch_pass1(const KParams& k, const ParticleSet& in, const unsigned* keys,
                         const int* cs, const NbrList* nl, const Pass1Out& out, float* rhop_sum,
                         float* w_sum, cudaStream_t s) {
    if (k.n <= 0) return cudaSuccess;
    if (nl)
        pass1_launch<true>(k, in, keys, cs, *nl, out, rhop_sum, w_sum, s);
    else
        pass1_launch<false>(k, in, keys, cs, NbrList{}, out, rhop_sum, w_sum, s);
    return cudaGetLastError();
}

cudaError_t launch_pass2_rates(const KParams& k, const ParticleSet& in, const unsigned* keys,
                               const int* cs, const NbrList* nl, const Pass1Out& p1,
                               float* rho_dt, float* vel_dt, int wall_rates, cudaStream_t s) {
    if (k.n <= 0) return cudaSuccess;
    pass2_launch<MODE_RATES>(k, in, keys, cs, nl, p1, rho_dt, vel_dt, wall_rates, ParticleSet{},
                             nullptr, nullptr, nullptr, s);
    return cudaGetLastError();
}

cudaError_t launch_pass2_step(const KParams& k, HalfStep half, const ParticleSet& in,
                              const unsigned* keys, const int* cs, const NbrList* nl,
                              const Pass1Out& p1, ParticleSet out, unsigned* out_hash,
                              unsigned* err, unsigned* disp, cudaStream_t s) {
    if (k.n <= 0) return cudaSuccess;
    if (half == HALF_PREDICT)
        pass2_launch<MODE_PRED>(k, in, keys, cs, nl, p1, nullptr, nullptr, 0, out, out_hash, err,
                                disp, s);
    else
        pass2_launch<MODE_CORR>(k, in, keys, cs, nl, p1, nullptr, nullptr, 0, out, out_hash, err,
                                disp, s);
    return cudaGetLastError();
}

}  // namespace sph
