// mesh.cu — cell list: particle -> cell hash, stable LSD radix sort of (hash, slot) pairs,
// cell ranges, and the permutation of the particle arrays into cell order.
//
// Reference counterparts: calcHashD/calcHash (src/lib/mesh.cu:26-70), sortParticles
// (src/lib/mesh.cu:73-86, a thrust::sort_by_key), reorderD/reorder (src/lib/mesh.cu:89-159),
// recoverD/recover (src/lib/mesh.cu:162-194).
//
// The sort is written for this project: reduce-then-scan LSD radix with 8-bit digits,
// 4096-key tiles (256 threads x 16 keys), warp-level stable ranking with __match_any_sync,
// tile-local reordering in shared memory so the scatter to global memory is in digit runs.
// No spin-waits, no allocation: all scratch is caller-provided.
#include <cuda_runtime.h>

#include <algorithm>

#include "sph_internal.h"

namespace sph {

namespace {

constexpr int RS_THREADS = 256;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_IPT = 16;
constexpr int RS_TILE = RS_THREADS * RS_IPT;  // 4096 keys
constexpr int RS_RADIX = 256;
constexpr int RS_MAX_PASSES = 4;

inline int rs_tiles(int n) { return (n + RS_TILE - 1) / RS_TILE; }
inline size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

struct SortScratch {
    unsigned* keys_alt;
    int* vals_alt;
    unsigned* hist;    // [RS_RADIX][tiles]
    unsigned* totals;  // [RS_MAX_PASSES][RS_RADIX]
};

SortScratch carve(void* base, int n) {
    char* p = static_cast<char*>(base);
    SortScratch s;
    size_t nn = (size_t)(n > 0 ? n : 1);
    s.keys_alt = reinterpret_cast<unsigned*>(p);
    p += align256(nn * sizeof(unsigned));
    s.vals_alt = reinterpret_cast<int*>(p);
    p += align256(nn * sizeof(int));
    s.hist = reinterpret_cast<unsigned*>(p);
    p += align256((size_t)RS_RADIX * (size_t)(rs_tiles(n) > 0 ? rs_tiles(n) : 1) * sizeof(unsigned));
    s.totals = reinterpret_cast<unsigned*>(p);
    return s;
}

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Per-tile digit histogram: hist[d * tiles + tile]; totals[d] accumulates over tiles.
__global__ void __launch_bounds__(RS_THREADS)
k_rs_upsweep(const unsigned* __restrict__ keys, int n, int shift, unsigned xmask,
             int check_bits, unsigned* __restrict__ hist, int tiles,
             unsigned* __restrict__ totals, unsigned* err, const unsigned* gate) {
    __shared__ unsigned cnt[RS_RADIX];
    if (gated_off(gate)) return;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    cnt[tid] = 0;
    __syncthreads();
    const long base = (long)blockIdx.x * RS_TILE + warp * (32 * RS_IPT) + lane;
    unsigned flags = 0;
#pragma unroll
    for (int r = 0; r < RS_IPT; r++) {
        long idx = base + r * 32;
        bool valid = idx < n;
        unsigned key = valid ? (__ldg(keys + idx) ^ xmask) : 0u;
        if (valid && check_bits < 32 && (key >> check_bits) != 0u) flags |= SPH_FLAG_KEY_RANGE;
        unsigned d = (key >> shift) & 0xffu;
        unsigned peers = __match_any_sync(0xffffffffu, valid ? d : 0x100u);
        if (valid && lane == __ffs(peers) - 1) atomicAdd(&cnt[d], __popc(peers));
    }
    __syncthreads();
    unsigned c = cnt[tid];
    hist[(size_t)tid * tiles + blockIdx.x] = c;
    if (c) atomicAdd(&totals[tid], c);
    raise_flags(err, flags);
}

// Exclusive scan of one digit's row of tile counts, offset by the counts of all smaller
// digits: after this, hist[d * tiles + t] is the first output slot of digit d in tile t.
__global__ void __launch_bounds__(RS_THREADS)
k_rs_scan(unsigned* __restrict__ hist, int tiles, const unsigned* __restrict__ totals,
          const unsigned* gate) {
    __shared__ unsigned wsum[RS_WARPS];
    __shared__ unsigned s_carry;
    if (gated_off(gate)) return;
    const int d = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // base = sum of totals of digits < d
    unsigned v = (tid < d) ? totals[tid] : 0u;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) wsum[warp] = v;
    __syncthreads();
    if (tid == 0) {
        unsigned b = 0;
        for (int w = 0; w < RS_WARPS; w++) b += wsum[w];
        s_carry = b;
    }
    __syncthreads();
    unsigned* row = hist + (size_t)d * tiles;
    for (int chunk = 0; chunk < tiles; chunk += RS_THREADS) {
        int idx = chunk + tid;
        unsigned x = idx < tiles ? row[idx] : 0u;
        unsigned incl = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            unsigned y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        __syncthreads();  // wsum reuse
        if (lane == 31) wsum[warp] = incl;
        __syncthreads();
        unsigned wpre = 0, btot = 0;
        for (int w = 0; w < RS_WARPS; w++) {
            unsigned t = wsum[w];
            if (w < warp) wpre += t;
            btot += t;
        }
        unsigned carry = s_carry;
        if (idx < tiles) row[idx] = carry + wpre + incl - x;
        __syncthreads();
        if (tid == 0) s_carry = carry + btot;
        __syncthreads();
    }
}

// Stable rank-and-scatter of one tile for one digit.
__global__ void __launch_bounds__(RS_THREADS)
k_rs_downsweep(const unsigned* __restrict__ keys_in, const int* __restrict__ vals_in,
               unsigned* __restrict__ keys_out, int* __restrict__ vals_out,
               const unsigned* __restrict__ hist, int n, int shift, unsigned xmask_in,
               unsigned xmask_out, int tiles, const unsigned* gate) {
    __shared__ unsigned s_cnt[RS_WARPS][RS_RADIX];
    __shared__ unsigned s_gbase[RS_RADIX];
    __shared__ unsigned s_tpre[RS_RADIX];
    __shared__ unsigned s_keys[RS_TILE];
    __shared__ int s_vals[RS_TILE];
    __shared__ unsigned s_wsum[RS_WARPS];

    if (gated_off(gate)) return;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
#pragma unroll
    for (int w = 0; w < RS_WARPS; w++) s_cnt[w][tid] = 0;
    __syncthreads();

    const long tile_base = (long)blockIdx.x * RS_TILE;
    const long wbase = tile_base + warp * (32 * RS_IPT) + lane;
    unsigned key[RS_IPT];
    int val[RS_IPT];
    unsigned lr[RS_IPT];
#pragma unroll
    for (int r = 0; r < RS_IPT; r++) {
        long idx = wbase + r * 32;
        bool valid = idx < n;
        key[r] = valid ? (__ldg(keys_in + idx) ^ xmask_in) : 0u;
        val[r] = valid ? (vals_in ? __ldg(vals_in + idx) : (int)idx) : 0;
    }
    const unsigned lt = lanemask_lt();
#pragma unroll
    for (int r = 0; r < RS_IPT; r++) {
        bool valid = wbase + r * 32 < n;
        unsigned d = (key[r] >> shift) & 0xffu;
        unsigned peers = __match_any_sync(0xffffffffu, valid ? d : 0x100u);
        unsigned c = valid ? s_cnt[warp][d] : 0u;
        __syncwarp();
        if (valid && lane == __ffs(peers) - 1) s_cnt[warp][d] = c + __popc(peers);
        __syncwarp();
        lr[r] = c + __popc(peers & lt);
    }
    __syncthreads();
    // per digit: exclusive prefix over warps, tile count, global base
    unsigned run = 0;
#pragma unroll
    for (int w = 0; w < RS_WARPS; w++) {
        unsigned v = s_cnt[w][tid];
        s_cnt[w][tid] = run;
        run += v;
    }
    s_gbase[tid] = hist[(size_t)tid * tiles + blockIdx.x];
    // exclusive scan of tile counts over digits
    unsigned incl = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        unsigned y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) s_wsum[warp] = incl;
    __syncthreads();
    unsigned wpre = 0;
    for (int w = 0; w < warp; w++) wpre += s_wsum[w];
    s_tpre[tid] = wpre + incl - run;
    __syncthreads();
#pragma unroll
    for (int r = 0; r < RS_IPT; r++) {
        if (wbase + r * 32 < n) {
            unsigned d = (key[r] >> shift) & 0xffu;
            unsigned lp = s_tpre[d] + s_cnt[warp][d] + lr[r];
            s_keys[lp] = key[r];
            s_vals[lp] = val[r];
        }
    }
    __syncthreads();
    const int tile_n = (int)min((long)RS_TILE, (long)n - tile_base);
    for (int e = tid; e < tile_n; e += RS_THREADS) {
        unsigned k = s_keys[e];
        unsigned d = (k >> shift) & 0xffu;
        unsigned g = s_gbase[d] + (unsigned)e - s_tpre[d];
        if (g < (unsigned)n) {  // always true for consistent histograms; guards the store
            keys_out[g] = k ^ xmask_out;
            vals_out[g] = s_vals[e];
        }
    }
}

// Gated memset: the graph-capturable stand-in for cudaMemsetAsync inside a gated rebuild.
__global__ void k_fill_u32(unsigned* __restrict__ p, unsigned value, long count,
                           const unsigned* gate) {
    if (gated_off(gate)) return;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < count;
         i += (long)gridDim.x * blockDim.x)
        p[i] = value;
}

cudaError_t fill_u32(unsigned* p, unsigned value, long count, const unsigned* gate,
                     cudaStream_t s) {
    if (!gate)
        return (value & 0xffu) * 0x01010101u == value
                   ? cudaMemsetAsync(p, (int)(value & 0xffu), (size_t)count * sizeof(unsigned), s)
                   : cudaErrorInvalidValue;
    const int blocks = (int)std::min<long>((count + 255) / 256, 152L * 8);
    k_fill_u32<<<blocks > 0 ? blocks : 1, 256, 0, s>>>(p, value, count, gate);
    return cudaGetLastError();
}

// ---------------------------------------------------------------- dense cell starts
__global__ void k_cell_mark(const unsigned* __restrict__ keys, int n, int num_cells,
                            int* __restrict__ cs, const unsigned* gate,
                            const int* __restrict__ type, unsigned char* __restrict__ fluid) {
    if (gated_off(gate)) return;
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    unsigned key = keys[k];
    if (fluid && key < (unsigned)num_cells && type[k] == SPH_TYPE_FLUID) fluid[key] = 1;
    // key num_cells starts the tail of slots outside every cell (park_inactive)
    if ((k == 0 || keys[k - 1] != key) && key <= (unsigned)num_cells) cs[key] = k;
}

constexpr int FILL_THREADS = 256;
constexpr int FILL_PER_THREAD = 4;
constexpr int FILL_CHUNK = FILL_THREADS * FILL_PER_THREAD;

// Suffix-min fill: an unmarked (empty) cell takes the start of the next non-empty cell.
// Each block owns FILL_CHUNK cells; the value flowing in from the right of the chunk is the
// first slot whose key is >= the chunk end (one binary search per block).
__global__ void __launch_bounds__(FILL_THREADS)
k_cell_fill(int* __restrict__ cs, int num_cells, const unsigned* __restrict__ keys, int n,
            const unsigned* gate) {
    __shared__ int s_carry;
    __shared__ int s_wmin[FILL_THREADS / 32];
    if (gated_off(gate)) return;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const long c0 = (long)blockIdx.x * FILL_CHUNK;
    if (tid == 0) {
        long target = c0 + FILL_CHUNK;
        int lo = 0, hi = n;
        while (lo < hi) {
            int mid = (int)(((long)lo + hi) >> 1);
            if ((long)keys[mid] < target) lo = mid + 1; else hi = mid;
        }
        s_carry = lo;
    }
    const int BIG = 0x7fffffff;
    int v[FILL_PER_THREAD];
    const long cbase = c0 + (long)tid * FILL_PER_THREAD;
#pragma unroll
    for (int j = 0; j < FILL_PER_THREAD; j++) {
        long c = cbase + j;
        v[j] = c < num_cells ? cs[c] : (c == num_cells ? min(cs[c], n) : BIG);
    }
    int tmin = v[FILL_PER_THREAD - 1];
#pragma unroll
    for (int j = FILL_PER_THREAD - 2; j >= 0; j--) tmin = min(tmin, v[j]);
    // inclusive suffix min within the warp
    int incl = tmin;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_down_sync(0xffffffffu, incl, o);
        if (lane + o < 32) incl = min(incl, y);
    }
    if (lane == 0) s_wmin[warp] = incl;
    __syncthreads();
    int right = s_carry;
    for (int w = warp + 1; w < FILL_THREADS / 32; w++) right = min(right, s_wmin[w]);
    int nxt = __shfl_down_sync(0xffffffffu, incl, 1);
    int excl = (lane < 31) ? min(nxt, right) : right;
#pragma unroll
    for (int j = FILL_PER_THREAD - 1; j >= 0; j--) {
        excl = min(excl, v[j]);
        long c = cbase + j;
        if (c <= num_cells) cs[c] = excl;
    }
}

// ---------------------------------------------------------------- drop-in kernels
__global__ void k_calc_hash(KParams k, const float* __restrict__ pos, int* __restrict__ hash,
                            int* __restrict__ index, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
    hash[i] = cell_hash_raw(k, x, y, z);
    index[i] = i;
}

__global__ void k_reorder(int num_cells, const float* __restrict__ pos,
                          const float* __restrict__ vel, const float* __restrict__ rho,
                          const float* __restrict__ p, const int* __restrict__ type,
                          const int* __restrict__ zone, float* __restrict__ s_pos,
                          float* __restrict__ s_vel, float* __restrict__ s_rho,
                          float* __restrict__ s_p, int* __restrict__ s_type,
                          int* __restrict__ s_zone, const int* __restrict__ hash,
                          const int* __restrict__ index, int* __restrict__ cs,
                          int* __restrict__ ce, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int h = hash[i];
    bool in = (unsigned)h < (unsigned)num_cells;
    if (i == 0 || h != hash[i - 1]) {
        if (in) cs[h] = i;
        if (i > 0) {
            int hp = hash[i - 1];
            if ((unsigned)hp < (unsigned)num_cells) ce[hp] = i;
        }
    }
    if (i == n - 1 && in) ce[h] = i + 1;
    int s = index[i];
    if ((unsigned)s >= (unsigned)n) return;
    s_pos[3 * i] = pos[3 * s];
    s_pos[3 * i + 1] = pos[3 * s + 1];
    s_pos[3 * i + 2] = pos[3 * s + 2];
    s_vel[3 * i] = vel[3 * s];
    s_vel[3 * i + 1] = vel[3 * s + 1];
    s_vel[3 * i + 2] = vel[3 * s + 2];
    s_rho[i] = rho[s];
    s_p[i] = p[s];
    s_type[i] = type[s];
    if (zone && s_zone) s_zone[i] = zone[s];
}

__global__ void k_recover(float* __restrict__ pos, float* __restrict__ vel,
                          float* __restrict__ rho, float* __restrict__ p,
                          const int* __restrict__ index, int* __restrict__ type,
                          int* __restrict__ zone, const float* __restrict__ s_pos,
                          const float* __restrict__ s_vel, const float* __restrict__ s_rho,
                          const float* __restrict__ s_p, const int* __restrict__ s_type,
                          const int* __restrict__ s_zone, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int r = index[i];
    if ((unsigned)r >= (unsigned)n) return;
    pos[3 * r] = s_pos[3 * i];
    pos[3 * r + 1] = s_pos[3 * i + 1];
    pos[3 * r + 2] = s_pos[3 * i + 2];
    vel[3 * r] = s_vel[3 * i];
    vel[3 * r + 1] = s_vel[3 * i + 1];
    vel[3 * r + 2] = s_vel[3 * i + 2];
    rho[r] = s_rho[i];
    p[r] = s_p[i];
    type[r] = s_type[i];
    if (zone && s_zone) zone[r] = s_zone[i];
}

// ---------------------------------------------------------------- resident-state kernels
template <class T>
__device__ __forceinline__ T signed_rho_t(int type, T rho) {
    return type == SPH_TYPE_FLUID ? rho : -rho;
}

// Record position of an FP64 position for slot key `key` (policies with FP64 masters):
// cell-local offsets (cell codes) or the rounded position (record_pos).
template <class P, class KT>
__device__ __forceinline__ float4 offsets_in_cell(const KParamsT<KT>& k, unsigned key,
                                                  const dvec4& xm, float w) {
    const float3 q = record_pos<P>(k, key, xm.x, xm.y, xm.z);
    return make_float4(q.x, q.y, q.z, w);
}

// Permute (perm) or copy (perm == NULL) a particle set.  With cell codes a permuting gather
// re-expresses positions as offsets in the new cells keys[k].
template <class P>
__global__ void k_gather(KParamsT<typename P::T> kp, const int* __restrict__ perm,
                         ParticleSetT<typename P::T> src, ParticleSetT<typename P::T> dst,
                         int with_tmp, const unsigned* __restrict__ keys, const unsigned* gate) {
    using T = typename P::T;
    using V = vec4_t<T>;
    if (gated_off(gate)) return;
    const int n = kp.n;
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int s = perm ? perm[k] : k;
    if ((unsigned)s >= (unsigned)n) s = k;  // a consistent permutation never takes this
    V a = src.rec[2 * (size_t)s];
    const V b = src.rec[2 * (size_t)s + 1];
    if constexpr (P::kMixed) {
        const dvec4 xm = src.xm[s];
        dst.xm[k] = xm;
        if (with_tmp) dst.txm[k] = src.txm[s];
        if (perm && P::kCodes) a = offsets_in_cell<P>(kp, keys[k], xm, a.w);
    } else {
        (void)keys;
        if (with_tmp) dst.tpos[k] = src.tpos[s];
    }
    dst.rec[2 * (size_t)k] = a;
    dst.rec[2 * (size_t)k + 1] = b;
    dst.xyz[k] = make4<T>(a.x, a.y, a.z, b.w > T(0) ? T(1) : T(-1));
    dst.type[k] = src.type[s];
    dst.id[k] = src.id[s];
    if (src.inst && dst.inst) dst.inst[k] = src.inst[s];
    if (with_tmp) dst.tvel[k] = src.tvel[s];
}

// Instance of particle i when instance b owns [off[b], off[b+1]) (upper bound search).
__device__ __forceinline__ int instance_of(const int* __restrict__ off, int n_inst, int i) {
    if (!off || n_inst <= 1) return 0;
    int lo = 0, hi = n_inst;  // off[lo] <= i < off[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(off + mid) <= i) lo = mid; else hi = mid;
    }
    return lo;
}

template <class P>
__global__ void k_upload_convert(KParamsT<typename P::T> kp, const float* __restrict__ pos,
                                 const float* __restrict__ vel, const float* __restrict__ rho,
                                 const float* __restrict__ p, const int* __restrict__ type,
                                 const int* __restrict__ inst_off, int n_inst,
                                 ParticleSetT<typename P::T> dst, unsigned* __restrict__ hash,
                                 unsigned* err) {
    using T = typename P::T;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kp.n) return;
    const float x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
    const float vx = vel[3 * i], vy = vel[3 * i + 1], vz = vel[3 * i + 2];
    const int t = type[i];
    const int inst = instance_of(inst_off, n_inst, i);
    unsigned f = 0;
    dst.type[i] = t;
    dst.id[i] = i;
    if (dst.inst) dst.inst[i] = inst;
    dst.tvel[i] = make4<T>(vx, vy, vz, T(0));
    dst.rec[2 * (size_t)i + 1] = make4<T>(vx, vy, vz, signed_rho_t<T>(t, (T)rho[i]));
    if constexpr (P::kMixed) {
        const dvec4 xm = {(double)x, (double)y, (double)z, (double)rho[i] - (double)kp.rho0};
        // the FP32 hash of the FP32 positions where the passes use them (record_pos)
        const unsigned h = P::kCodes ? slot_key(kp, inst, t == SPH_TYPE_FLUID, xm.x, xm.y, xm.z, &f)
                                     : slot_key(kp, inst, t == SPH_TYPE_FLUID, x, y, z, &f);
        dst.xm[i] = xm;
        dst.txm[i] = xm;
        dst.rec[2 * (size_t)i] = offsets_in_cell<P>(kp, h, xm, p[i]);
        hash[i] = h;
    } else {
        dst.rec[2 * (size_t)i] = make4<T>(x, y, z, (T)p[i]);
        dst.tpos[i] = make4<T>(x, y, z, (T)rho[i]);
        hash[i] = slot_key(kp, inst, t == SPH_TYPE_FLUID, (T)x, (T)y, (T)z, &f);
    }
    raise_flags(err, f);
}

// Upload into the current cell order.  Slot k of the sorted live set takes particle id[k] of
// the original-order arrays, so the cell starts and neighbour lists built for that order stay
// in use.  Every slot adds its displacement from the position its list was built at (xb) to
// the displacement box `disp` (the half step's rebuild test then decides, as after a pass-2
// update), and a particle whose kind changed (boundary lists hold fluid neighbours only) sets
// *force.
// Mixed precision: record positions as pass 2 writes them (record_pos: offsets in the slot's
// sorted cell, or the rounded FP64 position).
template <class P>
__global__ void k_upload_sorted(KParamsT<typename P::T> kp, const float* __restrict__ pos,
                                const float* __restrict__ vel, const float* __restrict__ rho,
                                const float* __restrict__ p, const int* __restrict__ type,
                                const unsigned* __restrict__ keys, const float4* __restrict__ xb,
                                ParticleSetT<typename P::T> dst, unsigned* __restrict__ hash,
                                unsigned* err, unsigned* disp, unsigned* force) {
    using T = typename P::T;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    DispBox box;
    unsigned* const iw = kp.inst_boxes ? disp : nullptr;  // per-instance boxes
    if (k < kp.n) {
        const int r = dst.id[k];
        if ((unsigned)r < (unsigned)kp.n) {
            const float x = pos[3 * r], y = pos[3 * r + 1], z = pos[3 * r + 2];
            const float vx = vel[3 * r], vy = vel[3 * r + 1], vz = vel[3 * r + 2];
            const int t = type[r];
            if (t != dst.type[k]) atomicOr(force, 1u);
            const int inst = dst.inst ? dst.inst[k] : 0;
            unsigned f = 0;
            dst.type[k] = t;
            dst.tvel[k] = make4<T>(vx, vy, vz, T(0));
            const T srho = signed_rho_t<T>(t, (T)rho[r]);
            dst.rec[2 * (size_t)k + 1] = make4<T>(vx, vy, vz, srho);
            vec4_t<T> a;
            unsigned nk;
            const unsigned key = keys[k];
            if constexpr (P::kMixed) {
                const dvec4 xm = {(double)x, (double)y, (double)z, (double)rho[r] - (double)kp.rho0};
                dst.xm[k] = xm;
                dst.txm[k] = xm;
                a = offsets_in_cell<P>(kp, key, xm, p[r]);
                nk = P::kCodes ? slot_key(kp, inst, t == SPH_TYPE_FLUID, xm.x, xm.y, xm.z, &f)
                               : slot_key(kp, inst, t == SPH_TYPE_FLUID, x, y, z, &f);
            } else {
                a = make4<T>(x, y, z, (T)p[r]);
                dst.tpos[k] = make4<T>(x, y, z, (T)rho[r]);
                nk = slot_key(kp, inst, t == SPH_TYPE_FLUID, (T)x, (T)y, (T)z, &f);
            }
            hash[k] = nk;
            // a particle entering or leaving the neighbour search (park_inactive) needs new
            // lists; one that stays outside it is in no list.  Marked as pass 2 marks it (a
            // box no skin covers, not a forced rebuild), so the adaptive skin of a host loop
            // follows the resident run's
            const bool out_now = inactive_key(kp, nk);
            const bool moved_out = out_now != inactive_key(kp, key);
            if (moved_out) {
                if (iw) atomicOr(iw + IW_ALL, 1u);  // later slots move: every instance rebuilds
                box.add_at(iw, inst, 3.0e38f, 3.0e38f, 3.0e38f);
                box.add_at(iw, inst, -3.0e38f, -3.0e38f, -3.0e38f);
            }
            dst.rec[2 * (size_t)k] = a;
            dst.xyz[k] = make4<T>(a.x, a.y, a.z, srho > T(0) ? T(1) : T(-1));
            raise_flags(err, f);
            if (xb && !out_now && !moved_out) {
                const float4 b = xb[k];
                box.add_at(iw, inst, (float)a.x - b.x, (float)a.y - b.y, (float)a.z - b.z);
            }
        } else {
            atomicOr(force, 1u);  // a consistent permutation never takes this
        }
    }
    // blockDim is 256, every thread gets here
    __shared__ unsigned s_box[6 * 8];
    __shared__ int s_inst[8];
    reduce_disp(kp, box, disp, s_box, s_inst);
}

// Cell keys of a resident set on the current grid (after the grid changed under it).
template <class P>
__global__ void k_rehash(KParamsT<typename P::T> kp, ParticleSetT<typename P::T> set,
                         unsigned* __restrict__ hash, unsigned* err) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kp.n) return;
    unsigned f = 0;
    const int inst = set.inst ? set.inst[i] : 0;
    const bool fluid = set.type[i] == SPH_TYPE_FLUID;
    if constexpr (P::kCodes) {  // the FP64 hash where the records hold cell-local offsets
        const dvec4 q = set.xm[i];
        hash[i] = slot_key(kp, inst, fluid, q.x, q.y, q.z, &f);
    } else {
        const auto q = set.xyz[i];
        hash[i] = slot_key(kp, inst, fluid, q.x, q.y, q.z, &f);
    }
    raise_flags(err, f);
}

template <class P>
__global__ void k_download_convert(int n, ParticleSetT<typename P::T> src, float* __restrict__ pos,
                                   float* __restrict__ vel, float* __restrict__ rho,
                                   float* __restrict__ p, int* __restrict__ type) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int r = src.id[k];
    if ((unsigned)r >= (unsigned)n) return;
    const auto a = src.rec[2 * (size_t)k];
    const auto v = src.rec[2 * (size_t)k + 1];
    if (pos) {
        if constexpr (P::kMixed) {
            const dvec4 xm = src.xm[k];
            pos[3 * r] = (float)xm.x;
            pos[3 * r + 1] = (float)xm.y;
            pos[3 * r + 2] = (float)xm.z;
        } else {
            pos[3 * r] = (float)a.x;
            pos[3 * r + 1] = (float)a.y;
            pos[3 * r + 2] = (float)a.z;
        }
    }
    if (vel) { vel[3 * r] = (float)v.x; vel[3 * r + 1] = (float)v.y; vel[3 * r + 2] = (float)v.z; }
    if (rho) rho[r] = (float)fabs((double)v.w);
    if (p) p[r] = (float)a.w;
    if (type) type[r] = src.type[k];
}

// The state in original order and full precision of the solver (FP64 positions of the FP64
// and mixed solvers, FP32 values widened otherwise).
template <class P>
__global__ void k_download_f64(int n, double rho0, ParticleSetT<typename P::T> src,
                               double* __restrict__ pos, double* __restrict__ vel,
                               double* __restrict__ rho, double* __restrict__ p) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int r = src.id[k];
    if ((unsigned)r >= (unsigned)n) return;
    const auto a = src.rec[2 * (size_t)k];
    const auto v = src.rec[2 * (size_t)k + 1];
    double x = (double)a.x, y = (double)a.y, z = (double)a.z;
    double rr = fabs((double)v.w);
    if constexpr (P::kMixed) {
        const dvec4 xm = src.xm[k];
        x = xm.x;
        y = xm.y;
        z = xm.z;
        if (src.type[k] == SPH_TYPE_FLUID) rr = rho0 + xm.w;
    }
    if (pos) { pos[3 * r] = x; pos[3 * r + 1] = y; pos[3 * r + 2] = z; }
    if (vel) { vel[3 * r] = v.x; vel[3 * r + 1] = v.y; vel[3 * r + 2] = v.z; }
    if (rho) rho[r] = rr;
    if (p) p[r] = (double)a.w;
}

// Signed density of a record: negative marks a boundary (non-fluid) particle.
__device__ __forceinline__ float signed_rho(int type, float rho) {
    return signed_rho_t<float>(type, rho);
}

// A sorted hash outside [0, num_cells) (a particle outside the grid) is clamped to the
// nearest end of the range, which keeps the keys sorted and every cell index in bounds.
__global__ void k_aos_to_set(int n, int num_cells, const float* __restrict__ s_pos,
                             const float* __restrict__ s_vel, const float* __restrict__ s_rho,
                             const float* __restrict__ s_p, const int* __restrict__ s_type,
                             const int* __restrict__ hash, ParticleSet dst,
                             unsigned* __restrict__ keys, unsigned* err) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int t = s_type[i];
    dst.rec[2 * (size_t)i] = make_float4(s_pos[3 * i], s_pos[3 * i + 1], s_pos[3 * i + 2], s_p[i]);
    dst.rec[2 * (size_t)i + 1] =
        make_float4(s_vel[3 * i], s_vel[3 * i + 1], s_vel[3 * i + 2], signed_rho(t, s_rho[i]));
    dst.xyz[i] = make_float4(s_pos[3 * i], s_pos[3 * i + 1], s_pos[3 * i + 2],
                             t == SPH_TYPE_FLUID ? 1.f : -1.f);
    dst.type[i] = t;
    int h = hash[i];
    unsigned f = 0;
    if (h < 0 || h >= num_cells) {
        f = SPH_FLAG_OUT_OF_GRID;
        h = h < 0 ? 0 : num_cells - 1;
    }
    keys[i] = (unsigned)h;
    raise_flags(err, f);
}

__global__ void k_ns_writeback(int n, const int* __restrict__ s_type,
                               const float4* __restrict__ self, float* __restrict__ s_rho,
                               float* __restrict__ s_p, float* __restrict__ dofv) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 a = self[i];
    if (s_type[i] != SPH_TYPE_FLUID) {
        s_p[i] = a.x;
        s_rho[i] = a.y;
    }
    dofv[i] = a.z;
}

inline int blocks_for(long n, int t) { return (int)((n + t - 1) / t); }

}  // namespace

// ---------------------------------------------------------------- internal API
int key_bits_for(int num_cells) {
    int b = 1;
    while (b < 31 && (1u << b) < (unsigned)num_cells) b++;
    return b;
}

size_t sort_scratch_bytes(int n) {
    size_t nn = (size_t)(n > 0 ? n : 1);
    size_t tiles = (size_t)(rs_tiles(n) > 0 ? rs_tiles(n) : 1);
    return align256(nn * sizeof(unsigned)) + align256(nn * sizeof(int)) +
           align256((size_t)RS_RADIX * tiles * sizeof(unsigned)) +
           align256((size_t)RS_MAX_PASSES * RS_RADIX * sizeof(unsigned));
}

cudaError_t radix_sort_pairs(const unsigned* keys_in, const int* vals_in, unsigned* keys_out,
                             int* vals_out, int n, int key_bits, void* scratch,
                             size_t scratch_bytes, unsigned* err, cudaStream_t s,
                             const unsigned* gate) {
    if (n <= 0) return cudaSuccess;
    if (key_bits < 1 || key_bits > 32 || !scratch || scratch_bytes < sort_scratch_bytes(n))
        return cudaErrorInvalidValue;
    const int passes = (key_bits + 7) / 8;
    // a gated sort must not need the ungated copies below
    if (gate && passes % 2 == 1 && (keys_in == keys_out || (vals_in && vals_in == vals_out)))
        return cudaErrorInvalidValue;
    SortScratch sc = carve(scratch, n);
    const int tiles = rs_tiles(n);
    const unsigned xm = key_bits == 32 ? 0x80000000u : 0u;  // signed order for full keys
    cudaError_t e = fill_u32(sc.totals, 0u, (long)RS_MAX_PASSES * RS_RADIX, gate, s);
    if (e != cudaSuccess) return e;
    const unsigned* kin = keys_in;
    const int* vin = vals_in;
    // In-place sorts with an odd pass count start from a copy, so no pass reads the buffer it
    // writes.
    if (passes % 2 == 1) {
        if (keys_in == keys_out) {
            e = cudaMemcpyAsync(sc.keys_alt, keys_in, (size_t)n * sizeof(unsigned),
                                cudaMemcpyDeviceToDevice, s);
            if (e != cudaSuccess) return e;
            kin = sc.keys_alt;
        }
        if (vals_in && vals_in == vals_out) {
            e = cudaMemcpyAsync(sc.vals_alt, vals_in, (size_t)n * sizeof(int),
                                cudaMemcpyDeviceToDevice, s);
            if (e != cudaSuccess) return e;
            vin = sc.vals_alt;
        }
    }
    for (int p = 0; p < passes; p++) {
        const bool to_out = ((passes - 1 - p) % 2) == 0;
        unsigned* kdst = to_out ? keys_out : sc.keys_alt;
        int* vdst = to_out ? vals_out : sc.vals_alt;
        const int shift = 8 * p;
        const unsigned xin = (p == 0) ? xm : 0u;
        const unsigned xout = (p == passes - 1) ? xm : 0u;
        unsigned* totals = sc.totals + (size_t)p * RS_RADIX;
        k_rs_upsweep<<<tiles, RS_THREADS, 0, s>>>(kin, n, shift, xin, p == 0 ? key_bits : 32,
                                                   sc.hist, tiles, totals, err, gate);
        k_rs_scan<<<RS_RADIX, RS_THREADS, 0, s>>>(sc.hist, tiles, totals, gate);
        k_rs_downsweep<<<tiles, RS_THREADS, 0, s>>>(kin, vin, kdst, vdst, sc.hist, n, shift, xin,
                                                     xout, tiles, gate);
        kin = kdst;
        vin = vdst;
    }
    return cudaGetLastError();
}

cudaError_t build_cell_starts(const unsigned* sorted_keys, int n, int num_cells, int* cs,
                              cudaStream_t s, const unsigned* gate, const int* type,
                              unsigned char* fluid_cells) {
    cudaError_t e = fill_u32(reinterpret_cast<unsigned*>(cs), 0x7f7f7f7fu, (long)num_cells + 1,
                             gate, s);
    if (e != cudaSuccess) return e;
    if (fluid_cells && type) {
        e = fill_u32(reinterpret_cast<unsigned*>(fluid_cells), 0u, ((long)num_cells + 4) / 4,
                     gate, s);
        if (e != cudaSuccess) return e;
    } else {
        fluid_cells = nullptr;
    }
    if (n > 0)
        k_cell_mark<<<blocks_for(n, 256), 256, 0, s>>>(sorted_keys, n, num_cells, cs, gate, type,
                                                       fluid_cells);
    k_cell_fill<<<blocks_for((long)num_cells + 1, FILL_CHUNK), FILL_THREADS, 0, s>>>(
        cs, num_cells, sorted_keys, n, gate);
    return cudaGetLastError();
}

template <class P>
cudaError_t launch_gather(const KParamsT<typename P::T>& k, const int* perm,
                          const ParticleSetT<typename P::T>& src, ParticleSetT<typename P::T> dst,
                          int with_tmp, const unsigned* keys, cudaStream_t s,
                          const unsigned* gate) {
    if (k.n <= 0) return cudaSuccess;
    if (P::kCodes && perm && !keys) return cudaErrorInvalidValue;
    k_gather<P><<<blocks_for(k.n, 256), 256, 0, s>>>(k, perm, src, dst, with_tmp, keys, gate);
    return cudaGetLastError();
}

template <class P>
cudaError_t launch_upload_convert(const KParamsT<typename P::T>& k, const float* pos,
                                  const float* vel, const float* rho, const float* p,
                                  const int* type, const int* inst_off, int n_inst,
                                  ParticleSetT<typename P::T> dst, unsigned* hash, unsigned* err,
                                  cudaStream_t s) {
    if (k.n <= 0) return cudaSuccess;
    k_upload_convert<P><<<blocks_for(k.n, 256), 256, 0, s>>>(k, pos, vel, rho, p, type, inst_off,
                                                             n_inst, dst, hash, err);
    return cudaGetLastError();
}

template <class P>
cudaError_t launch_upload_sorted(const KParamsT<typename P::T>& k, const float* pos,
                                 const float* vel, const float* rho, const float* p,
                                 const int* type, const unsigned* keys, const float4* xb,
                                 ParticleSetT<typename P::T> dst, unsigned* hash, unsigned* err,
                                 unsigned* disp, unsigned* force, cudaStream_t s) {
    if (k.n <= 0) return cudaSuccess;
    k_upload_sorted<P><<<blocks_for(k.n, 256), 256, 0, s>>>(k, pos, vel, rho, p, type, keys, xb,
                                                            dst, hash, err, disp, force);
    return cudaGetLastError();
}

template <class P>
cudaError_t launch_rehash(const KParamsT<typename P::T>& k, const ParticleSetT<typename P::T>& set,
                          unsigned* hash, unsigned* err, cudaStream_t s) {
    if (k.n <= 0) return cudaSuccess;
    k_rehash<P><<<blocks_for(k.n, 256), 256, 0, s>>>(k, set, hash, err);
    return cudaGetLastError();
}

template <class P>
cudaError_t launch_download_convert(const KParamsT<typename P::T>& k,
                                    const ParticleSetT<typename P::T>& src, float* pos,
                                    float* vel, float* rho, float* p, int* type, cudaStream_t s) {
    if (k.n <= 0) return cudaSuccess;
    k_download_convert<P><<<blocks_for(k.n, 256), 256, 0, s>>>(k.n, src, pos, vel, rho, p, type);
    return cudaGetLastError();
}

template <class P>
cudaError_t launch_download_f64(const KParamsT<typename P::T>& k,
                                const ParticleSetT<typename P::T>& src, double* pos, double* vel,
                                double* rho, double* p, cudaStream_t s) {
    if (k.n <= 0) return cudaSuccess;
    k_download_f64<P><<<blocks_for(k.n, 256), 256, 0, s>>>(k.n, (double)k.rho0, src, pos, vel,
                                                           rho, p);
    return cudaGetLastError();
}

#define SPH_MESH_INSTANTIATE(P)                                                                 \
    template cudaError_t launch_download_f64<P>(const KParamsT<P::T>&, const ParticleSetT<P::T>&,\
                                                double*, double*, double*, double*,             \
                                                cudaStream_t);                                  \
    template cudaError_t launch_gather<P>(const KParamsT<P::T>&, const int*,                    \
                                          const ParticleSetT<P::T>&, ParticleSetT<P::T>, int,   \
                                          const unsigned*, cudaStream_t, const unsigned*);      \
    template cudaError_t launch_upload_convert<P>(const KParamsT<P::T>&, const float*,          \
                                                  const float*, const float*, const float*,     \
                                                  const int*, const int*, int,                  \
                                                  ParticleSetT<P::T>, unsigned*, unsigned*,     \
                                                  cudaStream_t);                                \
    template cudaError_t launch_upload_sorted<P>(const KParamsT<P::T>&, const float*,           \
                                                 const float*, const float*, const float*,      \
                                                 const int*, const unsigned*, const float4*,    \
                                                 ParticleSetT<P::T>, unsigned*, unsigned*,      \
                                                 unsigned*, unsigned*, cudaStream_t);           \
    template cudaError_t launch_rehash<P>(const KParamsT<P::T>&, const ParticleSetT<P::T>&,     \
                                          unsigned*, unsigned*, cudaStream_t);                  \
    template cudaError_t launch_download_convert<P>(const KParamsT<P::T>&,                      \
                                                    const ParticleSetT<P::T>&, float*, float*,  \
                                                    float*, float*, int*, cudaStream_t);
SPH_MESH_INSTANTIATE(PrecF32)
SPH_MESH_INSTANTIATE(PrecF64)
SPH_MESH_INSTANTIATE(PrecMix)
SPH_MESH_INSTANTIATE(PrecMixC)
SPH_MESH_INSTANTIATE(PrecMixA)
#undef SPH_MESH_INSTANTIATE

cudaError_t launch_aos_to_set(const KParams& k, const float* s_pos, const float* s_vel,
                              const float* s_rho, const float* s_p, const int* s_type,
                              const int* hash, ParticleSet dst, unsigned* keys,
                              unsigned* err, cudaStream_t s) {
    if (k.n <= 0) return cudaSuccess;
    k_aos_to_set<<<blocks_for(k.n, 256), 256, 0, s>>>(k.n, k.num_cells, s_pos, s_vel, s_rho, s_p,
                                                      s_type, hash, dst, keys, err);
    return cudaGetLastError();
}

cudaError_t launch_ns_writeback(const KParams& k, const int* s_type, const float4* self,
                                float* s_rho, float* s_p, float* dofv, cudaStream_t s) {
    if (k.n <= 0) return cudaSuccess;
    k_ns_writeback<<<blocks_for(k.n, 256), 256, 0, s>>>(k.n, s_type, self, s_rho, s_p, dofv);
    return cudaGetLastError();
}

}  // namespace sph

// ---------------------------------------------------------------- C ABI (drop-in)
using namespace sph;

extern "C" int sph_calc_hash(const sph_params* p, const float* pos, int* hash, int* index,
                             int n, void* stream) {
    if (!p || n < 0 || (n > 0 && (!pos || !hash || !index))) return SPH_ERR_ARG;
    if (n == 0) return SPH_OK;
    KParams k = make_kparams(*p, n);
    k_calc_hash<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(k, pos, hash, index, n);
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

extern "C" int sph_sort_scratch_bytes(int n, size_t* bytes) {
    if (n < 0 || !bytes) return SPH_ERR_ARG;
    *bytes = sort_scratch_bytes(n);
    return SPH_OK;
}

extern "C" int sph_sort_particles(int* hash, int* index, int n, int key_bits, void* scratch,
                                  size_t scratch_bytes, void* stream) {
    if (n < 0 || key_bits < 1 || key_bits > 32 || (n > 0 && (!hash || !index)))
        return SPH_ERR_ARG;
    if (n <= 1) return SPH_OK;
    if (!scratch || scratch_bytes < sort_scratch_bytes(n)) return SPH_ERR_SCRATCH;
    cudaError_t e = radix_sort_pairs(reinterpret_cast<unsigned*>(hash), index,
                                     reinterpret_cast<unsigned*>(hash), index, n, key_bits,
                                     scratch, scratch_bytes, nullptr, (cudaStream_t)stream);
    return e == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

extern "C" int sph_reorder(const sph_params* p, const float* old_pos, const float* old_vel,
                           const float* old_rho, const float* old_p, const int* old_type,
                           const int* old_zone, float* s_pos, float* s_vel, float* s_rho,
                           float* s_p, int* s_type, int* s_zone, const int* hash,
                           const int* index, int* cell_start, int* cell_end, int n,
                           void* stream) {
    if (!p || n < 0 || !cell_start || !cell_end || p->num_cells <= 0) return SPH_ERR_ARG;
    if (n > 0 && (!old_pos || !old_vel || !old_rho || !old_p || !old_type || !s_pos || !s_vel ||
                  !s_rho || !s_p || !s_type || !hash || !index))
        return SPH_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    // every cell starts empty (src/lib/mesh.cu:149)
    if (cudaMemsetAsync(cell_start, 0xff, (size_t)p->num_cells * sizeof(int), s) != cudaSuccess)
        return SPH_ERR_CUDA;
    if (n == 0) return SPH_OK;
    k_reorder<<<blocks_for(n, 256), 256, 0, s>>>(p->num_cells, old_pos, old_vel, old_rho, old_p,
                                                 old_type, old_zone, s_pos, s_vel, s_rho, s_p,
                                                 s_type, s_zone, hash, index, cell_start, cell_end,
                                                 n);
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

extern "C" int sph_recover(float* pos, float* vel, float* rho, float* p, int n, const int* index,
                           int* type, int* zone, const float* s_pos, const float* s_vel,
                           const float* s_rho, const float* s_p, const int* s_type,
                           const int* s_zone, void* stream) {
    if (n < 0) return SPH_ERR_ARG;
    if (n == 0) return SPH_OK;
    if (!pos || !vel || !rho || !p || !index || !type || !s_pos || !s_vel || !s_rho || !s_p ||
        !s_type)
        return SPH_ERR_ARG;
    k_recover<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(
        pos, vel, rho, p, index, type, zone, s_pos, s_vel, s_rho, s_p, s_type, s_zone, n);
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}
