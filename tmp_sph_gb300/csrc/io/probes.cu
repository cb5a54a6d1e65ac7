// probes.cu — measurements of the resident state on the GPU: pressure probes, water-height
// gauges, the surge front and FP64 global reductions (mass, energy, extreme speed and density,
// the CFL step).
//
// Reference counterpart: output_fluid_file (src/io/io.cu:154-279) copies the whole state to
// the host every output interval and scans it there for the gauge heights (the largest z of
// fluid particles within 1.5 dx of a vertical line) and reads the pressure of four fixed
// particle indices.  Here one kernel scans the state where it lives and returns a few numbers;
// a pressure probe is a Shepard-normalised kernel average over the fluid around a point
// instead of the pressure of one particle, which has no fixed position in a Lagrangian flow.
//
// One launch of at most four blocks per SM strides over all particles.  Sums are
// accumulated in FP64: per thread, then per warp with shuffles, per block in shared memory,
// then one global atomic per block and quantity.  Extremes use the order-preserving map of a
// double onto a 64-bit unsigned integer, so atomicMax/atomicMin on the integers order the
// doubles.
#include <cuda_runtime.h>

#include <cstring>

#include "sph_internal.h"

namespace sph {

namespace {

constexpr int PROBE_THREADS = 256;

struct ProbeSet {
    sph_probe p[SPH_MAX_PROBES];
    int n;
};

__device__ __forceinline__ unsigned long long ord(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ double warp_min(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}

// Block reduction of one value with the warp reduction `op` (identity `id`), result valid in
// thread 0.  The leading barrier lets consecutive reductions reuse s_buf.
template <class Op>
__device__ __forceinline__ double block_reduce(double v, double* s_buf, Op op, double id) {
    v = op(v);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) s_buf[w] = v;
    __syncthreads();
    double r = id;
    if (w == 0) {
        r = lane < PROBE_THREADS / 32 ? s_buf[lane] : id;
        r = op(r);
    }
    return r;
}

// Accumulator layout (doubles / 64-bit words), ACC_WORDS in total:
enum {
    A_MASS = 0, A_KIN, A_POT, A_FLUID, A_PARKED,  // sums (doubles; counts summed as doubles)
    A_VMAX, A_RHOMAX, A_RHOMIN, A_FRONT,          // extremes (ordered 64-bit words)
    A_PROBE,                                      // per probe: num, den (doubles), max (word)
    ACC_WORDS = A_PROBE + 3 * SPH_MAX_PROBES
};

template <class P>
__global__ void __launch_bounds__(PROBE_THREADS)
k_probes(KParamsT<typename P::T> k, ParticleSetT<typename P::T> set, ProbeSet probes,
         double* __restrict__ acc) {
    __shared__ double s_buf[PROBE_THREADS / 32];
    __shared__ double s_num[SPH_MAX_PROBES], s_den[SPH_MAX_PROBES];
    __shared__ unsigned long long s_max[SPH_MAX_PROBES];
    for (int q = threadIdx.x; q < probes.n; q += blockDim.x) {
        s_num[q] = 0.0;
        s_den[q] = 0.0;
        s_max[q] = 0ull;
    }
    __syncthreads();
    const double mass = (double)k.mass, g = (double)k.g;
    const double kh2 = (double)k.kh * (double)k.kh, inv_h = 1.0 / (double)k.h;
    double mass_s = 0.0, kin = 0.0, pot = 0.0, fluid = 0.0, parked = 0.0;
    double vmax = 0.0, rmax = -1.0e300, rmin = 1.0e300, front = -1.0e300;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < k.n;
         i += (long)gridDim.x * blockDim.x) {
        const auto a = set.rec[2 * (size_t)i];
        const auto v = set.rec[2 * (size_t)i + 1];
        if (!(v.w > 0)) continue;  // fluid only
        double x = (double)a.x, y = (double)a.y, z = (double)a.z, rho = (double)v.w;
        if constexpr (P::kMixed) {
            const dvec4 xm = set.xm[i];  // FP64 position and rho - rho0
            x = xm.x;
            y = xm.y;
            z = xm.z;
            rho = (double)k.rho0 + xm.w;
        }
        const double vx = v.x, vy = v.y, vz = v.z, pr = a.w;
        const double v2 = vx * vx + vy * vy + vz * vz;
        fluid += 1.0;
        if (x == (double)k.park_x && y == (double)k.park_y && z == (double)k.park_z) parked += 1.0;
        mass_s += mass;
        kin += 0.5 * mass * v2;
        pot += -mass * g * z;
        vmax = fmax(vmax, sqrt(v2));
        rmax = fmax(rmax, rho);
        rmin = fmin(rmin, rho);
        front = fmax(front, x);
        for (int q = 0; q < probes.n; q++) {
            const sph_probe& pb = probes.p[q];
            if (pb.kind == SPH_PROBE_PRESSURE) {
                const double dx = x - pb.x, dy = y - pb.y, dz = z - pb.z;
                const double r2 = dx * dx + dy * dy + dz * dz;
                if (r2 < kh2) {
                    const double s = sqrt(r2) * inv_h, t = 1.0 - 0.5 * s;
                    const double w = (double)k.adh * t * t * t * t * (2.0 * s + 1.0);
                    atomicAdd(&s_num[q], pr * w);
                    atomicAdd(&s_den[q], w);
                }
            } else if (pb.kind == SPH_PROBE_HEIGHT) {
                if (fabs(x - pb.x) < pb.radius && fabs(y - pb.y) < pb.radius &&
                    (pb.zmax <= 0.f || z < pb.zmax))
                    atomicMax(&s_max[q], ord(z));
            }
        }
    }
    // block reductions, one global atomic per quantity
    const double b_mass = block_reduce(mass_s, s_buf, warp_sum, 0.0);
    const double b_kin = block_reduce(kin, s_buf, warp_sum, 0.0);
    const double b_pot = block_reduce(pot, s_buf, warp_sum, 0.0);
    const double b_fluid = block_reduce(fluid, s_buf, warp_sum, 0.0);
    const double b_parked = block_reduce(parked, s_buf, warp_sum, 0.0);
    const double b_vmax = block_reduce(vmax, s_buf, warp_max, 0.0);
    const double b_rmax = block_reduce(rmax, s_buf, warp_max, -1.0e300);
    const double b_rmin = block_reduce(rmin, s_buf, warp_min, 1.0e300);
    const double b_front = block_reduce(front, s_buf, warp_max, -1.0e300);
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long* u = reinterpret_cast<unsigned long long*>(acc);
        atomicAdd(&acc[A_MASS], b_mass);
        atomicAdd(&acc[A_KIN], b_kin);
        atomicAdd(&acc[A_POT], b_pot);
        atomicAdd(&acc[A_FLUID], b_fluid);
        atomicAdd(&acc[A_PARKED], b_parked);
        if (b_fluid > 0.0) {
            atomicMax(&u[A_VMAX], ord(b_vmax));
            atomicMax(&u[A_RHOMAX], ord(b_rmax));
            atomicMin(&u[A_RHOMIN], ord(b_rmin));
            atomicMax(&u[A_FRONT], ord(b_front));
        }
    }
    for (int q = threadIdx.x; q < probes.n; q += blockDim.x) {
        unsigned long long* u = reinterpret_cast<unsigned long long*>(acc);
        if (s_den[q] != 0.0) {
            atomicAdd(&acc[A_PROBE + 3 * q], s_num[q]);
            atomicAdd(&acc[A_PROBE + 3 * q + 1], s_den[q]);
        }
        if (s_max[q]) atomicMax(&u[A_PROBE + 3 * q + 2], s_max[q]);
    }
}

inline double unord(unsigned long long u) {
    const unsigned long long b = (u >> 63) ? (u & 0x7fffffffffffffffull) : ~u;
    double d;
    memcpy(&d, &b, sizeof(d));
    return d;
}

}  // namespace

size_t probe_acc_words() { return ACC_WORDS; }

template <class P>
cudaError_t launch_probes(const KParamsT<typename P::T>& k, const ParticleSetT<typename P::T>& set,
                          const sph_probe* probes, int nprobes, double* acc, cudaStream_t s) {
    if (nprobes < 0 || nprobes > SPH_MAX_PROBES) return cudaErrorInvalidValue;
    ProbeSet ps{};
    for (int q = 0; q < nprobes; q++) ps.p[q] = probes[q];
    ps.n = nprobes;
    cudaError_t e = cudaMemsetAsync(acc, 0, ACC_WORDS * sizeof(double), s);
    if (e == cudaSuccess)  // rho_min starts at the largest ordered word
        e = cudaMemsetAsync(acc + A_RHOMIN, 0xff, sizeof(double), s);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long blocks = ((long)k.n + PROBE_THREADS - 1) / PROBE_THREADS;
    const long cap = 4L * (sms > 0 ? sms : 1);
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    k_probes<P><<<(int)blocks, PROBE_THREADS, 0, s>>>(k, set, ps, acc);
    return cudaGetLastError();
}

void probe_results(const double* acc, const sph_probe* probes, int nprobes, double cfl, double h,
                   double cs, sph_stats* stats, double* values) {
    const unsigned long long* u = reinterpret_cast<const unsigned long long*>(acc);
    const bool any = acc[A_FLUID] > 0.0;
    if (stats) {
        stats->fluid = (long long)acc[A_FLUID];
        stats->parked = (long long)acc[A_PARKED];
        stats->mass = acc[A_MASS];
        stats->kinetic = acc[A_KIN];
        stats->potential = acc[A_POT];
        stats->max_speed = any ? unord(u[A_VMAX]) : 0.0;
        stats->rho_max = any ? unord(u[A_RHOMAX]) : 0.0;
        stats->rho_min = any ? unord(u[A_RHOMIN]) : 0.0;
        stats->front_x = any ? unord(u[A_FRONT]) : 0.0;
        stats->cfl_dt = cfl * h / (cs + stats->max_speed);
    }
    for (int q = 0; values && q < nprobes; q++) {
        const double num = acc[A_PROBE + 3 * q], den = acc[A_PROBE + 3 * q + 1];
        const unsigned long long m = u[A_PROBE + 3 * q + 2];
        if (probes[q].kind == SPH_PROBE_FRONT)
            values[q] = any ? unord(u[A_FRONT]) : 0.0;
        else if (probes[q].kind == SPH_PROBE_PRESSURE)
            values[q] = den != 0.0 ? num / den : 0.0;
        else
            values[q] = m ? unord(m) : 0.0;
    }
}

#define SPH_PROBE_INSTANTIATE(P)                                                                \
    template cudaError_t launch_probes<P>(const KParamsT<P::T>&, const ParticleSetT<P::T>&,     \
                                          const sph_probe*, int, double*, cudaStream_t);
SPH_PROBE_INSTANTIATE(PrecF32)
SPH_PROBE_INSTANTIATE(PrecF64)
SPH_PROBE_INSTANTIATE(PrecMix)
SPH_PROBE_INSTANTIATE(PrecMixC)
SPH_PROBE_INSTANTIATE(PrecMixA)
#undef SPH_PROBE_INSTANTIATE

}  // namespace sph
