// integrator.cu — midpoint predictor-corrector on the reference's sorted AoS arrays.
//
// Reference counterparts: PC_predictionD / PC_prediction (src/sph/sph_run.cu:425-470,521-535)
// and PC_correctionD / PC_correction (src/sph/sph_run.cu:473-519,537-550).  Only fluid
// particles (kind 1) are advanced; a fluid particle outside the escape box is parked with
// zero velocity, zero pressure and rest density; the step-n state is saved at (and read
// from) the particle's original index.  The resident solver fuses the same update into the
// second neighbour pass (equation/ns.cu).
#include <cuda_runtime.h>

#include "sph_internal.h"

namespace sph {
namespace {

__device__ __forceinline__ void park(const KParams& k, float* s_pos, float* s_vel, float* s_rho,
                                     float* s_p, int i) {
    s_pos[3 * i] = k.park_x;
    s_pos[3 * i + 1] = k.park_y;
    s_pos[3 * i + 2] = k.park_z;
    s_vel[3 * i] = 0.f;
    s_vel[3 * i + 1] = 0.f;
    s_vel[3 * i + 2] = 0.f;
    s_p[i] = 0.f;
    s_rho[i] = k.rho0;
}

__global__ void k_pc_prediction(KParams k, float* __restrict__ s_pos, float* __restrict__ s_vel,
                                float* __restrict__ s_rho, float* __restrict__ s_p,
                                const float* __restrict__ rho_dt,
                                const float* __restrict__ vel_dt,
                                const int* __restrict__ index, float* __restrict__ pos_tmp,
                                float* __restrict__ vel_tmp, float* __restrict__ rho_tmp,
                                const int* __restrict__ s_type) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.n || s_type[i] != SPH_TYPE_FLUID) return;
    const float x = s_pos[3 * i], y = s_pos[3 * i + 1], z = s_pos[3 * i + 2];
    if (escaped(k, x, y, z)) {
        park(k, s_pos, s_vel, s_rho, s_p, i);
        return;
    }
    const int r = index[i];
    if ((unsigned)r >= (unsigned)k.n) return;
    const float vx = s_vel[3 * i], vy = s_vel[3 * i + 1], vz = s_vel[3 * i + 2];
    const float rho0 = s_rho[i];
    pos_tmp[3 * r] = x; pos_tmp[3 * r + 1] = y; pos_tmp[3 * r + 2] = z;
    vel_tmp[3 * r] = vx; vel_tmp[3 * r + 1] = vy; vel_tmp[3 * r + 2] = vz;
    rho_tmp[r] = rho0;
    float rho = rho0 + rho_dt[i] * k.half_dt;
    if (k.clamp_density && rho < k.rho0) rho = k.rho0;
    s_rho[i] = rho;
    s_pos[3 * i] = x + vx * k.half_dt;
    s_pos[3 * i + 1] = y + vy * k.half_dt;
    s_pos[3 * i + 2] = z + vz * k.half_dt;
    s_vel[3 * i] = vx + vel_dt[3 * i] * k.half_dt;
    s_vel[3 * i + 1] = vy + vel_dt[3 * i + 1] * k.half_dt;
    s_vel[3 * i + 2] = vz + vel_dt[3 * i + 2] * k.half_dt;
    s_p[i] = eos_pressure(k, rho);
}

__global__ void k_pc_correction(KParams k, float* __restrict__ s_pos, float* __restrict__ s_vel,
                                float* __restrict__ s_rho, float* __restrict__ s_p,
                                const float* __restrict__ rho_dt,
                                const float* __restrict__ vel_dt,
                                const int* __restrict__ index,
                                const float* __restrict__ pos_tmp,
                                const float* __restrict__ vel_tmp,
                                const float* __restrict__ rho_tmp,
                                const int* __restrict__ s_type) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.n || s_type[i] != SPH_TYPE_FLUID) return;
    if (escaped(k, s_pos[3 * i], s_pos[3 * i + 1], s_pos[3 * i + 2])) {
        park(k, s_pos, s_vel, s_rho, s_p, i);
        return;
    }
    const int r = index[i];
    if ((unsigned)r >= (unsigned)k.n) return;
    const float rn = rho_tmp[r];
    float rho = rn + rho_dt[i] * k.half_dt;
    if (k.clamp_density && rho < k.rho0) rho = k.rho0;
    rho = 2.f * rho - rn;
    if (k.clamp_density && rho < k.rho0) rho = k.rho0;
    s_rho[i] = rho;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const float xn = pos_tmp[3 * r + c], vn = vel_tmp[3 * r + c];
        const float xs = xn + s_vel[3 * i + c] * k.half_dt;  // uses v at the half step
        const float vs = vn + vel_dt[3 * i + c] * k.half_dt;
        s_pos[3 * i + c] = 2.f * xs - xn;
        s_vel[3 * i + c] = 2.f * vs - vn;
    }
    s_p[i] = eos_pressure(k, rho);
}

inline int blocks_for(long n, int t) { return (int)((n + t - 1) / t); }

}  // namespace
}  // namespace sph

using namespace sph;

extern "C" int sph_pc_prediction(const sph_params* p, float* s_pos, float* s_vel, float* s_rho,
                                 float* s_p, const float* rho_dt, const float* vel_dt,
                                 const int* index, float* pos_tmp, float* vel_tmp,
                                 float* rho_tmp, int n, const int* s_type, void* stream) {
    if (!p || n < 0) return SPH_ERR_ARG;
    if (n == 0) return SPH_OK;
    if (!s_pos || !s_vel || !s_rho || !s_p || !rho_dt || !vel_dt || !index || !pos_tmp ||
        !vel_tmp || !rho_tmp || !s_type)
        return SPH_ERR_ARG;
    KParams k = make_kparams(*p, n);
    k_pc_prediction<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(
        k, s_pos, s_vel, s_rho, s_p, rho_dt, vel_dt, index, pos_tmp, vel_tmp, rho_tmp, s_type);
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

extern "C" int sph_pc_correction(const sph_params* p, float* s_pos, float* s_vel, float* s_rho,
                                 float* s_p, const float* rho_dt, const float* vel_dt,
                                 const int* index, const float* pos_tmp, const float* vel_tmp,
                                 const float* rho_tmp, int n, const int* s_type, void* stream) {
    if (!p || n < 0) return SPH_ERR_ARG;
    if (n == 0) return SPH_OK;
    if (!s_pos || !s_vel || !s_rho || !s_p || !rho_dt || !vel_dt || !index || !pos_tmp ||
        !vel_tmp || !rho_tmp || !s_type)
        return SPH_ERR_ARG;
    KParams k = make_kparams(*p, n);
    k_pc_correction<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(
        k, s_pos, s_vel, s_rho, s_p, rho_dt, vel_dt, index, pos_tmp, vel_tmp, rho_tmp, s_type);
    return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}
