// ref_shim.cu — the reference's own host-function signatures (C++ linkage), forwarding to
// the C ABI, so a reference driver links against this library unchanged apart from one
// sph_shim_set_reference_params() call after its cudaMemcpyToSymbol of the parameters.
//
// Signatures: src/header/mesh.cuh:14-33, src/header/ns.cuh:4, src/header/sph.cuh:26-28.
// The reference functions return nothing and report launch errors on stdout
// (src/lib/mesh.cu:64-69); these do the same, through sph_status_string.  They run on the
// legacy default stream, as the reference's do.  The sort and the neighbour passes need
// scratch; it is allocated on first use (as thrust does inside the reference's
// sortParticles) and grown when a call needs more.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "sph_internal.h"

struct SimParams;  // the reference's parameter struct, layout-compatible with sph_ref_simparams

namespace {

struct ShimState {
    std::mutex mu;
    bool have_params = false;
    sph_params P{};
    sph_ctx* ctx = nullptr;
    int ctx_capacity = 0;
    void* sort_scratch = nullptr;
    size_t sort_bytes = 0;
};

ShimState& shim() {
    static ShimState s;
    return s;
}

void report(const char* what, int st) {
    if (st != SPH_OK) std::printf("%s failed: %s\n", what, sph_status_string(st));
}

bool ensure_ctx(ShimState& s, int n) {
    if (s.ctx && s.ctx_capacity >= n) return sph_set_params(s.ctx, &s.P) == SPH_OK;
    if (s.ctx) sph_destroy(s.ctx);
    s.ctx = nullptr;
    sph_params p = s.P;
    p.num_particles = n;
    if (sph_create(&p, n, &s.ctx) != SPH_OK) return false;
    s.ctx_capacity = n;
    return true;
}

}  // namespace

extern "C" int sph_shim_set_reference_params(const sph_ref_simparams* p) {
    ShimState& s = shim();
    std::lock_guard<std::mutex> lk(s.mu);
    sph_params P;
    int st = sph_params_from_reference(p, &P);
    if (st != SPH_OK) return st;
    s.P = P;
    s.have_params = true;
    return SPH_OK;
}

extern "C" int sph_shim_set_params(const sph_params* p) {
    if (!p) return SPH_ERR_ARG;
    ShimState& s = shim();
    std::lock_guard<std::mutex> lk(s.mu);
    s.P = *p;
    s.have_params = true;
    return SPH_OK;
}

extern "C" int sph_shim_release(void) {
    ShimState& s = shim();
    std::lock_guard<std::mutex> lk(s.mu);
    if (s.ctx) sph_destroy(s.ctx);
    s.ctx = nullptr;
    s.ctx_capacity = 0;
    cudaFree(s.sort_scratch);
    s.sort_scratch = nullptr;
    s.sort_bytes = 0;
    return SPH_OK;
}

// --- the reference's declarations, reproduced because the shim must match them exactly ---

int iDivUp(int a, int b) { return a % b != 0 ? a / b + 1 : a / b; }

void computeGridSize(int n, int blockSize, int& numBlocks, int& numThreads) {
    numThreads = blockSize < n ? blockSize : n;
    numBlocks = numThreads > 0 ? iDivUp(n, numThreads) : 0;
}

void calcHash(float* pos, int* particleHash, int* particleIndex, int numParticles) {
    ShimState& s = shim();
    std::lock_guard<std::mutex> lk(s.mu);
    if (!s.have_params) return report("calcHashD launch", SPH_ERR_STATE);
    report("calcHashD launch", sph_calc_hash(&s.P, pos, particleHash, particleIndex, numParticles, nullptr));
}

void sortParticles(int* particleHash, int* particleIndex, int numParticles) {
    ShimState& s = shim();
    std::lock_guard<std::mutex> lk(s.mu);
    size_t need = 0;
    sph_sort_scratch_bytes(numParticles, &need);
    if (need > s.sort_bytes) {
        cudaFree(s.sort_scratch);
        s.sort_scratch = nullptr;
        s.sort_bytes = 0;
        if (cudaMalloc(&s.sort_scratch, need) != cudaSuccess) return report("sortParticles", SPH_ERR_NOMEM);
        s.sort_bytes = need;
    }
    // all 32 key bits, signed order: the same permutation thrust::sort_by_key gives
    report("sortParticles", sph_sort_particles(particleHash, particleIndex, numParticles, 32,
                                               s.sort_scratch, s.sort_bytes, nullptr));
}

void reorder(float* oldPos, float* oldVel, float* olddensity, float* oldpressure,
             int* oldparticle_type, int* oldparticle_zone, float* sortedPos, float* sortedVel,
             float* sorteddensity, float* sortedpressure, int* sortedparticle_type,
             int* sortedparticle_zone, int* particleHash, int* particleIndex, int* dcellStart,
             int* dCellEnd, int numParticles, SimParams* temps) {
    ShimState& s = shim();
    std::lock_guard<std::mutex> lk(s.mu);
    if (temps) {
        // the reference's reorder reads only temps->numCells (src/lib/mesh.cu:149)
        const sph_ref_simparams* r = reinterpret_cast<const sph_ref_simparams*>(temps);
        if (s.have_params)
            s.P.num_cells = r->numCells;
        else if (sph_params_from_reference(r, &s.P) == SPH_OK)
            s.have_params = true;
    }
    if (!s.have_params) return report("reorderD launch", SPH_ERR_STATE);
    report("reorderD launch",
           sph_reorder(&s.P, oldPos, oldVel, olddensity, oldpressure, oldparticle_type,
                       oldparticle_zone, sortedPos, sortedVel, sorteddensity, sortedpressure,
                       sortedparticle_type, sortedparticle_zone, particleHash, particleIndex,
                       dcellStart, dCellEnd, numParticles, nullptr));
}

void recover(float* d_pos, float* d_vel, float* d_density, float* d_pressure, int numParticles,
             int* d_particleIndex, int* d_particle_type, int* d_particle_zone, float* d_sortedpos,
             float* d_sortedvel, float* d_sorteddensity, float* d_sortedpressure,
             int* d_sorted_particle_type, int* d_sorted_particle_zone) {
    report("recoverD launch",
           sph_recover(d_pos, d_vel, d_density, d_pressure, numParticles, d_particleIndex,
                       d_particle_type, d_particle_zone, d_sortedpos, d_sortedvel, d_sorteddensity,
                       d_sortedpressure, d_sorted_particle_type, d_sorted_particle_zone, nullptr));
}

void SPH_NS_simpleversion(float* sortedPos, float* sortedVel, float* sorteddensity,
                          float* sortedpressure, int* sorted_particle_type, float* densitydt,
                          float* Veldt, int* cellStart, int* cellEnd, int numParticles,
                          int* particleHash, int timestep, float* dofv, float* rhop_sum,
                          float* w_sum) {
    (void)timestep;
    ShimState& s = shim();
    std::lock_guard<std::mutex> lk(s.mu);
    if (!s.have_params) return report("SPH_NS launch", SPH_ERR_STATE);
    if (!ensure_ctx(s, numParticles)) return report("SPH_NS launch", SPH_ERR_NOMEM);
    report("SPH_NS launch",
           sph_ns(s.ctx, sortedPos, sortedVel, sorteddensity, sortedpressure, sorted_particle_type,
                  densitydt, Veldt, cellStart, cellEnd, numParticles, particleHash, dofv, rhop_sum,
                  w_sum, nullptr));
}

void PC_prediction(float* sortedPos, float* sortedVel, float* sorteddensity, float* sortedpressure,
                   float* densitydt, float* Veldt, int* particleHash, int* particleIndex,
                   float* Pos_tmp, float* Vel_tmp, float* density_tmp, int numParticles,
                   int* sorted_particle_type) {
    (void)particleHash;
    ShimState& s = shim();
    std::lock_guard<std::mutex> lk(s.mu);
    if (!s.have_params) return report("PC_predictionD launch", SPH_ERR_STATE);
    report("PC_predictionD launch",
           sph_pc_prediction(&s.P, sortedPos, sortedVel, sorteddensity, sortedpressure, densitydt,
                             Veldt, particleIndex, Pos_tmp, Vel_tmp, density_tmp, numParticles,
                             sorted_particle_type, nullptr));
}

void PC_correction(float* sortedPos, float* sortedVel, float* sorteddensity, float* sortedpressure,
                   float* densitydt, float* Veldt, int* particleHash, int* particleIndex,
                   float* Pos_tmp, float* Vel_tmp, float* density_tmp, int numParticles,
                   int* sorted_particle_type) {
    (void)particleHash;
    ShimState& s = shim();
    std::lock_guard<std::mutex> lk(s.mu);
    if (!s.have_params) return report("PC_correctionD launch", SPH_ERR_STATE);
    report("PC_correctionD launch",
           sph_pc_correction(&s.P, sortedPos, sortedVel, sorteddensity, sortedpressure, densitydt,
                             Veldt, particleIndex, Pos_tmp, Vel_tmp, density_tmp, numParticles,
                             sorted_particle_type, nullptr));
}
