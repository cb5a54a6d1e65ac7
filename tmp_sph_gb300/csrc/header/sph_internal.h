// sph_internal.h — host-side declarations shared by the library's translation units:
// the resident-solver context and the launchers each .cu file provides.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "sph_gb300.h"
#include "sph_device.cuh"

namespace sph {

// ---------------------------------------------------------------- radix sort (lib/mesh.cu)
// Stable LSD radix sort of 32-bit unsigned keys with int values, 8-bit digits, keys sorted on
// bits [0, key_bits).  Scratch layout and size come from sort_scratch_bytes(); no allocation.
// vals_in == NULL means the values are the identity 0..n-1.  The sorted output lands in
// keys_out / vals_out (which may alias keys_in / vals_in).  err (may be NULL) receives
// SPH_FLAG_KEY_RANGE if a key has bits at or above key_bits.
size_t sort_scratch_bytes(int n);
// gate: see gated_off() — NULL sorts unconditionally.
cudaError_t radix_sort_pairs(const unsigned* keys_in, const int* vals_in, unsigned* keys_out,
                             int* vals_out, int n, int key_bits, void* scratch,
                             size_t scratch_bytes, unsigned* err, cudaStream_t s,
                             const unsigned* gate = nullptr);
int key_bits_for(int num_cells);

// ---------------------------------------------------------------- cell list (lib/mesh.cu)
// Dense cell starts: cell_start[c] = first sorted slot whose key >= c, for c in [0, C];
// cell_start[C] = n.  Keys must be sorted and < C.
cudaError_t build_cell_starts(const unsigned* sorted_keys, int n, int num_cells,
                              int* cell_start, cudaStream_t s, const unsigned* gate = nullptr);

// ---------------------------------------------------------------- resident state
// One particle set.  rec holds two float4 per particle, rec[2i] = (x, y, z, p) and
// rec[2i+1] = (vx, vy, vz, ±rho) with rho negated for boundary (non-fluid) particles: one
// aligned 32-byte record, the unit a neighbour gather reads.  type keeps the particle kind as
// given (0 wall, 1 fluid, 2 rigid, ...), id the original particle index; tpos/tvel hold the
// predictor's saved step-n state (x, y, z, rho) / (vx, vy, vz, 0).
struct ParticleSet {
    float4* rec = nullptr;
    float4* xyz = nullptr;  // sorted set only: dense (x, y, z, ±1) for candidate walks
    int* type = nullptr;
    int* id = nullptr;
    float4* tpos = nullptr;
    float4* tvel = nullptr;
};

// Pass-1 output.  nrec[2i] = (x, y, z, q) with q = p' - rho0 cs h dofv for fluid particles and
// q = p' for boundary particles, nrec[2i+1] = (vx, vy, vz, ±rho'): the record pass 2 gathers per
// neighbour.  self[i] = (p', rho', dofv, 0): the particle's own side.
struct Pass1Out {
    float4* nrec = nullptr;
    float4* self = nullptr;
};

enum HalfStep { HALF_PREDICT = 0, HALF_CORRECT = 1 };

// Per-half-step neighbour list: idx[i * cap + c] is the c-th neighbour of slot i (walk
// order), count[i] how many; count[i] > cap means the list overflowed for i and the passes
// walk the cells for it instead.  cap is a multiple of 16 (rows are 16-byte aligned).
// The list holds every pair closer than the list cutoff (KParams::kh2_list, the support
// radius plus a skin); xb (may be NULL) receives each slot's position when the list is built,
// from which the integrator tracks how far particles have moved since.
// Neighbour list: slot c of particle i at idx[(i / 32) * cap * 32 + c * 32 + i % 32] (each warp
// of 32 consecutive particles owns a block of cap x 32 slots), count[i] entries, and xb[i]
// the position i had when the list was built.
struct NbrList {
    int* idx = nullptr;
    int* count = nullptr;
    int cap = 0;
    float4* xb = nullptr;
};
// List slots per particle: 1.5x the lattice particles within kh (1 + skin), rounded up to 16.
int nbr_capacity_for(const sph_params& p, double skin = 0.0);

// Neighbour passes (equation/ns.cu).  nl == NULL walks the cells in every pass.
//  build : fills nl for the sorted set (walls keep only fluid neighbours unless walls_all).
//  pass 1: fills a Pass1Out — boundary particles get the extrapolated p and rho, fluid
//          particles their own p, rho and the velocity divergence.  rhop_sum / w_sum are
//          written when non-NULL.
//  pass 2: either rates only (rho_dt, AoS vel_dt) or rates + the predictor/corrector update
//          written into `out` (slot-aligned with `in`) with the next cell hash.
cudaError_t launch_nbr_build(const KParams& k, const ParticleSet& in, const unsigned* sorted_keys,
                             const int* cell_start, const NbrList& nl, int walls_all,
                             unsigned* err, cudaStream_t s, const unsigned* gate = nullptr);
cudaError_t launch_pass1(const KParams& k, const ParticleSet& in, const unsigned* sorted_keys,
                         const int* cell_start, const NbrList* nl, const Pass1Out& out,
                         float* rhop_sum, float* w_sum, cudaStream_t s);
cudaError_t launch_pass2_rates(const KParams& k, const ParticleSet& in,
                               const unsigned* sorted_keys, const int* cell_start,
                               const NbrList* nl, const Pass1Out& p1, float* rho_dt,
                               float* vel_dt, int wall_rates, cudaStream_t s);
// `out` may be `in` (the update is per particle; neighbours are read from p1).  disp (may be
// NULL) receives, by atomicMax on its float bits, the largest squared distance of a fluid
// particle from its position when the list was built (nl->xb).
cudaError_t launch_pass2_step(const KParams& k, HalfStep half, const ParticleSet& in,
                              const unsigned* sorted_keys, const int* cell_start,
                              const NbrList* nl, const Pass1Out& p1, ParticleSet out,
                              unsigned* out_hash, unsigned* err, unsigned* disp, cudaStream_t s);

// Resident-state glue (lib/mesh.cu).
// perm == NULL copies slot for slot.
cudaError_t launch_gather(const KParams& k, const int* perm, const ParticleSet& src,
                          ParticleSet dst, int with_tmp, cudaStream_t s,
                          const unsigned* gate = nullptr);
// Recompute the cell keys of `set` on the grid of `k` (k.n particles).
cudaError_t launch_rehash(const KParams& k, const ParticleSet& set, unsigned* hash, unsigned* err,
                          cudaStream_t s);
cudaError_t launch_upload_convert(const KParams& k, const float* pos, const float* vel,
                                  const float* rho, const float* p, const int* type,
                                  ParticleSet dst, unsigned* hash, unsigned* err,
                                  cudaStream_t s);
cudaError_t launch_download_convert(const KParams& k, const ParticleSet& src, float* pos,
                                    float* vel, float* rho, float* p, int* type,
                                    cudaStream_t s);
// Drop-in sph_ns glue: AoS sorted arrays -> SoA set (and back for the outputs).
cudaError_t launch_aos_to_set(const KParams& k, const float* s_pos, const float* s_vel,
                              const float* s_rho, const float* s_p, const int* s_type,
                              const int* hash, ParticleSet dst, unsigned* keys,
                              unsigned* err, cudaStream_t s);
cudaError_t launch_ns_writeback(const KParams& k, const int* s_type, const float4* self,
                                float* s_rho, float* s_p, float* dofv, cudaStream_t s);

// Per-phase device timing of sph_step (SPH_OPT_PROFILE).
enum Phase { PH_SORT = 0, PH_GATHER, PH_NBR, PH_PASS1, PH_PASS2, PH_COUNT };

}  // namespace sph

// The resident-solver context (sph/solver.cu).
struct sph_ctx {
    sph_params P{};
    int capacity = 0;
    int n = 0;
    int device = 0;
    bool loaded = false;
    bool rehash = false;  // the grid changed since the keys in hash_x were computed
    long long steps = 0;

    sph::ParticleSet x;   // integrator output, slot-aligned with the previous sorted order
    sph::ParticleSet y;   // cell-sorted order the neighbour passes read
    unsigned* hash_x = nullptr;      // next cell of every slot of x
    unsigned* keys_sorted = nullptr; // sorted cell keys of y
    int* perm = nullptr;             // y slot k came from x slot perm[k]
    sph::Pass1Out p1;                // pass-1 output
    int* cell_start = nullptr;       // [num_cells + 1]
    int cell_capacity = 0;
    void* sort_scratch = nullptr;
    size_t sort_scratch_bytes = 0;
    unsigned* err = nullptr;         // device error word

    // neighbour list, reused across half steps while every particle stays within skin/2 of
    // where it was when the list was built
    sph::NbrList nl;
    sph_params Pi{};                 // internal grid: cells of kh (1 + skin)
    double skin = 0.1;               // list skin as a fraction of the support radius kh
    unsigned* rb = nullptr;          // [0] rebuild gate, [1] max squared displacement (float
                                     // bits), [2] forced rebuild, [3] rebuild count

    // graph replay of one full step
    int opt_use_graph = 1;
    int opt_wall_rates = 0;
    int opt_profile = 0;
    int opt_nbr_list = 1;
    int opt_nbr_cap = 0;  // 0: nbr_capacity_for(P)
    int opt_cond_graph = 1;  // graph replay skips the rebuild kernels through conditional nodes
    cudaGraphExec_t graph = nullptr;
    cudaStream_t graph_stream = nullptr;
    int graph_n = -1;
    bool graph_conditional = false;  // rebuild kernels under conditional nodes
    cudaStream_t side_stream = nullptr;  // captures the conditional bodies
    // profiling events (PH_COUNT + 1 per half step) / accumulated milliseconds per phase
    cudaEvent_t ev[2 * (sph::PH_COUNT + 1)] = {};
    double phase_ms[sph::PH_COUNT] = {};
    long long phase_launches[sph::PH_COUNT] = {};
};
