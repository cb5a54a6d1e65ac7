// sph_internal.h — host-side declarations shared by the library's translation units:
// the resident-solver context and the launchers each .cu file provides.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <vector>

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
// cell_start[C] = n.  Keys must be sorted and < C.  With `type` and `fluid_cells` (C + 4 bytes),
// also marks the cells that hold a fluid particle.
cudaError_t build_cell_starts(const unsigned* sorted_keys, int n, int num_cells,
                              int* cell_start, cudaStream_t s, const unsigned* gate = nullptr,
                              const int* type = nullptr, unsigned char* fluid_cells = nullptr);

// ---------------------------------------------------------------- precision policies
// The resident solver in three precisions sharing one code path:
//  PrecF32 — FP32 state and arithmetic (the reference's precision; the drop-in path).
//  PrecF64 — FP64 state and arithmetic: the accuracy reference every result is measured
//            against ("an FP64 run of the same solver").
//  PrecMix — FP32 neighbour sums on relative positions rebuilt from cell-local offsets; FP64
//            master positions and density perturbation rho - rho0 for the integration.
//  PrecMixC — PrecMix with compensated (Neumaier) accumulation of the density and force sums.
//  PrecMixA — PrecMix's FP64 integration with the pair arithmetic of PrecF32: the neighbour
//            sums run on FP32 positions in the simulation's frame, rounded from the FP64 master
//            positions every half step (no cell-local offsets, no cell codes in the lists).
// kMixed: FP64 master positions and rho - rho0 (xm); kCodes: records hold cell-local offsets
// and list slots carry the neighbour's anchor cell (the relative-position decode).
struct PrecF32 {
    using T = float;
    static constexpr bool kMixed = false;
    static constexpr bool kCodes = false;
    static constexpr bool kComp = false;
    static constexpr int kId = SPH_PREC_FP32;
};
struct PrecF64 {
    using T = double;
    static constexpr bool kMixed = false;
    static constexpr bool kCodes = false;
    static constexpr bool kComp = false;
    static constexpr int kId = SPH_PREC_FP64;
};
struct PrecMix {
    using T = float;
    static constexpr bool kMixed = true;
    static constexpr bool kCodes = true;
    static constexpr bool kComp = false;
    static constexpr int kId = SPH_PREC_MIXED;
};
struct PrecMixC {
    using T = float;
    static constexpr bool kMixed = true;
    static constexpr bool kCodes = true;
    static constexpr bool kComp = true;
    static constexpr int kId = SPH_PREC_MIXED_COMP;
};
struct PrecMixA {
    using T = float;
    static constexpr bool kMixed = true;
    static constexpr bool kCodes = false;
    static constexpr bool kComp = false;
    static constexpr int kId = SPH_PREC_MIXED_ABS;
};
inline bool prec_is_mixed(int prec) {
    return prec == SPH_PREC_MIXED || prec == SPH_PREC_MIXED_COMP || prec == SPH_PREC_MIXED_ABS;
}
// Position a record of a policy with FP64 master positions holds for the neighbour sums: the
// offsets from the anchor cell of resident key `key` (cell codes), or the FP64 position
// rounded to FP32 (PrecMixA).
template <class P, class KT>
__device__ __forceinline__ float3 record_pos(const KParamsT<KT>& k, unsigned key, double x,
                                             double y, double z) {
    if constexpr (P::kCodes) {
        double ox, oy, oz;
        cell_origin(k, key, ox, oy, oz);
        return make_float3((float)(x - ox), (float)(y - oy), (float)(z - oz));
    } else {
        (void)k;
        (void)key;
        return make_float3((float)x, (float)y, (float)z);
    }
}
// The list slots carry a cell code above a 26-bit neighbour index.
inline bool prec_has_codes(int prec) {
    return prec == SPH_PREC_MIXED || prec == SPH_PREC_MIXED_COMP;
}

// ---------------------------------------------------------------- resident state
// One particle set.  rec holds two vec4 per particle, rec[2i] = (x, y, z, p) and
// rec[2i+1] = (vx, vy, vz, ±rho) with rho negated for boundary (non-fluid) particles: one
// aligned record (32 bytes in FP32), the unit a neighbour gather reads.  type keeps the
// particle kind as given (0 wall, 1 fluid, 2 rigid, ...), id the original particle index;
// tpos/tvel hold the predictor's saved step-n state (x, y, z, rho) / (vx, vy, vz, 0).
// Mixed precision (kMixed): xm holds the FP64 position and rho - rho0, txm the predictor's save
// of it (tpos is unused); x, y, z in rec and xyz are the offsets from the origin of the
// particle's anchor cell at the last list build (kCodes) or the FP64 position rounded to FP32
// (PrecMixA).
template <class T>
struct ParticleSetT {
    vec4_t<T>* rec = nullptr;
    vec4_t<T>* xyz = nullptr;  // sorted set only: dense (x, y, z, ±1) for candidate walks
    int* type = nullptr;
    int* id = nullptr;
    vec4_t<T>* tpos = nullptr;
    vec4_t<T>* tvel = nullptr;
    dvec4* xm = nullptr;
    dvec4* txm = nullptr;
    int* inst = nullptr;  // batched instances: the particle's instance (0 for one simulation)
};
using ParticleSet = ParticleSetT<float>;

// Pass-1 output.  nrec[2i] = (x, y, z, q) with q = p' - rho0 cs h dofv for fluid particles and
// q = p' for boundary particles, nrec[2i+1] = (vx, vy, vz, ±rho'): the record pass 2 gathers per
// neighbour.  self[i] = (p', rho', dofv, 0): the particle's own side.
template <class T>
struct Pass1OutT {
    vec4_t<T>* nrec = nullptr;
    vec4_t<T>* self = nullptr;
};
using Pass1Out = Pass1OutT<float>;

enum HalfStep { HALF_PREDICT = 0, HALF_CORRECT = 1 };

// Neighbour list: slot c of particle i at idx[(i / 32) * cap * 32 + (c / 4) * 128 + (i % 32) * 4
// + c % 4] (each warp of 32 consecutive particles owns a block of cap x 32 slots, its particles'
// slots four to an int4, side by side), count[i] entries, and xb[i]
// the position i had when the list was built (its record position).  The list
// holds every pair closer than the list cutoff (KParams::kh2_list, the support radius plus a
// skin), in candidate-walk order; count[i] > cap means the list overflowed for i and the
// passes walk the cells for it instead.  With cell codes (kCodes) each slot also holds, in
// bits 26-31, the neighbour's anchor relative to i's ((dz+1) << 4 | (dy+1) << 2 | (dx+1)),
// from which the passes rebuild relative positions out of the cell-local offsets.
struct NbrList {
    int* idx = nullptr;
    int* count = nullptr;
    int cap = 0;
    float4* xb = nullptr;
    // squared list cutoff chosen on the device at each rebuild (adaptive skin); NULL: the
    // constant block's kh2_list
    const float* cut2 = nullptr;
    // cells holding a fluid particle (marked with the cell starts); NULL: not known.  A
    // boundary particle keeps fluid neighbours only, so one with no such cell among its 27
    // has an empty list without walking them.
    const unsigned char* fluid_cells = nullptr;
    // per-instance decisions (KParams::inst_boxes): the instance words and the instance of
    // every slot; the build skips the particles of instances that keep their lists.  NULL:
    // every particle is rebuilt at cut2
    const unsigned* iw = nullptr;
    const int* inst = nullptr;
};
// List slots per particle: 1.5x the lattice particles within kh (1 + skin), rounded up to 16.
int nbr_capacity_for(const sph_params& p, double skin = 0.0);

// Neighbour passes (equation/ns.cu), one instantiation per precision policy P.
// nl == NULL walks the cells in every pass.
//  build : fills nl for the sorted set (walls keep only fluid neighbours unless walls_all).
//  pass 1: fills a Pass1Out — boundary particles get the extrapolated p and rho, fluid
//          particles their own p, rho and the velocity divergence.  rhop_sum / w_sum are
//          written when non-NULL (FP32 only).
//  pass 2: either rates only (rho_dt, AoS vel_dt; FP32 only) or rates + the
//          predictor/corrector update written into `out` (slot-aligned with `in`) with the
//          next cell hash.
template <class P>
cudaError_t launch_nbr_build(const KParamsT<typename P::T>& k,
                             const ParticleSetT<typename P::T>& in, const unsigned* sorted_keys,
                             const int* cell_start, const NbrList& nl, int walls_all,
                             unsigned* err, cudaStream_t s, const unsigned* gate = nullptr);
template <class P>
cudaError_t launch_pass1(const KParamsT<typename P::T>& k, const ParticleSetT<typename P::T>& in,
                         const unsigned* sorted_keys, const int* cell_start, const NbrList* nl,
                         const Pass1OutT<typename P::T>& out, float* rhop_sum, float* w_sum,
                         cudaStream_t s);
cudaError_t launch_pass2_rates(const KParams& k, const ParticleSet& in,
                               const unsigned* sorted_keys, const int* cell_start,
                               const NbrList* nl, const Pass1Out& p1, float* rho_dt,
                               float* vel_dt, int wall_rates, cudaStream_t s);
// `out` may be `in` (the update is per particle; neighbours are read from p1).  disp (may be
// NULL) receives, by atomicMax on its float bits, the largest squared distance of a fluid
// particle from its position when the list was built (nl->xb).
template <class P>
cudaError_t launch_pass2_step(const KParamsT<typename P::T>& k, HalfStep half,
                              const ParticleSetT<typename P::T>& in, const unsigned* sorted_keys,
                              const int* cell_start, const NbrList* nl,
                              const Pass1OutT<typename P::T>& p1,
                              ParticleSetT<typename P::T> out, unsigned* out_hash, unsigned* err,
                              unsigned* disp, cudaStream_t s);

// Resident-state glue (lib/mesh.cu), one instantiation per precision policy P.
// perm == NULL copies slot for slot.  With cell codes a permuting gather recomputes the
// cell-local offsets from the FP64 positions for the cells in `keys` (the new sorted keys).
template <class P>
cudaError_t launch_gather(const KParamsT<typename P::T>& k, const int* perm,
                          const ParticleSetT<typename P::T>& src, ParticleSetT<typename P::T> dst,
                          int with_tmp, const unsigned* keys, cudaStream_t s,
                          const unsigned* gate = nullptr);
// Recompute the cell keys of `set` on the grid of `k` (k.n particles).
template <class P>
cudaError_t launch_rehash(const KParamsT<typename P::T>& k, const ParticleSetT<typename P::T>& set,
                          unsigned* hash, unsigned* err, cudaStream_t s);
// inst_off (device, n_inst + 1 entries; may be NULL for one simulation): instance b owns
// particles [inst_off[b], inst_off[b+1]).
template <class P>
cudaError_t launch_upload_convert(const KParamsT<typename P::T>& k, const float* pos,
                                  const float* vel, const float* rho, const float* p,
                                  const int* type, const int* inst_off, int n_inst,
                                  ParticleSetT<typename P::T> dst, unsigned* hash, unsigned* err,
                                  cudaStream_t s);
// Lane-group variant of list pass 1 (equation/ns_groups.cu): k.lanes in {2, 4, 8, 16} lanes
// per particle over the one-lane list; launch_pass1 dispatches to it when k.lanes > 1.
template <class P>
cudaError_t launch_pass1_groups(const KParamsT<typename P::T>& k,
                                const ParticleSetT<typename P::T>& in, const unsigned* keys,
                                const int* cs, const NbrList& nl,
                                const Pass1OutT<typename P::T>& out, cudaStream_t s);

// Upload original-order arrays into the current sorted order (slot k takes particle id[k]),
// measuring displacements from the list-build positions xb into *disp; a changed particle
// kind sets *force.
template <class P>
cudaError_t launch_upload_sorted(const KParamsT<typename P::T>& k, const float* pos,
                                 const float* vel, const float* rho, const float* p,
                                 const int* type, const unsigned* keys, const float4* xb,
                                 ParticleSetT<typename P::T> dst, unsigned* hash, unsigned* err,
                                 unsigned* disp, unsigned* force, cudaStream_t s);
template <class P>
cudaError_t launch_download_convert(const KParamsT<typename P::T>& k,
                                    const ParticleSetT<typename P::T>& src, float* pos,
                                    float* vel, float* rho, float* p, int* type, cudaStream_t s);
template <class P>
cudaError_t launch_download_f64(const KParamsT<typename P::T>& k,
                                const ParticleSetT<typename P::T>& src, double* pos, double* vel,
                                double* rho, double* p, cudaStream_t s);
// Probes and FP64 reductions (io/probes.cu): launch_probes fills a device accumulator of
// probe_acc_words() doubles, probe_results turns its host copy into sph_stats and probe values.
size_t probe_acc_words();
template <class P>
cudaError_t launch_probes(const KParamsT<typename P::T>& k, const ParticleSetT<typename P::T>& set,
                          const sph_probe* probes, int nprobes, double* acc, cudaStream_t s);
void probe_results(const double* acc, const sph_probe* probes, int nprobes, double cfl, double h,
                   double cs, sph_stats* stats, double* values);
// Drop-in sph_ns glue: AoS sorted arrays -> SoA set (and back for the outputs).
cudaError_t launch_aos_to_set(const KParams& k, const float* s_pos, const float* s_vel,
                              const float* s_rho, const float* s_p, const int* s_type,
                              const int* hash, ParticleSet dst, unsigned* keys,
                              unsigned* err, cudaStream_t s);
cudaError_t launch_ns_writeback(const KParams& k, const int* s_type, const float4* self,
                                float* s_rho, float* s_p, float* dofv, cudaStream_t s);

// Layout of the rebuild block: four control words, the list skin control, then the
// displacement box (DISP_WORDS, 128-byte aligned).
constexpr int RB_SKIN = 4;  // skin of the current lists, as a fraction of kh (float bits)
constexpr int RB_HS = 5;    // half steps since the last build
constexpr int RB_CUT2 = 6;  // squared list cutoff kh^2 (1 + skin)^2 (float bits)
constexpr int RB_THR = 7;   // rebuild threshold (skin kh / 2)^2 on the box (float bits)
constexpr int RB_DISP = 32;
constexpr int RB_WORDS = RB_DISP + DISP_WORDS;

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
    // y is in the cell order its keys_sorted, cell starts and neighbour lists were built for,
    // on the current grid and options (a half step ran since the last upload or change), so an
    // upload of the same particles can go straight into that order
    bool sorted = false;
    long long steps = 0;

    int prec = SPH_PREC_FP32;   // SPH_OPT_PRECISION
    // FP32 and mixed precision use x, y, p1; FP64 uses xd, yd, p1d (the other is unallocated)
    sph::ParticleSet x;   // scratch: permutation target on a rebuild, download staging
    sph::ParticleSet y;   // live state in the cell-sorted order the neighbour passes read
    unsigned* hash_x = nullptr;      // next cell of every slot of x
    unsigned* keys_sorted = nullptr; // sorted cell keys of y
    int* perm = nullptr;             // y slot k came from x slot perm[k]
    unsigned char* fluid_cells = nullptr;  // cells holding fluid, per list build
    sph::Pass1Out p1;                // pass-1 output
    sph::ParticleSetT<double> xd, yd;
    sph::Pass1OutT<double> p1d;
    int* cell_start = nullptr;       // [num_cells + 1]
    int cell_capacity = 0;
    void* sort_scratch = nullptr;
    size_t sort_scratch_bytes = 0;
    unsigned* err = nullptr;         // device error word
    double* probe_acc = nullptr;     // probe / reduction accumulator (probe_acc_words())
    // asynchronous snapshots: original-order state written on the compute stream, copied to the
    // host on copy_stream while later steps run
    float* snap_f = nullptr;         // pos [3n], vel [3n], rho [n], p [n]
    int* snap_type = nullptr;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t snap_ready = nullptr, snap_done = nullptr;
    bool snap_pending = false;

    // neighbour list, reused across half steps while every particle stays within skin/2 of
    // where it was when the list was built
    sph::NbrList nl;
    sph_params Pi{};                 // internal grid: cells of kh (1 + skin), instances stacked
    int n_inst = 1;                  // batched instances (sph_upload_instances)
    std::vector<int> inst_off_h;     // their offsets, as last uploaded
    int gz_inst = 0;                 // grid height of one instance
    int* inst_off = nullptr;         // [SPH_MAX_INSTANCES + 1] instance particle offsets
    double skin = 0.1;               // list skin as a fraction of the support radius kh
    unsigned* rb = nullptr;          // [0] rebuild gate, [1] last half-diagonal^2 of the
                                     // displacement box (float bits), [2] forced rebuild,
                                     // [3] rebuild count, [RB_DISP ..] the displacement box

    // graph replay of one full step
    int opt_use_graph = 1;
    int opt_wall_rates = 0;
    int opt_profile = 0;
    int opt_nbr_list = 1;
    int opt_nbr_cap = 0;  // 0: nbr_capacity_for(P)
    int opt_cond_graph = 1;  // graph replay skips the rebuild kernels through conditional nodes
    int opt_threads = 0;     // neighbour kernels: threads per block (0: the precision's default)
    int opt_ppt = 1;         // neighbour kernels: particles per thread
    int opt_lanes = 0;       // list pass 1: lanes per particle (0: the precision's default)
    int opt_adaptive_skin = 1;  // list skin chosen at each rebuild, up to `skin`
    int opt_reach = 1;       // cells per list cutoff (SPH_OPT_CELL_DIVISIONS): walk reach
    bool opt_reach_set = false;  // set by the caller (else the precision's default)
    int opt_inst_decisions = 0;  // batched instances rebuild on their own decisions
    // per-instance rebuild words (IW_*, sph_device.cuh): a header and IW_STRIDE words for each
    // of up to SPH_MAX_INSTANCES instances
    unsigned* iw = nullptr;
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
