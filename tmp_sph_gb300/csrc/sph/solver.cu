// solver.cu — the resident solver: one context per simulation, state kept on the GPU in
// cell-sorted SoA order, whole predictor-corrector steps advanced with fused kernels.
//
// Reference counterpart: the step loop of src/sph/sph_run.cu:285-336 (hash, sort, reorder,
// SPH_NS, PC_prediction, recover, then the same for PC_correction).  Here one half step is
//
//   rebuild decision  ->  [radix sort (cell key, slot)  ->  gather y -> x -> y in cell order
//   + dense cell starts  ->  neighbour-list build (y)]  ->  pass 1 (y -> records p1)
//   ->  pass 2 + integrator (p1 -> y in place, next cell keys, displacement box)
//
// so the state never returns to original order inside a step (the original particle id
// travels with it and is used only by sph_download), there is no separate hash kernel
// (pass 2 writes the next keys), and no host synchronisation: a full step is a fixed list
// of launches, captured once as a CUDA graph and replayed.
//
// Verlet skin.  The cells are kh(1 + skin) wide and the list holds every pair closer than
// kh(1 + s) at build time, s <= skin (the adaptive skin below picks s at each rebuild).
// While the bounding box of all displacements since the build has a half-diagonal below
// s kh / 2, no two particles have closed in by more than s kh, so every pair now closer than
// kh is in the list and the bracketed kernels are skipped: k_decide (one thread, on the GPU)
// compares the box pass 2 recorded with that bound and writes a gate word the gated kernels
// read before doing any work.  The passes test r < kh themselves, so they evaluate the same
// pairs as a rebuild every half step; only the order of the sums within a particle can
// differ.  skin = 0 rebuilds every half step on the reference's cell size.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "sph_internal.h"

using namespace sph;

namespace {

template <class T>
cudaError_t dalloc(T** p, size_t count) {
    return cudaMalloc(reinterpret_cast<void**>(p), (count > 0 ? count : 1) * sizeof(T));
}

template <class T>
void free_set(ParticleSetT<T>& s) {
    cudaFree(s.rec); cudaFree(s.xyz); cudaFree(s.type); cudaFree(s.id);
    cudaFree(s.tpos); cudaFree(s.tvel); cudaFree(s.xm); cudaFree(s.txm); cudaFree(s.inst);
    s = ParticleSetT<T>{};
}

template <class T>
cudaError_t alloc_set(ParticleSetT<T>& s, int cap, bool mixed) {
    cudaError_t e;
    if ((e = dalloc(&s.rec, 2 * (size_t)cap)) != cudaSuccess) return e;
    if ((e = dalloc(&s.xyz, cap)) != cudaSuccess) return e;
    if ((e = dalloc(&s.type, cap)) != cudaSuccess) return e;
    if ((e = dalloc(&s.id, cap)) != cudaSuccess) return e;
    if ((e = dalloc(&s.tpos, cap)) != cudaSuccess) return e;
    if ((e = dalloc(&s.tvel, cap)) != cudaSuccess) return e;
    if ((e = dalloc(&s.inst, cap)) != cudaSuccess) return e;
    if (mixed) {
        if ((e = dalloc(&s.xm, cap)) != cudaSuccess) return e;
        if ((e = dalloc(&s.txm, cap)) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

template <class T>
void free_p1(Pass1OutT<T>& p) {
    cudaFree(p.nrec);
    cudaFree(p.self);
    p = Pass1OutT<T>{};
}

template <class T>
cudaError_t alloc_p1(Pass1OutT<T>& p, int cap) {
    cudaError_t e = dalloc(&p.nrec, 2 * (size_t)cap);
    if (e == cudaSuccess) e = dalloc(&p.self, cap);
    return e;
}

// The particle state of the context's precision: x, y, p1 (FP32, mixed) or xd, yd, p1d (FP64).
void free_state(sph_ctx* c) {
    free_set(c->x);
    free_set(c->y);
    free_p1(c->p1);
    free_set(c->xd);
    free_set(c->yd);
    free_p1(c->p1d);
}

cudaError_t alloc_state(sph_ctx* c) {
    const int cap = c->capacity;
    cudaError_t e;
    if (c->prec == SPH_PREC_FP64) {
        if ((e = alloc_set(c->xd, cap, false)) != cudaSuccess) return e;
        if ((e = alloc_set(c->yd, cap, false)) != cudaSuccess) return e;
        return alloc_p1(c->p1d, cap);
    }
    const bool mixed = prec_is_mixed(c->prec);
    if ((e = alloc_set(c->x, cap, mixed)) != cudaSuccess) return e;
    if ((e = alloc_set(c->y, cap, mixed)) != cudaSuccess) return e;
    return alloc_p1(c->p1, cap);
}

// The state arrays one precision policy works on.
template <class P> struct State {
    static ParticleSet& x(sph_ctx* c) { return c->x; }
    static ParticleSet& y(sph_ctx* c) { return c->y; }
    static Pass1Out& p1(sph_ctx* c) { return c->p1; }
};
template <> struct State<PrecF64> {
    static ParticleSetT<double>& x(sph_ctx* c) { return c->xd; }
    static ParticleSetT<double>& y(sph_ctx* c) { return c->yd; }
    static Pass1OutT<double>& p1(sph_ctx* c) { return c->p1d; }
};

// Calls f(P{}) for the context's precision policy.
template <class F>
auto with_prec(const sph_ctx* c, F&& f) {
    switch (c->prec) {
        case SPH_PREC_FP64: return f(PrecF64{});
        case SPH_PREC_MIXED: return f(PrecMix{});
        case SPH_PREC_MIXED_COMP: return f(PrecMixC{});
        case SPH_PREC_MIXED_ABS: return f(PrecMixA{});
        default: return f(PrecF32{});
    }
}

void drop_graph(sph_ctx* c) {
    if (c->graph) cudaGraphExecDestroy(c->graph);
    c->graph = nullptr;
    c->graph_stream = nullptr;
    c->graph_n = -1;
}

void release(sph_ctx* c) {
    drop_graph(c);
    if (c->side_stream) cudaStreamDestroy(c->side_stream);
    c->side_stream = nullptr;
    free_state(c);
    cudaFree(c->hash_x); cudaFree(c->keys_sorted); cudaFree(c->perm);
    cudaFree(c->cell_start); cudaFree(c->sort_scratch); cudaFree(c->err);
    cudaFree(c->fluid_cells);
    c->fluid_cells = nullptr;
    cudaFree(c->nl.idx); cudaFree(c->nl.count); cudaFree(c->nl.xb);
    c->nl = NbrList{};
    cudaFree(c->rb);
    c->rb = nullptr;
    cudaFree(c->iw);
    c->iw = nullptr;
    cudaFree(c->probe_acc);
    c->probe_acc = nullptr;
    cudaFree(c->inst_off);
    c->inst_off = nullptr;
    if (c->snap_pending && c->snap_done) cudaEventSynchronize(c->snap_done);
    cudaFree(c->snap_f);
    cudaFree(c->snap_type);
    c->snap_f = nullptr;
    c->snap_type = nullptr;
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
    if (c->snap_ready) cudaEventDestroy(c->snap_ready);
    if (c->snap_done) cudaEventDestroy(c->snap_done);
    c->copy_stream = nullptr;
    c->snap_ready = c->snap_done = nullptr;
    for (auto& e : c->ev)
        if (e) cudaEventDestroy(e);
}

int to_status(cudaError_t e) { return e == cudaSuccess ? SPH_OK : SPH_ERR_CUDA; }

// Device staging for host transfers, carved from buffers that hold nothing between steps
// (the scratch set's predictor arrays and the pass-1 neighbour records); the live state (y),
// the sorted keys, cell starts and neighbour list are untouched by an upload/download.
struct Staging {
    float* pos;   // 3n floats
    float* vel;   // 3n floats
    float* rho;   // n
    float* p;     // n
    int* type;    // n
};

Staging staging(sph_ctx* c, int n) {
    Staging s;
    const bool d = c->prec == SPH_PREC_FP64;
    s.pos = d ? reinterpret_cast<float*>(c->xd.tpos) : reinterpret_cast<float*>(c->x.tpos);
    s.vel = d ? reinterpret_cast<float*>(c->xd.tvel) : reinterpret_cast<float*>(c->x.tvel);
    // 8n floats (FP32 records) or 16n (FP64)
    float* a = d ? reinterpret_cast<float*>(c->p1d.nrec) : reinterpret_cast<float*>(c->p1.nrec);
    s.rho = a;
    s.p = a + n;
    s.type = reinterpret_cast<int*>(a + 2 * (size_t)n);
    return s;
}

bool params_ok(const sph_params* p) {
    return p && p->num_cells > 0 && p->grid_dim[0] > 0 && p->grid_dim[1] > 0 &&
           p->grid_dim[2] > 0 && p->cell_size > 0.f && p->h > 0.f && p->kh > 0.f &&
           p->rho0 > 0.f && p->cs > 0.f &&
           // the 27-cell walk needs cells at least as wide as the support radius
           p->cell_size >= p->kh &&
           (long long)p->grid_dim[0] * p->grid_dim[1] * p->grid_dim[2] == p->num_cells &&
           p->num_cells < (1 << 30);
}

constexpr int EV_PER_HALF = PH_COUNT + 1;


// Batched instances with a neighbour list rebuild on their own decisions (per-instance
// displacement boxes, skins and rebuild flags in c->iw).
bool per_instance(const sph_ctx* c) {
    return c->n_inst > 1 && c->opt_inst_decisions && c->opt_nbr_list && c->nl.idx;
}

// The neighbour list to use this half step, or NULL to walk the cells in every pass.
const NbrList* list_for(sph_ctx* c) {
    c->nl.fluid_cells = c->fluid_cells;
    const bool pi = per_instance(c);
    c->nl.iw = pi ? c->iw : nullptr;
    c->nl.inst = pi ? (c->prec == SPH_PREC_FP64 ? c->yd.inst : c->y.inst) : nullptr;
    return (c->opt_nbr_list && c->nl.idx) ? &c->nl : nullptr;
}

// Where pass 2 and an upload into the cell order put the displacements: the instance words
// or the one box of the rebuild block.
unsigned* disp_words(sph_ctx* c) { return per_instance(c) ? c->iw : c->rb + RB_DISP; }

// The resident solver's own grid: the caller's grid box with cells of kh (1 + skin) / reach,
// so a walk of the reach cells on each side of a particle's cell at the last rebuild still
// finds every particle within kh of it while no particle has moved more than skin/2.  skin = 0
// and reach 1 keep the caller's grid exactly (cells of kh).
sph_params internal_params(const sph_params& P, double skin, int reach) {
    if (!(skin > 0.0) && reach <= 1) return P;
    sph_params Q = P;
    float base = skin > 0.0 ? (float)((double)P.kh * (1.0 + skin)) : P.cell_size;
    if (base < P.cell_size) base = P.cell_size;
    Q.cell_size = reach > 1 ? (float)((double)base / (double)reach) : base;
    for (int c = 0; c < 3; c++) {
        float span = (Q.grid_max[c] - Q.grid_min[c]) / Q.cell_size;
        Q.grid_dim[c] = (int)ceilf(span);
        if (Q.grid_dim[c] < 1) Q.grid_dim[c] = 1;
    }
    Q.num_cells = Q.grid_dim[0] * Q.grid_dim[1] * Q.grid_dim[2];
    return Q;
}

// The solver's grid for n_inst batched instances: the instances' grids stacked along z, `reach`
// empty cell layers between consecutive instances, so no cell walk reaches another instance.
// *gz_local receives the height of one instance's grid.  Returns false when the stacked grid
// does not fit the key range.
// Height of one instance in the stacked grid: its own layers and at least `reach` empty ones,
// rounded up to a multiple of reach.
int instance_stride(int gz_local, int reach) {
    const int r = reach > 1 ? reach : 1;
    return (gz_local + r + r - 1) / r * r;
}

bool stacked_params(const sph_params& P, double skin, int reach, int n_inst, sph_params* out,
                    int* gz_local) {
    sph_params Q = internal_params(P, skin, reach);
    *gz_local = Q.grid_dim[2];
    if (n_inst > 1) {
        const long long gz = (long long)n_inst * instance_stride(Q.grid_dim[2], reach);
        const long long cells = (long long)Q.grid_dim[0] * Q.grid_dim[1] * gz;
        if (cells >= (1LL << 30)) return false;
        Q.grid_dim[2] = (int)gz;
        Q.num_cells = (int)cells;
    }
    *out = Q;
    return true;
}

// Lanes per particle of list pass 1: the option, or by default 2 in FP32 on cells of the list
// cutoff while the lists have a skin (4.96M-particle dam break: pass 1 −4%, step −1.6%), else
// 1.  On the default FP32 cells of a third of the cutoff the particles of a warp already
// gather shifted copies of each other's neighbour rows and one lane wins (pass 1 0.552
// against 0.600 ms, 1000 steps from rest 2.83 against 2.91 ms per step); without a skin the
// lists are rebuilt every half step and the build of interleaved windows costs 17% more (the
// step 6%); mixed precision and FP64 gain nothing (mixed: 3.64 ms per step either way).
static int pass1_lanes(const sph_ctx* c) {
    if (c->opt_lanes > 0) return c->opt_lanes;
    return c->prec == SPH_PREC_FP32 && c->skin > 0.0 && c->opt_reach == 1 ? 2 : 1;
}

// The FP32 pair arithmetic without cell codes: FP32 and the mixed policy on FP32 positions
// (SPH_PREC_MIXED_ABS), which share the FP32 defaults below.
static bool fp32_pairs(int prec) { return prec == SPH_PREC_FP32 || prec == SPH_PREC_MIXED_ABS; }

// Threads per block of the neighbour kernels: the option, or by default 256 in FP32 (their
// static shared memory is sized for 256 threads, so 128-thread blocks pack twice as much per
// SM and leave L1 less room: 4.96M dam break 3.26 against 3.32 ms per step, 7.50 against 7.60
// rebuilding every half step) and 128 in the other precisions (mixed precision's 56-register
// pass 2 keeps 36 warps per SM in 128-thread blocks, 32 in 256: 3.64 against 3.75 ms).
static int block_threads(const sph_ctx* c) {
    if (c->opt_threads > 0) return c->opt_threads;
    return fp32_pairs(c->prec) ? 256 : 128;
}

// Cells per list cutoff by default: 3 in FP32 (cells of about dx at h = 1.3 dx: the
// cell-sorted state is ordered along rows of single particles, so the lanes of a warp hold
// neighbours whose lists are shifted copies of each other and gather common lines; 4.96M dam
// break 2.85 against 3.28 ms per step), 1 in the other precisions (the passes of the
// cell-code precisions gain less, and FP64's are bound by its arithmetic).
static int default_reach(int prec) { return fp32_pairs(prec) ? 3 : 1; }

// Lane groups read interleaved list windows, one lane per particle plain ones.
static bool list_windows(const sph_ctx* c) { return pass1_lanes(c) > 1; }

template <class T>
KParamsT<T> resident_kparams(const sph_ctx* c) {
    KParamsT<T> k = make_kparams_t<T>(c->Pi, c->n);
    k.gz_local = c->gz_inst;
    k.threads = block_threads(c);
    k.ppt = c->opt_ppt;
    // lane groups need the list
    const bool groups = c->opt_nbr_list && c->nl.idx;
    k.lanes = groups ? pass1_lanes(c) : 1;
    k.list_win = k.lanes > 1;
    k.reach = c->opt_reach;
    k.reach_cell = (T)c->opt_reach * k.cell;
    k.gz_stride = c->n_inst > 1 ? instance_stride(c->gz_inst, c->opt_reach) : c->gz_inst;
    k.inst_boxes = per_instance(c) ? 1 : 0;
    k.inst_cells = c->n_inst > 1 ? c->Pi.grid_dim[0] * c->Pi.grid_dim[1] * k.gz_stride : 0;
    const double cut = (double)c->P.kh * (1.0 + (c->skin > 0.0 ? c->skin : 0.0));
    k.kh2_list = (T)(cut * cut);
    if (k.kh2_list < k.kh2) k.kh2_list = k.kh2;
    return k;
}

// Skin of the neighbour lists.  The cells are sized for the largest skin s_max (the option);
// with `adapt`, each rebuild picks the skin s <= s_max of the next lists from how long the last
// ones lasted.  A list of skin s costs passes over about (1 + s)^3 times the pairs within kh
// and lasts until the displacement box has grown to s kh / 2; with the box growing at the rate
// just seen, a list of skin s lasts n s / s_cur half steps.  Balancing the extra pass work of
// a larger skin against the rebuilds it saves (a rebuild costs about as much as three passes'
// share of skin pairs at s = 0.1: `ratio`) gives s ~ sqrt(ratio s_cur / n); the new skin is
// the geometric mean of that and the current one, within [s_min, s_max].  A flow at rest keeps
// tight lists (a dam break's first hundreds of steps); a surge widens them to s_max.
struct SkinControl {
    float kh, s_min, s_max, ratio;
    int adapt;
};

// Skin s for the next lists: the words of the list cutoff and of the rebuild threshold, and
// the half-step count restarted.
__device__ __forceinline__ void write_skin(unsigned* skin, unsigned* cut2, unsigned* thr,
                                           unsigned* hs, const SkinControl& sc, float s) {
    const float cut = sc.kh * (1.f + s), half = 0.5f * s * sc.kh;
    *skin = __float_as_uint(s);
    *cut2 = __float_as_uint(cut * cut);
    *thr = __float_as_uint(half * half);
    *hs = 0u;
}
__device__ __forceinline__ void set_skin(unsigned* rb, const SkinControl& sc, float s) {
    write_skin(rb + RB_SKIN, rb + RB_CUT2, rb + RB_THR, rb + RB_HS, sc, s);
}
__device__ __forceinline__ void set_inst_skin(unsigned* w, const SkinControl& sc, float s) {
    write_skin(w + IW_SKIN, w + IW_CUT2, w + IW_THR, w + IW_HS, sc, s);
}

// Skin of the lists a rebuild makes after lists of skin s lasted hs half steps (adaptive).
__device__ __forceinline__ float next_skin(const SkinControl& sc, float s, unsigned hs) {
    const float want = sqrtf(sc.ratio * s / (float)hs);
    return fminf(fmaxf(sqrtf(s * want), sc.s_min), sc.s_max);
}

// Squared half-diagonal of a displacement box (lo x, y, z, hi x, y, z, `stride` words apart),
// which is emptied for the next half step.
__device__ __forceinline__ float take_box(unsigned* box, int stride) {
    float hd2 = 0.f;
    for (int c = 0; c < 3; c++) {
        const unsigned lo = box[c * stride], hi = box[(3 + c) * stride];
        if (lo <= hi) {  // else no particle counted
            const float r = 0.5f * (ord_value(hi) - ord_value(lo));
            hd2 = fma_rn(r, r, hd2);
        }
        box[c * stride] = 0xffffffffu;
        box[(3 + c) * stride] = 0u;
    }
    return hd2;
}

// Skin of the first lists after an upload or a change of parameters.
__global__ void k_skin_init(unsigned* rb, SkinControl sc) {
    if (threadIdx.x == 0) set_skin(rb, sc, sc.adapt ? sc.s_min : sc.s_max);
}

SkinControl skin_control(const sph_ctx* c) {
    SkinControl sc;
    sc.kh = c->P.kh;
    sc.s_max = c->skin > 0.0 ? (float)c->skin : 0.f;
    sc.s_min = std::min(sc.s_max, 0.02f);
    sc.ratio = 1.f;
    sc.adapt = (c->opt_adaptive_skin && sc.s_max > 0.f) ? 1 : 0;
    return sc;
}

__global__ void k_inst_reset(unsigned* iw, int n_inst, SkinControl sc, int skin_too,
                             int counts_too);

cudaError_t reset_skin(sph_ctx* c, cudaStream_t s) {
    k_skin_init<<<1, 32, 0, s>>>(c->rb, skin_control(c));
    if (c->n_inst > 1) k_inst_reset<<<1, 256, 0, s>>>(c->iw, c->n_inst, skin_control(c), 1, 0);
    return cudaGetLastError();
}

// The same, between calls on any stream: the device is idle first, so no half step in flight
// reads the skin words while they change.
cudaError_t reset_skin_sync(sph_ctx* c) {
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = reset_skin(c, nullptr);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    return e;
}

// Rebuild decision, one thread: rebuild when forced, when the cells are walked every half
// step (no list), or when the box of all displacements since the last build (written by the
// previous pass 2 or upload, sph_device.cuh) has a half-diagonal beyond skin/2, its square
// compared with the threshold of the current lists.  A rebuild picks the next skin (above).
// The box is emptied for the next half step.  In a graph built with conditional nodes it also
// sets the condition of the node that holds the rebuild kernels, so a half step without a
// rebuild launches none of them.
__global__ void k_decide(unsigned* rb, SkinControl sc, int always,
                         cudaGraphConditionalHandle cond, int set_cond) {
    const float hd2 = take_box(rb + RB_DISP, DISP_STRIDE);
    const bool forced = rb[2] != 0u;
    const bool rebuild = always || forced || !(hd2 <= __uint_as_float(rb[RB_THR]));
    const unsigned hs = rb[RB_HS] + 1u;
    rb[0] = rebuild ? 1u : 0u;
    rb[1] = __float_as_uint(hd2);
    if (rebuild) {
        float s = __uint_as_float(rb[RB_SKIN]);
        if (sc.adapt && !always && !forced && s > 0.f) s = next_skin(sc, s, hs);
        set_skin(rb, sc, s);
        rb[2] = 0u;
        rb[3] += 1u;
    } else {
        rb[RB_HS] = hs;
    }
    if (set_cond) cudaGraphSetConditional(cond, rebuild ? 1u : 0u);
}

// The same decision for each instance of a batch on its own box and skin (one block): an
// instance rebuilds when forced (rb[2], or IW_ALL when a particle left or rejoined the search
// and the slots after it moved) or when its own box has outgrown its own lists, exactly as
// k_decide decides for it alone.  rb[0] (the gate of the rebuild kernels, and the condition)
// is set when any instance rebuilds; rb[1] and RB_SKIN report the largest box and skin, rb[3]
// counts the half steps that rebuilt any.
__global__ void k_decide_inst(unsigned* rb, unsigned* iw, int n_inst, SkinControl sc,
                              cudaGraphConditionalHandle cond, int set_cond) {
    __shared__ unsigned s_max[2 * 32];
    const bool forced = rb[2] != 0u || iw[IW_ALL] != 0u;
    int any = 0;
    unsigned hd2_max = 0u, skin_max = 0u;  // float bits of non-negative values
    for (int b = (int)threadIdx.x; b < n_inst; b += (int)blockDim.x) {
        unsigned* w = inst_words(iw, b);
        const float hd2 = take_box(w + IW_BOX, 1);
        const bool rebuild = forced || !(hd2 <= __uint_as_float(w[IW_THR]));
        const unsigned hs = w[IW_HS] + 1u;
        w[IW_REBUILD] = rebuild ? 1u : 0u;
        w[IW_HD2] = __float_as_uint(hd2);
        if (rebuild) {
            float s = __uint_as_float(w[IW_SKIN]);
            if (sc.adapt && !forced && s > 0.f) s = next_skin(sc, s, hs);
            set_inst_skin(w, sc, s);
            w[IW_COUNT] += 1u;
        } else {
            w[IW_HS] = hs;
        }
        any |= rebuild ? 1 : 0;
        hd2_max = max(hd2_max, hd2 == hd2 ? __float_as_uint(hd2) : 0x7f800000u);
        skin_max = max(skin_max, w[IW_SKIN]);
    }
    any = __syncthreads_or(any);
    hd2_max = __reduce_max_sync(0xffffffffu, hd2_max);
    skin_max = __reduce_max_sync(0xffffffffu, skin_max);
    if ((threadIdx.x & 31) == 0) {
        s_max[threadIdx.x >> 5] = hd2_max;
        s_max[32 + (threadIdx.x >> 5)] = skin_max;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 1; q < (int)(blockDim.x >> 5); q++) {
            hd2_max = max(hd2_max, s_max[q]);
            skin_max = max(skin_max, s_max[32 + q]);
        }
        rb[0] = any ? 1u : 0u;
        rb[1] = hd2_max;
        rb[RB_SKIN] = skin_max;
        if (any) {
            rb[2] = 0u;
            iw[IW_ALL] = 0u;
            rb[3] += 1u;
        }
        if (set_cond) cudaGraphSetConditional(cond, any ? 1u : 0u);
    }
}

// Per-instance words of the n_inst instances: the first skin and the half-step counts
// (skin_too), empty boxes, and with counts_too no rebuild pending or counted.
__global__ void k_inst_reset(unsigned* iw, int n_inst, SkinControl sc, int skin_too,
                             int counts_too) {
    for (int b = (int)threadIdx.x; b < n_inst; b += (int)blockDim.x) {
        unsigned* w = inst_words(iw, b);
        if (skin_too) set_inst_skin(w, sc, sc.adapt ? sc.s_min : sc.s_max);
        for (int c = 0; c < 3; c++) {
            w[IW_BOX + c] = 0xffffffffu;
            w[IW_BOX + 3 + c] = 0u;
        }
        if (counts_too) {
            w[IW_REBUILD] = 0u;
            w[IW_COUNT] = 0u;
            w[IW_HD2] = 0u;
        }
    }
    if (threadIdx.x == 0 && counts_too) iw[IW_ALL] = 0u;
}

// Per-instance rebuilds: the slots of the instances that keep their lists are sorted on the
// keys they were sorted on last time.  Those keys are in order and each instance's keys lie in
// its own key range, so the stable sort leaves these slots where they are, and their lists,
// list-build positions and cell offsets stay valid.
__global__ void k_keep_keys(int n, const int* __restrict__ inst, const unsigned* __restrict__ iw,
                            const unsigned* __restrict__ keys_sorted, unsigned* __restrict__ hash,
                            const unsigned* gate) {
    if (gated_off(gate)) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (!iw[IW_STRIDE * (inst[i] + 1) + IW_REBUILD]) hash[i] = keys_sorted[i];
}

// Empty displacement box (before an upload fills it, and at allocation).
__global__ void k_disp_reset(unsigned* rb) {
    const int c = (int)threadIdx.x;
    if (c < 6) rb[RB_DISP + c * DISP_STRIDE] = c < 3 ? 0xffffffffu : 0u;
}

// Conditional-node capture of a half step: the rebuild kernels go into the body of an IF node
// (captured on `side`), whose condition k_decide sets.
struct CondCapture {
    cudaStream_t side;
    cudaGraphConditionalHandle handle;
};

// Sort, gather, cell starts and list build, each kernel gated on rb[0].  `ev` as half_step.
template <class P>
cudaError_t rebuild_lists(sph_ctx* c, const KParamsT<typename P::T>& k, cudaStream_t s,
                          cudaEvent_t* ev) {
    // with park_inactive, key num_cells marks the slots outside the neighbour search
    const int bits = key_bits_for(c->Pi.num_cells + (c->P.park_inactive ? 1 : 0));
    const NbrList* nl = list_for(c);
    const unsigned* gate = c->rb;
    cudaError_t e;
    if (per_instance(c)) {
        k_keep_keys<<<(c->n + 255) / 256, 256, 0, s>>>(c->n, State<P>::y(c).inst, c->iw,
                                                       c->keys_sorted, c->hash_x, gate);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    e = radix_sort_pairs(c->hash_x, nullptr, c->keys_sorted, c->perm, c->n, bits, c->sort_scratch,
                         c->sort_scratch_bytes, c->err, s, gate);
    if (e != cudaSuccess) return e;
    if (ev) cudaEventRecord(ev[PH_GATHER], s);
    // permute the live set y into cell order through x, then copy it back
    auto& x = State<P>::x(c);
    auto& y = State<P>::y(c);
    if ((e = launch_gather<P>(k, c->perm, y, x, 1, c->keys_sorted, s, gate)) != cudaSuccess)
        return e;
    if ((e = launch_gather<P>(k, nullptr, x, y, 1, nullptr, s, gate)) != cudaSuccess) return e;
    if ((e = build_cell_starts(c->keys_sorted, c->n, c->Pi.num_cells, c->cell_start, s, gate,
                               y.type, c->fluid_cells)) !=
        cudaSuccess)
        return e;
    if (ev) cudaEventRecord(ev[PH_NBR], s);
    if (nl && (e = launch_nbr_build<P>(k, y, c->keys_sorted, c->cell_start, *nl, 0, c->err, s,
                                       gate)) != cudaSuccess)
        return e;
    return cudaSuccess;
}

// Adds an IF node (condition cc.handle) after the current capture dependencies of `s` and
// captures the rebuild kernels into its body on cc.side.
template <class P>
cudaError_t capture_conditional_rebuild(sph_ctx* c, const KParamsT<typename P::T>& k,
                                        cudaStream_t s, const CondCapture& cc) {
    cudaStreamCaptureStatus st;
    cudaGraph_t cg = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    cudaError_t e = cudaStreamGetCaptureInfo(s, &st, nullptr, &cg, &deps, nullptr, &nd);
    if (e != cudaSuccess) return e;
    if (st != cudaStreamCaptureStatusActive) return cudaErrorStreamCaptureInvalidated;
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = cc.handle;
    cp.conditional.type = cudaGraphCondTypeIf;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    if ((e = cudaGraphAddNode(&node, cg, deps, nullptr, nd, &cp)) != cudaSuccess) return e;
    if ((e = cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1,
                                                 cudaStreamSetCaptureDependencies)) != cudaSuccess)
        return e;
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    if ((e = cudaStreamBeginCaptureToGraph(cc.side, body, nullptr, nullptr, 0,
                                           cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
        return e;
    e = rebuild_lists<P>(c, k, cc.side, nullptr);
    cudaGraph_t out = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(cc.side, &out);
    return e != cudaSuccess ? e : e2;
}

// One half step (see the file comment).  `ev` (may be NULL) receives PH_COUNT + 1 timestamps;
// `cc` (may be NULL) puts the rebuild kernels under a conditional node of the capture.
template <class P>
cudaError_t half_step(sph_ctx* c, HalfStep half, cudaStream_t s, cudaEvent_t* ev,
                      const CondCapture* cc = nullptr) {
    const KParamsT<typename P::T> k = resident_kparams<typename P::T>(c);
    auto& y = State<P>::y(c);
    auto& p1 = State<P>::p1(c);
    const NbrList* nl = list_for(c);
    cudaError_t e;
    if (ev) cudaEventRecord(ev[PH_SORT], s);
    if (per_instance(c))
        k_decide_inst<<<1, 256, 0, s>>>(c->rb, c->iw, c->n_inst, skin_control(c),
                                        cc ? cc->handle : 0, cc ? 1 : 0);
    else
        k_decide<<<1, 1, 0, s>>>(c->rb, skin_control(c), nl ? 0 : 1, cc ? cc->handle : 0,
                                 cc ? 1 : 0);
    e = cc ? capture_conditional_rebuild<P>(c, k, s, *cc) : rebuild_lists<P>(c, k, s, ev);
    if (e != cudaSuccess) return e;
    if (ev) cudaEventRecord(ev[PH_PASS1], s);
    if ((e = launch_pass1<P>(k, y, c->keys_sorted, c->cell_start, nl, p1, nullptr, nullptr,
                             s)) != cudaSuccess)
        return e;
    if (ev) cudaEventRecord(ev[PH_PASS2], s);
    // in place: pass 2 reads its neighbours from the pass-1 records
    e = launch_pass2_step<P>(k, half, y, c->keys_sorted, c->cell_start, nl, p1, y, c->hash_x,
                             c->err, disp_words(c), s);
    if (ev) cudaEventRecord(ev[PH_COUNT], s);
    return e;
}

cudaError_t full_step(sph_ctx* c, cudaStream_t s, cudaEvent_t* ev,
                      const CondCapture* cc = nullptr) {
    return with_prec(c, [&](auto tag) {
        using P = decltype(tag);
        cudaError_t e = half_step<P>(c, HALF_PREDICT, s, ev, cc);
        if (e != cudaSuccess) return e;
        return half_step<P>(c, HALF_CORRECT, s, ev ? ev + EV_PER_HALF : nullptr,
                            cc ? cc + 1 : nullptr);
    });
}

// The step graph with the rebuild kernels under two conditional nodes (one per half step).
cudaError_t build_conditional_graph(sph_ctx* c, cudaStream_t s, cudaGraph_t* out) {
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaGraphCreate(&g, 0);
    if (e != cudaSuccess) return e;
    CondCapture cc[2];
    for (int h = 0; h < 2 && e == cudaSuccess; h++) {
        cc[h].side = c->side_stream;
        e = cudaGraphConditionalHandleCreate(&cc[h].handle, g, 1u, cudaGraphCondAssignDefault);
    }
    if (e == cudaSuccess)
        e = cudaStreamBeginCaptureToGraph(s, g, nullptr, nullptr, 0,
                                          cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        e = full_step(c, s, nullptr, cc);
        cudaGraph_t g2 = nullptr;
        const cudaError_t e2 = cudaStreamEndCapture(s, &g2);
        if (e == cudaSuccess) e = e2;
    }
    if (e != cudaSuccess) {
        cudaGraphDestroy(g);
        cudaGetLastError();
        return e;
    }
    *out = g;
    return cudaSuccess;
}

// Next half step rebuilds the cell and neighbour lists whatever the displacement.
cudaError_t force_rebuild(sph_ctx* c, cudaStream_t s) {
    c->sorted = false;
    return cudaMemsetAsync(c->rb + 2, 1, sizeof(unsigned), s);
}

void free_list(NbrList& nl) {
    cudaFree(nl.idx);
    cudaFree(nl.count);
    cudaFree(nl.xb);
    nl = NbrList{};
}

cudaError_t alloc_list(sph_ctx* c) {
    // the option is rounded up to a multiple of 16, like the derived capacity
    int cap = c->opt_nbr_cap > 0 ? (c->opt_nbr_cap + 15) & ~15 : nbr_capacity_for(c->P, c->skin);
    if (c->nl.idx && c->nl.cap == cap) return cudaSuccess;
    free_list(c->nl);
    // warp-interleaved blocks of cap x 32 slots: whole warps, the last one padded
    const size_t rows = ((size_t)(c->capacity > 0 ? c->capacity : 1) + 31) & ~(size_t)31;
    cudaError_t e = dalloc(&c->nl.idx, (size_t)cap * rows);
    if (e == cudaSuccess) e = dalloc(&c->nl.count, c->capacity);
    if (e == cudaSuccess) e = dalloc(&c->nl.xb, c->capacity);
    if (e != cudaSuccess) {
        free_list(c->nl);
        return e;
    }
    c->nl.cap = cap;
    c->nl.cut2 = reinterpret_cast<const float*>(c->rb + RB_CUT2);
    return cudaSuccess;
}

}  // namespace

extern "C" int sph_create(const sph_params* p, int capacity, sph_ctx** out) {
    if (!out) return SPH_ERR_ARG;
    *out = nullptr;
    if (!params_ok(p) || capacity < 0) return SPH_ERR_ARG;
    sph_ctx* c = new (std::nothrow) sph_ctx();
    if (!c) return SPH_ERR_NOMEM;
    c->P = *p;
    c->opt_reach = default_reach(c->prec);
    stacked_params(*p, c->skin, c->opt_reach, 1, &c->Pi, &c->gz_inst);
    c->capacity = capacity;
    cudaGetDevice(&c->device);
    cudaError_t e = cudaSuccess;
    const int cap = capacity;
    if (e == cudaSuccess) e = alloc_state(c);
    if (e == cudaSuccess) e = dalloc(&c->hash_x, cap);
    if (e == cudaSuccess) e = dalloc(&c->keys_sorted, cap);
    if (e == cudaSuccess) e = dalloc(&c->perm, cap);
    c->cell_capacity = std::max(p->num_cells, c->Pi.num_cells);
    if (e == cudaSuccess) e = dalloc(&c->cell_start, (size_t)c->cell_capacity + 1);
    if (e == cudaSuccess) e = cudaMalloc(&c->fluid_cells, (size_t)c->cell_capacity + 4);
    c->sort_scratch_bytes = sort_scratch_bytes(cap);
    if (e == cudaSuccess) e = cudaMalloc(&c->sort_scratch, c->sort_scratch_bytes);
    if (e == cudaSuccess) e = dalloc(&c->err, 1);
    if (e == cudaSuccess) e = cudaMemset(c->err, 0, sizeof(unsigned));
    if (e == cudaSuccess) e = dalloc(&c->probe_acc, probe_acc_words());
    if (e == cudaSuccess) e = dalloc(&c->inst_off, SPH_MAX_INSTANCES + 1);
    if (e == cudaSuccess) e = dalloc(&c->snap_f, 8 * (size_t)cap);
    if (e == cudaSuccess) e = dalloc(&c->snap_type, cap);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->snap_ready, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->snap_done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = dalloc(&c->rb, RB_WORDS);
    if (e == cudaSuccess) e = cudaMemset(c->rb, 0, RB_WORDS * sizeof(unsigned));
    if (e == cudaSuccess) e = dalloc(&c->iw, (size_t)(SPH_MAX_INSTANCES + 1) * IW_STRIDE);
    if (e == cudaSuccess)
        e = cudaMemset(c->iw, 0, (size_t)(SPH_MAX_INSTANCES + 1) * IW_STRIDE * sizeof(unsigned));
    if (e == cudaSuccess) {
        k_disp_reset<<<1, 32>>>(c->rb);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = reset_skin(c, nullptr);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->side_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = alloc_list(c);
    for (auto& ev : c->ev)
        if (e == cudaSuccess) e = cudaEventCreate(&ev);
    if (e != cudaSuccess) {
        release(c);
        delete c;
        cudaGetLastError();
        return e == cudaErrorMemoryAllocation ? SPH_ERR_NOMEM : SPH_ERR_CUDA;
    }
    *out = c;
    return SPH_OK;
}

extern "C" int sph_destroy(sph_ctx* c) {
    if (!c) return SPH_ERR_ARG;
    release(c);
    delete c;
    return SPH_OK;
}

// Grows the cell-start array to hold `cells` + 1 entries; the only allocation outside
// sph_create besides the neighbour list (a grid with more cells).
static cudaError_t ensure_cells(sph_ctx* c, int cells) {
    if (cells <= c->cell_capacity) return cudaSuccess;
    int* cs = nullptr;
    unsigned char* fc = nullptr;
    cudaError_t e = dalloc(&cs, (size_t)cells + 1);
    if (e == cudaSuccess) e = cudaMalloc(&fc, (size_t)cells + 4);
    if (e != cudaSuccess) {
        cudaFree(cs);
        cudaGetLastError();
        return e;
    }
    cudaFree(c->cell_start);
    cudaFree(c->fluid_cells);
    c->cell_start = cs;
    c->fluid_cells = fc;
    c->cell_capacity = cells;
    return cudaSuccess;
}

extern "C" int sph_set_params(sph_ctx* c, const sph_params* p) {
    if (!c || !params_ok(p)) return SPH_ERR_ARG;
    sph_params pi;
    int gz_local;
    if (!stacked_params(*p, c->skin, c->opt_reach, c->n_inst, &pi, &gz_local)) return SPH_ERR_ARG;
    if (ensure_cells(c, std::max(p->num_cells, pi.num_cells)) != cudaSuccess) return SPH_ERR_NOMEM;
    c->P = *p;
    c->Pi = pi;
    c->gz_inst = gz_local;
    c->rehash = c->loaded;
    c->sorted = false;
    drop_graph(c);
    // and the neighbour list, when the support radius holds more lattice neighbours
    if (alloc_list(c) != cudaSuccess) {
        cudaGetLastError();
        return SPH_ERR_NOMEM;
    }
    if (reset_skin_sync(c) != cudaSuccess) return SPH_ERR_CUDA;  // kh may have changed
    return cudaMemset(c->rb + 2, 1, sizeof(unsigned)) == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

extern "C" int sph_get_params(const sph_ctx* c, sph_params* out) {
    if (!c || !out) return SPH_ERR_ARG;
    *out = c->P;
    return SPH_OK;
}

// A new cell size: the solver's grid and the cell arrays for it, the keys recomputed and the
// lists rebuilt at the next half step.
static int set_reach(sph_ctx* c, int reach) {
    sph_params pi;
    int gz_local;
    if (!stacked_params(c->P, c->skin, reach, c->n_inst, &pi, &gz_local)) return SPH_ERR_ARG;
    if (ensure_cells(c, pi.num_cells) != cudaSuccess) return SPH_ERR_NOMEM;
    c->opt_reach = reach;
    c->Pi = pi;
    c->gz_inst = gz_local;
    c->rehash = c->loaded;  // the keys pass 2 wrote index the old grid
    c->sorted = false;
    drop_graph(c);
    return cudaMemset(c->rb + 2, 1, sizeof(unsigned)) == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

extern "C" int sph_ctx_set_option(sph_ctx* c, int option, int value) {
    if (!c) return SPH_ERR_ARG;
    switch (option) {
        case SPH_OPT_USE_GRAPH: c->opt_use_graph = value != 0; drop_graph(c); return SPH_OK;
        case SPH_OPT_CONDITIONAL_GRAPH:
            c->opt_cond_graph = value != 0;
            drop_graph(c);
            return SPH_OK;
        case SPH_OPT_BLOCK_THREADS:
            // 0: the precision's default
            if (value != 0 && (value < 32 || value > 256 || value % 32)) return SPH_ERR_ARG;
            c->opt_threads = value;
            drop_graph(c);
            return SPH_OK;
        case SPH_OPT_PARTICLES_PER_THREAD:
            if (value < 1 || value > 64) return SPH_ERR_ARG;
            c->opt_ppt = value;
            drop_graph(c);
            return SPH_OK;
        case SPH_OPT_ADAPTIVE_SKIN:
            c->opt_adaptive_skin = value != 0;
            if (reset_skin_sync(c) != cudaSuccess) return SPH_ERR_CUDA;
            break;  // the next lists take the first skin of the new mode
        case SPH_OPT_LANES_PER_PARTICLE:
        case SPH_OPT_PASS1_LANES: {
            // 0: the default of the precision
            if (value != 0 && value != 1 && value != 2 && value != 4 && value != 8 && value != 16)
                return SPH_ERR_ARG;
            const bool win = list_windows(c);
            c->opt_lanes = value;
            drop_graph(c);
            if (win == list_windows(c)) return SPH_OK;
            break;  // the slot order of the lists changed: rebuild
        }
        case SPH_OPT_WALL_RATES: c->opt_wall_rates = value != 0; return SPH_OK;
        case SPH_OPT_INSTANCE_DECISIONS: {
            const int v = value != 0;
            if (v == c->opt_inst_decisions) return SPH_OK;
            c->opt_inst_decisions = v;
            drop_graph(c);
            // the boxes move between the rebuild block and the instance words: new lists
            return force_rebuild(c, nullptr) == cudaSuccess && cudaDeviceSynchronize() == cudaSuccess
                       ? SPH_OK
                       : SPH_ERR_CUDA;
        }
        case SPH_OPT_CELL_DIVISIONS: {
            // 0: the precision's default
            if (value < 0 || value > 3) return SPH_ERR_ARG;
            const int reach = value > 0 ? value : default_reach(c->prec);
            c->opt_reach_set = value > 0;
            if (reach == c->opt_reach) return SPH_OK;
            const int st = set_reach(c, reach);
            if (st != SPH_OK) return st;
            break;
        }
        case SPH_OPT_PRECISION: {
            if (value != SPH_PREC_FP32 && value != SPH_PREC_FP64 && !prec_is_mixed(value))
                return SPH_ERR_ARG;
            if (value == c->prec) return SPH_OK;
            drop_graph(c);
            free_state(c);
            c->prec = value;
            c->loaded = false;
            c->sorted = false;
            c->n = 0;
            if (alloc_state(c) != cudaSuccess) {
                cudaGetLastError();
                free_state(c);
                c->prec = SPH_PREC_FP32;
                alloc_state(c);
                cudaGetLastError();
                return SPH_ERR_NOMEM;
            }
            // the cell size follows the precision unless it was set
            if (!c->opt_reach_set && default_reach(c->prec) != c->opt_reach) {
                const int st = set_reach(c, default_reach(c->prec));
                if (st != SPH_OK) return st;
            }
            return SPH_OK;
        }
        case SPH_OPT_PROFILE: c->opt_profile = value != 0; return SPH_OK;
        case SPH_OPT_NEIGHBOR_LIST:
            c->opt_nbr_list = value != 0;
            drop_graph(c);
            break;
        case SPH_OPT_NEIGHBOR_CAP:
        case SPH_OPT_SKIN_PERMILLE:
            if (value < 0 || (option == SPH_OPT_SKIN_PERMILLE && value > 2000)) return SPH_ERR_ARG;
            if (option == SPH_OPT_NEIGHBOR_CAP) {
                c->opt_nbr_cap = value;
            } else {
                if (c->P.num_cells <= 0) return SPH_ERR_STATE;
                sph_params pi;
                int gz_local;
                if (!stacked_params(c->P, value / 1000.0, c->opt_reach, c->n_inst, &pi, &gz_local))
                    return SPH_ERR_ARG;
                if (ensure_cells(c, pi.num_cells) != cudaSuccess) return SPH_ERR_NOMEM;
                c->skin = value / 1000.0;
                c->Pi = pi;
                c->gz_inst = gz_local;
                c->rehash = c->loaded;
                if (reset_skin_sync(c) != cudaSuccess) return SPH_ERR_CUDA;
            }
            drop_graph(c);
            if (alloc_list(c) != cudaSuccess) {
                cudaGetLastError();
                return SPH_ERR_NOMEM;
            }
            break;
        default: return SPH_ERR_ARG;
    }
    // the cell and neighbour lists no longer match: rebuild them next half step
    c->sorted = false;
    return cudaMemset(c->rb + 2, 1, sizeof(unsigned)) == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

extern "C" int sph_ctx_get_option(const sph_ctx* c, int option, int* value) {
    if (!c || !value) return SPH_ERR_ARG;
    switch (option) {
        case SPH_OPT_USE_GRAPH: *value = c->opt_use_graph; break;
        case SPH_OPT_WALL_RATES: *value = c->opt_wall_rates; break;
        case SPH_OPT_PROFILE: *value = c->opt_profile; break;
        case SPH_OPT_NEIGHBOR_LIST: *value = c->opt_nbr_list; break;
        case SPH_OPT_NEIGHBOR_CAP: *value = c->nl.idx ? c->nl.cap : c->opt_nbr_cap; break;
        case SPH_OPT_SKIN_PERMILLE: *value = (int)std::lround(c->skin * 1000.0); break;
        case SPH_OPT_CONDITIONAL_GRAPH: *value = c->opt_cond_graph; break;
        case SPH_OPT_PRECISION: *value = c->prec; break;
        case SPH_OPT_BLOCK_THREADS: *value = block_threads(c); break;
        case SPH_OPT_PARTICLES_PER_THREAD: *value = c->opt_ppt; break;
        case SPH_OPT_ADAPTIVE_SKIN: *value = c->opt_adaptive_skin; break;
        case SPH_OPT_CELL_DIVISIONS: *value = c->opt_reach; break;
        case SPH_OPT_INSTANCE_DECISIONS: *value = c->opt_inst_decisions; break;
        case SPH_OPT_LANES_PER_PARTICLE:
        case SPH_OPT_PASS1_LANES: *value = pass1_lanes(c); break;
        default: return SPH_ERR_ARG;
    }
    return SPH_OK;
}

// Upload n particles of n_inst instances (offsets: host array of n_inst + 1, NULL for one).
static int upload_impl(sph_ctx* c, const float* pos, const float* vel, const float* rho,
                       const float* p, const int* type, const int* offsets, int n_inst, int n,
                       int from_host, void* stream) {
    if (!c || n < 0 || n > c->capacity) return SPH_ERR_ARG;
    if (n > 0 && (!pos || !vel || !rho || !p || !type)) return SPH_ERR_ARG;
    // list slots with cell codes keep the neighbour index in 26 bits
    if (prec_has_codes(c->prec) && n >= (1 << 26)) return SPH_ERR_ARG;
    if (n_inst < 1 || n_inst > SPH_MAX_INSTANCES) return SPH_ERR_ARG;
    if (n_inst > 1) {
        if (!offsets || offsets[0] != 0 || offsets[n_inst] != n) return SPH_ERR_ARG;
        for (int b = 0; b < n_inst; b++)
            if (offsets[b + 1] < offsets[b]) return SPH_ERR_ARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
    // the same particles again (same count and instances) after a half step: keep the cell
    // order, cell starts and neighbour lists, and let the displacement test decide
    const bool same_inst = n_inst == c->n_inst &&
                           (n_inst == 1 || std::equal(offsets, offsets + n_inst + 1,
                                                      c->inst_off_h.begin(), c->inst_off_h.end()));
    const bool into_order = c->sorted && c->loaded && !c->rehash && n == c->n && n > 0 && same_inst;
    if (n_inst != c->n_inst) {
        sph_params pi;
        int gz_local;
        if (!stacked_params(c->P, c->skin, c->opt_reach, n_inst, &pi, &gz_local)) return SPH_ERR_ARG;
        if (ensure_cells(c, pi.num_cells) != cudaSuccess) return SPH_ERR_NOMEM;
        c->Pi = pi;
        c->gz_inst = gz_local;
        c->n_inst = n_inst;
        drop_graph(c);
    }
    if (n_inst > 1 && !into_order &&
        cudaMemcpyAsync(c->inst_off, offsets, (size_t)(n_inst + 1) * sizeof(int),
                        cudaMemcpyHostToDevice, s) != cudaSuccess)
        return SPH_ERR_CUDA;
    if (n_inst > 1) c->inst_off_h.assign(offsets, offsets + n_inst + 1);
    else c->inst_off_h.clear();
    if (n != c->n) drop_graph(c);
    c->n = n;
    c->steps = 0;
    c->loaded = true;
    c->rehash = false;  // the upload computes the keys on the current grid
    if (n == 0) return SPH_OK;
    const float* dpos = pos;
    const float* dvel = vel;
    const float* drho = rho;
    const float* dp = p;
    const int* dtype = type;
    if (from_host) {
        Staging st = staging(c, n);
        float* spos = st.pos;
        float* svel = st.vel;
        float* srho = st.rho;
        float* sp = st.p;
        int* stype = st.type;
        if (cudaMemcpyAsync(spos, pos, (size_t)n * 12, cudaMemcpyHostToDevice, s) != cudaSuccess ||
            cudaMemcpyAsync(svel, vel, (size_t)n * 12, cudaMemcpyHostToDevice, s) != cudaSuccess ||
            cudaMemcpyAsync(srho, rho, (size_t)n * 4, cudaMemcpyHostToDevice, s) != cudaSuccess ||
            cudaMemcpyAsync(sp, p, (size_t)n * 4, cudaMemcpyHostToDevice, s) != cudaSuccess ||
            cudaMemcpyAsync(stype, type, (size_t)n * 4, cudaMemcpyHostToDevice, s) != cudaSuccess)
            return SPH_ERR_CUDA;
        dpos = spos; dvel = svel; drho = srho; dp = sp; dtype = stype;
    }
    if (into_order) {
        // the displacement box restarts from the uploaded positions; a pending forced rebuild
        // (rb[2]) stays
        k_disp_reset<<<1, 32, 0, s>>>(c->rb);
        if (c->n_inst > 1)
            k_inst_reset<<<1, 256, 0, s>>>(c->iw, c->n_inst, skin_control(c), 0, 0);
        if (cudaGetLastError() != cudaSuccess) return SPH_ERR_CUDA;
        const NbrList* nl = list_for(c);
        return to_status(with_prec(c, [&](auto tag) {
            using P = decltype(tag);
            return launch_upload_sorted<P>(resident_kparams<typename P::T>(c), dpos, dvel, drho,
                                           dp, dtype, c->keys_sorted, nl ? nl->xb : nullptr,
                                           State<P>::y(c), c->hash_x, c->err,
                                           disp_words(c), c->rb + 2, s);
        }));
    }
    // the state goes straight into the live set, hashed on the solver's grid; the first half
    // step sorts it
    if (cudaMemsetAsync(c->rb, 0, 4 * sizeof(unsigned), s) != cudaSuccess ||
        reset_skin(c, s) != cudaSuccess || force_rebuild(c, s) != cudaSuccess)
        return SPH_ERR_CUDA;
    if (n_inst > 1) {
        k_inst_reset<<<1, 256, 0, s>>>(c->iw, n_inst, skin_control(c), 0, 1);
        if (cudaGetLastError() != cudaSuccess) return SPH_ERR_CUDA;
    }
    return to_status(with_prec(c, [&](auto tag) {
        using P = decltype(tag);
        return launch_upload_convert<P>(resident_kparams<typename P::T>(c), dpos, dvel, drho, dp,
                                        dtype, n_inst > 1 ? c->inst_off : nullptr, n_inst,
                                        State<P>::y(c), c->hash_x, c->err, s);
    }));
}

extern "C" int sph_upload(sph_ctx* c, const float* pos, const float* vel, const float* rho,
                          const float* p, const int* type, int n, int from_host, void* stream) {
    return upload_impl(c, pos, vel, rho, p, type, nullptr, 1, n, from_host, stream);
}

extern "C" int sph_upload_instances(sph_ctx* c, const float* pos, const float* vel,
                                    const float* rho, const float* p, const int* type,
                                    const int* offsets, int n_inst, int n, int from_host,
                                    void* stream) {
    return upload_impl(c, pos, vel, rho, p, type, offsets, n_inst, n, from_host, stream);
}

extern "C" int sph_instances(const sph_ctx* c, int* n_inst) {
    if (!c || !n_inst) return SPH_ERR_ARG;
    *n_inst = c->n_inst;
    return SPH_OK;
}

extern "C" int sph_download(sph_ctx* c, float* pos, float* vel, float* rho, float* p, int* type,
                            int to_host, void* stream) {
    if (!c) return SPH_ERR_ARG;
    if (!c->loaded) return SPH_ERR_STATE;
    const int n = c->n;
    if (n == 0) return SPH_OK;
    cudaStream_t s = (cudaStream_t)stream;
    auto convert = [&](float* dpos, float* dvel, float* drho, float* dp, int* dtype) {
        return with_prec(c, [&](auto tag) {
            using P = decltype(tag);
            return launch_download_convert<P>(resident_kparams<typename P::T>(c), State<P>::y(c),
                                              dpos, dvel, drho, dp, dtype, s);
        });
    };
    if (!to_host) return to_status(convert(pos, vel, rho, p, type));
    Staging st = staging(c, n);
    float* spos = pos ? st.pos : nullptr;
    float* svel = vel ? st.vel : nullptr;
    float* srho = rho ? st.rho : nullptr;
    float* sp = p ? st.p : nullptr;
    int* stype = type ? st.type : nullptr;
    if (convert(spos, svel, srho, sp, stype) != cudaSuccess) return SPH_ERR_CUDA;
    if ((pos && cudaMemcpyAsync(pos, spos, (size_t)n * 12, cudaMemcpyDeviceToHost, s) != cudaSuccess) ||
        (vel && cudaMemcpyAsync(vel, svel, (size_t)n * 12, cudaMemcpyDeviceToHost, s) != cudaSuccess) ||
        (rho && cudaMemcpyAsync(rho, srho, (size_t)n * 4, cudaMemcpyDeviceToHost, s) != cudaSuccess) ||
        (p && cudaMemcpyAsync(p, sp, (size_t)n * 4, cudaMemcpyDeviceToHost, s) != cudaSuccess) ||
        (type && cudaMemcpyAsync(type, stype, (size_t)n * 4, cudaMemcpyDeviceToHost, s) != cudaSuccess))
        return SPH_ERR_CUDA;
    return SPH_OK;
}

extern "C" int sph_download_f64(sph_ctx* c, double* pos, double* vel, double* rho, double* p,
                                int to_host, void* stream) {
    if (!c) return SPH_ERR_ARG;
    if (!c->loaded) return SPH_ERR_STATE;
    const int n = c->n;
    if (n == 0) return SPH_OK;
    cudaStream_t s = (cudaStream_t)stream;
    auto convert = [&](double* dpos, double* dvel, double* drho, double* dp) {
        return with_prec(c, [&](auto tag) {
            using P = decltype(tag);
            return launch_download_f64<P>(resident_kparams<typename P::T>(c), State<P>::y(c),
                                          dpos, dvel, drho, dp, s);
        });
    };
    if (!to_host) return to_status(convert(pos, vel, rho, p));
    // staging in buffers that hold nothing between steps: the scratch set's records
    // (>= 32 B per particle) for positions and the pass-1 records for velocities, the scratch
    // set's predictor arrays (>= 16 B per particle) for density and pressure
    const bool d = c->prec == SPH_PREC_FP64;
    double* spos = d ? reinterpret_cast<double*>(c->xd.rec) : reinterpret_cast<double*>(c->x.rec);
    double* svel = d ? reinterpret_cast<double*>(c->p1d.nrec) : reinterpret_cast<double*>(c->p1.nrec);
    double* srho = d ? reinterpret_cast<double*>(c->xd.tpos) : reinterpret_cast<double*>(c->x.tpos);
    double* sp = d ? reinterpret_cast<double*>(c->xd.tvel) : reinterpret_cast<double*>(c->x.tvel);
    if (convert(pos ? spos : nullptr, vel ? svel : nullptr, rho ? srho : nullptr,
                p ? sp : nullptr) != cudaSuccess)
        return SPH_ERR_CUDA;
    if ((pos && cudaMemcpyAsync(pos, spos, (size_t)n * 24, cudaMemcpyDeviceToHost, s) != cudaSuccess) ||
        (vel && cudaMemcpyAsync(vel, svel, (size_t)n * 24, cudaMemcpyDeviceToHost, s) != cudaSuccess) ||
        (rho && cudaMemcpyAsync(rho, srho, (size_t)n * 8, cudaMemcpyDeviceToHost, s) != cudaSuccess) ||
        (p && cudaMemcpyAsync(p, sp, (size_t)n * 8, cudaMemcpyDeviceToHost, s) != cudaSuccess))
        return SPH_ERR_CUDA;
    return SPH_OK;
}

extern "C" int sph_probe_read(sph_ctx* c, const sph_probe* probes, int nprobes, double* values,
                              double cfl, sph_stats* stats, void* stream) {
    if (!c || nprobes < 0 || nprobes > SPH_MAX_PROBES || (nprobes > 0 && (!probes || !values)))
        return SPH_ERR_ARG;
    if (!c->loaded) return SPH_ERR_STATE;
    cudaStream_t s = (cudaStream_t)stream;
    std::vector<double> acc(probe_acc_words(), 0.0);
    if (c->n > 0) {
        const cudaError_t e = with_prec(c, [&](auto tag) {
            using P = decltype(tag);
            return launch_probes<P>(resident_kparams<typename P::T>(c), State<P>::y(c), probes,
                                    nprobes, c->probe_acc, s);
        });
        if (e != cudaSuccess ||
            cudaMemcpyAsync(acc.data(), c->probe_acc, acc.size() * sizeof(double),
                            cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return SPH_ERR_CUDA;
    }
    probe_results(acc.data(), probes, nprobes, cfl, c->P.h, c->P.cs, stats, values);
    return SPH_OK;
}

extern "C" int sph_snapshot_wait(sph_ctx* c) {
    if (!c) return SPH_ERR_ARG;
    if (!c->snap_pending) return SPH_OK;
    const cudaError_t e = cudaEventSynchronize(c->snap_done);
    c->snap_pending = false;
    return to_status(e);
}

extern "C" int sph_snapshot_query(sph_ctx* c, int* done) {
    if (!c || !done) return SPH_ERR_ARG;
    if (!c->snap_pending) {
        *done = 1;
        return SPH_OK;
    }
    const cudaError_t e = cudaEventQuery(c->snap_done);
    if (e == cudaErrorNotReady) {
        *done = 0;
        return SPH_OK;
    }
    *done = 1;
    return to_status(e);
}

extern "C" int sph_snapshot_begin(sph_ctx* c, float* pos, float* vel, float* rho, float* p,
                                  int* type, void* stream) {
    if (!c) return SPH_ERR_ARG;
    if (!c->loaded) return SPH_ERR_STATE;
    // the snapshot buffers are reused: the previous snapshot's copies must have finished
    int st = sph_snapshot_wait(c);
    if (st != SPH_OK) return st;
    const int n = c->n;
    if (n == 0) return SPH_OK;
    cudaStream_t s = (cudaStream_t)stream;
    float* spos = c->snap_f;
    float* svel = c->snap_f + 3 * (size_t)n;
    float* srho = c->snap_f + 6 * (size_t)n;
    float* sp = c->snap_f + 7 * (size_t)n;
    const cudaError_t e = with_prec(c, [&](auto tag) {
        using P = decltype(tag);
        return launch_download_convert<P>(resident_kparams<typename P::T>(c), State<P>::y(c),
                                          pos ? spos : nullptr, vel ? svel : nullptr,
                                          rho ? srho : nullptr, p ? sp : nullptr,
                                          type ? c->snap_type : nullptr, s);
    });
    if (e != cudaSuccess || cudaEventRecord(c->snap_ready, s) != cudaSuccess ||
        cudaStreamWaitEvent(c->copy_stream, c->snap_ready, 0) != cudaSuccess)
        return SPH_ERR_CUDA;
    cudaStream_t cs = c->copy_stream;
    if ((pos && cudaMemcpyAsync(pos, spos, (size_t)n * 12, cudaMemcpyDeviceToHost, cs) != cudaSuccess) ||
        (vel && cudaMemcpyAsync(vel, svel, (size_t)n * 12, cudaMemcpyDeviceToHost, cs) != cudaSuccess) ||
        (rho && cudaMemcpyAsync(rho, srho, (size_t)n * 4, cudaMemcpyDeviceToHost, cs) != cudaSuccess) ||
        (p && cudaMemcpyAsync(p, sp, (size_t)n * 4, cudaMemcpyDeviceToHost, cs) != cudaSuccess) ||
        (type && cudaMemcpyAsync(type, c->snap_type, (size_t)n * 4, cudaMemcpyDeviceToHost, cs) != cudaSuccess) ||
        cudaEventRecord(c->snap_done, cs) != cudaSuccess)
        return SPH_ERR_CUDA;
    c->snap_pending = true;
    return SPH_OK;
}

static int step_impl(sph_ctx* c, int nsteps, void* stream);

extern "C" int sph_step(sph_ctx* c, int nsteps, void* stream) {
    if (!c || nsteps < 0) return SPH_ERR_ARG;
    if (!c->loaded) return SPH_ERR_STATE;
    const int st = step_impl(c, nsteps, stream);
    // after a half step the live set is in the order of its cell and neighbour lists
    if (st != SPH_OK) c->sorted = false;
    else if (nsteps > 0 && c->n > 0) c->sorted = true;
    return st;
}

static int step_impl(sph_ctx* c, int nsteps, void* stream) {
    if (c->n == 0 || nsteps == 0) {
        c->steps += nsteps;
        return SPH_OK;
    }
    cudaStream_t s = (cudaStream_t)stream;
    if (c->rehash) {
        // the grid changed (sph_set_params, skin option): the keys pass 2 wrote for the
        // current positions index the old grid
        const cudaError_t e = with_prec(c, [&](auto tag) {
            using P = decltype(tag);
            return launch_rehash<P>(resident_kparams<typename P::T>(c), State<P>::y(c), c->hash_x,
                                    c->err, s);
        });
        if (e != cudaSuccess) return SPH_ERR_CUDA;
        c->rehash = false;
    }
    if (c->opt_profile) {
        for (int i = 0; i < nsteps; i++) {
            cudaError_t e = full_step(c, s, c->ev);
            if (e != cudaSuccess) return SPH_ERR_CUDA;
            if (cudaEventSynchronize(c->ev[2 * EV_PER_HALF - 1]) != cudaSuccess) return SPH_ERR_CUDA;
            for (int h = 0; h < 2; h++)
                for (int ph = 0; ph < PH_COUNT; ph++) {
                    if (ph == PH_NBR && !list_for(c)) continue;
                    float ms = 0.f;
                    cudaEventElapsedTime(&ms, c->ev[EV_PER_HALF * h + ph],
                                         c->ev[EV_PER_HALF * h + ph + 1]);
                    c->phase_ms[ph] += ms;
                    c->phase_launches[ph] += 1;
                }
            c->steps++;
        }
        return SPH_OK;
    }
    const bool graph_ok = c->opt_use_graph && s != nullptr;
    if (!graph_ok) {
        for (int i = 0; i < nsteps; i++) {
            if (full_step(c, s, nullptr) != cudaSuccess) return SPH_ERR_CUDA;
            c->steps++;
        }
        return SPH_OK;
    }
    if (!c->graph || c->graph_stream != s || c->graph_n != c->n) {
        drop_graph(c);
        cudaGraph_t g = nullptr;
        // rebuild kernels under conditional nodes when the driver takes them, else gated
        if (c->opt_cond_graph && c->side_stream && build_conditional_graph(c, s, &g) == cudaSuccess) {
            if (cudaGraphInstantiate(&c->graph, g, 0) != cudaSuccess) {
                c->graph = nullptr;
                cudaGetLastError();
            }
            cudaGraphDestroy(g);
            g = nullptr;
        }
        c->graph_conditional = c->graph != nullptr;
        if (!c->graph) {
            if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
                return SPH_ERR_CUDA;
            cudaError_t e = full_step(c, s, nullptr);
            cudaError_t e2 = cudaStreamEndCapture(s, &g);
            if (e != cudaSuccess || e2 != cudaSuccess) {
                if (g) cudaGraphDestroy(g);
                cudaGetLastError();
                return SPH_ERR_CUDA;
            }
            const cudaError_t ei = cudaGraphInstantiate(&c->graph, g, 0);
            cudaGraphDestroy(g);
            if (ei != cudaSuccess) {
                c->graph = nullptr;
                cudaGetLastError();
                return SPH_ERR_CUDA;
            }
        }
        c->graph_stream = s;
        c->graph_n = c->n;
    }
    for (int i = 0; i < nsteps; i++) {
        if (cudaGraphLaunch(c->graph, s) != cudaSuccess) return SPH_ERR_CUDA;
        c->steps++;
    }
    return SPH_OK;
}

extern "C" int sph_step_host(sph_ctx* c, float* pos, float* vel, float* rho, float* p, int* type,
                             int n, int nsteps, void* stream) {
    int st = sph_upload(c, pos, vel, rho, p, type, n, 1, stream);
    if (st != SPH_OK) return st;
    st = sph_step(c, nsteps, stream);
    if (st != SPH_OK) return st;
    st = sph_download(c, pos, vel, rho, p, nullptr, 1, stream);
    if (st != SPH_OK) return st;
    return cudaStreamSynchronize((cudaStream_t)stream) == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

extern "C" int sph_ctx_sorted_view(sph_ctx* c, const int** cell_start, const int** sorted_id,
                                   const int** sorted_hash, int* num_cells) {
    if (!c) return SPH_ERR_ARG;
    if (num_cells) *num_cells = c->Pi.num_cells;
    if (cell_start) *cell_start = c->cell_start;
    if (sorted_id) *sorted_id = c->prec == SPH_PREC_FP64 ? c->yd.id : c->y.id;
    if (sorted_hash) *sorted_hash = reinterpret_cast<const int*>(c->keys_sorted);
    return SPH_OK;
}

extern "C" int sph_read_error_flags(sph_ctx* c, unsigned* flags, void* stream) {
    if (!c || !flags) return SPH_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    unsigned h = 0;
    if (cudaMemcpyAsync(&h, c->err, sizeof(unsigned), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess ||
        cudaMemsetAsync(c->err, 0, sizeof(unsigned), s) != cudaSuccess)
        return SPH_ERR_CUDA;
    *flags = h;
    return SPH_OK;
}

extern "C" int sph_steps_taken(const sph_ctx* c, long long* steps) {
    if (!c || !steps) return SPH_ERR_ARG;
    *steps = c->steps;
    return SPH_OK;
}

extern "C" int sph_profile_read(sph_ctx* c, double* ms, long long* launches, int reset) {
    if (!c) return SPH_ERR_ARG;
    for (int i = 0; i < PH_COUNT; i++) {
        if (ms) ms[i] = c->phase_ms[i];
        if (launches) launches[i] = c->phase_launches[i];
        if (reset) {
            c->phase_ms[i] = 0.0;
            c->phase_launches[i] = 0;
        }
    }
    return SPH_OK;
}

// ---------------------------------------------------------------- drop-in SPH_NS
extern "C" int sph_ns(sph_ctx* c, float* s_pos, float* s_vel, float* s_rho, float* s_p,
                      const int* s_type, float* rho_dt, float* vel_dt, const int* cell_start,
                      const int* cell_end, int n, const int* hash, float* dofv, float* rhop_sum,
                      float* w_sum, void* stream) {
    (void)cell_start;
    (void)cell_end;  // the dense cell starts are rebuilt from the sorted hash
    if (!c || n < 0 || n > c->capacity) return SPH_ERR_ARG;
    if (c->prec == SPH_PREC_FP64) return SPH_ERR_STATE;  // the drop-in runs the FP32 kernels
    if (n == 0) return SPH_OK;
    if (!s_pos || !s_vel || !s_rho || !s_p || !s_type || !rho_dt || !vel_dt || !hash || !dofv)
        return SPH_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    KParams k = make_kparams(c->P, n);
    k.park_inactive = 0;  // the drop-in takes the caller's cells as they are
    if (launch_aos_to_set(k, s_pos, s_vel, s_rho, s_p, s_type, hash, c->x, c->keys_sorted,
                          c->err, s) != cudaSuccess)
        return SPH_ERR_CUDA;
    if (build_cell_starts(c->keys_sorted, n, c->P.num_cells, c->cell_start, s) != cudaSuccess)
        return SPH_ERR_CUDA;
    // the drop-in builds and uses its list within this call, with the constant cutoff
    NbrList dl = c->nl;
    dl.cut2 = nullptr;
    dl.fluid_cells = nullptr;
    const NbrList* nl = list_for(c) ? &dl : nullptr;
    if (nl && launch_nbr_build<PrecF32>(k, c->x, c->keys_sorted, c->cell_start, *nl,
                                        c->opt_wall_rates, c->err, s) != cudaSuccess)
        return SPH_ERR_CUDA;
    if (launch_pass1<PrecF32>(k, c->x, c->keys_sorted, c->cell_start, nl, c->p1, rhop_sum,
                              w_sum, s) != cudaSuccess)
        return SPH_ERR_CUDA;
    if (launch_pass2_rates(k, c->x, c->keys_sorted, c->cell_start, nl, c->p1, rho_dt, vel_dt,
                           c->opt_wall_rates, s) != cudaSuccess)
        return SPH_ERR_CUDA;
    if (launch_ns_writeback(k, s_type, c->p1.self, s_rho, s_p, dofv, s) != cudaSuccess)
        return SPH_ERR_CUDA;
    // the resident state (y) is untouched, but the cell and neighbour lists now describe these
    // arrays: a later sph_step rebuilds them first
    return force_rebuild(c, s) == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

extern "C" int sph_read_list_skin(sph_ctx* c, float* skin, void* stream) {
    if (!c || !skin) return SPH_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    unsigned h = 0;
    if (cudaMemcpyAsync(&h, c->rb + RB_SKIN, sizeof(unsigned), cudaMemcpyDeviceToHost, s) !=
            cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return SPH_ERR_CUDA;
    std::memcpy(skin, &h, sizeof(float));
    return SPH_OK;
}

extern "C" int sph_read_instance_rebuild_counts(sph_ctx* c, unsigned* counts, int n,
                                                void* stream) {
    if (!c || !counts || n < 1 || n > c->n_inst) return SPH_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    if (c->n_inst == 1 || !per_instance(c)) {
        // one decision for all: every instance rebuilt with the whole set
        unsigned h = 0;
        if (sph_read_rebuild_count(c, &h, stream) != SPH_OK) return SPH_ERR_CUDA;
        for (int b = 0; b < n; b++) counts[b] = h;
        return SPH_OK;
    }
    if (cudaMemcpy2DAsync(counts, sizeof(unsigned), c->iw + IW_STRIDE + IW_COUNT,
                          IW_STRIDE * sizeof(unsigned), sizeof(unsigned), (size_t)n,
                          cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return SPH_ERR_CUDA;
    return SPH_OK;
}

extern "C" int sph_read_rebuild_count(sph_ctx* c, unsigned* count, void* stream) {
    if (!c || !count) return SPH_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    unsigned h = 0;
    if (cudaMemcpyAsync(&h, c->rb + 3, sizeof(unsigned), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return SPH_ERR_CUDA;
    *count = h;
    return SPH_OK;
}
