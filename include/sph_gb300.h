/*
 * sph_gb300.h — C ABI of the GB300-native weakly-compressible delta-SPH hot path.
 *
 * The hot path is the one the reference CUDA solver runs every half step:
 *   cell-list build (particle -> cell hash, stable radix sort, permutation of the particle
 *   arrays, cell start/end)  ->  neighbour pass 1 (wall pressure extrapolation, fluid
 *   velocity divergence)  ->  neighbour pass 2 (continuity with delta density diffusion,
 *   momentum with pressure, acoustic damper, artificial viscosity, gravity)  ->  midpoint
 *   predictor-corrector integrator.
 *
 * Two families of entry points:
 *
 *  1. Drop-in functions.  Same arguments, layout and meaning as the reference's host
 *     functions (AoS float[3N] positions/velocities, int cellStart/cellEnd with -1 for an
 *     empty cell, one thread of work per particle).  Every pointer is a caller-owned device
 *     buffer.  Each function returns an sph_status and takes an explicit stream
 *     (a cudaStream_t passed as void*, NULL = legacy default stream).  The reference
 *     functions return nothing and read their constants from a __constant__ SimParams;
 *     here the constants travel in an sph_params (by value into every kernel) or in an
 *     sph_ctx.
 *
 *  2. Resident solver (sph_ctx).  Keeps the particle state on the GPU in cell-sorted SoA
 *     order and advances whole predictor-corrector steps with fused kernels; optionally
 *     replays each step as a CUDA graph.  This is the fast path; its physics is the same.
 *
 * No function here allocates device memory except sph_create (everything a context needs),
 * and sph_set_params / sph_ctx_set_option when a new grid or list needs more room than the
 * context holds.
 * All functions are host functions; none is thread-safe on the same sph_ctx.
 */
#ifndef SPH_GB300_H
#define SPH_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status codes */
typedef enum sph_status {
    SPH_OK = 0,
    SPH_ERR_ARG = -1,        /* bad argument (NULL pointer, n < 0, n > capacity, ...) */
    SPH_ERR_CUDA = -2,       /* a CUDA runtime call or kernel launch failed */
    SPH_ERR_NOMEM = -3,      /* device allocation failed (sph_create / sph_ctx_reserve) */
    SPH_ERR_DEVICE = -4,     /* a kernel raised a device error flag (see SPH_FLAG_*) */
    SPH_ERR_STATE = -5,      /* call out of order (e.g. sph_step before sph_upload) */
    SPH_ERR_SCRATCH = -6     /* caller-provided scratch too small */
} sph_status;

/* Device error flags, read with sph_read_error_flags. */
#define SPH_FLAG_OUT_OF_GRID   0x1u  /* a particle hashed outside the grid; its cell index was clamped */
#define SPH_FLAG_KEY_RANGE     0x2u  /* a sort key was outside [0, 2^key_bits) */
#define SPH_FLAG_NONFINITE     0x4u  /* a non-finite position was seen by the hash kernel */
#define SPH_FLAG_NEIGHBOR_OVERFLOW 0x8u  /* a particle had more neighbours than the list holds;
                                            it walked its cells instead (results unaffected) */

/* EOS selector: the reference hard-codes the linear form p = cs^2 (rho - rho0)
 * (src/sph/sph_run.cu:467,515); TAIT is p = B((rho/rho0)^gamma - 1), B = rho0 cs^2/gamma. */
#define SPH_EOS_LINEAR 0
#define SPH_EOS_TAIT   1

/* Particle kinds, as in the reference: 0 wall, 1 fluid, 2 rigid (every non-1 kind is
 * treated as a boundary particle; src/sph/sph_run.cu:36). */
#define SPH_TYPE_WALL  0
#define SPH_TYPE_FLUID 1
#define SPH_TYPE_RIGID 2

/* ---------------------------------------------------------------- parameters */
/* Constants of one simulation.  The reference keeps the same quantities in
 * `SimParams` (src/header/data_struct.cuh:4-44), copied once to `__constant__ par`
 * (src/sph/sph_run.cu:105). */
typedef struct sph_params {
    int   num_particles;     /* N = fluid + boundary particles */
    int   num_boundary;      /* boundary (non-fluid) particle count, informational */
    float dt;                /* full predictor-corrector step (timeStep) */
    float gravity;           /* z acceleration (g, negative = down) */
    float cell_size;         /* gridSize */
    float grid_min[3];       /* gridxmin, gridymin, gridzmin */
    float grid_max[3];       /* gridxmax, gridymax, gridzmax */
    int   grid_dim[3];       /* gridxdim, gridydim, gridzdim */
    int   num_cells;         /* gx*gy*gz; cell hash = (z*gy + y)*gx + x */
    float dx;                /* particleR: lattice spacing */
    float h;                 /* smoothing length */
    float kh;                /* support radius 2h */
    float eta;               /* 0.1 h regulariser */
    float delta;             /* delta-SPH diffusion coefficient */
    float alpha;             /* artificial viscosity coefficient (afa) */
    float adh;               /* Wendland C2 3-D normalisation 21/(16 pi h^3) */
    float mass;              /* particleMass = dx^3 rho0 */
    float rho0;              /* restDensity */
    float cs;                /* numerical speed of sound */
    int   eos;               /* SPH_EOS_LINEAR or SPH_EOS_TAIT */
    float tait_gamma;        /* gamma of the Tait EOS (7) */
    float tait_b;            /* B = rho0 cs^2 / gamma */
    int   clamp_density;     /* 1: rho >= rho0 after each update (reference behaviour) */
    float escape_min[3];     /* a fluid particle outside [escape_min, escape_max] ... */
    float escape_max[3];
    float escape_park[3];    /* ... is parked here with v = 0, p = 0, rho = rho0 */
    int   park_inactive;     /* 0: parked particles stay in the neighbour search at the
                              * parking point (reference behaviour); 1: a fluid particle outside
                              * the escape box leaves it (sorted after every cell, no pairs) */
    int   reserved[7];
} sph_params;

/* Inputs from which sph_params_derive computes the derived constants with the same
 * mixed double/float rounding as the reference's main (src/sph/sph_run.cu:60-101). */
typedef struct sph_config {
    float  dx;               /* lattice spacing */
    double h_factor;         /* h = h_factor * dx (reference: 1.5) */
    float  rho0;             /* 1000 */
    float  cs;               /* speed of sound (reference: 25) */
    float  gravity;          /* -9.81 */
    float  delta;            /* reference: 0.2 */
    float  alpha;            /* reference: 0.05 */
    float  dt;               /* > 0: fixed step; <= 0: dt = cfl * h / cs */
    float  cfl;              /* used when dt <= 0 */
    int    eos;              /* SPH_EOS_LINEAR / SPH_EOS_TAIT */
    float  tait_gamma;       /* 7 */
    float  domain_min[3];    /* tank box; the grid is this box padded by `pad` */
    float  domain_max[3];
    double pad;              /* reference: 0.1 m on every side */
    double cell_factor;      /* cell size = cell_factor * kh (reference: 1) */
    float  escape_min[3];
    float  escape_max[3];
    float  escape_park[3];
    int    num_particles;
    int    num_boundary;
    int    clamp_density;
} sph_config;

/* Layout-compatible copy of the reference's SimParams (src/header/data_struct.cuh:4-44),
 * so a reference driver can hand its host-side `temps` to sph_params_from_reference. */
typedef struct sph_ref_simparams {
    float timeStep, time;
    int numParticles, boundary_p_num;
    float gravity;
    float gridSize, gridxmin, gridymin, gridzmin, gridxmax, gridymax, gridzmax;
    int gridxdim, gridydim, gridzdim, numCells;
    int hash_max, hash_min;
    float pre_set_domain_x_min, pre_set_domain_x_max, pre_set_domain_y_min,
          pre_set_domain_y_max, pre_set_domain_z_min, pre_set_domain_z_max;
    float particleR, h, kh, eta, delta, afa;
    float SpikyKern, LapKern, Poly6Kern;
    float minDist;
    float particleMass, restDensity;
    float viscosity, stiffness;
    float cs;
    float adh;
    float namuta_threshold_1, namuta_threshold_2;
    float CFL, Ma, conc_0, conc_t, PST_R, PST_n, w_deltar;
    int ngp, nnode, n_edge, num_vp, max_nspnode, nele;
    float mat_para[3];
} sph_ref_simparams;

/* Derive parameters from a config.  Replaces the host block of src/sph/sph_run.cu:60-101. */
int sph_params_derive(const sph_config* cfg, sph_params* out);

/* The reference's own hard-coded case (src/sph/sph_run.cu:11-22,60-101): h = 1.5 dx,
 * delta 0.2, alpha 0.05, cs 25, dt 2e-4, linear EOS, tank vlx*vly*vlz padded by 0.1 m,
 * escape box x<=3.23, y<=1, z<=1 parked at (0, 0.5, -0.08) (src/sph/sph_run.cu:437-447). */
int sph_params_reference(float dx, float vlx, float vly, float vlz,
                         int num_particles, int num_boundary, sph_params* out);

/* Convert a reference SimParams into sph_params (linear EOS, reference escape box). */
int sph_params_from_reference(const sph_ref_simparams* in, sph_params* out);
/* And back (fields the hot path does not use are zero). */
int sph_params_to_reference(const sph_params* in, sph_ref_simparams* out);

const char* sph_status_string(int status);
/* Library version string. */
const char* sph_version(void);

/* Measured FP32 arithmetic peak (no reference counterpart: the denominator of the solver's
 * FP32 roofline fraction).  Launches blocks x 256 threads of independent fused multiply-add
 * chains, `iters` rounds of 128 FMAs each, once to warm up and once timed by CUDA events on
 * `stream`; *flops receives the flops of the timed launch, *ms its duration.  sink: device
 * buffer of blocks * 256 floats (overwritten).  Synchronises the stream. */
int sph_measure_fp32_peak(float* sink, int blocks, int iters, double* flops, double* ms,
                          void* stream);

/* ---------------------------------------------------------------- drop-in functions */
/* calcHash (src/header/mesh.cuh:20, src/lib/mesh.cu:26-70): hash[i] = cell of pos[3i..3i+2],
 * index[i] = i.  The cell coordinate is floorf((p - grid_min)/cell_size) in IEEE FP32,
 * bit-identical to the reference for every in-grid position. */
int sph_calc_hash(const sph_params* p, const float* pos, int* hash, int* index, int n,
                  void* stream);

/* sortParticles (src/header/mesh.cuh:23, src/lib/mesh.cu:73-86): stable sort of (hash, index)
 * pairs by hash, in place.  key_bits = 32 sorts the full signed int range (same order as the
 * reference's thrust::sort_by_key); key_bits in [1,31] requires 0 <= hash < 2^key_bits and
 * runs ceil(key_bits/8) passes.  Scratch is caller-provided (sph_sort_scratch_bytes). */
int sph_sort_scratch_bytes(int n, size_t* bytes);
int sph_sort_particles(int* hash, int* index, int n, int key_bits,
                       void* scratch, size_t scratch_bytes, void* stream);

/* sph_sort_particles without a scratch argument and without allocating: no counterpart in
 * the reference.  For callers bound to the three-argument sortParticles form that may not
 * allocate device memory during a run.  Scratch is a fixed array of this library (one per
 * device, about 9.5 MB); n > SPH_SORT_NOALLOC_MAX_N returns SPH_ERR_SCRATCH.  The first call
 * on a device looks up that array's address (make it before any stream capture); later calls
 * outside a capture look it up again (so a cudaDeviceReset between calls is harmless), calls
 * inside one use the last address.  Nothing in the array needs to start at zero.  Calls on one
 * device whose executions overlap race on the shared array: order them on one stream or with
 * events. */
#define SPH_SORT_NOALLOC_MAX_N (1 << 20)
int sph_sort_particles_noalloc(int* hash, int* index, int n, int key_bits, void* stream);

/* reorder (src/header/mesh.cuh:29, src/lib/mesh.cu:89-159): cell_start[c] = first sorted
 * slot of cell c or -1 if empty, cell_end[c] = one past its last slot (untouched for an
 * empty cell), and gathers pos, vel (AoS), rho, p, type, zone into sorted order.
 * zone arrays may be NULL. */
int sph_reorder(const sph_params* p,
                const float* old_pos, const float* old_vel, const float* old_rho,
                const float* old_p, const int* old_type, const int* old_zone,
                float* s_pos, float* s_vel, float* s_rho, float* s_p, int* s_type, int* s_zone,
                const int* hash, const int* index, int* cell_start, int* cell_end, int n,
                void* stream);

/* recover (src/header/mesh.cuh:33, src/lib/mesh.cu:162-194): scatter sorted arrays back to
 * original order through index. zone arrays may be NULL. */
int sph_recover(float* pos, float* vel, float* rho, float* p, int n, const int* index,
                int* type, int* zone,
                const float* s_pos, const float* s_vel, const float* s_rho, const float* s_p,
                const int* s_type, const int* s_zone, void* stream);

/* PC_prediction / PC_correction (src/header/sph.cuh:26,28, src/sph/sph_run.cu:425-550):
 * midpoint predictor and corrector on sorted AoS arrays; the saved step-n state
 * (pos_tmp, vel_tmp, rho_tmp) is indexed by original particle id index[i]. */
int sph_pc_prediction(const sph_params* p, float* s_pos, float* s_vel, float* s_rho,
                      float* s_p, const float* rho_dt, const float* vel_dt, const int* index,
                      float* pos_tmp, float* vel_tmp, float* rho_tmp, int n,
                      const int* s_type, void* stream);
int sph_pc_correction(const sph_params* p, float* s_pos, float* s_vel, float* s_rho,
                      float* s_p, const float* rho_dt, const float* vel_dt, const int* index,
                      const float* pos_tmp, const float* vel_tmp, const float* rho_tmp, int n,
                      const int* s_type, void* stream);

/* ---------------------------------------------------------------- resident solver */
typedef struct sph_ctx sph_ctx;

/* Solver options (sph_ctx_set_option). */
#define SPH_OPT_USE_GRAPH     1  /* 1: sph_step replays one captured CUDA graph per step */
#define SPH_OPT_WALL_RATES    2  /* 1: sph_ns also fills rho_dt/vel_dt rows of boundary particles */
#define SPH_OPT_PROFILE       3  /* 1: sph_step times each phase with CUDA events (no graph; syncs per step) */
#define SPH_OPT_NEIGHBOR_LIST 4  /* 1 (default): one cell walk per half step fills a neighbour
                                    list both passes iterate; 0: each pass walks the cells */
#define SPH_OPT_NEIGHBOR_CAP  5  /* list slots per particle; 0 (default) = 1.5x the lattice
                                    neighbours of the list sphere (reallocates the list) */
#define SPH_OPT_SKIN_PERMILLE 6  /* neighbour-list skin in thousandths of the support radius kh
                                    (default 100; the cells are kh (1 + skin) wide).  The list
                                    keeps every pair closer than kh (1 + skin) and is rebuilt,
                                    cell list included, only when the bounding box of all
                                    displacements since the last build has a half-diagonal over
                                    skin/2 (decided on the GPU each half step); 0 rebuilds every
                                    half step as the reference does.  With
                                    SPH_OPT_ADAPTIVE_SKIN the lists use a skin up to this one */
#define SPH_OPT_CONDITIONAL_GRAPH 7  /* 1 (default): the replayed step graph holds the rebuild
                                    kernels under conditional nodes, so a half step that keeps
                                    its lists launches none of them; 0: they are launched and
                                    return at once (also the fallback when the driver refuses
                                    conditional nodes) */
#define SPH_OPT_PRECISION     8  /* SPH_PREC_* below; set before sph_upload (the state is
                                    reallocated; the uploaded state is dropped) */
#define SPH_OPT_BLOCK_THREADS 9  /* threads per block of the neighbour kernels: 32..256, a
                                    multiple of 32; 0 (default): 256 in FP32, 128 in the
                                    other precisions */
#define SPH_OPT_PARTICLES_PER_THREAD 10  /* particles each thread of the neighbour kernels
                                    handles, grid-stride (1..64, default 1) */
/* 11 is not used (it selected a two-particles-per-thread mode, measured slower and removed) */
#define SPH_OPT_ADAPTIVE_SKIN 13  /* 1 (default): each list rebuild picks the skin of the next
                             lists, between 0.02 and SPH_OPT_SKIN_PERMILLE, from how long the
                             last lists lasted (tight lists for slow flow, wide for fast); 0: the
                             lists always use SPH_OPT_SKIN_PERMILLE */
#define SPH_OPT_LANES_PER_PARTICLE 12  /* lanes of a warp per particle in list pass 1 (the
                             wall extrapolation and velocity divergence): 1 (one thread per
                             particle), 2, 4, 8 or 16 (a group of lanes shares a particle's list
                             and reduces its sums); 0 (default): 2 in FP32 with a list skin
                             on cells of the list cutoff (SPH_OPT_CELL_DIVISIONS 1), else 1.  With groups the lists store their entries interleaved in
                             windows of eight (a change rebuilds them).  Pass 2 runs one lane
                             per particle (groups were slower there at every size measured) */
#define SPH_OPT_PASS1_LANES 14  /* the same as SPH_OPT_LANES_PER_PARTICLE */
/* 15 is not used (it selected lane groups in pass 2, removed) */
#define SPH_OPT_CELL_DIVISIONS 16  /* cells per list cutoff of the resident grid: 1 (cells
                             of kh (1 + skin), the 27 around a particle's cell walked), 2 (cells
                             of half that, 125 walked) or 3 (a third, about dx at h = 1.3 dx:
                             343 walked, the reference's gridSize = dx of
                             opt_src_v4/sph/sph_run.cu:73); 0 (default): 3 in FP32, 1 in the
                             other precisions.  Smaller cells give the list build
                             fewer candidates for more cell lookups, and order the particles of
                             the cell-sorted state along finer x rows */
#define SPH_OPT_INSTANCE_DECISIONS 17  /* batched instances (sph_upload_instances) with a
                             neighbour list: 1: each instance keeps its own displacement box,
                             list skin and rebuild decision, so its lists are rebuilt in the same
                             half steps, with the same skins, as in a run of it alone and it
                             evolves bit for bit as it would alone (the slots of the instances
                             that keep their lists stay in place through the sort, and their
                             lists are not rebuilt); 0 (default): one box and one decision for
                             the whole batch, the fastest instance rebuilding all.  Every half
                             step in which any instance rebuilds still sorts and permutes the
                             whole batch, so similar instances, whose rebuilds fall in different
                             half steps, rebuild more often in all with 1 (64 dam breaks, 1000
                             steps: 42.5 against 31.8 ms per step).  With park_inactive, a
                             particle that leaves or rejoins the neighbour search moves the
                             slots after it and every instance rebuilds */


/* Precision of the resident solver (SPH_OPT_PRECISION); none has a reference counterpart. */
#define SPH_PREC_FP32  0  /* FP32 state and arithmetic, the reference's precision (default) */
#define SPH_PREC_FP64  1  /* FP64 state and arithmetic: the accuracy reference for the others */
#define SPH_PREC_MIXED 2  /* FP32 neighbour sums on relative positions rebuilt from cell-local
                             offsets; FP64 positions and density perturbation (rho - rho0) for
                             the time integration; n < 2^26 */
#define SPH_PREC_MIXED_COMP 3  /* SPH_PREC_MIXED with compensated (Neumaier) accumulation of the
                             density and force sums */
#define SPH_PREC_MIXED_ABS 4  /* FP64 master positions and density perturbation for the time
                             integration, as SPH_PREC_MIXED, but the neighbour sums run on FP32
                             positions in the simulation's own frame (rounded from the FP64
                             ones every half step) instead of cell-local offsets: the FP32
                             pair arithmetic, no per-pair cell code */

/* Phases reported by sph_profile_read: [0] radix sort, [1] gather + cell starts,
 * [2] neighbour-list build, [3] neighbour pass 1, [4] neighbour pass 2 + integrator;
 * summed over half steps. */
#define SPH_PHASE_COUNT 5

/* Create a context on the current CUDA device for up to `capacity` particles (allocates all
 * state and scratch once).  p may describe fewer particles than capacity. */
int sph_create(const sph_params* p, int capacity, sph_ctx** out);
int sph_destroy(sph_ctx* ctx);
int sph_set_params(sph_ctx* ctx, const sph_params* p);
int sph_get_params(const sph_ctx* ctx, sph_params* out);
int sph_ctx_set_option(sph_ctx* ctx, int option, int value);
/* The value an option has in effect (a default resolved: SPH_OPT_PASS1_LANES and
 * SPH_OPT_LANES_PER_PARTICLE give pass 1's lanes for the context's precision;
 * SPH_OPT_SKIN_PERMILLE the largest skin). */
int sph_ctx_get_option(const sph_ctx* ctx, int option, int* value);

/* SPH_NS_simpleversion (src/header/ns.cuh:4, src/equation/ns.cu:5-131 and :134-249): both
 * neighbour passes on sorted AoS arrays.  Writes dofv, rho_dt, vel_dt (AoS) and, for boundary
 * particles, the extrapolated pressure and density in place in s_p / s_rho.  rhop_sum and
 * w_sum (the wall extrapolation sums) are written when non-NULL.  Rows of rho_dt / vel_dt
 * for boundary particles are zero unless SPH_OPT_WALL_RATES is set (the integrator never
 * reads them).  cell_start/cell_end/hash are the outputs of sph_reorder/sph_calc_hash. */
int sph_ns(sph_ctx* ctx, float* s_pos, float* s_vel, float* s_rho, float* s_p,
           const int* s_type, float* rho_dt, float* vel_dt, const int* cell_start,
           const int* cell_end, int n, const int* hash, float* dofv, float* rhop_sum,
           float* w_sum, void* stream);

/* Load a particle state given in original order (AoS pos/vel [3n], rho, p, type [n]) from
 * host (from_host = 1) or device memory.  Resets the step counter.  After sph_step has run, an
 * upload of the same number of particles (and, batched, the same offsets) keeps the cell order
 * and neighbour lists: the next half step rebuilds them only if a particle moved more than half
 * the skin from where the lists were built, or changed kind.  The results equal those of a
 * continued sph_step run given the state it would hold (a loop of sph_step_host calls in FP32
 * gives the bits of one resident run). */
int sph_upload(sph_ctx* ctx, const float* pos, const float* vel, const float* rho,
               const float* p, const int* type, int n, int from_host, void* stream);
/* Batched instances (no reference counterpart): n particles of n_inst independent simulations
 * that share this context's sph_params (same tank, grid and constants), each in its own
 * coordinates; instance b owns particles [offsets[b], offsets[b+1]) of the arrays (`offsets`:
 * host array of n_inst + 1 ints, offsets[0] = 0, offsets[n_inst] = n).  Every kernel then
 * advances all instances in one launch.  The solver's grid stacks the instances along z with an
 * empty cell layer between them, so no neighbour search crosses instances and each instance
 * evolves exactly as it would alone.  Allocates when the stacked grid needs more cells than the
 * context holds.  sph_download returns all n particles in upload order; sph_probe_read reduces
 * over all instances.  sph_upload returns the context to one simulation. */
#define SPH_MAX_INSTANCES 4096
int sph_upload_instances(sph_ctx* ctx, const float* pos, const float* vel, const float* rho,
                         const float* p, const int* type, const int* offsets, int n_inst, int n,
                         int from_host, void* stream);
int sph_instances(const sph_ctx* ctx, int* n_inst);
/* Write the current state back in original order; any pointer may be NULL. */
int sph_download(sph_ctx* ctx, float* pos, float* vel, float* rho, float* p, int* type,
                 int to_host, void* stream);
/* The same in double (no reference counterpart): FP64 positions and density of the FP64 and
 * mixed-precision solvers without rounding to float, FP32 values widened otherwise.  For
 * accuracy studies against an FP64 run. */
int sph_download_f64(sph_ctx* ctx, double* pos, double* vel, double* rho, double* p,
                     int to_host, void* stream);
/* Advance nsteps full predictor-corrector steps (two cell-list builds, four neighbour passes
 * per step), asynchronously on `stream`. */
int sph_step(sph_ctx* ctx, int nsteps, void* stream);
/* End-to-end call with host buffers: upload, nsteps steps, download into the same buffers;
 * synchronises the stream before returning. */
int sph_step_host(sph_ctx* ctx, float* pos, float* vel, float* rho, float* p, int* type,
                  int n, int nsteps, void* stream);
/* Views of the last cell-list rebuild for diagnostics / tests (device pointers owned by ctx):
 * dense cell starts [num_cells + 1], original id per slot, sorted cell key per slot, and the
 * number of cells of the solver's grid (cells of kh (1 + skin)). */
int sph_ctx_sorted_view(sph_ctx* ctx, const int** cell_start, const int** sorted_id,
                        const int** sorted_hash, int* num_cells);
/* Read and clear the device error flags (synchronises the stream). */
int sph_read_error_flags(sph_ctx* ctx, unsigned* flags, void* stream);
/* Steps taken since the last upload. */
int sph_steps_taken(const sph_ctx* ctx, long long* steps);
/* Accumulated milliseconds and launch counts per phase under SPH_OPT_PROFILE
 * (arrays of SPH_PHASE_COUNT); reset != 0 clears them. */
int sph_profile_read(sph_ctx* ctx, double* ms, long long* launches, int reset);
/* Cell-list / neighbour-list rebuilds since the last upload (synchronises the stream); with
 * per-instance decisions (SPH_OPT_INSTANCE_DECISIONS), the half steps in which any instance
 * rebuilt. */
int sph_read_rebuild_count(sph_ctx* ctx, unsigned* count, void* stream);
/* List rebuilds of each of the first n instances of a batch since the upload (host array of n;
 * synchronises the stream).  Without per-instance decisions every instance reports the count
 * of sph_read_rebuild_count. */
int sph_read_instance_rebuild_counts(sph_ctx* ctx, unsigned* counts, int n, void* stream);
/* Skin of the current neighbour lists as a fraction of kh (synchronises the stream); with
 * per-instance decisions, the largest skin of the instances. */
int sph_read_list_skin(sph_ctx* ctx, float* skin, void* stream);

/* ---------------------------------------------------------------- probes and reductions */
/* Measurements of the resident state computed on the GPU (no reference counterpart: the
 * reference copies the whole state to the host every output interval and scans it there for
 * its gauges, src/io/io.cu:236-279). */
#define SPH_PROBE_PRESSURE 0  /* Shepard-normalised Wendland average of fluid pressure within kh
                                 of (x, y, z); 0 when no fluid is in range */
#define SPH_PROBE_HEIGHT   1  /* water height: largest z of fluid particles with |x - x0| < radius,
                                 |y - y0| < radius and, if zmax > 0, z < zmax (the reference's
                                 gauges use radius 1.5 dx); 0 when none */
#define SPH_PROBE_FRONT    2  /* surge front: largest x of any fluid particle */
#define SPH_MAX_PROBES 32
typedef struct sph_probe {
    int   kind;
    float x, y, z;
    float radius;
    float zmax;
} sph_probe;

/* Global FP64 reductions over the fluid particles. */
typedef struct sph_stats {
    long long fluid;     /* fluid particles */
    long long parked;    /* of which parked at escape_park after leaving the escape box */
    double mass;         /* sum of masses */
    double kinetic;      /* sum m |v|^2 / 2 */
    double potential;    /* sum -m g z (gravity along z) */
    double max_speed;
    double rho_min, rho_max;
    double front_x;      /* largest x */
    double cfl_dt;       /* cfl h / (cs + max_speed): the step a CFL rule with this number
                            would take now (the solver itself keeps the fixed dt) */
} sph_stats;

/* Evaluate nprobes (<= SPH_MAX_PROBES) probes into values[] (Pa or m) and, if stats is not
 * NULL, the reductions with CFL number cfl.  One kernel over the resident state; synchronises
 * the stream to return the numbers. */
int sph_probe_read(sph_ctx* ctx, const sph_probe* probes, int nprobes, double* values,
                   double cfl, sph_stats* stats, void* stream);

/* ---------------------------------------------------------------- output */
/* Asynchronous snapshot (no reference counterpart: the reference copies the state to the host
 * synchronously before each output, src/sph/sph_run.cu:262-267).  Writes the state in original
 * order into buffers of the context on `stream`, then copies it into the given host buffers
 * (pinned for the copy to overlap; any may be NULL) on an internal copy stream, so steps
 * launched after this call run while the copy is in flight.  A second snapshot waits for the
 * first one's copies. */
int sph_snapshot_begin(sph_ctx* ctx, float* pos, float* vel, float* rho, float* p, int* type,
                       void* stream);
/* Wait until the last snapshot is in the host buffers. */
int sph_snapshot_wait(sph_ctx* ctx);
/* *done = 1 when the last snapshot's copies have completed (or there is none), else 0. */
int sph_snapshot_query(sph_ctx* ctx, int* done);
/* Legacy-VTK particle file in the reference's layout (src/io/io.cu:154-199,
 * opt_src_v3/io/io.cu:121-200): UNSTRUCTURED_GRID POINTS with POINT_DATA "p" and "velocity",
 * plus "type" when given; binary = 1 writes big-endian floats, 0 text. */
int sph_write_vtk(const char* path, int n, const float* pos, const float* vel, const float* p,
                  const int* type, int binary);

/* ---------------------------------------------------------------- reference-signature shim */
/* The library also exports, with C++ linkage, the reference's own host functions calcHash,
 * sortParticles, reorder, recover, SPH_NS_simpleversion, PC_prediction, PC_correction,
 * iDivUp and computeGridSize (src/header/mesh.cuh:14-33, ns.cuh:4, sph.cuh:26-28), forwarding
 * to the functions above on the legacy default stream.  The reference functions read their
 * constants from `__constant__ par`; a reference driver hands the same SimParams to the shim
 * once, right after its cudaMemcpyToSymbol (src/sph/sph_run.cu:105). */
int sph_shim_set_reference_params(const sph_ref_simparams* p);
/* Or full sph_params (EOS, escape box and other options the reference hard-codes). */
int sph_shim_set_params(const sph_params* p);
/* Free the shim's lazily allocated scratch and context. */
int sph_shim_release(void);

/* ---------------------------------------------------------------- initial conditions */
/* Seeded dam-break generator: fluid block on a lattice at (i+1/2)dx, `wall_layers` lattice
 * layers outside the floor and four side walls of the tank (open top), an optional box
 * obstacle of rigid particles, uniform jitter of +-jitter*dx per coordinate.  Replaces the
 * reference's missing input files read by ini_fluid (src/io/io.cu:6-111). */
typedef struct sph_dam_break {
    float  dx;
    float  tank[3];          /* tank interior size, origin at 0 */
    float  block[3];         /* water block size at the x=0, y=0 corner, from the floor */
    int    wall_layers;      /* 3 */
    int    has_obstacle;
    float  obstacle_min[3];  /* obstacle box (rigid particles fill it on the lattice) */
    float  obstacle_max[3];
    float  jitter;           /* fraction of dx */
    unsigned long long seed;
    int    hydrostatic;      /* 1: p = rho0 |g| (H - z) and rho from the EOS inverse */
    float  rho0, gravity, cs;
    int    eos;
    float  tait_gamma;
} sph_dam_break;

/* Count particles (fluid, boundary) without generating them. */
int sph_dam_break_count(const sph_dam_break* d, int* n_fluid, int* n_boundary);
/* Fill host arrays (pos/vel [3n], rho, p [n], type [n]); boundary particles first, then
 * fluid, as in the reference's input ordering (walls at indices < nb). */
int sph_dam_break_generate(const sph_dam_break* d, float* pos, float* vel, float* rho,
                           float* p, int* type, int n);
/* Write the seven whitespace text files ini_fluid reads (h_pos.dat, h_vel.dat, h_ac.dat,
 * rhop.dat, p.dat, particle_type.dat, particle_zone.dat) into directory `dir`
 * (src/io/io.cu:10-111); zone is written as 0. */
int sph_write_dat(const char* dir, const float* pos, const float* vel, const float* rho,
                  const float* p, const int* type, int n);
/* Read them back (the inverse of sph_write_dat / the reference's ini_fluid). */
int sph_read_dat(const char* dir, float* pos, float* vel, float* ac, float* rho, float* p,
                 int* type, int* zone, int n);

#ifdef __cplusplus
}
#endif

#endif /* SPH_GB300_H */
