/*
 * b2d.h — C ABI of the GB300 implementation of binary2d's explicit
 * finite-volume Runge–Kutta step on the block mesh.
 *
 * Drop-in boundary.  The reference exposes the step as the Rust generic
 *
 *     scheme::advance<H: Hydrodynamics>(state: State<H::Conserved>, hydro: H,
 *         mesh: &Mesh, physics: &Physics, fold: usize, timestep: &mut f64,
 *         block_data: &HashMap<BlockIndex, BlockData<C>>, runtime: &Runtime)
 *         -> Result<State<C>, HydroError>                    (src/scheme.rs:323-349)
 *
 * called once per loop iteration by main.rs:run (src/main.rs:159-167).  The
 * functions below replace that call: a context owns the device copy of the
 * `State` (conserved fields, time, iteration, per-block source ledger) and of
 * the `BlockData` background (scheme.rs:36-58), and b2d_advance() performs
 * `fold` Runge–Kutta steps with one dt computed at the start, exactly as
 * scheme::advance does.
 *
 * Conventions
 *  - Plain C types only; every buffer argument is caller-owned host memory
 *    unless the name says `device`.
 *  - Conserved arrays use the reference's block layout
 *    [num_blocks][num_blocks][block_size][block_size][nf], blocks in
 *    mesh.block_indexes() order (src/mesh.rs:84-89: i outer, j inner), zones
 *    row-major within a block (i ↔ x, j ↔ y, j contiguous), nf = 3 for
 *    isothermal (Σ, Σvx, Σvy) and 4 for Euler (Σ, Σvx, Σvy, E).
 *  - Source ledgers (ItemizedChange, src/state.rs:27-36) use
 *    [num_blocks][num_blocks][7][nf] with items ordered sink1, sink2, grav1,
 *    grav2, buffer, cooling, fake_mass.
 *  - A context is not thread-safe: one host thread drives it, as main.rs
 *    drives scheme::advance from one thread.
 *  - No C++ exception crosses this boundary; every call returns a b2d_status.
 *  - There is no CPU fallback: without a usable CUDA device b2d_create fails
 *    with B2D_ERR_CUDA.
 */
#ifndef B2D_H
#define B2D_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------ */
/* Status codes.  The hydro errors mirror HydroErrorType (src/physics.rs:25-36). */
typedef enum b2d_status {
    B2D_OK                 = 0,
    B2D_ERR_NEG_DENSITY    = 1,  /* HydroErrorType::NegativeDensity            */
    B2D_ERR_NEG_PRESSURE   = 2,  /* HydroErrorType::NegativePressure           */
    B2D_ERR_UNBOUND_ORBIT  = 3,  /* HydroErrorType::OrbitalEvolutionError      */
    B2D_ERR_TIMEOUT        = 4,  /* a bounded device wait gave up               */
    B2D_ERR_CUDA           = 5,  /* CUDA runtime error (message via b2d_last_error) */
    B2D_ERR_INVALID        = 6,  /* bad argument                                */
    B2D_ERR_UNSUPPORTED    = 7   /* option combination not built                */
} b2d_status;

/* Hydro systems, AnyHydro (src/app.rs:28-33). */
enum { B2D_ISOTHERMAL = 0, B2D_EULER = 1 };

/* Arithmetic of the stage kernels. */
enum {
    B2D_PREC_FP64        = 0,  /* FP64 stencil, FP64 state: parity path                */
    B2D_PREC_FP32_STATE64 = 1, /* FP32 stencil, FP64 state                             */
    B2D_PREC_FP32_COMP   = 2   /* FP32 stencil, FP32 state + FP32 compensation word    */
};

/* ViscosityModel (src/physics.rs:97-103), SinkModel (src/physics.rs:109-115). */
enum { B2D_VISC_CONSTANT_NU = 0, B2D_VISC_ALPHA = 1 };
enum { B2D_SINK_IMPARTIAL = 0, B2D_SINK_TORQUE_FREE = 1 };

/* Euler cooling law: the reference's T^4 law (src/physics.rs:701-738), or
 * β-cooling, which has no counterpart in the reference (a new option). */
enum { B2D_COOLING_T4 = 0, B2D_COOLING_BETA = 1 };

/*
 * Run configuration: Mesh (src/mesh.rs:19-33), the Isothermal / Euler hydro
 * parameters (src/physics.rs:256-303) and Physics (src/physics.rs:121-218)
 * flattened into one plain struct.  Optional fields of the reference
 * (Option<f64>) carry a has_* flag.  The deprecated aliases nu / alpha /
 * lambda (physics.rs:211-230) are resolved by the host before filling this.
 */
typedef struct b2d_config {
    /* Mesh */
    int32_t num_blocks;
    int32_t block_size;
    double  domain_radius;

    /* Hydro */
    int32_t hydro_kind;            /* B2D_ISOTHERMAL | B2D_EULER            */
    int32_t density_index;         /* Euler, default 2                      */
    double  mach_number;           /* Isothermal                            */
    double  gamma_law_index;       /* Euler                                 */
    double  cooling_coefficient;   /* Euler, T^4 law                        */
    double  pressure_floor;        /* Euler, valid if has_pressure_floor    */
    double  density_floor;         /* valid if has_density_floor            */
    int32_t has_pressure_floor;
    int32_t has_density_floor;
    int32_t cooling_slow_start;    /* Euler                                 */
    int32_t cooling_kind;          /* B2D_COOLING_T4 | B2D_COOLING_BETA     */
    double  cooling_beta;          /* β of β-cooling                        */

    /* Physics */
    double  buffer_rate;
    double  buffer_scale;
    double  binary_eccentricity;
    double  binary_mass_ratio;
    double  lambda_multiplier;
    double  viscosity;             /* ν or α, per viscosity_kind            */
    int32_t viscosity_kind;        /* B2D_VISC_*                            */
    int32_t sink_model;            /* B2D_SINK_*                            */
    double  cfl;
    double  plm;
    double  plm_density_trigger;   /* valid if has_plm_density_trigger      */
    double  fake_mass_threshold;
    double  fake_mass_rate;
    double  mach_ceiling;          /* valid if has_mach_ceiling             */
    double  sink_radius;
    double  sink_rate;
    double  softening_length;      /* valid if has_softening_length         */
    double  dt_min;                /* valid if has_dt_min                   */
    int32_t has_plm_density_trigger;
    int32_t one_body;
    int32_t rk_order;              /* 1, 2 or 3                             */
    int32_t has_mach_ceiling;
    int32_t has_softening_length;
    int32_t has_dt_min;
} b2d_config;

/*
 * Where and why a step failed: HydroError (src/physics.rs:47-71) carries the
 * error type and value, the zone position and the binary position.
 */
typedef struct b2d_error {
    int32_t code;          /* b2d_status                                    */
    int32_t run;           /* run index within a batch                      */
    int32_t block_i, block_j, zone_i, zone_j;
    double  value;         /* offending Σ or p                              */
    double  x, y;          /* zone centre                                   */
    double  time;          /* stage time at which it failed                 */
    double  binary[4];     /* x1, y1, x2, y2 of the binary at that time     */
} b2d_error;

typedef struct b2d_ctx b2d_ctx;

/* ------------------------------------------------------------------------ */
/* Context life cycle. */

/* Create a context for `nruns` runs (nruns = 1 for the reference's single
 * run).  `cfgs` points to nruns configurations; runs may differ in mesh size
 * and physics but share hydro kind, rk_order and precision.  Replaces the
 * set-up of main.rs:run (tokio runtime, BlockData table; src/main.rs:114-122). */
b2d_ctx* b2d_create(const b2d_config* cfgs, int32_t nruns, int32_t precision,
                    b2d_status* status);
void     b2d_destroy(b2d_ctx* ctx);

/* Message of the last error raised on this thread (static storage). */
const char* b2d_last_error(void);

/* Number of conserved fields (3 or 4) of a context. */
int32_t b2d_num_fields(const b2d_ctx* ctx);

/* ------------------------------------------------------------------------ */
/* State transfer.  Replaces moving a State into / out of scheme::advance
 * (src/scheme.rs:323-331, state.rs:57-62) and building BlockData's
 * initial_conserved background (scheme.rs:46-57). */

/* Upload one run's conserved state and background (both in block layout),
 * its time and iteration (Rational64 as numerator / denominator).  Resets that
 * run's source ledger to zero unless `ledger` is non-NULL. */
b2d_status b2d_upload_state(b2d_ctx* ctx, int32_t run, const double* cons,
                            const double* background, const double* ledger,
                            double time, int64_t iteration_num,
                            int64_t iteration_den);

/* Upload only the conserved state of one run (background and ledger kept). */
b2d_status b2d_upload_conserved(b2d_ctx* ctx, int32_t run, const double* cons);

/* Download one run's conserved state (block layout), time and iteration.
 * Any output pointer may be NULL. */
b2d_status b2d_download_state(b2d_ctx* ctx, int32_t run, double* cons,
                              double* time, int64_t* iteration_num,
                              int64_t* iteration_den);

/* Download one run's per-block integrated source terms
 * (BlockState::integrated_source_terms, src/state.rs:44-49). */
b2d_status b2d_download_ledger(b2d_ctx* ctx, int32_t run, double* ledger);

/* Per-block orbital-element change (BlockState::orbital_elements_change,
 * src/state.rs:44-49; ItemizedChange::perturbation, state.rs:258-281):
 * [num_blocks][num_blocks][7][4] of (a, M, q, e) per ledger item.  Uploading
 * a state resets it to zero; these calls move it to and from the host. */
b2d_status b2d_download_elements(b2d_ctx* ctx, int32_t run, double* elements);

/* Pipelined host transfers (no reference counterpart: the reference keeps its
 * state in host memory).  Both calls return at once; the bytes move on two
 * copy streams through double-buffered device staging while the context's
 * stream computes, so in a loop of upload / advance_async / download the
 * copies of one step overlap the neighbouring steps' advances.  Buffers
 * should be page-locked (b2d_pin_host) for the copies to be asynchronous.
 *   b2d_upload_conserved_async — like b2d_upload_conserved, queued: `cons`
 *     must stay unchanged until a download queued after it has landed;
 *   b2d_download_async — the state as queued at this point, into `cons`;
 *   b2d_transfers_wait — pending = 0: every queued transfer has landed;
 *   pending = 1: every download but the newest has landed. */
b2d_status b2d_upload_conserved_async(b2d_ctx* ctx, int32_t run, const double* cons);
b2d_status b2d_download_async(b2d_ctx* ctx, int32_t run, double* cons);
b2d_status b2d_transfers_wait(b2d_ctx* ctx, int32_t pending);
b2d_status b2d_upload_elements(b2d_ctx* ctx, int32_t run, const double* elements);

/* ------------------------------------------------------------------------ */
/* The step.  scheme::advance (src/scheme.rs:323-349): dt = cfl·dx / max
 * signal speed (floored by dt_min), then `fold` RK steps of
 * try_advance_rk (scheme.rs:88-173) with the RK averaging of
 * state.rs:183-252.  All runs of the context advance together, each with its
 * own dt.  `dt_out` (nruns doubles) may be NULL; `err_out` may be NULL.
 * On a hydro error the context's state is left as it was before the call,
 * like the caller's copy of State in main.rs:159-205. */
b2d_status b2d_advance(b2d_ctx* ctx, int32_t fold, double* dt_out,
                       b2d_error* err_out);

/* Enqueue an advance on the context's stream without waiting for it and
 * without reading back dt or errors (for timing loops and graphs); a later
 * b2d_synchronize() reports any error. */
b2d_status b2d_advance_async(b2d_ctx* ctx, int32_t fold);
b2d_status b2d_synchronize(b2d_ctx* ctx, double* dt_out, b2d_error* err_out);

/* Massless tracer particles of one run (no counterpart in the reference's
 * code; its README names them).  `xy` holds n (x, y) pairs.  Each RK stage
 * moves a tracer with the stage input's gas velocity, bilinearly interpolated
 * between the four surrounding cell centres, with the same weighted averages
 * as the state, and wraps it into the periodic domain.  n = 0 removes them. */
b2d_status b2d_set_tracers(b2d_ctx* ctx, int32_t run, int64_t n, const double* xy);
b2d_status b2d_get_tracers(b2d_ctx* ctx, int32_t run, double* xy);

/* State::max_signal_speed (src/state.rs:121-133) of one run. */
b2d_status b2d_max_signal_speed(b2d_ctx* ctx, int32_t run, double* out);

/* ------------------------------------------------------------------------ */
/* Initial conditions.  BlockState::from_model (src/state.rs:74-86) for the
 * reference's initial models (AnyModel, src/app.rs:41-48):
 *   B2D_MODEL_INFINITE_DISK        disks.rs:137-157
 *   B2D_MODEL_INFINITE_ALPHA_DISK  disks.rs:172-193
 *   B2D_MODEL_FINITE_DISK          disks.rs:11-115 (disk_mass, disk_width,
 *                                  disk_radius, disk_softening)
 *   B2D_MODEL_RESIDUAL_TEST        disks.rs:208-228
 * optionally modified by a synthetic cavity and seeded multiplicative noise
 * (both new: the reference has neither):
 *   Σ ← Σ · max(cavity_floor, exp(-(cavity_radius / r)^12))
 *         · (1 + noise · (2u - 1)),  u ~ U[0,1) from a counter hash of
 *   (seed, run, global zone i, global zone j).
 * cavity_radius = 0 disables the cavity; noise = 0 disables the noise.  The
 * model's Mach number is used where the hydro has none (Euler).  The result
 * is written in block layout.  Runs on the host. */
enum {
    B2D_MODEL_INFINITE_DISK = 0,
    B2D_MODEL_INFINITE_ALPHA_DISK = 1,
    B2D_MODEL_FINITE_DISK = 2,
    B2D_MODEL_RESIDUAL_TEST = 3
};

typedef struct b2d_disk_model {
    double   surface_density;
    double   mach_number;      /* model Mach number (Euler); isothermal uses the hydro's */
    double   cavity_radius;
    double   cavity_floor;
    double   noise;
    uint64_t seed;
    int32_t  run;
    int32_t  kind;             /* B2D_MODEL_*                                 */
    double   disk_mass;        /* finite disk                                 */
    double   disk_width;
    double   disk_radius;
    double   disk_softening;
    double   core_radius;      /* synthetic: solid-body rotation inside this radius (0: none) */
    double   edge_width;       /* synthetic: velocity tapered to rest over this width inside
                                  the domain radius (0: none)                 */
} b2d_disk_model;

b2d_status b2d_initial_state(const b2d_config* cfg, const b2d_disk_model* model,
                             double* cons);

/* ------------------------------------------------------------------------ */
/* Tuning / introspection. */

/* Tile shape of the stage kernel for a context: width in zones along j (a
 * multiple of 32 dividing block_size) and height along i (dividing
 * block_size).  The paired-column FP32 kernel (precision FP32_COMP,
 * isothermal) also takes 128-, 256- or 512-column tiles that span whole
 * blocks of 64 columns or more side by side.  0 keeps the current value. */
b2d_status b2d_set_tile(b2d_ctx* ctx, int32_t tile_w, int32_t tile_h);
b2d_status b2d_get_tile(const b2d_ctx* ctx, int32_t* tile_w, int32_t* tile_h);

/* Row chunks of the FP32 stage kernels (the paired-column kernel: FP32_COMP,
 * isothermal, tile width 64, 128, 256 or 512; the TMA-staged kernel: FP32 tiles
 * whose width is a multiple of 32, at most 128).  rows > 0: every column strip of tile
 * width is covered in ceil(N / rows) row chunks of near-equal height (at most
 * `rows`; 8 <= rows <= block_size), each of which may cross one block
 * boundary, so that the stage's CTAs can fill whole waves of the GPU; the
 * tile height then applies only to the other stage kernels.  0 (default):
 * block-aligned tiles of the tile height.  No reference counterpart: the
 * reference advances block by block (src/scheme.rs:323-349); results and
 * per-block ledgers do not depend on the tiling. */
b2d_status b2d_set_strip_rows(b2d_ctx* ctx, int32_t rows);
b2d_status b2d_get_strip_rows(const b2d_ctx* ctx, int32_t* rows);

/* Tile autotuner: times every tile shape that divides the block size (width
 * 32..128, or 256 for FP64; height 8..128), the paired FP32 kernel's tiles
 * that span blocks (128, 256 or 512 columns) and, where that kernel runs, the
 * strip rows that fill one, two or three whole waves of its resident CTAs, over `reps` advances of `fold` steps with CUDA events; keeps
 * the fastest (b2d_get_tile and b2d_get_strip_rows report it).  The
 * context's state is unchanged. */
b2d_status b2d_autotune(b2d_ctx* ctx, int32_t fold, int32_t reps, int32_t* tile_w,
                        int32_t* tile_h, double* ms_per_stage);

/* Use (1) or bypass (0) CUDA-graph replay of advance. Default 1. */
b2d_status b2d_set_graphs(b2d_ctx* ctx, int32_t enable);

/* Kernel launches issued by this context since creation. */
int64_t b2d_launch_count(const b2d_ctx* ctx);

/* Launches per advance of `fold` steps (for reporting). */
int64_t b2d_launches_per_advance(const b2d_ctx* ctx, int32_t fold);

/* Run `reps` advances of `fold` steps with CUDA events recorded around every
 * stage-kernel launch on the context's stream; returns the average stage
 * kernel duration in ms. */
b2d_status b2d_time_stages(b2d_ctx* ctx, int32_t fold, int32_t reps,
                           double* ms_per_stage);

/* Event instrumentation of subsequent advances (graphs are bypassed while
 * on); b2d_stage_stats reports the stage launches timed and their total ms. */
b2d_status b2d_set_instrument(b2d_ctx* ctx, int32_t enable);
b2d_status b2d_stage_stats(const b2d_ctx* ctx, int64_t* count, double* total_ms);

/* The context's CUDA stream (a cudaStream_t), for event timing by callers. */
b2d_status b2d_stream(const b2d_ctx* ctx, void** stream);

/* Page-lock / release a caller-owned host buffer (cudaHostRegister) so that
 * uploads and downloads from it are DMA transfers. */
b2d_status b2d_pin_host(void* ptr, uint64_t bytes);
b2d_status b2d_unpin_host(void* ptr);

/* Select the CUDA device used by contexts created afterwards on this thread. */
b2d_status b2d_set_device(int32_t device);

/* ------------------------------------------------------------------------ */
/* Row slabs: one run split across contexts (one per GPU or process), each
 * advancing the blocks of its own block rows.  No counterpart in the
 * reference, which advances every block of a run in one process; its block
 * dataflow joins each block with its 3x3 neighbours and extends a 2-zone
 * halo (src/scheme.rs:119-133; periodic neighbours, src/mesh.rs:101-110), so
 * an advance of a split run is, per context:
 *   1. b2d_max_signal_speed of each context's slab, reduced with max over
 *      the contexts (State::max_signal_speed, src/state.rs:121-133);
 *   2. b2d_slab_begin(fold, global maxima): dt and the stage times;
 *   3. per stage: exchange halo rows — b2d_slab_rows(get) of the slab's first
 *      and last two zone rows, b2d_slab_rows(put) of the neighbours' into the
 *      two rows above and below the slab (periodically) — then b2d_slab_stage;
 *   4. b2d_slab_end: the orbital-element ledger of the slab's blocks, dt and
 *      errors as b2d_advance reports them.
 * The per-block ledgers of the slab's blocks are this context's; a caller
 * sums them with the other slabs' (each block has one owner).  The results
 * equal an unsplit run's with the same block-aligned tiles bit for bit, at
 * every precision (a slab's stage launches cover its block-aligned tiles of
 * the tile height; row chunks apply to whole runs only). */

/* Make block rows [block_row_lo, block_row_hi) of `run` this context's slab
 * ((0, 0): the whole run again).  The stage kernel then covers only the
 * slab's tiles, b2d_max_signal_speed the slab's zones (recomputed here), and
 * the orbital-element ledger the slab's blocks. */
b2d_status b2d_set_slab(b2d_ctx* ctx, int32_t run, int32_t block_row_lo, int32_t block_row_hi);

/* Start an advance of `fold` RK steps whose dt comes from amax[run], the
 * maximum signal speed of each run over all of its slabs. */
b2d_status b2d_slab_begin(b2d_ctx* ctx, int32_t fold, const double* amax);

/* Run the next RK stage of the advance begun by b2d_slab_begin. */
b2d_status b2d_slab_stage(b2d_ctx* ctx);

/* Finish the advance after its last stage (as b2d_advance returns: dt of
 * each run, hydro errors with the state kept as it was before the advance). */
b2d_status b2d_slab_end(b2d_ctx* ctx, double* dt_out, b2d_error* err_out);

/* Copy zone rows [row0, row0 + nrows) (periodic) of the next stage's input
 * (between advances: of the current state) to (put = 0) or from (put = 1)
 * `rows`, as stored: [nf][nrows][N] FP64 words (FP64 and FP64-state
 * contexts) or [nf][2][nrows][N] FP32 words, hi then lo (compensated FP32
 * state); either is nf * nrows * N * 8 bytes.  Rows got from one context
 * are put into another of the same precision. */
b2d_status b2d_slab_rows(b2d_ctx* ctx, int32_t run, int32_t row0, int32_t nrows, double* rows, int32_t put);

/* ------------------------------------------------------------------------ */
/* One RK stage that allocates nothing.  No counterpart in the reference: it
 * serves callers that cannot call cudaMalloc — a host code that owns a fixed
 * device memory pool and forbids allocation by libraries, or an
 * allocator-less runtime.
 *
 * Performs one try_advance_rk stage with the FP64 kernel on caller-owned
 * device buffers: state planes [nf][N][N] (N = num_blocks · block_size,
 * field-major, j contiguous) for the stage input, background, optional RK
 * base (NULL: no averaging) and output; per-block ledgers
 * [num_blocks][num_blocks][7][nf] in, base and out, with
 *   out = (in + Σ sources · dx · dy) · (1 - bf) + base · bf   (base given)
 *   out =  in + Σ sources · dx · dy                            (no base);
 * `time` is the stage time, `dt` the step.  If d_max_speed is non-NULL the
 * max signal speed of the output is written there (device double).
 *
 * Its scratch is one file-scope __device__ array of 4 MiB that every GPU that
 * loads the library holds until exit; meshes whose tile partials and
 * geometry tables do not fit, and block sizes that are neither a multiple of
 * 32 nor at most 256, are rejected with B2D_ERR_INVALID.  The first
 * call on a device looks up the array's device address (cudaGetSymbolAddress)
 * and should come before any stream capture.  All calls share the array:
 * calls that overlap on the GPU (other streams, other host threads) race.
 * The call synchronizes `stream` (a cudaStream_t, NULL for the default
 * stream) to report hydro errors through err_out. */
b2d_status b2d_stage_noalloc(const b2d_config* cfg, const double* d_in,
                             const double* d_background, const double* d_base,
                             double* d_out, const double* d_ledger_in,
                             const double* d_ledger_base, double* d_ledger_out,
                             double time, double dt, double bf,
                             double* d_max_speed, b2d_error* err_out,
                             void* stream);

#ifdef __cplusplus
}
#endif

#endif /* B2D_H */
