/*
 * asph.h — C ABI of the GB300 anisotropic-SPH warm-rain step.
 *
 * The reference (Forbu/sph_cuda, a single file asph_h100.cu) has no library
 * interface: its boundaries are (1) the CLI flags and the asph_tXXXXXXs.bin
 * dump files written by main() (asph_h100.cu:753-1176) and (2) the raw
 * kernel launches of its host loop (asph_h100.cu:958-1161).  Every entry
 * point below replaces one block of that host loop; the comment on each
 * names the reference lines it stands for.
 *
 * Conventions
 *  - Plain C types only: no CUDA or torch types appear in a signature.  A
 *    stream is passed as `void*` holding a cudaStream_t (NULL = the legacy
 *    default stream, which is what the reference uses).
 *  - Every call returns an `int` status (ASPH_OK or an ASPH_ERR_* code) and
 *    never calls exit(); asph_last_error() gives a one-line reason for the
 *    last failure on the calling thread.
 *  - The context owns all device memory.  Host buffers passed to get/set
 *    calls are caller-owned and are copied; pinned host memory makes the
 *    copies asynchronous-capable but is not required.
 *  - One context belongs to one stream and is not thread-safe; distinct
 *    contexts may be driven from distinct threads.
 *  - Particle fields are float32, stored on the device as 16-byte field
 *    groups (pos = x,y,z,rho_old ; vel = u,v,w,- ; thq = theta,qv,qc,-) in
 *    Morton order, the layout the reference uses (asph_h100.cu:829-838).
 */
#ifndef ASPH_H_
#define ASPH_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ASPH_ABI_VERSION 2

/* ---- status codes ------------------------------------------------------ */
#define ASPH_OK             0
#define ASPH_ERR_CUDA       1   /* a CUDA runtime call failed (reference: CK -> exit 1, asph_h100.cu:41-43) */
#define ASPH_ERR_CONFIG     2   /* invalid parameters (reference: Morton limit -> exit 1, asph_h100.cu:785-788) */
#define ASPH_ERR_CFL_ABORT  3   /* CFL trip limit exceeded (reference: return 2, asph_h100.cu:1061-1066) */
#define ASPH_ERR_TIMEOUT    4   /* a bounded device-side wait gave up */
#define ASPH_ERR_ARG        5   /* NULL pointer / bad argument */
#define ASPH_ERR_NOMEM      6   /* device or host allocation failed */
#define ASPH_ERR_IO         7   /* dump file could not be written */
#define ASPH_ERR_STATE      8   /* call out of order (e.g. step before init) */
#define ASPH_ERR_NONFINITE  9   /* a particle position or velocity became NaN/Inf; the run was stopped */
#define ASPH_ERR_DENSE     10   /* a search window held more than ASPH_MAX_CANDIDATES particles; the run was stopped */
#define ASPH_MAX_CANDIDATES 65536

/* ---- parameter presets ------------------------------------------------- */
#define ASPH_PRESET_REFERENCE 0 /* the reference's constexpr physics, 1 particle per cell (asph_h100.cu:48-120) */
#define ASPH_PRESET_SMALL_65K      1 /* 65,536 particles, 10x10x5 km, h 200/50 m, one bubble */
#define ASPH_PRESET_BUBBLE_2M      2 /* 2,097,152 particles, 20x20x8 km, h 150/40 m, three bubbles, sort every step */
#define ASPH_PRESET_LARGE_16M      3 /* 16,777,216 particles, 40x40x10 km, h 160/20 m, 95% RH below 1 km */
#define ASPH_PRESET_ADJOINT_262K      4 /* 262,144 particles in the SMALL_65K box (adjoint workload) */

#define ASPH_INIT_REFERENCE 0   /* one particle at each cell centre + hash noise (asph_h100.cu:210-227) */
#define ASPH_INIT_LATTICE   1   /* jittered lattice + Gaussian bubbles + Gaussian noise */

#define ASPH_QV_REFERENCE 0     /* qv_ref = qv0 exp(-z/2500) exp(-max(z-5000,0)/1000) (asph_h100.cu:149-153) */
#define ASPH_QV_RH        1     /* qv_ref = RH(z) * qsat(T_ref, p_ref) */

#define ASPH_MAX_BUBBLES 8

/* Every constexpr of asph_h100.cu:48-120 becomes a runtime field. */
typedef struct AsphParams {
    /* grid (asph_h100.cu:48-57): cells per axis; the cell edge is the kernel
     * length on that axis, the support is 2 cells (q < 2) */
    int32_t nx, ny, nz;
    float   dx, dy, dz;
    /* particles and initial state */
    int32_t n_particles;
    int32_t init_mode;                 /* ASPH_INIT_* */
    int32_t lat_nx, lat_ny, lat_nz;    /* ASPH_INIT_LATTICE: lattice counts, product = n_particles */
    float   jitter;                    /* uniform jitter as a fraction of the lattice spacing */
    uint32_t seed;
    float   noise;                     /* REFERENCE: hash-noise amplitude [K] (--noise); LATTICE: Gaussian sigma [K] */
    int32_t n_bubbles;
    float   bubble_x[ASPH_MAX_BUBBLES], bubble_y[ASPH_MAX_BUBBLES], bubble_z[ASPH_MAX_BUBBLES];
    float   bubble_r[ASPH_MAX_BUBBLES], bubble_amp[ASPH_MAX_BUBBLES];  /* theta' = amp exp(-(d/r)^2) */
    /* sounding (asph_h100.cu:66-76, 136-153) */
    float   th0, n2, cs;
    int32_t qv_mode;                   /* ASPH_QV_* */
    float   qv0, rh, rh_bl, z_bl;      /* RH(z) = rh_bl below z_bl, rh above */
    /* dissipation (asph_h100.cu:84-91) */
    float   alpha_av, beta_av, h_av;   /* beta_av = 0 reproduces the reference exactly */
    float   sponge_sigma, sponge_frac, dthdt_cap;
    /* surface forcing (asph_h100.cu:100-105) */
    int32_t surface_flux;
    float   c_h, c_e, beta_moist, v_bg, dts_skin, ramp;
    /* warm-rain microphysics (asph_h100.cu:111-120) */
    float   qc_auto, rate_auto, v_rain, theta_cap, qv_cap;
    int32_t accretion, rain_evap;      /* Kessler accretion / rain evaporation (absent in the reference: 0) */
    float   k_accr;                    /* accretion rate constant [1/s] */
    /* time stepping and CFL control (asph_h100.cu:728-742, 794-797, 1040-1078) */
    float   dt_request;                /* --dt ; <= 0 means the static bound */
    float   cfl;
    int32_t max_trip, strict_cfl;
    int32_t adaptive_dt;               /* 1: adopt the closed-loop dt (reference); 0: keep dt fixed */
    int32_t sort_every;                /* 0: displacement-gated cadence (reference); k>0: every k steps */
    int32_t permute_acc;               /* 0: reference (acc keeps its pre-sort order); 1: acc follows its particle */
    float   pmass;                     /* particle mass [kg]; 0: rho0 * Lx*Ly*Lz / n_particles */
    /* coarse dump strides (asph_h100.cu:737) */
    int32_t dump_sx, dump_sy, dump_sz;
    int32_t reserved[16];
} AsphParams;

/* Host-side SoA view of the particle state, in the context's current
 * (Morton-sorted) order.  Any pointer may be NULL to skip that field. */
typedef struct AsphHostState {
    float *x, *y, *z;       /* position [m] */
    float *u, *v, *w;       /* velocity [m/s] */
    float *th, *qv, *qc;    /* potential temperature [K], vapour and cloud water [kg/kg] */
    float *rho;             /* current density [kg/m^3] */
    float *ax, *ay, *az;    /* last acceleration [m/s^2] (needed by the first half kick) */
    float *prs;             /* perturbation pressure p' [Pa] */
    float *dthdt;           /* viscous-heating tendency [K/s] */
} AsphHostState;

/* Device control block: the values the reference keeps in host variables
 * of its step loop (asph_h100.cu:931-942, 1040-1078). */
typedef struct AsphControl {
    double  simt;           /* simulated time [s] */
    double  since_sort;     /* time since the last sort [s] */
    float   dt;             /* dt of the next step [s] */
    float   dt_cap, dt_floor, dt_static;
    float   dt_required;    /* last closed-loop CFL bound */
    float   sort_dt;        /* displacement-gated sort interval [s] */
    float   umax, vmax, wmax;  /* last |u|,|v|,|w| maxima */
    int32_t step;           /* completed steps */
    int32_t trips;          /* consecutive CFL violations */
    int32_t sort_count;
    int32_t aborted;        /* 1 after a CFL abort: later steps do nothing */
    int32_t clamp_pending;  /* a CFL trip asked for the velocity clamp */
    int32_t do_sort;        /* the next step starts with a sort */
    int32_t error;          /* device error word (ASPH_ERR_TIMEOUT ...) */
    int32_t surf_count;     /* particles in the lowest layer at the last sort */
    int32_t deferred;       /* targets the last brick density pass left to its
                               warp-per-target kernel (outside the staged bricks) */
    int32_t split_regions;  /* brick regions the last density pass split into halves
                               because they overflowed the staging capacity */
} AsphControl;

/* ---- library / parameters ---------------------------------------------- */
int         asph_abi_version(void);
/* sizeof(AsphParams) as compiled into the library (FFI layout check). */
int         asph_params_size(void);
const char* asph_last_error(void);
const char* asph_status_string(int status);
/* Fill `p` with a preset.  nx,ny,nz > 0 override the preset grid (used by
 * ASPH_PRESET_REFERENCE, which mirrors --nx/--ny/--nz, asph_h100.cu:760-762). */
int asph_params_preset(AsphParams* p, int preset, int nx, int ny, int nz);
/* Validate parameters (Morton limit 1024 cells/axis, asph_h100.cu:785-788). */
int asph_params_check(const AsphParams* p);

/* ---- context ------------------------------------------------------------ */
typedef struct asph_ctx asph_ctx;
/* Allocate every device buffer the reference allocates (asph_h100.cu:827-872). */
int asph_create(const AsphParams* p, void* stream, asph_ctx** out);
int asph_destroy(asph_ctx* ctx);
/* Initial state, initial sort, initial force evaluation
 * (asph_h100.cu:885-921): kernel_init, kernel_iota, sort, density,
 * kernel_eos_micro, kernel_momentum. */
int asph_init(asph_ctx* ctx);
/* Replace the particle state with host arrays (x..qc and rho required, the
 * rest optional) and reset the cell table; the next sort rebuilds it. */
int asph_set_state(asph_ctx* ctx, const AsphHostState* st);
int asph_get_state(asph_ctx* ctx, AsphHostState* st);
/* Rain grid (nx*ny*nz cells) and surface precipitation (nx*ny). */
int asph_get_rain(asph_ctx* ctx, float* rain, float* precip2d);
int asph_set_rain(asph_ctx* ctx, const float* rain, const float* precip2d);
int asph_get_control(asph_ctx* ctx, AsphControl* c);
/* Set simt, dt and the sort flag (tests and restarts). */
int asph_set_time(asph_ctx* ctx, double simt, float dt, int do_sort);

/* ---- granular steps (one block of the reference step each) -------------- */
/* keys -> stable radix sort -> gather -> cell table + surface list
 * (asph_h100.cu:963-977: kernel_morton_keys, SortPairs, kernel_gather,
 * memset, kernel_build_pairs). */
int asph_sort_build(asph_ctx* ctx);
/* Sort outputs: unsorted keys of the pre-sort order, sorted keys, the
 * permutation, cellRange (2*nx*ny*nz ints: start,end per cell, {0,0} for an
 * empty cell) and the surface list in ascending order. */
int asph_get_sort(asph_ctx* ctx, uint32_t* keys_in, uint32_t* keys_sorted,
                  uint32_t* perm, int32_t* cell_range, int32_t* surf_list,
                  int32_t* surf_count);
/* half kick + drift + surface flux (asph_h100.cu:981-998). */
int asph_kick_drift_flux(asph_ctx* ctx);
/* summation density + EOS + saturation adjustment + autoconversion
 * (+ accretion/evaporation when enabled) (asph_h100.cu:1002-1008). */
int asph_density_eos(asph_ctx* ctx);
/* momentum (asph_h100.cu:1013); with integrate != 0 also theta update,
 * second half kick and sponge (asph_h100.cu:1019-1026). */
int asph_momentum(asph_ctx* ctx, int integrate);
/* rain sedimentation (asph_h100.cu:1028-1036). */
int asph_rain(asph_ctx* ctx);
/* closed-loop CFL control on the device (asph_h100.cu:1040-1078). */
int asph_cfl(asph_ctx* ctx);
/* nsteps full steps (asph_h100.cu:958-1078) as one CUDA graph per step
 * pair, no host synchronisation inside; returns ASPH_ERR_CFL_ABORT if the
 * trip limit was exceeded during the call. */
int asph_step(asph_ctx* ctx, int nsteps);
/* Queue nsteps without waiting; asph_sync() collects the status. */
int asph_step_async(asph_ctx* ctx, int nsteps);
int asph_sync(asph_ctx* ctx);
/* Kernel launches of one step: the kernel nodes of the step's CUDA graph
 * (captured here, without running, if no step ran yet). */
int asph_step_kernels(asph_ctx* ctx, int* n);

/* nsteps steps launched without a graph, with CUDA events between the
 * phases (the reference's per-phase timers, asph_h100.cu:931-954, 1149-1157).
 * phase_ms[ASPH_NPHASES] receives the summed milliseconds of: 0 cell-table
 * clear + sort reset, 1 digit histogram + radix passes, 2 gather / kick /
 * drift / flux / keys, 3 density + EOS + microphysics, 4 momentum +
 * integration + rain + CFL, 5 the whole step. */
#define ASPH_NPHASES 6
int asph_step_profiled(asph_ctx* ctx, int nsteps, float* phase_ms);

/* Execution options (setting one drops the captured step graphs).
 * ASPH_OPT_PAIR_PATH: 0 = automatic (brick-staged shared-memory pair
 * kernels where the grid allows), 1 = per-target global path everywhere
 * (same results to rounding; for testing), 2 = the density pass takes one
 * warp per target for every target (the kernel that serves targets outside
 * the staged bricks; same pairs, in the reference's order).
 * ASPH_OPT_PAIR_SHAPE: brick shape of the density pass, 0 = 8x8x8,
 * 1 = 8x8x4, 2 = 8x4x4, 3 = 4x4x4 cells, -1 = automatic (set); get returns
 * the shape in use, -1 for the global path.  A shape whose staged region
 * does not suit the grid or the particle density is ASPH_ERR_ARG.
 * ASPH_OPT_SORT_EVERY: sort cadence, 0 = displacement-gated (the
 * reference), k > 0 = every k steps (the AsphParams field sort_every).
 * ASPH_OPT_TARGETS_PER_THREAD: targets each thread of the momentum pass
 * takes, 1, 2 (default) or 4, so that a warp covers 32, 64 or 128
 * consecutive targets (about 32 k / ppc cells, ppc = particles per cell);
 * 0 restores the default.  Results do not depend on it.
 * ASPH_OPT_SORT_AHEAD: 1 (default) = with a sort every step, a run of
 * several steps (asph_step, asph_step_async with nsteps >= 2) sorts the
 * next step's keys beside the current step's density and momentum passes,
 * which neither read the sort's inputs later nor its outputs, and the next
 * step's gather applies it; 0 = every step sorts at its start.  Results are
 * bit-identical either way; between calls the context always holds the
 * last applied sort. */
#define ASPH_OPT_PAIR_PATH  1
#define ASPH_OPT_PAIR_SHAPE 2
#define ASPH_OPT_SORT_EVERY 3
#define ASPH_OPT_TARGETS_PER_THREAD 4
#define ASPH_OPT_SORT_AHEAD 5
int asph_set_option(asph_ctx* ctx, int option, int value);
int asph_get_option(asph_ctx* ctx, int option, int* value);

/* Neighbour lists of the last density pass (pairs with 0 < q < 2 accepted
 * by the reference's window rule, asph_h100.cu:296-327): count[i] per
 * particle (-1 if it overflowed ASPH_NBR_CAP) and list[q*N + i], q < count[i]
 * (slot-major, N*ASPH_NBR_CAP entries).  Either pointer may be NULL. */
#define ASPH_NBR_CAP 192
int asph_get_neighbours(asph_ctx* ctx, int32_t* count, int32_t* list);

/* ---- diagnostics and output ----------------------------------------------- */
/* FP64 totals: KE, PE, IE, water, p_z, mass (asph_h100.cu:650-668). */
int asph_audit(asph_ctx* ctx, double out[6]);
/* Coarse dump in the reference format (asph_h100.cu:1080-1120), file name
 * <outdir>/asph_t%06.0fs.bin; `path` (may be NULL) receives the name. */
int asph_dump(asph_ctx* ctx, const char* outdir, char* path, int path_len);
/* The same dump in two halves, so that the device-to-host copy and the file
 * write overlap the next steps: asph_dump_begin queues the coarse fields,
 * the column diagnostics and the control block into pinned host memory on
 * the context's stream (and restarts the precipitation accumulator, like
 * asph_column_diag); steps may be queued after it; asph_dump_finish waits
 * for that copy only, writes the file of the state at begin and fills
 * diag[4] (may be NULL) as asph_column_diag does.  One dump in flight per
 * context. */
int asph_dump_begin(asph_ctx* ctx);
int asph_dump_finish(asph_ctx* ctx, const char* outdir, char* path, int path_len, float diag[4]);
/* Column diagnostics of the dump line (asph_h100.cu:1095-1105): cloud
 * cover [%], max ql [kg/kg], max |w| [m/s], mean precipitation [mm];
 * resets the precipitation accumulator like the reference. */
int asph_column_diag(asph_ctx* ctx, float out[4]);

/* ---- source-term hook ---------------------------------------------------------
 * The reference's header defers radiation and ice/mixed-phase physics to
 * "NN, additive source terms" (asph_h100.cu:14-15) without an interface.
 * With the hook on, every step adds per-particle tendencies of theta [K/s],
 * qv and qc [1/s] in its theta update (asph_h100.cu:562-571): theta +=
 * (dthdt + S_theta) dt, qv += S_qv dt, qc += S_qc dt, then the caps.  The
 * tendencies belong to particles: they are given in the context's current
 * order and follow their particles through every later sort, so a set of
 * tendencies stays attached until it is replaced.
 *   asph_source_enable      allocates (zeroed) / detaches the buffer
 *   asph_source_set         host arrays, any may be NULL (zero)
 *   asph_source_set_device  a device float4[N] array {S_theta, S_qv, S_qc, -}
 *                           (e.g. a model's output tensor), copied on the
 *                           context's stream
 *   asph_state_device       copies the current pos {x,y,z,rho_old}, vel
 *                           {u,v,w,-} and thq {theta,qv,qc,-} (float4[N]
 *                           each, any may be NULL) into caller device
 *                           buffers on the context's stream
 * The adjoint window runs without the hook. */
int asph_source_enable(asph_ctx* ctx, int on);
int asph_source_set(asph_ctx* ctx, const float* dtheta, const float* dqv, const float* dqc);
int asph_source_set_device(asph_ctx* ctx, const void* tendencies);
int asph_state_device(asph_ctx* ctx, void* pos, void* vel, void* thq);

/* ---- state snapshots and restart files -------------------------------------
 * No counterpart in the reference (it cannot restart; its dumps are coarse
 * averages, asph_h100.cu:680-703).  A snapshot holds, in device memory,
 * everything a context needs to continue bit for bit: the particle field
 * groups, the cell table and surface flags of the last sort, the rain grid,
 * the surface precipitation and the control block.  save/restore are queued
 * on the context's stream; a snapshot fits only contexts with its particle
 * count and grid.  Restart files hold the same content on disk; reading one
 * needs a context created with the same particle count and grid, whose
 * parameters then govern the continued run. */
typedef struct asph_snapshot asph_snapshot;
int asph_snapshot_create(asph_ctx* ctx, asph_snapshot** out);
int asph_snapshot_save(asph_ctx* ctx, asph_snapshot* snap);
int asph_snapshot_restore(asph_ctx* ctx, const asph_snapshot* snap);
int asph_snapshot_destroy(asph_snapshot* snap);
int asph_checkpoint_write(asph_ctx* ctx, const char* path);
int asph_checkpoint_read(asph_ctx* ctx, const char* path);

/* ---- ensemble ----------------------------------------------------------------
 * No counterpart in the reference.  n_members independent simulations of
 * any sizes, each a full context (own parameters, dt, CFL control and sort
 * cadence) on its own stream.  One ensemble step is one CUDA graph launch on
 * `stream` (NULL: the ensemble's own stream) that forks into every member's
 * step and joins; members run concurrently on the GPU.  A member's results
 * equal those of the same parameters run alone with the same options.
 * asph_ens_member() lends a member's context for state, audit and dump calls
 * (ordered after the queued ensemble steps); the ensemble keeps ownership.
 * asph_ens_tune() times every brick shape that suits each member (and the
 * per-target path), crossed with the momentum pass's targets per thread
 * (1, 2, 4: the cells one warp covers) and with the sort cadences in
 * sort_choices (none: keep each member's own), trial_steps steps each from
 * a snapshot, keeps the fastest per member and restores the member's
 * state; chosen (may be NULL, else 3 ints per member) receives {shape (-1:
 * per-target path), sort cadence, targets per thread}. */
typedef struct asph_ens asph_ens;
int asph_ens_create(const AsphParams* members, int n_members, void* stream, asph_ens** out);
int asph_ens_destroy(asph_ens* ens);
int asph_ens_size(asph_ens* ens);
int asph_ens_member(asph_ens* ens, int k, asph_ctx** ctx);
int asph_ens_init(asph_ens* ens);
int asph_ens_step(asph_ens* ens, int nsteps);
int asph_ens_step_async(asph_ens* ens, int nsteps);
int asph_ens_sync(asph_ens* ens);
int asph_ens_tune(asph_ens* ens, int trial_steps, const int* sort_choices, int n_sort_choices, int* chosen);

/* ---- adjoint window -----------------------------------------------------------
 * No counterpart in the reference.  Gradients of a loss L of the final cloud
 * water (and theta) after nsteps steps with respect to the initial theta of
 * every particle and the viscosity coefficients alpha, beta.  The window
 * step is the full step with the sort moved after the kick/drift/flux, so
 * the neighbour lists hold exactly the pairs with q < 2; the sort
 * (permutation), the lists and dt are held fixed in the adjoint.  The
 * forward saves a device snapshot every `every` steps; the backward
 * recomputes each segment from its snapshot, recording the per-step values
 * the reverse needs, and runs the hand-written reverse kernels.
 *   asph_adj_create    sizes the checkpoints and the segment tape for ctx
 *   asph_adj_forward   runs the window from ctx's current state (its order
 *                      is the order of dL_dtheta0) and leaves ctx at the end
 *   asph_adj_backward  dL_dqc, dL_dtheta (N each), dL_dxyz (3 x N: x, y, z),
 *                      any of them NULL: dL/d(final field) in the final
 *                      state's order; writes
 *                      dL_dtheta0[N] and dL_dalpha_beta[2] (may be NULL);
 *                      ctx is left at the end of the window
 * ASPH_ERR_STATE: a CFL trip or a neighbour-list overflow inside the window. */
typedef struct asph_adj asph_adj;
int asph_adj_create(asph_ctx* ctx, int nsteps, int every, asph_adj** out);
int asph_adj_forward(asph_adj* adj);
int asph_adj_backward(asph_adj* adj, const float* dL_dqc, const float* dL_dtheta, const float* dL_dxyz,
                      float* dL_dtheta0, double* dL_dalpha_beta);
int asph_adj_destroy(asph_adj* adj);
/* Viscosity coefficients alpha (asph_h100.cu:84) and beta of the running
 * context (the adjoint's parameters). */
int asph_set_viscosity(asph_ctx* ctx, float alpha, float beta);

/* ---- stable key sort without allocation -----------------------------------
 * No counterpart in the reference.  For callers that must not call
 * cudaMalloc/cudaFree (a latency-critical loop where cudaFree would
 * synchronise the device, a host callback or foreign-language runtime that
 * must not block in the allocator, an application whose memory pool owns all
 * device memory): sorts n 32-bit keys (device pointer `keys`) stably,
 * writing the sorted keys and the permutation (sorted position -> input
 * index) to caller-owned device buffers.  Same kernels and same result as
 * the sort of asph_sort_build.  The sort runs over whole 8-bit digits, bits
 * [0, 8*ceil(key_bits/8)): keys must be below 2^key_bits (Morton keys of a
 * grid are) for that to be the sort over bits [0, key_bits).  Scratch lives
 * in a static device array sized for ASPH_NOALLOC_MAX_KEYS keys (about 5 MB,
 * held by every GPU that loads the library until exit); larger n returns
 * ASPH_ERR_ARG.  All calls share that array: calls that overlap on the GPU
 * race and must be serialised by the caller.  The outputs must not alias
 * `keys` or each other.  The first call in each CUDA context looks up the
 * array's address in that context.  Every call waits for `stream` and
 * reads the device error word back, so it must never be made while any
 * stream on the device is being captured into a graph.  Returns
 * ASPH_ERR_TIMEOUT if a bounded device wait gave up. */
#define ASPH_NOALLOC_MAX_KEYS 524288
int asph_sort_keys_noalloc(const uint32_t* keys, uint32_t* keys_sorted, uint32_t* perm, int n, int key_bits,
                           void* stream);

#ifdef __cplusplus
}
#endif
#endif /* ASPH_H_ */
