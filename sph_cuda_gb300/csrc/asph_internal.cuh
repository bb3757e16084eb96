// asph_internal.cuh — device-side control block, buffer sets and the
// launch functions shared by the kernel files and the C-ABI layer.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "asph_phys.cuh"
#include "../../include/asph.h"

namespace asph {

constexpr int TPB = 256;
constexpr int SORT_TPB = 256;
constexpr int SORT_ITEMS = 16;
constexpr int SORT_TILE = SORT_TPB * SORT_ITEMS;   // keys per radix tile
constexpr int MAX_PASSES = 4;                      // 30-bit keys / 8-bit digits
constexpr unsigned SPIN_LIMIT = 1u << 24;          // bounded device waits
constexpr int NBR_CAP = ASPH_NBR_CAP;              // neighbour-list slots per particle

// Device-resident step control: the host variables of the reference step
// loop (asph_h100.cu:931-942, 1040-1078) live here so that a step needs no
// host round trip.
struct DevCtl {
    double simt, since_sort;
    float dt, dt_required, sort_dt;
    float umax, vmax, wmax;
    int step, trips, sort_count, aborted, clamp_pending, do_sort, error, surf_count;
    int sorted_this_step;
    unsigned defer_n;          // targets queued for the density pass's deferred kernel
    unsigned defer_done;       // finished blocks of the deferred kernel (the last resets defer_n)
    unsigned defer_last;       // targets the last density pass deferred
    unsigned split_n;          // brick regions split into halves in the running density pass
    unsigned split_last;       // ... in the last density pass
    unsigned gmax[3];          // float bits of |u|,|v|,|w| maxima (atomicMax)
    unsigned epoch;            // radix look-back epoch
    unsigned hist[MAX_PASSES][256];
    unsigned tile_ctr[MAX_PASSES];
    // incremental sort (sort lane 1): keys that changed since the last sort
    unsigned inc_m;            // how many changed this step
    int inc_on;                // 1: this step sorts incrementally
    unsigned iepoch;           // look-back epoch of the changed-key sort
    unsigned ihist[MAX_PASSES][256];
    unsigned itile_ctr[MAX_PASSES];
};

// Buffers of one context.  Particle buffers hold 16-byte field groups.
struct Bufs {
    float4* pos[2];     // x, y, z, rho_old (rho gathered for the density pass)
    float4* vel[2];     // u, v, w, -
    float4* thq[2];     // theta, qv, qc, -
    float2* rp;         // rho_new, p'
    float4* ms[2];      // written by the density pass for the momentum pass: (x, y, z, p'), (u, v, w, rho)
    float4* acc;        // ax, ay, az, -
    float*  dthdt;
    uint32_t* kin;      // keys of the current order (input of the next sort)
    uint32_t* kbuf[2];  // radix ping-pong keys
    uint32_t* vbuf[2];  // radix ping-pong values
    uint32_t* skeys;    // sorted keys of the last sort (points into kbuf)
    uint32_t* perm;     // permutation of the last sort (points into vbuf)
    // the next step's sort, run ahead beside this step's pair passes (see
    // launch_sort_ahead); the next gather applies it and copies it into
    // skeys/perm
    uint32_t* skeys_ahead;
    uint32_t* perm_ahead;
    uint64_t* status;   // look-back words [pass][tile][digit]
    // incremental sort: unchanged indices, changed keys/indices (ping-pong),
    // per-block counts, the changed-key sort's look-back words
    uint32_t* inc_u;
    uint32_t* inc_uk;   // the unchanged particles' keys, in the order of inc_u
    uint32_t* inc_k[2];
    uint32_t* inc_i[2];
    uint32_t* inc_cnt;
    uint64_t* inc_status;
    int inc_max, inc_tiles, inc_blocks;
    int2*   range;      // cell table, {start,end}, {0,0} when empty
    uint8_t* surf;      // 1 when the particle was in the lowest layer at the last sort
    float*  rain[2];    // Eulerian rain mass per cell [kg]
    float*  rain_delta; // this step's deposits when the microphysics reads the grid
    float*  precip;     // accumulated surface precipitation [kg/m^2]
    DevCtl* ctl;
    float4* snd;        // sounding tables: rho_ref, pres_ref, thvr (3 x snd_n nodes)
    int2*   spans;      // per brick of the density pass, by the brick's Morton id (its keys >> log2 of the
                        // brick's key count): its span of targets in the sorted order, {0,0} when empty
    int*    nbr;        // neighbour lists of the density pass, slot-major [NBR_CAP][N]
    int*    nbr_cnt;    // neighbours per particle, -1 when the list overflowed
    int*    defer;      // targets of the density pass left to its deferred kernel (N slots)
    int ntiles, npasses;
    int pc, vc, qc, rc; // current index of pos/vel/thq/rain ping-pong pairs
    int force_global;   // 1: pair passes take the per-target global path, 2: density warp per target
    int shape;          // brick shape index of the density pass, -1: automatic
    int m_tpt;          // targets per thread of the momentum pass (1, 2 or 4; 0: the default, 2)
    cudaStream_t aux;   // second stream: the full sort runs beside the incremental one (a graph branch)
    cudaEvent_t ev_fork, ev_join;
    cudaStream_t aux2;  // third stream: the next step's sort beside this step's pair passes
    cudaEvent_t ev_fork2, ev_join2;
    float4* src;        // source-term hook: per-particle tendencies (theta, qv, qc), NULL when off
    float4* src_tmp;    // the tendencies in the order of the current step (written by the gather)
};

// Mode bits of the gather/integrate pass.
enum : int {
    G_SORTED    = 1,    // gather through the permutation when a sort ran
    G_INTEGRATE = 2,    // half kick + drift + surface flux
    G_FORCE     = 4,    // the sort ran unconditionally (granular call)
    G_AHEAD     = 8,    // apply the sort run ahead (skeys_ahead/perm_ahead) and copy it into skeys/perm
};
// Mode bits of the momentum pass.
enum : int {
    M_INTEGRATE = 1,    // theta update, second half kick, sponge, velocity maxima
    M_RAIN      = 2,    // rain sedimentation blocks appended to the grid
    M_CFL       = 4,    // the CFL control follows (a one-block kernel)
};

// Record a failure for asph_last_error() (asph_capi.cu); returns `code`.
int set_error(int code, const char* msg);

// ---- launch functions (asph_kernels.cu / asph_sort.cu) --------------------
void launch_init(const Phys& P, const Bufs& B, const float* bub, int nbub, int init_mode,
                 int lat_nx, int lat_ny, int lat_nz, float jitter, uint32_t seed, float noise,
                 cudaStream_t s);
void launch_keys(const Phys& P, const Bufs& B, cudaStream_t s);
void launch_sort_prep(const Phys& P, const Bufs& B, int force, int clear_delta, cudaStream_t s);
void launch_sort(const Phys& P, Bufs& B, int force, cudaStream_t s);
// The next step's sort, enqueued right after this step's gather wrote the
// keys of the drifted positions: the same stable sort of the same keys, into
// skeys_ahead/perm_ahead, on its own stream branch so that it runs beside
// the density and momentum passes (which read neither its inputs' future
// values nor its outputs).  It runs whatever the step gating says; only a
// sort-every-step cadence may use it, and the next gather decides as
// always whether a sort is applied.
void launch_sort_ahead(const Phys& P, Bufs& B, cudaStream_t s);
// Sizes of the incremental sort's buffers for N particles.
void sort_inc_sizes(int N, int* max_keys, int* tiles, int* blocks);
void launch_gather(const Phys& P, const Bufs& B, int mode, cudaStream_t s);
void launch_density(const Phys& P, const Bufs& B, cudaStream_t s);
void launch_momentum(const Phys& P, const Bufs& B, int mode, int use_lists, cudaStream_t s);
// Targets per thread the momentum pass uses (the option, else the default).
int momentum_tpt(const Bufs& B);
void launch_rain(const Phys& P, const Bufs& B, cudaStream_t s);
// Brick shape index the density pass uses (-1: per-target global path),
// the number of shapes, and whether shape k suits the grid and density.
int pair_shape(const Phys& P, const Bufs& B);
// Entries of Bufs::spans: Morton ids of the smallest brick shape.
size_t pair_span_slots(const Phys& P);
// log2 of the key count of the brick shape in use (its spans are indexed by
// key >> shift), -1 on the global path.
int pair_span_shift(const Phys& P, const Bufs& B);
// Every brick's span by binary search in the sorted keys: for spans that the
// last sort's gather did not write (restored sorted keys, another brick shape).
void launch_brick_spans(const Phys& P, const Bufs& B, cudaStream_t s);
int pair_shape_count();
bool pair_shape_fits(const Phys& P, int k);
void launch_cfl(const Phys& P, const Bufs& B, cudaStream_t s);
void launch_clamp(const Phys& P, const Bufs& B, cudaStream_t s);
// FP64 constants of the conservation audit, evaluated on the host in double
// from the float parameters: the Exner coefficient g^2/(cp th0 N^2)
// (asph_h100.cu:140) and the particle mass rho0 Lx Ly Lz / N
// (asph_h100.cu:75-76 for one particle per cell), unless a mass is given.
struct AuditConst {
    double th0, n2, a_exner, pmass;
    int N;
};
AuditConst audit_constants(const AsphParams& p);
void launch_audit(const Phys& P, const AuditConst& A, const Bufs& B, double* partial, int nblk, double* out,
                  cudaStream_t s);
void launch_surf_flags(const Phys& P, const Bufs& B, uint8_t* flags, cudaStream_t s);
void launch_coarse(const Phys& P, const Bufs& B, float* out, int sx, int sy, int sz, int cx, int cy,
                   int cz, float4* coldiag, cudaStream_t s);

}  // namespace asph
