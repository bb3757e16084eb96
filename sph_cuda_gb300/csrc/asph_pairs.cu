// asph_pairs.cu — the two pair passes of the step, for sm_103a:
//   D  density (lagged Shepard) + EOS + microphysics (asph_h100.cu:286-402)
//   M  momentum + integration + rain sedimentation + CFL control
//      (asph_h100.cu:415-599, 1040-1078)
//
// Candidate set (identical to the reference): for target i, every particle
// listed by the cell table in the cells within +-2 of i's *current* cell,
// x/y wrapped, z clipped at the walls; the table is the one built at the
// last sort (positions have drifted since), distances are raw coordinate
// differences in cell units (no minimum image).  D and M see the same
// positions and table, so they accept the same pairs: D enumerates the
// candidates once and records each target's accepted neighbours (self
// excluded) in a slot-major list; M walks that list.
//
// D, brick path.  One CTA per Morton-aligned brick of BX x BY x BZ cells;
// the brick's targets are one contiguous span of the sorted order and the
// block has about as many threads as a brick has targets.  The CTA copies
// the particles of every table cell within H cells of the brick into shared
// memory, bucketed row-major by region cell, so that each row of a target's
// 5 x 5 x 5 window is one contiguous span of shared memory; each thread
// walks its target's row spans in one flattened loop, queues accepted
// candidates in a small per-thread list in shared memory, and drains the
// list (density sums + neighbour-list writes) in uniform loops.  H = 2 (the
// stencil) covers every target still in a cell of its brick; H = 3 also
// covers one cell of drift since the sort.  A region that overflows the
// staging capacity is split into its two Morton-aligned halves (each a
// contiguous sub-span of the targets with a smaller region), and a half
// that overflows once more; a target whose window leaves the staged region,
// and the targets of a quarter that still overflows, are queued for the
// deferred pass.
//
// Deferred pass.  One warp per queued target: the lanes read the window's
// cell ranges from the global table in parallel and test the candidates 32
// at a time in the reference's order, so the neighbour list comes out in
// that order.
//
// Global path.  One thread per target walking the cell table in global
// memory, the reference's loop structure; used for grids narrower than the
// staged region, and by M for a target whose list overflowed or was not
// produced on the current positions.
#include "asph_device.cuh"
#include "../../include/asph.h"

namespace asph {

constexpr int MAX_HALO = 3;      // widest staged halo (cells around a brick)
constexpr int DENSITY_REGS = 48; // register cap of the brick kernel (its launch plan counts on it)
constexpr int DLIST = 30;        // most queued accepted candidates per thread (D); a launch may use fewer
// Momentum blocks of 128 threads: a block ends with its slowest warp, and
// smaller blocks waste less of an SM on warps that wait for it (measured at
// 2M from init: 0.298 / 0.260 / 0.257 / 0.271 ms at 32 / 64 / 128 / 256).
constexpr int M_TPB = 128;
constexpr int M_MINB = 1024 / M_TPB;                     // resident blocks that keep 64 registers
// Rain cells per thread of a rain block: 1,024 cells a block, so that the
// rain advection adds few blocks (and few finished-block atomics) to the
// pass (momentum at 2M from init: 0.262 / 0.245 / 0.256 ms at 256 / 1,024 /
// 4,096 cells a block).
constexpr int M_RAIN_CELLS = 8;
constexpr int M_TPT = 2;         // default targets per thread of the momentum pass (1, 2 or 4 per launch)

template <int BX, int BY, int BZ, int H>
struct BrickGeom {
    static_assert((BX == BY && BY == BZ) || (BX == 2 * BY && BY == BZ) || (BX == BY && BX == 2 * BZ),
                  "brick must be a Morton-aligned key range");
    static_assert(H >= STENCIL && H <= MAX_HALO, "halo must cover the stencil");
    static constexpr int RX = BX + 2 * H, RY = BY + 2 * H, RZ = BZ + 2 * H;
    static constexpr int R = RX * RY * RZ;
    static constexpr int KEYS = BX * BY * BZ;
    static constexpr int LOG2K = KEYS >= 512 ? 9 : KEYS >= 256 ? 8 : KEYS >= 128 ? 7 : KEYS >= 64 ? 6
                               : KEYS >= 32 ? 5 : KEYS >= 16 ? 4 : 3;
    static_assert((1 << LOG2K) == KEYS, "brick key count is a power of two");
};

// The two Morton-aligned halves of a brick: the top bit of a brick-local
// key is z's for a cube, y's for BX = BY = 2 BZ and x's for BX = 2 BY = 2 BZ,
// so the lower half of the brick's keys is the half with the smaller
// coordinate along that axis, and each half is again a contiguous span of
// the sorted order.
template <int BX, int BY, int BZ>
struct BrickHalves {
    static constexpr bool cube = BX == BY && BY == BZ;
    static constexpr bool flat = BX == BY && BX == 2 * BZ;   // next split along y
    static constexpr int X = cube || flat ? BX : BX / 2;
    static constexpr int Y = flat ? BY / 2 : BY;
    static constexpr int Z = cube ? BZ / 2 : BZ;
    static constexpr int DX = BX - X, DY = BY - Y, DZ = BZ - Z;   // offset of the upper half
};

struct PairCfg {
    int nbx, nby, nbz, nbricks;
    int cap;            // staged particles that fit in shared memory
    int dlist;          // drain-queue depth of this launch (<= DLIST; queues drain above dlist - 4)
};

namespace {

__device__ __forceinline__ int lower_bound_u32(const uint32_t* __restrict__ a, int n, uint32_t key) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(&a[mid]) < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// Exclusive scan of one int per thread over the block (any multiple of 32
// up to 1024 threads).
__device__ __forceinline__ int block_excl_scan_int(int v, int* s_warp, int* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = lane < nw ? s_warp[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < nw) s_warp[lane] = w;
    }
    __syncthreads();
    const int off = warp ? s_warp[warp - 1] : 0;
    *total = s_warp[nw - 1];
    __syncthreads();
    return x - v + off;
}

// Walk the reference window of one target through the global cell table.
// At most ASPH_MAX_CANDIDATES candidates are visited: a denser window can
// only come from a blown-up state (the reference would spend quadratic
// time on it), so the run is stopped with ASPH_ERR_DENSE instead.
template <class F>
__device__ __forceinline__ void for_window_global(const Phys& P, const int2* __restrict__ range, DevCtl* ctl, float x,
                                                  float y, float z, F&& f) {
    const int ix = cell_ix(x, P.inv_dx, P.nx), iy = cell_ix(y, P.inv_dy, P.ny), iz = cell_ix(z, P.inv_dz, P.nz);
    const int z0 = max(iz - STENCIL, 0), z1 = min(iz + STENCIL, P.nz - 1);
    int budget = ASPH_MAX_CANDIDATES;
    for (int jz = z0; jz <= z1; ++jz)
        for (int jy = iy - STENCIL; jy <= iy + STENCIL; ++jy) {
            const int cy = wrapi(jy, P.ny);
            const int2* row = range + (size_t)(jz * P.ny + cy) * P.nx;
            for (int jx = ix - STENCIL; jx <= ix + STENCIL; ++jx) {
                const int2 rg = row[wrapi(jx, P.nx)];
                budget -= rg.y - rg.x;
                if (budget < 0) {
                    stop_run(ctl, ASPH_ERR_DENSE);
                    return;
                }
                for (int j = rg.x; j < rg.y; ++j) f(j);
            }
        }
}

// Span of one window row (cells ix-2 .. ix+2) inside the staged region.
// (Culling the span geometrically with a drift bound was measured slower at
// 0.6 particles per cell: the per-row arithmetic costs more than the candidates it
// removes.)
__device__ __forceinline__ void row_span(const int* s_off, int la_m2, int& k, int& kend) {
    k = s_off[la_m2];
    kend = s_off[la_m2 + 2 * STENCIL + 1];
}

// Region-local window of a target: returns false if it leaves the region.
template <int BX, int BY, int BZ, int H>
__device__ __forceinline__ bool local_window(const Phys& P, int ox, int oy, int oz, float x, float y, float z,
                                             int& lx, int& ly, int& zlo, int& zhi) {
    using G = BrickGeom<BX, BY, BZ, H>;
    const int ix = cell_ix(x, P.inv_dx, P.nx), iy = cell_ix(y, P.inv_dy, P.ny), iz = cell_ix(z, P.inv_dz, P.nz);
    lx = ix - (ox - H);
    lx += lx < 0 ? P.nx : 0; lx -= lx >= P.nx ? P.nx : 0;
    ly = iy - (oy - H);
    ly += ly < 0 ? P.ny : 0; ly -= ly >= P.ny ? P.ny : 0;
    const int rz0 = oz - H;
    zlo = max(iz - STENCIL, 0) - rz0;
    zhi = min(iz + STENCIL, P.nz - 1) - rz0;
    return lx >= STENCIL && lx < G::RX - STENCIL && ly >= STENCIL && ly < G::RY - STENCIL && zlo >= 0 &&
           zhi < G::RZ;
}

// Offsets of the staged region of a brick: s_off[l] = first slot of region
// cell l (row-major, H cells around the brick, x/y wrapped), s_off[R] =
// the total, s_start[l] = the cell's first global index, and (when it fits,
// total <= cap) s_gidx[k] = the global index of slot k.  A cell's particles
// take consecutive slots in index order.  The cell-table loads are strided
// over the block with four in flight per thread; the scan runs in shared
// memory.
template <int BX, int BY, int BZ, int H>
__device__ int region_offsets(const Phys& P, const int2* __restrict__ range, int ox, int oy, int oz, int* s_off,
                              int* s_start, int* s_gidx, int cap, int* s_warp) {
    using G = BrickGeom<BX, BY, BZ, H>;
    const int T = blockDim.x;
    const int rx0 = ox - H, ry0 = oy - H, rz0 = oz - H;
    for (int lb = threadIdx.x; lb < G::R; lb += 4 * T) {
        int2 rg[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int l = lb + u * T;
            rg[u] = make_int2(0, 0);
            if (l < G::R) {
                const int lx = l % G::RX, ly = (l / G::RX) % G::RY, lz = l / (G::RX * G::RY);
                const int gz = rz0 + lz;
                if (gz >= 0 && gz < P.nz) {
                    int gx = rx0 + lx, gy = ry0 + ly;
                    gx += gx < 0 ? P.nx : 0; gx -= gx >= P.nx ? P.nx : 0;
                    gy += gy < 0 ? P.ny : 0; gy -= gy >= P.ny ? P.ny : 0;
                    rg[u] = range[(size_t)(gz * P.ny + gy) * P.nx + gx];
                }
            }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int l = lb + u * T;
            if (l < G::R) {
                s_start[l] = rg[u].x;
                s_off[l] = rg[u].y - rg[u].x;
            }
        }
    }
    __syncthreads();
    const int chunk = (G::R + T - 1) / T;
    const int l0 = threadIdx.x * chunk, l1 = min(l0 + chunk, G::R);
    int run = 0;
    for (int l = l0; l < l1; ++l) run += s_off[l];
    int total;
    int excl = block_excl_scan_int(run, s_warp, &total);
    const bool map = total <= cap;
    for (int l = l0; l < l1; ++l) {
        const int c = s_off[l];
        s_off[l] = excl;
        if (map) {
            const int g = s_start[l];
            for (int k = 0; k < c; ++k) s_gidx[excl + k] = g + k;
        }
        excl += c;
    }
    if (threadIdx.x == 0) s_off[G::R] = total;
    __syncthreads();
    return total;
}

// Neighbour-list writer of one target (slot-major, coalesced over targets).
struct NbrOut {
    int* p;      // the next slot of target i's list
    size_t N;    // slot stride
    int n;
    __device__ __forceinline__ NbrOut(int* nbr, int n0, int N_, int i) : p(nbr + i), N((size_t)N_), n(n0) {}
    __device__ __forceinline__ void push(int j) {
        if (n < NBR_CAP) {
            *p = j;
            p += N;
        }
        ++n;
    }
};

}  // namespace

// ===========================================================================
// D: density + EOS + microphysics, neighbour lists
// ===========================================================================
struct DArgs {
    const float4* pos;      // x, y, z, rho_old
    const int2* range;
    const uint32_t* skeys;  // sorted keys of the table's order
    const int2* spans;      // per brick: its span of targets in the sorted order
    DOut out;
    int* nbr;
    int* nbr_cnt;
    int* defer;             // targets queued for the deferred pass (count in ctl->defer_n)
    DevCtl* ctl;
};

// Every brick's span of targets in the sorted order: the brick is a
// Morton-aligned key range, found by binary search in the sorted keys (one
// thread per brick).  The gather writes the same spans when a sort runs; this
// kernel serves sorted keys that the gather did not see (a restored state,
// another brick shape).
template <int BX, int BY, int BZ>
__global__ void k_brick_spans(const __grid_constant__ Phys P, const uint32_t* __restrict__ skeys, int2* spans,
                              PairCfg C) {
    using G = BrickGeom<BX, BY, BZ, STENCIL>;
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= C.nbricks) return;
    const int bxi = b % C.nbx, byi = (b / C.nbx) % C.nby, bzi = b / (C.nbx * C.nby);
    const uint32_t base = morton3((uint32_t)(bxi * BX), (uint32_t)(byi * BY), (uint32_t)(bzi * BZ));
    spans[base >> G::LOG2K] =
        make_int2(lower_bound_u32(skeys, P.N, base), lower_bound_u32(skeys, P.N, base + (uint32_t)G::KEYS));
}

__device__ __forceinline__ DSum density_target_global(const Phys& P, const DArgs& A, int i, float4 pi, FF rr) {
    DSum s{0.f, 0.f, 0.f};
    NbrOut L{A.nbr, 0, P.N, i};
    for_window_global(P, A.range, A.ctl, pi.x, pi.y, pi.z, [&](int j) {
        const float4 pj = A.pos[j];
        const float r2 = r2_pair(P, pi.x, pi.y, pi.z, pj.x, pj.y, pj.z);
        if (r2 < 4.0f) {
            dsum_add(s, r2, pj.w, rr);
            if (r2 >= 1e-12f) L.push(j);
        }
    });
    A.nbr_cnt[i] = L.n <= NBR_CAP ? L.n : -1;
    return s;
}

__global__ __launch_bounds__(256) void k_density_global(const __grid_constant__ Phys P,
                                                        const __grid_constant__ DArgs A) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (A.ctl->aborted || i >= P.N) return;
    const float dt = A.ctl->dt;
    const float4 pi = A.pos[i];
    const FF rr = snd_eval(P.snd_rho, P.snd_n, pi.z);
    const DSum s = density_target_global(P, A, i, pi, rr);
    density_eos_epilogue(P, A.out, i, pi, s, rr, dt);
}

// Pointers into the density pass's dynamic shared memory.
struct DSmem {
    float4* sp;               // staged particles: x, y, z, rho_old
    int* s_gidx;              // global index of a staged slot
    int* s_off;               // region cell -> first slot (R + 1)
    int* s_start;             // region cell -> first global index (R)
    unsigned short* s_list;   // drain queue, DLIST x T (reuses s_start after staging)
    int* s_warp;
    int* s_work;              // work items {ox, oy, oz, ts, te}: the root, then two per split level
};
constexpr int DENSITY_SPLITS = 2;   // an overflowing brick is split into halves, then quarters

// The work item at M.s_work + 5 * slot: the targets [ts, te) of the
// Morton-aligned brick with origin (ox, oy, oz) cells.  Stage the region,
// walk and drain.  A region that overflows the staging capacity is split
// into its two halves (each its own region and a contiguous sub-span of the
// targets), SPLITS times at most; targets the staged region still does not
// cover go to the deferred pass.  Work items live in shared memory, so
// nothing stays in registers across the first half's pass.
template <int BX, int BY, int BZ, int H, int SPLITS>
__device__ __forceinline__ void density_region(const Phys& P, const DArgs& A, const PairCfg& C, const DSmem& M,
                                               int slot) {
    using G = BrickGeom<BX, BY, BZ, H>;
    const int T = blockDim.x;
    // the work item was written by thread 0 before the call, and the shared
    // arrays of an earlier region are no longer read
    __syncthreads();
    const int* w = M.s_work + 5 * slot;
    const int ox = w[0], oy = w[1], oz = w[2], ts = w[3], te = w[4];
    const float dt = A.ctl->dt;
    float4* sp = M.sp;
    int* s_gidx = M.s_gidx;
    int* s_off = M.s_off;
    int* s_start = M.s_start;
    unsigned short* s_list = M.s_list;

    // ---- stage the region: counts, scan (row-major by region cell), copy
    const int total = region_offsets<BX, BY, BZ, H>(P, A.range, ox, oy, oz, s_off, s_start, s_gidx, C.cap, M.s_warp);
    const bool staged = total <= C.cap;
    if constexpr (SPLITS > 0) {
        if (!staged) {
            using S = BrickHalves<BX, BY, BZ>;
            const int c0 = 1 + 2 * (DENSITY_SPLITS - SPLITS);   // this level's two child slots
            if (threadIdx.x == 0) {
                atomicAdd(&A.ctl->split_n, 1u);
                const uint32_t half = morton3((uint32_t)ox, (uint32_t)oy, (uint32_t)oz) + (uint32_t)(G::KEYS / 2);
                const int mid = ts + lower_bound_u32(A.skeys + ts, te - ts, half);
                int* a = M.s_work + 5 * c0;
                a[0] = ox; a[1] = oy; a[2] = oz; a[3] = ts; a[4] = mid;
                a[5] = ox + S::DX; a[6] = oy + S::DY; a[7] = oz + S::DZ; a[8] = mid; a[9] = te;
            }
            density_region<S::X, S::Y, S::Z, H, SPLITS - 1>(P, A, C, M, c0);       // (starts with a barrier)
            density_region<S::X, S::Y, S::Z, H, SPLITS - 1>(P, A, C, M, c0 + 1);
            return;
        }
    }
    if (staged) {
        // slots strided over the block, copied global -> shared asynchronously:
        // every slot of the thread in flight at once, no registers held (density
        // 0.538 -> 0.527 ms at 2M against four register loads in flight)
        for (int k = threadIdx.x; k < total; k += T) {
            const unsigned d = (unsigned)__cvta_generic_to_shared(sp + k);
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(A.pos + s_gidx[k]) : "memory");
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    }
    __syncthreads();


    // ---- targets, one warp-synchronous round of 32 targets at a time
    const int lane = threadIdx.x & 31;
    for (int base = ts + (threadIdx.x & ~31); base < te; base += T) {
        const int i = base + lane;
        const bool active = i < te;
        float4 pi = make_float4(0.f, 0.f, 0.f, 0.f);
        FF rr{0.f, 0.f};
        DSum s{0.f, 0.f, 0.f};
        int lx = 0, ly = 0, zlo = 0, zhi = -1;
        bool fast = false;
        if (active) {
            pi = A.pos[i];
            rr = snd_eval(P.snd_rho, P.snd_n, pi.z);
            fast = staged && local_window<BX, BY, BZ, H>(P, ox, oy, oz, pi.x, pi.y, pi.z, lx, ly, zlo, zhi);
        }
        // targets the staged region does not cover go to the deferred pass
        const unsigned dm = __ballot_sync(0xffffffffu, active && !fast);
        if (dm) {
            const int lead = __ffs(dm) - 1;
            unsigned at = 0;
            if (lane == lead) at = atomicAdd(&A.ctl->defer_n, (unsigned)__popc(dm));
            at = __shfl_sync(0xffffffffu, at, lead);
            if (active && !fast) A.defer[at + __popc(dm & ((1u << lane) - 1u))] = i;
        }
        NbrOut L{A.nbr, 0, P.N, i};
        // the lanes' queues are the columns of the DLIST x T array (entry e of
        // this lane at qlane[e T]); n counts the queued entries in units of T,
        // so a push is one store and one add (density 0.5255 -> 0.5194 ms at 2M
        // against indexing by the entry count)
        unsigned short* const qlane = s_list + threadIdx.x;
        const int qlim = (C.dlist - 4) * T;
        int n = 0;
        // all lanes drain their queues together, in lockstep
#define ASPH_DRAIN()                                                                  \
    do {                                                                              \
        const int nmax_ = __reduce_max_sync(0xffffffffu, n);                          \
        for (int q = 0; q < nmax_; q += T) {                                          \
            if (q < n) {                                                              \
                const int kq = qlane[q];                                              \
                const float4 pj = sp[kq];                                             \
                const float r2 = r2_pair(P, pi.x, pi.y, pi.z, pj.x, pj.y, pj.z);      \
                dsum_add(s, r2, pj.w, rr);                                            \
                if (r2 >= 1e-12f) L.push(s_gidx[kq]);                                 \
            }                                                                         \
        }                                                                             \
        n = 0;                                                                        \
    } while (0)
        // flattened walk of the window rows in the staged region, branch
        // free: every step advances a finished row (la = region cell of the
        // row's first cell; rows step by RX, planes by RX * RY) and tests one
        // candidate, with selects, so the lanes never diverge.  Lanes past
        // their last row (la >= la_end) see empty rows.  The warp votes once
        // per 4 steps, so queues drain at dlist - 4 (drains run on fuller queues
        // than with a vote per 8 steps, which matters most in clustered states).
        int la = 0, la_end = 0, cy = 0, k = 0, kend = 0;
        if (fast) {
            la = (zlo * G::RY + ly - STENCIL) * G::RX + lx - STENCIL;
            la_end = la + (zhi - zlo + 1) * (G::RX * G::RY);
            row_span(s_off, la, k, kend);
        }
        for (;;) {
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const bool adv = k >= kend;
                int la2 = la + G::RX, cy2 = cy + 1;
                const bool wrap = cy2 == 2 * STENCIL + 1;
                la2 += wrap ? G::RX * G::RY - (2 * STENCIL + 1) * G::RX : 0;
                cy2 = wrap ? 0 : cy2;
                la = adv ? la2 : la;
                cy = adv ? cy2 : cy;
                if (adv) {   // predicated loads: only lanes that change rows read the offsets
                    if (la < la_end) {
                        k = s_off[la];
                        kend = s_off[la + 2 * STENCIL + 1];
                    } else {
                        kend = k;
                    }
                }
                const bool valid = k < kend;
                const float4 pj = sp[valid ? k : 0];
                if (valid && r2_pair(P, pi.x, pi.y, pi.z, pj.x, pj.y, pj.z) < 4.0f) {
                    qlane[n] = (unsigned short)k;
                    n += T;
                }
                k += valid ? 1 : 0;
            }
            if (__any_sync(0xffffffffu, n > qlim)) ASPH_DRAIN();
            if (__all_sync(0xffffffffu, la >= la_end)) break;
        }
        ASPH_DRAIN();
#undef ASPH_DRAIN
        if (active && fast) {
            A.nbr_cnt[i] = L.n <= NBR_CAP ? L.n : -1;
            density_eos_epilogue(P, A.out, i, pi, s, rr, dt);
        }
    }
}

// DENSITY_REGS = 48 registers keep 4 blocks of up to 320 threads per SM (the
// shared-memory limit at the default staging capacity).
template <int BX, int BY, int BZ, int H>
__global__ __maxnreg__(DENSITY_REGS) void k_density_brick(const __grid_constant__ Phys P, const __grid_constant__ DArgs A,
                                                       PairCfg C) {
    using G = BrickGeom<BX, BY, BZ, H>;
    extern __shared__ __align__(16) unsigned char smem[];
    const int T = blockDim.x;
    __shared__ int s_warp[32];
    __shared__ int s_work[5 * (1 + 2 * DENSITY_SPLITS)];
    __shared__ int s_run;
    DSmem M;
    M.sp = reinterpret_cast<float4*>(smem);
    M.s_gidx = reinterpret_cast<int*>(M.sp + C.cap);
    M.s_off = M.s_gidx + C.cap;
    M.s_start = M.s_off + (G::R + 1);
    M.s_list = reinterpret_cast<unsigned short*>(M.s_start);
    M.s_warp = s_warp;
    M.s_work = s_work;
    (void)T;
    if (threadIdx.x == 0) s_run = A.ctl->aborted ? 0 : 1;   // one decision per block (barriers follow)
    __syncthreads();
    if (!s_run) return;
    const int b = blockIdx.x;
    const int bxi = b % C.nbx, byi = (b / C.nbx) % C.nby, bzi = b / (C.nbx * C.nby);
    if (threadIdx.x == 0) {
        const int2 sp2 =
            A.spans[morton3((uint32_t)(bxi * BX), (uint32_t)(byi * BY), (uint32_t)(bzi * BZ)) >> G::LOG2K];
        s_work[0] = bxi * BX; s_work[1] = byi * BY; s_work[2] = bzi * BZ; s_work[3] = sp2.x; s_work[4] = sp2.y;
    }
    density_region<BX, BY, BZ, H, DENSITY_SPLITS>(P, A, C, M, 0);   // (starts with a barrier)
}

// Deferred pass: one warp per queued target.  The lanes read the ranges of
// the window's cells (c = dz * 25 + dy * 5 + dx, the reference's loop order)
// and their prefix counts into shared memory, then test the candidates 32
// at a time: candidate g lies in the last cell whose prefix is <= g.
// Accepted neighbours are appended in candidate order by ballot, so the list
// has the order of the reference's loop; the sums are reduced over the warp
// in a fixed tree.
constexpr int DEF_TPB = 256;
constexpr int WIN_CELLS = (2 * STENCIL + 1) * (2 * STENCIL + 1) * (2 * STENCIL + 1);
static_assert(WIN_CELLS <= 128, "a window's cells fit four per lane");

__global__ __launch_bounds__(DEF_TPB) void k_density_deferred(const __grid_constant__ Phys P,
                                                              const __grid_constant__ DArgs A) {
    __shared__ int s_cs[DEF_TPB / 32][128];   // first table index of window cell c
    __shared__ int s_cp[DEF_TPB / 32][128];   // candidates in the cells before c
    __shared__ int s_run;
    DevCtl* ctl = A.ctl;
    if (threadIdx.x == 0) s_run = ctl->aborted ? 0 : 1;   // one decision per block: every thread
    __syncthreads();                                       // reaches the barrier at the end
    const unsigned nq = !s_run ? 0u : (A.defer ? ctl->defer_n : (unsigned)P.N);   // no queue: every target
    const int lane = threadIdx.x & 31;
    int* cs = s_cs[threadIdx.x >> 5];
    int* cp = s_cp[threadIdx.x >> 5];
    const float dt = ctl->dt;
    const unsigned nwarps = (gridDim.x * DEF_TPB) >> 5;
    for (unsigned t = (blockIdx.x * DEF_TPB + threadIdx.x) >> 5; t < nq; t += nwarps) {
        const int i = A.defer ? A.defer[t] : (int)t;
        const float4 pi = A.pos[i];
        const int ix = cell_ix(pi.x, P.inv_dx, P.nx), iy = cell_ix(pi.y, P.inv_dy, P.ny);
        const int iz = cell_ix(pi.z, P.inv_dz, P.nz);
        const int z0 = max(iz - STENCIL, 0), z1 = min(iz + STENCIL, P.nz - 1);
        const int ncell = (z1 - z0 + 1) * (2 * STENCIL + 1) * (2 * STENCIL + 1);
        int total = 0;
        int2 rgs[4];   // the four cell-range loads in flight together
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int c = u * 32 + lane;
            rgs[u] = make_int2(0, 0);
            if (c < ncell) {
                const int dz = c / 25, r = c - dz * 25, dy = r / 5, dx = r - dy * 5;
                const int gy = wrapi(iy - STENCIL + dy, P.ny), gx = wrapi(ix - STENCIL + dx, P.nx);
                rgs[u] = A.range[(size_t)((z0 + dz) * P.ny + gy) * P.nx + gx];
            }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int c = u * 32 + lane;
            const int2 rg = rgs[u];
            const int cnt = rg.y - rg.x;
            int x = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            cs[c] = rg.x;
            cp[c] = total + x - cnt;
            total += __shfl_sync(0xffffffffu, x, 31);
        }
        __syncwarp();
        if (total > ASPH_MAX_CANDIDATES) {   // same stop as the global walk's budget (total is warp-uniform)
            if (lane == 0) stop_run(ctl, ASPH_ERR_DENSE);
            break;
        }
        const FF rr = snd_eval(P.snd_rho, P.snd_n, pi.z);
        DSum s{0.f, 0.f, 0.f};
        int nb = 0;
        for (int g0 = 0; g0 < total; g0 += 64) {
            // two rounds of 32 candidates: both rounds' loads in flight together
            int jr[2];
            float4 pr[2];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int g = g0 + 32 * h + lane;
                jr[h] = 0;
                if (g < total) {
                    int lo = 0, hi = ncell - 1;   // cp[lo] <= g
                    while (lo < hi) {
                        const int mid = (lo + hi + 1) >> 1;
                        if (cp[mid] <= g) lo = mid; else hi = mid - 1;
                    }
                    jr[h] = cs[lo] + (g - cp[lo]);
                    pr[h] = A.pos[jr[h]];
                }
            }
#pragma unroll
            for (int h = 0; h < 2; ++h) {
            const int g = g0 + 32 * h + lane;
            bool push = false;
            const int j = jr[h];
            if (g < total) {
                const float4 pj = pr[h];
                const float r2 = r2_pair(P, pi.x, pi.y, pi.z, pj.x, pj.y, pj.z);
                if (r2 < 4.0f) {
                    dsum_add(s, r2, pj.w, rr);
                    push = r2 >= 1e-12f;
                }
            }
            const unsigned m = __ballot_sync(0xffffffffu, push);
            if (push) {
                const int n = nb + __popc(m & ((1u << lane) - 1u));
                if (n < NBR_CAP) A.nbr[(size_t)n * P.N + i] = j;
            }
            nb += __popc(m);
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            s.S1 += __shfl_xor_sync(0xffffffffu, s.S1, o);
            s.S2 += __shfl_xor_sync(0xffffffffu, s.S2, o);
            s.T += __shfl_xor_sync(0xffffffffu, s.T, o);
        }
        if (lane == 0) {
            A.nbr_cnt[i] = nb <= NBR_CAP ? nb : -1;
            density_eos_epilogue(P, A.out, i, pi, s, rr, dt);
        }
        __syncwarp();   // cs and cp are rewritten for the next target
    }
    if (A.defer) {   // the last block to finish empties the queue for the next pass
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            if (atomicAdd(&ctl->defer_done, 1u) == gridDim.x - 1) {
                ctl->defer_last = ctl->defer_n;
                ctl->defer_n = 0u;
                ctl->split_last = ctl->split_n;
                ctl->split_n = 0u;
                ctl->defer_done = 0u;
            }
        }
    }
}

// ===========================================================================
// M: momentum + integrate + rain + CFL (list-driven)
// ===========================================================================
struct MArgs {
    const float4* pos;     // x, y, z, -
    const float4* vel;     // velocities after the first half kick
    const float2* rp;      // rho, p'
    const int2* range;
    const int* nbr;
    const int* nbr_cnt;
    int use_lists;         // lists (and ms0/ms1) were produced on the current positions and velocities
    const float4* ms0;     // x, y, z, p' of the density pass
    const float4* ms1;     // u, v, w, rho of the density pass
    MOut out;
    const float* rain_in;
    const float* rain_delta;
    float* rain_out;
    float* precip;
    DevCtl* ctl;
    int part_blocks;       // chunks of particle work (TPT x M_TPB targets each) ...
    int rain_blocks;       // ... then chunks of rain cells (M_RAIN_CELLS x M_TPB each)
};

// Out of line: targets without a usable neighbour list come here.
__device__ __noinline__ MSum momentum_target_global(const Phys& P, const MArgs& A, const MTarget T) {
    MSum s{0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for_window_global(P, A.range, A.ctl, T.x, T.y, T.z, [&](int j) {
        const float4 pj = A.pos[j];
        const float r2t = r2_pair(P, T.x, T.y, T.z, pj.x, pj.y, pj.z);
        if (r2t >= 4.0f || r2t < 1e-12f) return;   // also excludes j == i
        const float2 rj = A.rp[j];
        const float4 vj = A.vel[j];
        msum_add(P, s, T, make_float4(pj.x, pj.y, pj.z, rj.y), make_float4(vj.x, vj.y, vj.z, rj.x));
    });
    return s;
}

// The TPT x M_TPB targets of particle chunk `ch`: the lanes of warp w on
// targets w * 32 * TPT + lane + 32 r, so that a warp waits on the longest sum
// of its lanes' lists rather than on the longest list of each round; a warp
// covers 32 TPT consecutive targets, about 32 TPT / ppc cells.
template <int TPT>
__device__ __forceinline__ void momentum_chunk(const Phys& P, const MArgs& A, int mode, int ch, bool aborted,
                                               float dt, float3& m) {
    const int tbase = ch * (M_TPB * TPT) + (threadIdx.x >> 5) * (32 * TPT) + (threadIdx.x & 31);
    for (int r = 0; r < TPT; ++r) {
        const int i = tbase + 32 * r;
        if (i >= P.N) continue;
        if (aborted) {
            if (mode & M_INTEGRATE) A.out.vel_out[i] = A.vel[i];
            continue;
        }
        // (x, y, z, p') and (u, v, w, rho): packed by the density pass
        // when the lists are current, else from the state buffers
        float4 a, b;
        if (A.use_lists) {
            a = A.ms0[i];
            b = A.ms1[i];
        } else {
            const float4 p = A.pos[i], v = A.vel[i];
            const float2 rr = A.rp[i];
            a = make_float4(p.x, p.y, p.z, rr.y);
            b = make_float4(v.x, v.y, v.z, rr.x);
        }
        MTarget T;
        T.x = a.x; T.y = a.y; T.z = a.z;
        T.u = b.x; T.v = b.y; T.w = b.z;
        T.rhoi = fmaxf(b.w, 1e-3f);
        T.irhoi = __frcp_rn(T.rhoi);
        T.pri = a.w;
        MSum s{0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        const int cnt = A.use_lists ? A.nbr_cnt[i] : -1;
        if (cnt >= 0) {
            // four neighbours' loads in flight before their arithmetic
            int q = 0;
            const int* lp = A.nbr + i;   // slot q of the list at lp[q N]
            const size_t N = (size_t)P.N;
            for (; q + 4 <= cnt; q += 4) {
                int jj[4];
                float4 pp[4], vv[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) jj[u] = lp[u * N];
                lp += 4 * N;
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    pp[u] = A.ms0[jj[u]];
                    vv[u] = A.ms1[jj[u]];
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) msum_add(P, s, T, pp[u], vv[u]);
            }
            if (q < cnt) {   // the last 1-3 neighbours as one batch, their loads in flight together
                int jj[3];
                float4 pp[3], vv[3];
#pragma unroll
                for (int u = 0; u < 3; ++u) jj[u] = q + u < cnt ? lp[u * N] : i;
#pragma unroll
                for (int u = 0; u < 3; ++u) {
                    pp[u] = A.ms0[jj[u]];
                    vv[u] = A.ms1[jj[u]];
                }
#pragma unroll
                for (int u = 0; u < 3; ++u)
                    if (q + u < cnt) msum_add(P, s, T, pp[u], vv[u]);
            }
        } else {
            s = momentum_target_global(P, A, T);
        }
        const float3 mi = momentum_epilogue(P, A.out, i, T, s, (mode & M_INTEGRATE) != 0, dt);
        m = make_float3(fmaxf(m.x, mi.x), fmaxf(m.y, mi.y), fmaxf(m.z, mi.z));
    }
}

// The M_RAIN_CELLS x M_TPB rain cells of rain chunk `rc`.
__device__ __forceinline__ void rain_chunk(const Phys& P, const MArgs& A, int rc, bool aborted, float dt) {
#pragma unroll
    for (int r = 0; r < M_RAIN_CELLS; ++r) {
        const int cid = (rc * M_RAIN_CELLS + r) * M_TPB + threadIdx.x;
        if (cid < P.ncell && !aborted) rain_cell(P, cid, dt, A.rain_in, A.rain_delta, A.rain_out, A.precip);
    }
}

template <int TPT>
__global__ __launch_bounds__(M_TPB, M_MINB) void k_momentum(const __grid_constant__ Phys P, const __grid_constant__ MArgs A,
                                                    int mode) {
    __shared__ float s_max[3][M_TPB / 32];
    DevCtl* ctl = A.ctl;
    const bool aborted = ctl->aborted != 0;
    const float dt = ctl->dt;
    float3 m = make_float3(0.f, 0.f, 0.f);
    const int chunks = A.part_blocks + A.rain_blocks;
    if ((int)blockIdx.x >= A.part_blocks) {
        if ((int)blockIdx.x < chunks) rain_chunk(P, A, blockIdx.x - A.part_blocks, aborted, dt);
    } else {
        momentum_chunk<TPT>(P, A, mode, blockIdx.x, aborted, dt, m);
        if (mode & M_INTEGRATE) {   // the particle blocks' velocity maxima
            float mx = warp_max(m.x), my = warp_max(m.y), mz = warp_max(m.z);
            const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
            if (lane == 0) { s_max[0][warp] = mx; s_max[1][warp] = my; s_max[2][warp] = mz; }
            __syncthreads();
            if (threadIdx.x == 0) {
                float a = 0.f, b = 0.f, c = 0.f;
                for (int w = 0; w < M_TPB / 32; ++w) {
                    a = fmaxf(a, s_max[0][w]); b = fmaxf(b, s_max[1][w]); c = fmaxf(c, s_max[2][w]);
                }
                atomicMax(&ctl->gmax[0], __float_as_uint(a));
                atomicMax(&ctl->gmax[1], __float_as_uint(b));
                atomicMax(&ctl->gmax[2], __float_as_uint(c));
            }
        }
    }
}

// The CFL control after a momentum pass (asph_h100.cu:1040-1078), in a
// kernel of its own: one launch costs less than a finished-block atomic from
// each of the pass's ~11,600 blocks to find the last one (momentum 0.242 ->
// 0.234 ms at 2M).
__global__ void k_cfl_final(const __grid_constant__ Phys P, DevCtl* ctl) {
    if (threadIdx.x == 0 && !ctl->aborted) cfl_control(P, ctl);
}

// ===========================================================================
// launch
// ===========================================================================
namespace {

struct Shape {
    int bx, by, bz;
};
constexpr Shape SHAPES[] = {{8, 8, 8}, {8, 8, 4}, {8, 4, 4}, {4, 4, 4}};
constexpr int MAX_STAGE = 4096;      // staged particles per brick at most
constexpr double STAGE_MARGIN = 1.35;

int region_cells(const Shape& s, int h) { return (s.bx + 2 * h) * (s.by + 2 * h) * (s.bz + 2 * h); }

// Staged halo: with a sort every step the targets are in (or next to) the
// cells of their brick, and the stencil alone is staged; slower cadences
// stage one more cell of drift.  Targets outside either go to the deferred pass.
int halo_for(const Phys& P) { return P.sort_every == 1 ? STENCIL : MAX_HALO; }

// Largest brick whose region fits the grid without wrapping onto itself
// and whose expected staged count (with a margin) fits the cap.
bool fits(const Phys& P, int k) {
    const Shape& s = SHAPES[k];
    if (P.nx < s.bx + 2 * MAX_HALO || P.ny < s.by + 2 * MAX_HALO) return false;
    return region_cells(s, MAX_HALO) * ((double)P.N / (double)P.ncell) * STAGE_MARGIN <= MAX_STAGE;
}

int pick_shape(const Phys& P) {
    for (int k = 0; k < 4; ++k)
        if (fits(P, k)) return k;
    return -1;
}

int shape_in_use(const Phys& P, const Bufs& B) {
    if (B.force_global) return -1;
    return B.shape >= 0 ? B.shape : pick_shape(P);
}

struct Launch {
    PairCfg C;
    int threads;
    size_t smem;
};

// Shared memory per SM and reserved per block (queried once; GB300 values as fallback).
void smem_limits(int* per_sm, int* reserved) {
    static int sm = 0, res = -1;
    if (!sm) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess || sm <= 0)
            sm = 228 * 1024;
        if (cudaDeviceGetAttribute(&res, cudaDevAttrReservedSharedMemoryPerBlock, dev) != cudaSuccess || res < 0)
            res = 1024;
    }
    *per_sm = sm;
    *reserved = res;
}


Launch plan(const Phys& P, const Shape& s, int h) {
    Launch L;
    L.C.nbx = (P.nx + s.bx - 1) / s.bx;
    L.C.nby = (P.ny + s.by - 1) / s.by;
    L.C.nbz = (P.nz + s.bz - 1) / s.bz;
    L.C.nbricks = L.C.nbx * L.C.nby * L.C.nbz;
    const double ppc = (double)P.N / (double)P.ncell;
    const int R = region_cells(s, h);
    // about one thread per expected target (the lattice keeps brick counts
    // close to the mean), in whole warps, 64..512
    int t = (int)(s.bx * s.by * s.bz * ppc * 1.04 + 31) / 32 * 32;
    L.threads = t < 64 ? 64 : (t > 512 ? 512 : t);
    // s_start (R ints) while staging; the drain queue after
    auto smem_for = [&](size_t cap, int dlist) {
        const size_t queue = (size_t)dlist * L.threads * 2, start = (size_t)4 * R;
        return cap * 16 + cap * 4 + (size_t)4 * (R + 1) + ((queue > start ? queue : start) + 15) / 16 * 16;
    };
    // staging capacity: at least the expected region count times STAGE_MARGIN;
    // the most resident blocks the registers allow come first, then the
    // deepest drain queue (fuller drains) that still fits them, then all the
    // shared memory left for staging, so that clustered bricks overflow less
    // often (an overflowing brick is split into halves)
    int need = (int)(R * ppc * STAGE_MARGIN) + 64;
    need = (need + 63) & ~63;
    need = need > MAX_STAGE ? MAX_STAGE : need;
    int per_sm, reserved;
    smem_limits(&per_sm, &reserved);
    const int by_regs = 65536 / (DENSITY_REGS * L.threads);
    int cap = need, dlist = 16;
    bool found = false;
    for (int b = by_regs < 8 ? by_regs : 8; b >= 1 && !found; --b) {
        const size_t budget = (size_t)(per_sm / b - reserved - 512);   // 512: the kernel's static arrays
        for (int d = DLIST; d >= 16 && !found; d -= 2) {
            if (smem_for(need, d) > budget) continue;
            int c = MAX_STAGE;
            while (c > need && smem_for(c, d) > budget) c -= 64;
            cap = c;
            dlist = d;
            found = true;
        }
    }
    L.C.cap = cap;
    L.C.dlist = dlist;
    L.smem = smem_for(cap, dlist);
    return L;
}

// Blocks of the deferred pass: 4 per SM (32 warps), each warp looping over the queue.
int deferred_blocks() {
    static int blocks = 0;
    if (!blocks) {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 152;
        blocks = 4 * sms;
    }
    return blocks;
}

template <int BX, int BY, int BZ, int H>
void launch_dh(const Phys& P, const DArgs& A, cudaStream_t s) {
    const Launch L = plan(P, Shape{BX, BY, BZ}, H);
    cudaFuncSetAttribute(k_density_brick<BX, BY, BZ, H>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.smem);
    cudaFuncSetAttribute(k_density_brick<BX, BY, BZ, H>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    k_density_brick<BX, BY, BZ, H><<<L.C.nbricks, L.threads, L.smem, s>>>(P, A, L.C);
    k_density_deferred<<<deferred_blocks(), DEF_TPB, 0, s>>>(P, A);
}

template <int BX, int BY, int BZ>
void launch_d(const Phys& P, const DArgs& A, cudaStream_t s) {
    if (halo_for(P) == STENCIL) launch_dh<BX, BY, BZ, STENCIL>(P, A, s);
    else launch_dh<BX, BY, BZ, MAX_HALO>(P, A, s);
}

inline int blocks_for(int n, int tpb) { return n <= 0 ? 1 : (n + tpb - 1) / tpb; }

}  // namespace

int pair_shape(const Phys& P, const Bufs& B) { return shape_in_use(P, B); }
size_t pair_span_slots(const Phys& P) {
    const size_t keys = (size_t)1 << P.key_bits;
    return keys >> 6 > 0 ? keys >> 6 : 1;   // the smallest shape, 4 x 4 x 4, has 64 keys
}
int pair_span_shift(const Phys& P, const Bufs& B) {
    const int k = shape_in_use(P, B);
    if (k < 0) return -1;
    const int keys = SHAPES[k].bx * SHAPES[k].by * SHAPES[k].bz;
    int sh = 0;
    while ((1 << sh) < keys) ++sh;
    return sh;
}
void launch_brick_spans(const Phys& P, const Bufs& B, cudaStream_t s) {
    const int k = shape_in_use(P, B);
    if (k < 0) return;
    const Shape& sh = SHAPES[k];
    const Launch L = plan(P, sh, MAX_HALO);
    const int blocks = (L.C.nbricks + 255) / 256;
    switch (k) {
        case 0: k_brick_spans<8, 8, 8><<<blocks, 256, 0, s>>>(P, B.skeys, B.spans, L.C); break;
        case 1: k_brick_spans<8, 8, 4><<<blocks, 256, 0, s>>>(P, B.skeys, B.spans, L.C); break;
        case 2: k_brick_spans<8, 4, 4><<<blocks, 256, 0, s>>>(P, B.skeys, B.spans, L.C); break;
        default: k_brick_spans<4, 4, 4><<<blocks, 256, 0, s>>>(P, B.skeys, B.spans, L.C); break;
    }
}
int pair_shape_count() { return (int)(sizeof(SHAPES) / sizeof(SHAPES[0])); }
bool pair_shape_fits(const Phys& P, int k) { return k >= 0 && k < pair_shape_count() && fits(P, k); }

void launch_density(const Phys& P, const Bufs& B, cudaStream_t s) {
    DArgs A;
    A.pos = B.pos[B.pc];
    A.range = B.range;
    A.skeys = B.skeys;
    A.out.thq = B.thq[B.qc];
    A.out.rp = B.rp;
    A.out.vel = B.vel[B.vc];
    A.out.ms0 = B.ms[0];
    A.out.ms1 = B.ms[1];
    const bool reads = P.accretion || P.rain_evap;
    A.out.rain_cur = B.rain[B.rc];
    A.out.rain_dep = reads ? B.rain_delta : B.rain[B.rc];
    A.spans = B.spans;
    A.nbr = B.nbr;
    A.nbr_cnt = B.nbr_cnt;
    A.defer = B.defer;
    A.ctl = B.ctl;
    if (B.force_global == 2) {   // warp per target for every target
        A.defer = nullptr;
        k_density_deferred<<<deferred_blocks(), DEF_TPB, 0, s>>>(P, A);
        return;
    }
    switch (shape_in_use(P, B)) {
        case 0: launch_d<8, 8, 8>(P, A, s); break;
        case 1: launch_d<8, 8, 4>(P, A, s); break;
        case 2: launch_d<8, 4, 4>(P, A, s); break;
        case 3: launch_d<4, 4, 4>(P, A, s); break;
        default: k_density_global<<<blocks_for(P.N, 256), 256, 0, s>>>(P, A); break;
    }
}

int momentum_tpt(const Bufs& B) { return B.m_tpt > 0 ? B.m_tpt : M_TPT; }

void launch_momentum(const Phys& P, const Bufs& B, int mode, int use_lists, cudaStream_t s) {
    MArgs A;
    A.pos = B.pos[B.pc];
    A.vel = B.vel[B.vc];
    A.rp = B.rp;
    A.range = B.range;
    A.nbr = B.nbr;
    A.nbr_cnt = B.nbr_cnt;
    A.use_lists = use_lists;
    A.ms0 = B.ms[0];
    A.ms1 = B.ms[1];
    A.out.thq = B.thq[B.qc];
    A.out.acc = B.acc;
    A.out.dthdt = B.dthdt;
    A.out.vel_out = B.vel[1 - B.vc];
    A.out.src_cur = B.src ? B.src_tmp : nullptr;
    A.out.src_keep = B.src;
    A.rain_in = B.rain[B.rc];
    A.rain_delta = (P.accretion || P.rain_evap) ? B.rain_delta : nullptr;
    A.rain_out = B.rain[1 - B.rc];
    A.precip = B.precip;
    A.ctl = B.ctl;
    const int tpt = momentum_tpt(B);
    A.part_blocks = blocks_for(P.N, M_TPB * tpt);
    const int rain_blocks = (mode & M_RAIN) ? blocks_for(P.ncell, M_TPB * M_RAIN_CELLS) : 0;
    A.rain_blocks = rain_blocks;
    const int grid = A.part_blocks + rain_blocks;
    if (tpt == 1)
        k_momentum<1><<<grid, M_TPB, 0, s>>>(P, A, mode);
    else if (tpt == 4)
        k_momentum<4><<<grid, M_TPB, 0, s>>>(P, A, mode);
    else
        k_momentum<2><<<grid, M_TPB, 0, s>>>(P, A, mode);
    if (mode & M_CFL) k_cfl_final<<<1, 32, 0, s>>>(P, A.ctl);
}

}  // namespace asph
