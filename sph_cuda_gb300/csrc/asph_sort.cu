// asph_sort.cu — stable LSD radix sort of the Morton keys with the
// identity as values, written for sm_103a.
//
// Replaces cub::DeviceRadixSort::SortPairs(keys, iota) of the reference
// (asph_h100.cu:866-871, 903-904, 966-967).  A stable sort of (key, i) has
// one answer, std::stable_sort by key, so the permutation is bit-identical
// to CUB's whatever the implementation.
//
// Design (one "onesweep" pass per 8-bit digit):
//  * one upfront histogram kernel counts the digits of every pass;
//  * each pass kernel takes a tile of SORT_TILE keys (tile ids handed out by
//    an atomic counter so that a tile only ever waits on tiles that already
//    started), ranks keys inside the tile with __match_any_sync warp
//    ranking (stable: iteration order within a warp, warp order within the
//    tile), publishes its per-digit counts and resolves its global offsets
//    by decoupled look-back over 64-bit epoch-tagged status words (no
//    per-sort memset of the status array), then scatters through shared
//    memory so that global writes are runs of consecutive addresses.
//  * every wait is bounded (SPIN_LIMIT); on expiry the kernel records
//    ASPH_ERR_TIMEOUT in the control block and carries on.
#include "asph_internal.cuh"
#include "../../include/asph.h"

namespace asph {

namespace {

constexpr uint64_t FLAG_AGG = 1ull << 30;
constexpr uint64_t FLAG_PRE = 2ull << 30;
constexpr uint64_t CNT_MASK = (1ull << 30) - 1;

__device__ __forceinline__ bool sort_runs(const DevCtl* ctl, int force) {
    return force || (ctl->do_sort && !ctl->aborted);
}

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Exclusive scan of one value per thread over a 256-thread block.
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* s_warp, uint32_t* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < (SORT_TPB / 32) ? s_warp[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < (SORT_TPB / 32)) s_warp[lane] = w;
    }
    __syncthreads();
    uint32_t off = warp ? s_warp[warp - 1] : 0u;
    *total = s_warp[SORT_TPB / 32 - 1];
    __syncthreads();
    return x - v + off;
}

}  // namespace

// Clears the cell table before it is rebuilt (the reference's
// cudaMemsetAsync(cellRange), asph_h100.cu:971-972), resets the sort
// counters, and zeroes this step's rain deposits.
__global__ void k_sort_prep(Phys P, int2* __restrict__ range, float* __restrict__ delta,
                            DevCtl* __restrict__ ctl, int force, int clear_delta) {
    const bool run = sort_runs(ctl, force);
    const int stride = gridDim.x * blockDim.x;
    const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
    if (clear_delta) {
        float4* d4 = reinterpret_cast<float4*>(delta);
        const int n4 = P.ncell >> 2;
        for (int i = t0; i < n4; i += stride) d4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int i = (n4 << 2) + t0; i < P.ncell; i += stride) delta[i] = 0.f;
    }
    if (!run) return;
    if (blockIdx.x == 0) {
        for (int i = threadIdx.x; i < MAX_PASSES * 256; i += blockDim.x) (&ctl->hist[0][0])[i] = 0u;
        if (threadIdx.x < MAX_PASSES) ctl->tile_ctr[threadIdx.x] = 0u;
        if (threadIdx.x == 0) {
            ctl->epoch += 1u;
            ctl->surf_count = 0;
            ctl->sorted_this_step = 1;
            ctl->sort_count += 1;
        }
    }
    int4* r4 = reinterpret_cast<int4*>(range);   // 16-byte aligned allocation
    const int n4 = P.ncell >> 1;
    for (int i = t0; i < n4; i += stride) r4[i] = make_int4(0, 0, 0, 0);
    if ((P.ncell & 1) && t0 == 0) range[P.ncell - 1] = make_int2(0, 0);
}

// Digit histograms of every pass in one read of the keys.
__global__ __launch_bounds__(SORT_TPB) void k_hist(const uint32_t* __restrict__ keys, int N, int npasses,
                                                   DevCtl* __restrict__ ctl, int force) {
    if (!sort_runs(ctl, force)) return;
    __shared__ uint32_t h[MAX_PASSES][256];
    for (int i = threadIdx.x; i < MAX_PASSES * 256; i += blockDim.x) (&h[0][0])[i] = 0u;
    __syncthreads();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        uint32_t k = keys[i];
        for (int p = 0; p < npasses; ++p) atomicAdd(&h[p][(k >> (8 * p)) & 255u], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < npasses * 256; i += blockDim.x) {
        uint32_t c = (&h[0][0])[i];
        if (c) atomicAdd(&(&ctl->hist[0][0])[i], c);
    }
}

__global__ __launch_bounds__(SORT_TPB, 4) void k_radix_pass(
    const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin, uint32_t* __restrict__ kout,
    uint32_t* __restrict__ vout, uint64_t* __restrict__ status, int N, int ntiles, int pass,
    DevCtl* __restrict__ ctl, int force) {
    if (!sort_runs(ctl, force)) return;
    constexpr int NW = SORT_TPB / 32;
    __shared__ uint32_t s_whist[NW][256];
    __shared__ uint32_t s_keys[SORT_TILE];
    __shared__ uint32_t s_vals[SORT_TILE];
    __shared__ uint32_t s_texcl[256];
    __shared__ uint32_t s_gbase[256];
    __shared__ uint32_t s_scan[NW];
    __shared__ uint32_t s_tile;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) s_tile = atomicAdd(&ctl->tile_ctr[pass], 1u);
    for (int i = tid; i < NW * 256; i += SORT_TPB) (&s_whist[0][0])[i] = 0u;
    __syncthreads();
    const int tile = (int)s_tile;
    const int shift = 8 * pass;
    const int base = tile * SORT_TILE;
    const unsigned epoch = ctl->epoch;

    uint32_t k[SORT_ITEMS], v[SORT_ITEMS], r[SORT_ITEMS];
    uint32_t d[SORT_ITEMS];
#pragma unroll
    for (int it = 0; it < SORT_ITEMS; ++it) {
        const int e = base + warp * 32 * SORT_ITEMS + it * 32 + lane;
        const bool ok = e < N;
        k[it] = ok ? kin[e] : 0u;
        v[it] = ok ? (vin ? vin[e] : (uint32_t)e) : 0u;
        d[it] = ok ? ((k[it] >> shift) & 255u) : 256u;
    }
    // Stable rank inside the warp: iteration order, then lane order.
    const unsigned ltm = lanemask_lt();
#pragma unroll
    for (int it = 0; it < SORT_ITEMS; ++it) {
        const unsigned peers = __match_any_sync(0xffffffffu, d[it]);
        const int leader = __ffs(peers) - 1;
        uint32_t old = 0u;
        if (d[it] < 256u) old = s_whist[warp][d[it]];
        __syncwarp();
        if (d[it] < 256u && lane == leader) s_whist[warp][d[it]] = old + __popc(peers);
        __syncwarp();
        r[it] = old + __popc(peers & ltm);
    }
    __syncthreads();

    // Per digit (thread = digit): warp-exclusive prefixes and the tile count.
    const int dg = tid;
    uint32_t run = 0u;
#pragma unroll
    for (int w = 0; w < NW; ++w) {
        uint32_t c = s_whist[w][dg];
        s_whist[w][dg] = run;
        run += c;
    }
    const uint32_t tile_cnt = run;

    // Publish the aggregate, then look back for the exclusive prefix.
    uint64_t* st = status + ((size_t)pass * ntiles) * 256;
    const uint64_t ep = (uint64_t)epoch << 32;
    uint32_t excl = 0u;
    if (tile == 0) {
        atomicExch((unsigned long long*)&st[dg], (unsigned long long)(ep | FLAG_PRE | tile_cnt));
    } else {
        atomicExch((unsigned long long*)&st[(size_t)tile * 256 + dg],
                   (unsigned long long)(ep | FLAG_AGG | tile_cnt));
        int t = tile - 1;
        unsigned spins = 0;
        while (t >= 0) {
            const uint64_t w = *(volatile const uint64_t*)&st[(size_t)t * 256 + dg];
            if ((uint32_t)(w >> 32) != epoch || (w & (3ull << 30)) == 0) {
                if (++spins > SPIN_LIMIT) {
                    ctl->error = ASPH_ERR_TIMEOUT;
                    break;
                }
                continue;
            }
            excl += (uint32_t)(w & CNT_MASK);
            if (w & FLAG_PRE) break;
            --t;
        }
        atomicExch((unsigned long long*)&st[(size_t)tile * 256 + dg],
                   (unsigned long long)(ep | FLAG_PRE | (uint64_t)(excl + tile_cnt)));
    }

    // Global start of each digit (scan of the histogram) and the tile-local
    // start of each digit (scan of the tile counts).
    uint32_t tot;
    const uint32_t gstart = block_excl_scan(ctl->hist[pass][dg], s_scan, &tot);
    const uint32_t texcl = block_excl_scan(tile_cnt, s_scan, &tot);
    s_texcl[dg] = texcl;
    s_gbase[dg] = gstart + excl;
    __syncthreads();

    // Local scatter into digit order, then coalesced runs to global.
#pragma unroll
    for (int it = 0; it < SORT_ITEMS; ++it) {
        if (d[it] < 256u) {
            const uint32_t lp = s_texcl[d[it]] + s_whist[warp][d[it]] + r[it];
            s_keys[lp] = k[it];
            s_vals[lp] = v[it];
        }
    }
    __syncthreads();
    const int nvalid = min(SORT_TILE, N - base);
    for (int j = tid; j < nvalid; j += SORT_TPB) {
        const uint32_t key = s_keys[j];
        const uint32_t dd = (key >> shift) & 255u;
        const uint32_t o = s_gbase[dd] + (uint32_t)j - s_texcl[dd];
        if (o < (uint32_t)N) {   // only false after a timed-out look-back
            kout[o] = key;
            vout[o] = s_vals[j];
        }
    }
}

void launch_sort_prep(const Phys& P, const Bufs& B, int force, int clear_delta, cudaStream_t s) {
    int blocks = (P.ncell / 2 + TPB - 1) / TPB;
    blocks = blocks < 1 ? 1 : (blocks > 152 * 16 ? 152 * 16 : blocks);
    k_sort_prep<<<blocks, TPB, 0, s>>>(P, B.range, B.rain_delta, B.ctl, force, clear_delta);
}

void launch_sort(const Phys& P, Bufs& B, int force, cudaStream_t s) {
    if (P.N <= 0) return;
    int hb = (P.N + TPB * 8 - 1) / (TPB * 8);
    hb = hb > 152 * 8 ? 152 * 8 : hb;
    k_hist<<<hb, SORT_TPB, 0, s>>>(B.kin, P.N, B.npasses, B.ctl, force);
    for (int p = 0; p < B.npasses; ++p) {
        const uint32_t* ki = p == 0 ? B.kin : B.kbuf[(p - 1) & 1];
        const uint32_t* vi = p == 0 ? nullptr : B.vbuf[(p - 1) & 1];
        k_radix_pass<<<B.ntiles, SORT_TPB, 0, s>>>(ki, vi, B.kbuf[p & 1], B.vbuf[p & 1], B.status, P.N,
                                                   B.ntiles, p, B.ctl, force);
    }
}

}  // namespace asph
