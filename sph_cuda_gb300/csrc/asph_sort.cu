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

// Gate of a sort launch (`force`): 0 the step's gating (the control
// block's do_sort, nothing after an abort), 1 a forced full sort (granular
// call), GATE_AHEAD the next step's sort run ahead, which always runs (the
// gather that would apply it still follows the step's gating).
constexpr int GATE_AHEAD = 2;

__device__ __forceinline__ bool sort_runs(const DevCtl* ctl, int force) {
    return force || (ctl->do_sort && !ctl->aborted);
}

// Sort lane 0 is the full sort of all keys; lane 1 sorts the keys that
// changed since the last sort (incremental path).  The step launches both;
// the control block decides which one works.
__device__ __forceinline__ bool lane_runs(const DevCtl* ctl, int force, int sort_lane) {
    const bool go = force == GATE_AHEAD || (ctl->do_sort && !ctl->aborted);
    if (sort_lane == 0) return force == 1 || (go && !ctl->inc_on);
    return force != 1 && go && ctl->inc_on;
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
__global__ void k_sort_prep(Phys P, int2* __restrict__ range, int2* __restrict__ spans, int nspans,
                            float* __restrict__ delta, DevCtl* __restrict__ ctl, int force, int clear_delta) {
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
    for (int i = t0; i < nspans; i += stride) spans[i] = make_int2(0, 0);   // brick spans, rebuilt with the table
}

// Digit histograms of every pass in one read of the keys.
__global__ __launch_bounds__(SORT_TPB) void k_hist(const uint32_t* __restrict__ keys, int N, int npasses,
                                                   DevCtl* __restrict__ ctl, int force, int sort_lane) {
    if (!lane_runs(ctl, force, sort_lane)) return;
    if (sort_lane) N = min(N, (int)ctl->inc_m);
    unsigned* ghist = sort_lane ? &ctl->ihist[0][0] : &ctl->hist[0][0];
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
        if (c) atomicAdd(&ghist[i], c);
    }
}

__global__ __launch_bounds__(SORT_TPB, 4) void k_radix_pass(
    const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin, uint32_t* __restrict__ kout,
    uint32_t* __restrict__ vout, uint64_t* __restrict__ status, int N, int ntiles, int pass,
    DevCtl* __restrict__ ctl, int force, int sort_lane) {
    if (!lane_runs(ctl, force, sort_lane)) return;
    if (sort_lane) N = min(N, (int)ctl->inc_m);
    unsigned* const tile_ctr = sort_lane ? ctl->itile_ctr : ctl->tile_ctr;
    const unsigned* const ghist = sort_lane ? ctl->ihist[pass] : ctl->hist[pass];
    constexpr int NW = SORT_TPB / 32;
    __shared__ uint32_t s_whist[NW][256];
    __shared__ uint32_t s_keys[SORT_TILE];
    __shared__ uint32_t s_vals[SORT_TILE];
    __shared__ uint32_t s_texcl[256];
    __shared__ uint32_t s_gbase[256];
    __shared__ uint32_t s_scan[NW];
    __shared__ uint32_t s_tile;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) s_tile = atomicAdd(&tile_ctr[pass], 1u);
    for (int i = tid; i < NW * 256; i += SORT_TPB) (&s_whist[0][0])[i] = 0u;
    __syncthreads();
    const int tile = (int)s_tile;
    const int shift = 8 * pass;
    const int base = tile * SORT_TILE;
    if (base >= N && tile > 0) return;   // lane 1 launches for its largest count
    const unsigned epoch = sort_lane ? ctl->iepoch : ctl->epoch;

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
    const uint32_t gstart = block_excl_scan(ghist[dg], s_scan, &tot);
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
    const int nvalid = max(0, min(SORT_TILE, N - base));
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

// ---------------------------------------------------------------------------
// Incremental sort.  The particles are in the order of the last sort, whose
// sorted keys are B.skeys.  A particle whose key did not change keeps its
// place in that sorted sequence, so the unchanged particles, in index order,
// are already sorted by (key, index); only the changed ones need a sort.
// Their stable sort merged with the unchanged sequence by (key, index) is
// exactly the stable sort of all keys, bit for bit.  When more than a
// fixed share changed (inc_max), the full sort runs instead.
// ---------------------------------------------------------------------------
namespace {
constexpr int INC_TPB = 256;
constexpr int INC_CHUNK = INC_TPB * 8;   // keys per compaction block
constexpr int MERGE_ITEMS = 8;           // outputs per merge thread

__device__ __forceinline__ bool inc_step_sorts(const DevCtl* ctl, int gate) {
    return gate == GATE_AHEAD || (ctl->do_sort && !ctl->aborted);
}
}  // namespace

__global__ __launch_bounds__(INC_TPB) void k_inc_count(const uint32_t* __restrict__ kin,
                                                       const uint32_t* __restrict__ sprev, int N,
                                                       uint32_t* __restrict__ cnt, const DevCtl* __restrict__ ctl,
                                                       int gate) {
    if (!inc_step_sorts(ctl, gate)) return;
    __shared__ uint32_t s_red[INC_TPB / 32];
    const int base = blockIdx.x * INC_CHUNK;
    const int end = min(base + INC_CHUNK, N);
    uint32_t c = 0;
    for (int e = base + threadIdx.x; e < end; e += INC_TPB) c += kin[e] != sprev[e] ? 1u : 0u;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < INC_TPB / 32; ++w) t += s_red[w];
        cnt[blockIdx.x] = t;
    }
}

// One block: block counts -> exclusive offsets; decides the path.
__global__ void k_inc_scan(uint32_t* __restrict__ cnt, int nblocks, int inc_max, DevCtl* __restrict__ ctl,
                           int gate) {
    __shared__ uint32_t s_warp[32];
    __shared__ uint32_t s_carry;
    if (!inc_step_sorts(ctl, gate)) {
        if (threadIdx.x == 0) ctl->inc_on = 0;
        return;
    }
    if (threadIdx.x == 0) s_carry = 0u;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int b0 = 0; b0 < nblocks; b0 += blockDim.x) {
        const int b = b0 + threadIdx.x;
        const uint32_t v = b < nblocks ? cnt[b] : 0u;
        uint32_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) s_warp[warp] = x;
        __syncthreads();
        if (warp == 0) {
            uint32_t w = lane < nw ? s_warp[lane] : 0u;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += y;
            }
            if (lane < nw) s_warp[lane] = w;
        }
        __syncthreads();
        const uint32_t carry = s_carry;
        const uint32_t off = carry + (warp ? s_warp[warp - 1] : 0u) + x - v;
        if (b < nblocks) cnt[b] = off;
        __syncthreads();
        if (threadIdx.x == 0) s_carry = carry + s_warp[nw - 1];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const uint32_t m = s_carry;
        ctl->inc_m = m;
        ctl->inc_on = m <= (uint32_t)inc_max ? 1 : 0;
        ctl->iepoch += 1u;
    }
    for (int i = threadIdx.x; i < MAX_PASSES * 256; i += blockDim.x) (&ctl->ihist[0][0])[i] = 0u;
    if (threadIdx.x < MAX_PASSES) ctl->itile_ctr[threadIdx.x] = 0u;
}

// Split into the unchanged indices (in order) and the changed keys/indices.
__global__ __launch_bounds__(INC_TPB) void k_inc_split(const uint32_t* __restrict__ kin,
                                                       const uint32_t* __restrict__ sprev, int N,
                                                       const uint32_t* __restrict__ off, uint32_t* __restrict__ uidx,
                                                       uint32_t* __restrict__ ukey, uint32_t* __restrict__ ck,
                                                       uint32_t* __restrict__ ci, const DevCtl* __restrict__ ctl,
                                                       int gate) {
    if (!inc_step_sorts(ctl, gate) || !ctl->inc_on) return;
    __shared__ uint32_t s_warp[INC_TPB / 32];
    const int base = blockIdx.x * INC_CHUNK;
    uint32_t oc = off[blockIdx.x];          // changed before this block
    uint32_t ou = (uint32_t)base - oc;      // unchanged before this block
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int r = 0; r < INC_CHUNK; r += INC_TPB) {
        const int e = base + r + threadIdx.x;
        const bool in = e < N;
        const uint32_t k = in ? kin[e] : 0u;
        const bool ch = in && k != sprev[e];
        const unsigned m = __ballot_sync(0xffffffffu, ch);
        if (lane == 0) s_warp[warp] = __popc(m);
        __syncthreads();
        uint32_t before = 0, total = 0;
        for (int w = 0; w < INC_TPB / 32; ++w) {
            const uint32_t c = s_warp[w];
            if (w < warp) before += c;
            total += c;
        }
        const unsigned lt = (1u << lane) - 1u;
        const uint32_t rc = before + __popc(m & lt);                       // changed before e in this round
        const uint32_t ru = (uint32_t)(warp * 32 + lane) - rc;             // unchanged before e in this round
        if (ch) {
            ck[oc + rc] = k;
            ci[oc + rc] = (uint32_t)e;
        } else if (in) {
            uidx[ou + ru] = (uint32_t)e;
            ukey[ou + ru] = k;
        }
        oc += total;
        ou += (uint32_t)min(INC_TPB, max(0, N - (base + r))) - total;
        __syncthreads();
    }
}

// Merge of the unchanged sequence (uidx, keys ukey) and the sorted changed
// sequence (ck, ci) by (key, index): merge path, MERGE_ITEMS outputs per
// thread, staged in shared memory so that the block writes its tile of the
// output coalesced.  The split wrote the unchanged keys beside their indices,
// so a merge-path probe is one load, not a dependent pair.
__device__ __forceinline__ bool key_idx_less(uint32_t ka, uint32_t ia, uint32_t kb, uint32_t ib) {
    return ka < kb || (ka == kb && ia < ib);
}
__global__ __launch_bounds__(INC_TPB) void k_inc_merge(const uint32_t* __restrict__ uidx,
                                                       const uint32_t* __restrict__ ukey,
                                                       const uint32_t* __restrict__ ck,
                                                       const uint32_t* __restrict__ ci, int N,
                                                       uint32_t* __restrict__ skeys, uint32_t* __restrict__ perm,
                                                       const DevCtl* __restrict__ ctl, int gate) {
    if (!inc_step_sorts(ctl, gate) || !ctl->inc_on) return;
    __shared__ uint32_t s_k[INC_TPB * MERGE_ITEMS], s_i[INC_TPB * MERGE_ITEMS];
    const int m = (int)ctl->inc_m, nu = N - m;
    const long long t0 = (long long)blockIdx.x * INC_TPB * MERGE_ITEMS;   // the block's first output
    const long long p0 = t0 + (long long)threadIdx.x * MERGE_ITEMS;
    if (p0 < N) {
        int lo = (int)max(0LL, p0 - nu), hi = (int)min(p0, (long long)m);
        while (lo < hi) {   // how many changed keys come first among the first p0 outputs
            const int mid = (lo + hi) >> 1;
            const long long u = p0 - 1 - mid;
            if (key_idx_less(ck[mid], ci[mid], ukey[u], uidx[u])) lo = mid + 1;
            else hi = mid;
        }
        int b = lo, a = (int)p0 - lo;
        for (int j = 0; j < MERGE_ITEMS && p0 + j < N; ++j) {
            bool take_c = b < m;
            uint32_t ua = 0, ku = 0;
            if (a < nu) {
                ua = uidx[a];
                ku = ukey[a];
                take_c = take_c && key_idx_less(ck[b], ci[b], ku, ua);
            }
            const int o = threadIdx.x * MERGE_ITEMS + j;
            if (take_c) {
                s_k[o] = ck[b];
                s_i[o] = ci[b];
                ++b;
            } else {
                s_k[o] = ku;
                s_i[o] = ua;
                ++a;
            }
        }
    }
    __syncthreads();
    const int nout = (int)min((long long)INC_TPB * MERGE_ITEMS, (long long)N - t0);
    for (int e = threadIdx.x; e < nout; e += INC_TPB) {
        skeys[t0 + e] = s_k[e];
        perm[t0 + e] = s_i[e];
    }
}

void sort_inc_sizes(int N, int* max_keys, int* tiles, int* blocks) {
    *max_keys = N / 8 > 0 ? N / 8 : 1;   // above this share of changed keys the full sort runs
    *tiles = (*max_keys + SORT_TILE - 1) / SORT_TILE;
    *blocks = (N + INC_CHUNK - 1) / INC_CHUNK;
}

void launch_sort_prep(const Phys& P, const Bufs& B, int force, int clear_delta, cudaStream_t s) {
    int blocks = (P.ncell / 2 + TPB - 1) / TPB;
    blocks = blocks < 1 ? 1 : (blocks > 152 * 16 ? 152 * 16 : blocks);
    const int shift = pair_span_shift(P, B);
    const int nspans = shift >= 0 ? (int)(((size_t)1 << P.key_bits) >> shift) : 0;
    k_sort_prep<<<blocks, TPB, 0, s>>>(P, B.range, B.spans, nspans, B.rain_delta, B.ctl, force, clear_delta);
}

void launch_sort(const Phys& P, Bufs& B, int force, cudaStream_t s) {
    if (P.N <= 0) return;
    const bool inc = !force && B.inc_u;
    if (inc) {
        // decide the path: count the changed keys (lane 1 runs when few changed)
        k_inc_count<<<B.inc_blocks, INC_TPB, 0, s>>>(B.kin, B.skeys, P.N, B.inc_cnt, B.ctl, 0);
        k_inc_scan<<<1, 1024, 0, s>>>(B.inc_cnt, B.inc_blocks, B.inc_max, B.ctl, 0);
    }
    // Exactly one of the two sorts does work; the device flag decides.  With
    // both, the full sort runs on the second stream (in a captured step, a
    // graph branch) so that its kernels, which then return at once, are off
    // the incremental sort's path; they share no buffers once the flag is set.
    const bool fork = inc && B.aux;
    cudaStream_t fs = fork ? B.aux : s;
    if (fork) {
        cudaEventRecord(B.ev_fork, s);
        cudaStreamWaitEvent(B.aux, B.ev_fork, 0);
    }
    int hb = (P.N + TPB * 8 - 1) / (TPB * 8);
    hb = hb > 152 * 8 ? 152 * 8 : hb;
    k_hist<<<hb, SORT_TPB, 0, fs>>>(B.kin, P.N, B.npasses, B.ctl, force, 0);
    for (int p = 0; p < B.npasses; ++p) {
        const uint32_t* ki = p == 0 ? B.kin : B.kbuf[(p - 1) & 1];
        const uint32_t* vi = p == 0 ? nullptr : B.vbuf[(p - 1) & 1];
        k_radix_pass<<<B.ntiles, SORT_TPB, 0, fs>>>(ki, vi, B.kbuf[p & 1], B.vbuf[p & 1], B.status, P.N,
                                                    B.ntiles, p, B.ctl, force, 0);
    }
    if (fork) cudaEventRecord(B.ev_join, B.aux);
    if (inc) {
        k_inc_split<<<B.inc_blocks, INC_TPB, 0, s>>>(B.kin, B.skeys, P.N, B.inc_cnt, B.inc_u, B.inc_uk, B.inc_k[0],
                                                     B.inc_i[0] + 0, B.ctl, 0);
        // the changed keys: stable radix sort of (key, index), lane 1
        int ib = (B.inc_max + TPB * 8 - 1) / (TPB * 8);
        ib = ib < 1 ? 1 : (ib > 152 * 8 ? 152 * 8 : ib);
        k_hist<<<ib, SORT_TPB, 0, s>>>(B.inc_k[0], B.inc_max, B.npasses, B.ctl, 0, 1);
        const uint32_t* ki = B.inc_k[0];
        const uint32_t* vi = B.inc_i[0];
        for (int p = 0; p < B.npasses; ++p) {
            uint32_t* ko = B.inc_k[(p + 1) & 1];
            uint32_t* vo = B.inc_i[(p + 1) & 1];
            k_radix_pass<<<B.inc_tiles, SORT_TPB, 0, s>>>(ki, vi, ko, vo, B.inc_status, B.inc_max, B.inc_tiles, p,
                                                          B.ctl, 0, 1);
            ki = ko;
            vi = vo;
        }
        const int mb = (P.N + INC_TPB * MERGE_ITEMS - 1) / (INC_TPB * MERGE_ITEMS);
        k_inc_merge<<<mb, INC_TPB, 0, s>>>(B.inc_u, B.inc_uk, ki, vi, P.N, B.skeys, B.perm, B.ctl, 0);
    }
    if (fork) cudaStreamWaitEvent(s, B.ev_join, 0);
}

// Resets the full sort's histograms and tile counters and opens a new
// look-back epoch, for a sort run ahead (k_sort_prep does it for the step's
// own sort, together with the table clear that must wait for the step's
// pair passes).
__global__ void k_sort_state(DevCtl* __restrict__ ctl) {
    for (int i = threadIdx.x; i < MAX_PASSES * 256; i += blockDim.x) (&ctl->hist[0][0])[i] = 0u;
    if (threadIdx.x < MAX_PASSES) ctl->tile_ctr[threadIdx.x] = 0u;
    if (threadIdx.x == 0) ctl->epoch += 1u;
}

void launch_sort_ahead(const Phys& P, Bufs& B, cudaStream_t s) {
    if (P.N <= 0) return;
    // branch off the caller's stream; the caller's later work does not wait
    // for it until the join at the end
    cudaEventRecord(B.ev_fork2, s);
    cudaStreamWaitEvent(B.aux2, B.ev_fork2, 0);
    cudaStream_t a = B.aux2;
    k_sort_state<<<1, 256, 0, a>>>(B.ctl);
    k_inc_count<<<B.inc_blocks, INC_TPB, 0, a>>>(B.kin, B.skeys, P.N, B.inc_cnt, B.ctl, GATE_AHEAD);
    k_inc_scan<<<1, 1024, 0, a>>>(B.inc_cnt, B.inc_blocks, B.inc_max, B.ctl, GATE_AHEAD);
    // the full sort (when too many keys changed) on a branch of its own; its
    // passes alternate between skeys_ahead and the key buffer that is not
    // skeys, ending in skeys_ahead, so the last applied sort stays intact
    cudaEventRecord(B.ev_fork, a);
    cudaStreamWaitEvent(B.aux, B.ev_fork, 0);
    int hb = (P.N + TPB * 8 - 1) / (TPB * 8);
    hb = hb > 152 * 8 ? 152 * 8 : hb;
    k_hist<<<hb, SORT_TPB, 0, B.aux>>>(B.kin, P.N, B.npasses, B.ctl, GATE_AHEAD, 0);
    uint32_t* kscr = B.kbuf[B.skeys == B.kbuf[0] ? 1 : 0];
    uint32_t* vscr = B.vbuf[B.perm == B.vbuf[0] ? 1 : 0];
    const uint32_t* ki = B.kin;
    const uint32_t* vi = nullptr;
    for (int p = 0; p < B.npasses; ++p) {
        const bool last_parity = ((B.npasses - 1 - p) & 1) == 0;
        uint32_t* ko = last_parity ? B.skeys_ahead : kscr;
        uint32_t* vo = last_parity ? B.perm_ahead : vscr;
        k_radix_pass<<<B.ntiles, SORT_TPB, 0, B.aux>>>(ki, vi, ko, vo, B.status, P.N, B.ntiles, p, B.ctl,
                                                       GATE_AHEAD, 0);
        ki = ko;
        vi = vo;
    }
    cudaEventRecord(B.ev_join, B.aux);
    // the incremental sort
    k_inc_split<<<B.inc_blocks, INC_TPB, 0, a>>>(B.kin, B.skeys, P.N, B.inc_cnt, B.inc_u, B.inc_uk, B.inc_k[0],
                                                 B.inc_i[0], B.ctl, GATE_AHEAD);
    int ib = (B.inc_max + TPB * 8 - 1) / (TPB * 8);
    ib = ib < 1 ? 1 : (ib > 152 * 8 ? 152 * 8 : ib);
    k_hist<<<ib, SORT_TPB, 0, a>>>(B.inc_k[0], B.inc_max, B.npasses, B.ctl, GATE_AHEAD, 1);
    const uint32_t* ik = B.inc_k[0];
    const uint32_t* iv = B.inc_i[0];
    for (int p = 0; p < B.npasses; ++p) {
        uint32_t* ko = B.inc_k[(p + 1) & 1];
        uint32_t* vo = B.inc_i[(p + 1) & 1];
        k_radix_pass<<<B.inc_tiles, SORT_TPB, 0, a>>>(ik, iv, ko, vo, B.inc_status, B.inc_max, B.inc_tiles, p,
                                                      B.ctl, GATE_AHEAD, 1);
        ik = ko;
        iv = vo;
    }
    const int mb = (P.N + INC_TPB * MERGE_ITEMS - 1) / (INC_TPB * MERGE_ITEMS);
    k_inc_merge<<<mb, INC_TPB, 0, a>>>(B.inc_u, B.inc_uk, ik, iv, P.N, B.skeys_ahead, B.perm_ahead, B.ctl,
                                       GATE_AHEAD);
    cudaStreamWaitEvent(a, B.ev_join, 0);
    cudaEventRecord(B.ev_join2, a);
}

}  // namespace asph
