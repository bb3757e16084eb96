// asph_kernels.cu — the particle and cell kernels of one step, for sm_103a.
//
// Step structure (reference order, asph_h100.cu:958-1078) and the fused
// kernels that carry it here:
//   sort      k_sort_prep + k_hist + k_radix_pass x passes   (asph_sort.cu)
//   G         k_gather: gather through the permutation + cell table +
//             [CFL clamp] + half kick + drift + surface flux + next keys
//   D, M      the pair passes, in asph_pairs.cu
#include "asph_device.cuh"
#include "../../include/asph.h"

namespace asph {


// ---------------------------------------------------------------------------
// Initial state (asph_h100.cu:210-227 for the reference lattice).
// ---------------------------------------------------------------------------
struct InitArgs {
    float bx[ASPH_MAX_BUBBLES], by[ASPH_MAX_BUBBLES], bz[ASPH_MAX_BUBBLES], br[ASPH_MAX_BUBBLES],
        ba[ASPH_MAX_BUBBLES];
    int nbub, mode, lnx, lny, lnz;
    float jitter, noise;
    uint32_t seed;
};

__global__ void k_init(const __grid_constant__ Phys P, const __grid_constant__ InitArgs A,
                       float4* __restrict__ pos, float4* __restrict__ vel, float4* __restrict__ thq,
                       float2* __restrict__ rp, float4* __restrict__ acc, float* __restrict__ dthdt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    float x, y, z, th, qv;
    if (A.mode == ASPH_INIT_REFERENCE) {
        const int ix = i % P.nx, iy = (i / P.nx) % P.ny, iz = i / (P.nx * P.ny);
        x = (ix + 0.5f) * P.dx;
        y = (iy + 0.5f) * P.dy;
        z = (iz + 0.5f) * P.dz;
        th = theta_ref(P, z) + A.noise * hash_noise(ix, iy, iz);
        qv = fmaxf(qv_ref(P, z) * (1.0f + 0.02f * hash_noise(ix + 17, iy + 31, iz + 7)), 0.f);
    } else {
        const int ix = i % A.lnx, iy = (i / A.lnx) % A.lny, iz = i / (A.lnx * A.lny);
        // Positions use explicitly rounded float operations (no contraction
        // into FMAs), so that a host restatement in float reproduces them,
        // and with them the Morton keys, bit for bit.  2u - 1 is exact.
        const float sx = P.lx / A.lnx, sy = P.ly / A.lny, sz = P.lz / A.lnz;
        const float jx = __fmul_rn(A.jitter, 2.f * uniform24(A.seed, (uint32_t)i, 0u) - 1.f);
        const float jy = __fmul_rn(A.jitter, 2.f * uniform24(A.seed, (uint32_t)i, 1u) - 1.f);
        const float jz = __fmul_rn(A.jitter, 2.f * uniform24(A.seed, (uint32_t)i, 2u) - 1.f);
        x = __fmul_rn(__fadd_rn((float)ix + 0.5f, jx), sx);
        y = __fmul_rn(__fadd_rn((float)iy + 0.5f, jy), sy);
        z = __fmul_rn(__fadd_rn((float)iz + 0.5f, jz), sz);
        th = theta_ref(P, z);
        for (int b = 0; b < A.nbub; ++b) {
            const float ddx = x - A.bx[b], ddy = y - A.by[b], ddz = z - A.bz[b];
            const float d2 = (ddx * ddx + ddy * ddy + ddz * ddz) / (A.br[b] * A.br[b]);
            th += A.ba[b] * expf(-d2);
        }
        if (A.noise > 0.f) th += A.noise * normal01(A.seed, (uint32_t)i, 3u);
        qv = qv_ref(P, z);
    }
    // The initial density is rho_ref(z).  The reference lattice takes the
    // reference's float evaluation (asph_h100.cu:224).  The config lattice
    // evaluates the sounding in double (asph_h100.cu:136-146) and rounds
    // once: there p' = c_s^2 (rho - rho_ref) of the first density pass is a
    // small residual (the Shepard sum reproduces rho_ref in the interior),
    // and one float ulp of a particle's starting density moves its p' by
    // ~2e-4 Pa, so the start must be the correctly rounded profile.
    float rho0;
    if (A.mode == ASPH_INIT_REFERENCE) {
        rho0 = rho_ref(P, z);
    } else {
        constexpr double G_D = 9.80665, RD_D = 287.05, CP_D = 1004.0, P0_D = 100000.0;
        const double th0 = P.th0, n2 = P.n2, zd = z;
        const double a = G_D * G_D / (CP_D * th0 * n2);
        const double th = th0 * exp(n2 * zd / G_D);
        const double ex = 1.0 - a * (1.0 - exp(-n2 * zd / G_D));
        rho0 = (float)(P0_D * pow(ex, CP_D / RD_D) / (RD_D * th * ex));
    }
    pos[i] = make_float4(x, y, z, rho0);
    vel[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    thq[i] = make_float4(th, qv, 0.f, 0.f);
    rp[i] = make_float2(rho0, 0.f);
    acc[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    dthdt[i] = 0.f;
}

// Keys of the current positions (asph_h100.cu:229-240); used after init
// and set_state.  Inside a step the gather pass writes the keys.
__global__ void k_keys(const __grid_constant__ Phys P, const float4* __restrict__ pos,
                       const float2* __restrict__ rp, float4* __restrict__ pos_out,
                       uint32_t* __restrict__ keys) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    float4 p = pos[i];
    keys[i] = key_of(P, p.x, p.y, p.z);
    if (pos_out) { p.w = rp[i].x; pos_out[i] = p; }
}

// ---------------------------------------------------------------------------
// G: gather (asph_h100.cu:245-256) + cell table (asph_h100.cu:258-278) +
// CFL clamp (asph_h100.cu:669-675) + kick (535-544) + drift (545-561) +
// surface flux (606-626) + keys of the new positions for the next sort.
// ---------------------------------------------------------------------------
struct GArgs {
    const float4 *pos_src, *vel_src, *thq_src;
    float4 *pos_dst, *vel_dst, *thq_dst;
    const float2* rp;
    const float4* acc;
    const uint32_t *perm, *skeys;
    uint32_t *perm_out, *skeys_out;   // non-NULL: the sort was run ahead; copy it into the last-sort buffers
    int2* range;
    int2* spans;         // brick spans of the density pass by Morton id (NULL: global path) ...
    int span_shift;      // ... a brick's id is its keys >> span_shift
    uint8_t* surf;
    uint32_t* kin;
    const float4* src;   // source-term tendencies (NULL: hook off) ...
    float4* src_tmp;     // ... follow their particles through the gather
    DevCtl* ctl;
};

__global__ __launch_bounds__(TPB) void k_gather(const __grid_constant__ Phys P, const __grid_constant__ GArgs A,
                                                int mode) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    DevCtl* ctl = A.ctl;
    const bool aborted = ctl->aborted != 0;
    const bool sorted = (mode & G_SORTED) && (((mode & G_FORCE) != 0) || (ctl->do_sort && !aborted));
    const bool integ = (mode & G_INTEGRATE) && !aborted;
    __shared__ float s_Ts, s_qs, s_dt;
    __shared__ int s_clamp;
    if (threadIdx.x == 0) {
        float Ts, qs;
        surface_targets(P, ctl->simt, Ts, qs);
        s_Ts = Ts; s_qs = qs; s_dt = ctl->dt; s_clamp = ctl->clamp_pending;
    }
    __syncthreads();
    if (i < P.N) {
        const int s = sorted ? (int)A.perm[i] : i;
        float4 p = A.pos_src[s];
        float4 v = A.vel_src[s];
        float4 t = A.thq_src[s];
        const float rho = A.rp[s].x;
        bool surf;
        if (sorted) {
            // keys decode to cells inside the grid; the bounds test only guards
            // against a sort that gave up (error word set)
            const uint32_t kc = A.skeys[i];
            if (A.skeys_out) {
                A.skeys_out[i] = kc;
                A.perm_out[i] = (uint32_t)s;
            }
            const int c = cid_of_key(P, kc);
            const bool cin = (unsigned)c < (unsigned)P.ncell;
            if (i == 0) {
                if (cin) A.range[c].x = 0;
            } else {
                const uint32_t kp = A.skeys[i - 1];
                if (kc != kp) {
                    const int cp = cid_of_key(P, kp);
                    if (cin) A.range[c].x = i;
                    if ((unsigned)cp < (unsigned)P.ncell) A.range[cp].y = i;
                }
            }
            if (i == P.N - 1 && cin) A.range[c].y = P.N;
            if (A.spans) {   // the same boundaries at brick granularity
                const uint32_t bc = kc >> A.span_shift;
                if (i == 0) {
                    A.spans[bc].x = 0;
                } else {
                    const uint32_t bp = A.skeys[i - 1] >> A.span_shift;
                    if (bc != bp) {
                        A.spans[bc].x = i;
                        A.spans[bp].y = i;
                    }
                }
                if (i == P.N - 1) A.spans[bc].y = P.N;
            }
            surf = ((int)__fmul_rn(p.z, P.inv_dz)) == 0;
            A.surf[i] = surf ? 1 : 0;
            const unsigned m = __ballot_sync(__activemask(), surf);
            if (surf && (threadIdx.x & 31) == __ffs(m) - 1) atomicAdd((int*)&ctl->surf_count, __popc(m));
        } else {
            surf = A.surf[i] != 0;
        }
        if (integ) {
            const float dt = s_dt;
            if (s_clamp) {
                const float vmax = 0.5f * P.cs;
                const float s2 = v.x * v.x + v.y * v.y + v.z * v.z;
                if (s2 > vmax * vmax) {
                    const float f = vmax / sqrtf(s2);
                    v.x *= f; v.y *= f; v.z *= f;
                }
            }
            const float4 a = A.acc[P.permute_acc ? s : i];
            const float hdt = 0.5f * dt;
            v.x += a.x * hdt; v.y += a.y * hdt; v.z += a.z * hdt;
            p.x += v.x * dt; p.y += v.y * dt; p.z += v.z * dt;
            for (int k = 0; k < 64 && p.x < 0.f; ++k) p.x += P.lx;
            for (int k = 0; k < 64 && p.x >= P.lx; ++k) p.x -= P.lx;
            for (int k = 0; k < 64 && p.y < 0.f; ++k) p.y += P.ly;
            for (int k = 0; k < 64 && p.y >= P.ly; ++k) p.y -= P.ly;
            if (p.z < 0.f) { p.z = -p.z; v.z = fabsf(v.z); }
            if (p.z > P.lz) { p.z = 2.f * P.lz - p.z; v.z = -fabsf(v.z); }
            if (P.surface_flux && surf && p.z < P.dz) {
                const float Pi = powf(fmaxf(snd_eval(P.snd_p, P.snd_n, p.z).v(), 1.f) / P0, R_D / CP);
                const float Ta = t.x * Pi;
                t.x += P.c_h * P.v_bg * (s_Ts - Ta) * dt / P.dz;
                t.y += P.beta_moist * P.c_e * P.v_bg * (s_qs - t.y) * dt / P.dz;
                t.x = fminf(fmaxf(t.x, 100.f), P.theta_cap);
                t.y = fminf(fmaxf(t.y, 0.f), P.qv_cap);
            }
            if (!(isfinite(p.x) && isfinite(p.y) && isfinite(p.z) && isfinite(v.x) && isfinite(v.y) &&
                  isfinite(v.z)))
                stop_run(ctl, ASPH_ERR_NONFINITE);
        }
        A.pos_dst[i] = make_float4(p.x, p.y, p.z, rho);
        A.vel_dst[i] = v;
        A.thq_dst[i] = t;
        if (A.src) A.src_tmp[i] = A.src[s];
        A.kin[i] = key_of(P, p.x, p.y, p.z);
    }
}

// Standalone rain pass (granular API).
__global__ void k_rain(const __grid_constant__ Phys P, const float* __restrict__ rin, const float* __restrict__ delta,
                       float* __restrict__ rout, float* __restrict__ precip, const DevCtl* __restrict__ ctl) {
    const int cid = blockIdx.x * blockDim.x + threadIdx.x;
    if (ctl->aborted || cid >= P.ncell) return;
    rain_cell(P, cid, ctl->dt, rin, delta, rout, precip);
}

// Velocity maxima (asph_h100.cu:631-647) + control (granular API).
__global__ void k_maxvel(const __grid_constant__ Phys P, const float4* __restrict__ vel, DevCtl* __restrict__ ctl) {
    float mx = 0.f, my = 0.f, mz = 0.f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.N; i += gridDim.x * blockDim.x) {
        const float4 v = vel[i];
        mx = fmaxf(mx, fabsf(v.x)); my = fmaxf(my, fabsf(v.y)); mz = fmaxf(mz, fabsf(v.z));
    }
    mx = warp_max(mx); my = warp_max(my); mz = warp_max(mz);
    if ((threadIdx.x & 31) == 0) {
        atomicMax(&ctl->gmax[0], __float_as_uint(mx));
        atomicMax(&ctl->gmax[1], __float_as_uint(my));
        atomicMax(&ctl->gmax[2], __float_as_uint(mz));
    }
}
__global__ void k_cfl_ctl(const __grid_constant__ Phys P, DevCtl* __restrict__ ctl) {
    if (threadIdx.x == 0 && !ctl->aborted) cfl_control(P, ctl);
}

// Emergency clamp |v| <= 0.5 c_s when a CFL trip is pending
// (asph_h100.cu:669-675, 1067-1068).
__global__ void k_clamp(const __grid_constant__ Phys P, float4* __restrict__ vel, DevCtl* __restrict__ ctl) {
    if (!ctl->clamp_pending) return;
    const float vmax = 0.5f * P.cs;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.N; i += gridDim.x * blockDim.x) {
        float4 v = vel[i];
        const float s2 = v.x * v.x + v.y * v.y + v.z * v.z;
        if (s2 > vmax * vmax) {
            const float f = vmax / sqrtf(s2);
            v.x *= f; v.y *= f; v.z *= f;
            vel[i] = v;
        }
    }
}
__global__ void k_clamp_done(DevCtl* ctl) { ctl->clamp_pending = 0; }

// ---------------------------------------------------------------------------
// FP64 conservation audit (asph_h100.cu:650-668), deterministic two-stage.
// Every per-particle term is formed in double from the float32 state,
// including the Exner function of the reference sounding, so that the six
// totals are FP64 sums of FP64 terms.
// ---------------------------------------------------------------------------
__global__ void k_audit_partial(const __grid_constant__ Phys P, const __grid_constant__ AuditConst A,
                                const float4* __restrict__ pos, const float4* __restrict__ vel,
                                const float4* __restrict__ thq, double* __restrict__ partial) {
    constexpr double G_D = 9.80665, RD_D = 287.05, CP_D = 1004.0, P0_D = 100000.0;
    double a[5] = {0, 0, 0, 0, 0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.N; i += gridDim.x * blockDim.x) {
        const float4 p = pos[i], v = vel[i], t = thq[i];
        const double ex = 1.0 - A.a_exner * (1.0 - exp(-A.n2 * (double)p.z / G_D));   // asph_h100.cu:139-142
        const double pr = P0_D * pow(ex, CP_D / RD_D);                                 // asph_h100.cu:143-145
        const double Pi = pow(fmax(pr, 1.0) / P0_D, RD_D / CP_D);
        a[0] += 0.5 * ((double)v.x * v.x + (double)v.y * v.y + (double)v.z * v.z);
        a[1] += G_D * p.z;
        a[2] += CP_D * t.x * Pi;
        a[3] += (double)t.y + (double)t.z;
        a[4] += (double)v.z;
    }
    __shared__ double s[5][TPB];
    for (int c = 0; c < 5; ++c) s[c][threadIdx.x] = a[c];
    __syncthreads();
    for (int o = TPB / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o)
            for (int c = 0; c < 5; ++c) s[c][threadIdx.x] += s[c][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x < 5) partial[blockIdx.x * 5 + threadIdx.x] = s[threadIdx.x][0];
}
__global__ void k_audit_final(const __grid_constant__ AuditConst A, const double* __restrict__ partial, int nblk,
                              double* __restrict__ out) {
    if (threadIdx.x < 5) {
        double acc = 0.0;
        for (int b = 0; b < nblk; ++b) acc += partial[b * 5 + threadIdx.x];
        out[threadIdx.x] = acc * A.pmass;
    }
    if (threadIdx.x == 5) out[5] = A.pmass * (double)A.N;
}

// Surface-layer flags of the current order (exported surface list).
__global__ void k_surf_flags(const __grid_constant__ Phys P, const uint8_t* __restrict__ surf, uint8_t* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < P.N) out[i] = surf[i];
}

// ---------------------------------------------------------------------------
// Coarse dump + column diagnostics (asph_h100.cu:680-723).
// ---------------------------------------------------------------------------
__global__ void k_coarse(const __grid_constant__ Phys P, const int2* __restrict__ range, const float4* __restrict__ vel,
                         const float4* __restrict__ thq, float* __restrict__ out, int sx, int sy, int sz, int cx,
                         int cy, int cz) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= cx * cy * cz) return;
    const int cxx = idx % cx, cyy = (idx / cx) % cy, czz = idx / (cx * cy);
    float a[6] = {0, 0, 0, 0, 0, 0};
    int n = 0;
    const int ix1 = min((cxx + 1) * sx, P.nx), iy1 = min((cyy + 1) * sy, P.ny), iz1 = min((czz + 1) * sz, P.nz);
    for (int iz = czz * sz; iz < iz1; ++iz)
        for (int iy = cyy * sy; iy < iy1; ++iy)
            for (int ix = cxx * sx; ix < ix1; ++ix) {
                const int2 rg = range[(size_t)(iz * P.ny + iy) * P.nx + ix];
                for (int j = rg.x; j < rg.y; ++j) {
                    const float4 t = thq[j], v = vel[j];
                    a[0] += t.x; a[1] += t.y; a[2] += t.z;
                    a[3] += v.x; a[4] += v.y; a[5] += v.z;
                    n++;
                }
            }
    const float inv = n ? 1.f / (float)n : 0.f;
    for (int c = 0; c < 6; ++c) out[(size_t)idx * 6 + c] = a[c] * inv;
}
__global__ void k_coldiag(const __grid_constant__ Phys P, const int2* __restrict__ range, const float4* __restrict__ thq,
                          const float4* __restrict__ vel, float4* __restrict__ coldiag) {
    const int col = blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= P.nxy) return;
    const int iy = col / P.nx, ix = col % P.nx;
    float th = 0.f, qv = 0.f, qlmax = 0.f, wmax = 0.f;
    int n = 0;
    for (int k = 0; k < P.nz; ++k) {
        const int2 rg = range[(size_t)(k * P.ny + iy) * P.nx + ix];
        for (int j = rg.x; j < rg.y; ++j) {
            th += thq[j].x; qv += thq[j].y;
            qlmax = fmaxf(qlmax, thq[j].z);
            wmax = fmaxf(wmax, fabsf(vel[j].z));
            n++;
        }
    }
    if (n) { const float inv = 1.f / (float)n; th *= inv; qv *= inv; }
    coldiag[col] = make_float4(th, qv, qlmax, wmax);
}

// ---------------------------------------------------------------------------
// launch functions
// ---------------------------------------------------------------------------
static inline int blocks_for(int n) { return n <= 0 ? 1 : (n + TPB - 1) / TPB; }

void launch_init(const Phys& P, const Bufs& B, const float* bub, int nbub, int init_mode, int lat_nx, int lat_ny,
                 int lat_nz, float jitter, uint32_t seed, float noise, cudaStream_t s) {
    InitArgs A{};
    A.nbub = nbub;
    for (int b = 0; b < nbub && b < ASPH_MAX_BUBBLES; ++b) {
        A.bx[b] = bub[5 * b + 0]; A.by[b] = bub[5 * b + 1]; A.bz[b] = bub[5 * b + 2];
        A.br[b] = bub[5 * b + 3]; A.ba[b] = bub[5 * b + 4];
    }
    A.mode = init_mode; A.lnx = lat_nx; A.lny = lat_ny; A.lnz = lat_nz;
    A.jitter = jitter; A.noise = noise; A.seed = seed;
    k_init<<<blocks_for(P.N), TPB, 0, s>>>(P, A, B.pos[B.pc], B.vel[B.vc], B.thq[B.qc], B.rp, B.acc, B.dthdt);
}

void launch_keys(const Phys& P, const Bufs& B, cudaStream_t s) {
    k_keys<<<blocks_for(P.N), TPB, 0, s>>>(P, B.pos[B.pc], B.rp, nullptr, B.kin);
}

void launch_gather(const Phys& P, const Bufs& B, int mode, cudaStream_t s) {
    GArgs A;
    A.pos_src = B.pos[B.pc]; A.vel_src = B.vel[B.vc]; A.thq_src = B.thq[B.qc];
    A.pos_dst = B.pos[1 - B.pc]; A.vel_dst = B.vel[1 - B.vc]; A.thq_dst = B.thq[1 - B.qc];
    A.rp = B.rp; A.acc = B.acc; A.range = B.range;
    if (mode & G_AHEAD) {
        A.perm = B.perm_ahead; A.skeys = B.skeys_ahead; A.perm_out = B.perm; A.skeys_out = B.skeys;
    } else {
        A.perm = B.perm; A.skeys = B.skeys; A.perm_out = nullptr; A.skeys_out = nullptr;
    }
    A.span_shift = pair_span_shift(P, B);
    A.spans = A.span_shift >= 0 ? B.spans : nullptr;
    A.surf = B.surf; A.kin = B.kin; A.ctl = B.ctl;
    A.src = B.src; A.src_tmp = B.src_tmp;
    k_gather<<<blocks_for(P.N), TPB, 0, s>>>(P, A, mode);
}

void launch_rain(const Phys& P, const Bufs& B, cudaStream_t s) {
    k_rain<<<blocks_for(P.ncell), TPB, 0, s>>>(P, B.rain[B.rc], (P.accretion || P.rain_evap) ? B.rain_delta : nullptr,
                                               B.rain[1 - B.rc], B.precip, B.ctl);
}

void launch_cfl(const Phys& P, const Bufs& B, cudaStream_t s) {
    k_maxvel<<<152 * 4, TPB, 0, s>>>(P, B.vel[B.vc], B.ctl);
    k_cfl_ctl<<<1, 32, 0, s>>>(P, B.ctl);
}

void launch_clamp(const Phys& P, const Bufs& B, cudaStream_t s) {
    k_clamp<<<152 * 4, TPB, 0, s>>>(P, B.vel[B.vc], B.ctl);
    k_clamp_done<<<1, 1, 0, s>>>(B.ctl);
}

void launch_audit(const Phys& P, const AuditConst& A, const Bufs& B, double* partial, int nblk, double* out,
                  cudaStream_t s) {
    k_audit_partial<<<nblk, TPB, 0, s>>>(P, A, B.pos[B.pc], B.vel[B.vc], B.thq[B.qc], partial);
    k_audit_final<<<1, 32, 0, s>>>(A, partial, nblk, out);
}

void launch_surf_flags(const Phys& P, const Bufs& B, uint8_t* flags, cudaStream_t s) {
    k_surf_flags<<<blocks_for(P.N), TPB, 0, s>>>(P, B.surf, flags);
}

void launch_coarse(const Phys& P, const Bufs& B, float* out, int sx, int sy, int sz, int cx, int cy, int cz,
                   float4* coldiag, cudaStream_t s) {
    k_coarse<<<blocks_for(cx * cy * cz), TPB, 0, s>>>(P, B.range, B.vel[B.vc], B.thq[B.qc], out, sx, sy, sz, cx, cy, cz);
    k_coldiag<<<blocks_for(P.nxy), TPB, 0, s>>>(P, B.range, B.thq[B.qc], B.vel[B.vc], coldiag);
}

}  // namespace asph
