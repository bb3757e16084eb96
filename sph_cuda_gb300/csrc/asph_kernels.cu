// asph_kernels.cu — the particle and cell kernels of one step, for sm_103a.
//
// Step structure (reference order, asph_h100.cu:958-1078) and the fused
// kernels that carry it here:
//   sort      k_sort_prep + k_hist + k_radix_pass x passes   (asph_sort.cu)
//   G         k_gather: gather through the permutation + cell table +
//             [CFL clamp] + half kick + drift + surface flux + next keys
//   D         k_density: summation density + EOS + saturation adjustment
//             + autoconversion (+ accretion, rain evaporation)
//   M         k_momentum: pressure gradient + viscosity + buoyancy +
//             heating, then theta update, second half kick, sponge,
//             velocity maxima; extra blocks advect the rain grid; the last
//             block to finish runs the closed-loop CFL control.
#include "asph_internal.cuh"
#include "../../include/asph.h"

namespace asph {

namespace {

__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Surface skin temperature ramp (asph_h100.cu:989-992).
__device__ __forceinline__ void surface_targets(const Phys& P, double simt, float& Ts, float& qs_sfc) {
    float r = fminf(fmaxf((float)simt / P.ramp, 0.f), 1.f);
    float sw = r * r * (3.f - 2.f * r);
    Ts = P.th0 + P.dts_skin * sw;
    qs_sfc = qsat(Ts, pres_ref(P, 0.f));
}

// Closed-loop CFL control (asph_h100.cu:1040-1078), run by one thread.
__device__ void cfl_control(const Phys& P, DevCtl* ctl) {
    const float ux = __uint_as_float(atomicOr(&ctl->gmax[0], 0u));
    const float uy = __uint_as_float(atomicOr(&ctl->gmax[1], 0u));
    const float uz = __uint_as_float(atomicOr(&ctl->gmax[2], 0u));
    ctl->gmax[0] = ctl->gmax[1] = ctl->gmax[2] = 0u;
    ctl->umax = ux; ctl->vmax = uy; ctl->wmax = uz;
    const float dt = ctl->dt;
    ctl->simt += (double)dt;
    ctl->since_sort = (ctl->sorted_this_step ? 0.0 : ctl->since_sort) + (double)dt;
    ctl->sorted_this_step = 0;
    ctl->step += 1;
    ctl->clamp_pending = 0;

    const float dt_required =
        P.cfl * fminf(fminf(P.dx / (P.cs + ux), P.dy / (P.cs + uy)), P.dz / (P.cs + uz)) * 0.90f;
    ctl->dt_required = dt_required;
    float adopt = fminf(P.dt_cap, dt_required);
    if (adopt < P.dt_floor) {
        ctl->trips += 1;
        if (P.strict_cfl || ctl->trips > P.max_trip) {
            ctl->aborted = 1;
            ctl->do_sort = 0;
            return;
        }
        ctl->clamp_pending = 1;
        adopt = fmaxf(P.dt_floor, P.cfl * fminf(fminf(P.dx, P.dy), P.dz) / (1.5f * P.cs) * 0.90f);
    } else if (adopt < 0.98f * dt) {
        ctl->trips = 0;
    }
    const float dt_next = P.adaptive_dt ? adopt : dt;
    ctl->dt = dt_next;
    const float dz_move = 0.3f * P.dz / fmaxf(uz, 0.5f);
    const float dh_move = 0.3f * P.dx / fmaxf(fmaxf(ux, uy), 0.5f);
    ctl->sort_dt = fminf(fmaxf(fminf(dz_move, dh_move), dt_next), 15.0f);
    if (P.sort_every > 0)
        ctl->do_sort = (ctl->step % P.sort_every) == 0;
    else
        ctl->do_sort = ctl->since_sort >= (double)ctl->sort_dt;
}

}  // namespace

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
        const float sx = P.lx / A.lnx, sy = P.ly / A.lny, sz = P.lz / A.lnz;
        const float jx = A.jitter * (2.f * uniform24(A.seed, (uint32_t)i, 0u) - 1.f);
        const float jy = A.jitter * (2.f * uniform24(A.seed, (uint32_t)i, 1u) - 1.f);
        const float jz = A.jitter * (2.f * uniform24(A.seed, (uint32_t)i, 2u) - 1.f);
        x = (ix + 0.5f + jx) * sx;
        y = (iy + 0.5f + jy) * sy;
        z = (iz + 0.5f + jz) * sz;
        th = theta_ref(P, z);
        for (int b = 0; b < A.nbub; ++b) {
            const float ddx = x - A.bx[b], ddy = y - A.by[b], ddz = z - A.bz[b];
            const float d2 = (ddx * ddx + ddy * ddy + ddz * ddz) / (A.br[b] * A.br[b]);
            th += A.ba[b] * expf(-d2);
        }
        if (A.noise > 0.f) th += A.noise * normal01(A.seed, (uint32_t)i, 3u);
        qv = qv_ref(P, z);
    }
    pos[i] = make_float4(x, y, z, rho_ref(P, z));
    vel[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    thq[i] = make_float4(th, qv, 0.f, 0.f);
    rp[i] = make_float2(rho_ref(P, z), 0.f);
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
    int2* range;
    uint8_t* surf;
    uint32_t* kin;
    DevCtl* ctl;
};

__global__ __launch_bounds__(TPB) void k_gather(const __grid_constant__ Phys P, const __grid_constant__ GArgs A,
                                                int mode) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const DevCtl* ctl = A.ctl;
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
    if (i >= P.N) return;

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
        surf = ((int)__fmul_rn(p.z, P.inv_dz)) == 0;
        A.surf[i] = surf ? 1 : 0;
        const unsigned m = __ballot_sync(__activemask(), surf);
        if (surf && (threadIdx.x & 31) == __ffs(m) - 1) atomicAdd((int*)&A.ctl->surf_count, __popc(m));
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
            const float Pi = powf(fmaxf(pres_ref(P, p.z), 1.f) / P0, R_D / CP);
            const float Ta = t.x * Pi;
            t.x += P.c_h * P.v_bg * (s_Ts - Ta) * dt / P.dz;
            t.y += P.beta_moist * P.c_e * P.v_bg * (s_qs - t.y) * dt / P.dz;
            t.x = fminf(fmaxf(t.x, 100.f), P.theta_cap);
            t.y = fminf(fmaxf(t.y, 0.f), P.qv_cap);
        }
    }
    A.pos_dst[i] = make_float4(p.x, p.y, p.z, rho);
    A.vel_dst[i] = v;
    A.thq_dst[i] = t;
    A.kin[i] = key_of(P, p.x, p.y, p.z);
}

// ---------------------------------------------------------------------------
// D: summation density with lagged Shepard normalisation
// (asph_h100.cu:286-333) + EOS / saturation adjustment / autoconversion
// (asph_h100.cu:340-402) + Kessler accretion and rain evaporation.
// ---------------------------------------------------------------------------
struct DArgs {
    const float4* pos;      // x, y, z, rho_old
    const int2* range;
    float4* thq;
    float2* rp;             // out: rho_new, p'
    const float* rain_cur;  // read for accretion / evaporation
    float* rain_dep;        // deposits (rain_cur itself when nothing reads it)
    DevCtl* ctl;
};

__global__ __launch_bounds__(TPB) void k_density(const __grid_constant__ Phys P, const __grid_constant__ DArgs A) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (A.ctl->aborted) return;
    if (i >= P.N) return;
    const float dt = A.ctl->dt;
    const float4 pi = A.pos[i];
    const int ix = cell_ix(pi.x, P.inv_dx, P.nx);
    const int iy = cell_ix(pi.y, P.inv_dy, P.ny);
    const int iz = cell_ix(pi.z, P.inv_dz, P.nz);
    const int z0 = max(iz - STENCIL, 0), z1 = min(iz + STENCIL, P.nz - 1);

    float S1 = 0.f, S2 = 0.f;
    for (int jz = z0; jz <= z1; ++jz) {
        for (int jy = iy - STENCIL; jy <= iy + STENCIL; ++jy) {
            const int cy = jy < 0 ? jy + P.ny : (jy >= P.ny ? jy - P.ny : jy);
            const int2* row = A.range + (size_t)(jz * P.ny + cy) * P.nx;
            for (int jx = ix - STENCIL; jx <= ix + STENCIL; ++jx) {
                const int cx = jx < 0 ? jx + P.nx : (jx >= P.nx ? jx - P.nx : jx);
                const int2 rg = row[cx];
                for (int j = rg.x; j < rg.y; ++j) {
                    const float4 pj = A.pos[j];
                    const float dx = (pi.x - pj.x) * P.inv_dx;
                    const float dy = (pi.y - pj.y) * P.inv_dy;
                    const float dz = (pi.z - pj.z) * P.inv_dz;
                    const float r2 = dx * dx + dy * dy + dz * dz;
                    if (r2 < 4.0f) {
                        const float W = w3(sqrtf(r2));
                        S1 += W;
                        S2 += W / fmaxf(pj.w, 1e-3f);
                    }
                }
            }
        }
    }
    const float z = pi.z;
    const float rref = rho_ref(P, z);
    const float rr = S2 > 1e-20f ? S1 / S2 : rref;
    const float rho = fminf(fmaxf(rr, 0.5f * rref), 2.0f * rref);

    // --- EOS (asph_h100.cu:352-361)
    const float r = fmaxf(rho, 1e-3f);
    float dd = r - rref;
    dd = fminf(fmaxf(dd, -0.3f * rref), 0.3f * rref);
    const float ppr = P.cs * P.cs * dd;
    const float pfl = fmaxf(pres_ref(P, z) + ppr, 1.0f);
    const float Pi = powf(pfl / P0, R_D / CP);

    float4 t = A.thq[i];
    float th = t.x, qv = t.y, qc = t.z;
    float T = th * Pi;
    const float qs = qsat(T, pfl);
    // --- saturation adjustment, 3 Newton iterations (asph_h100.cu:370-385)
    if (qv > qs || qc > 0.f) {
        float dqc = 0.f;
        for (int it = 0; it < 3; ++it) {
            const float Tn = T + (L_V / CP) * dqc;
            const float esn = esat(Tn);
            const float qsn = qsat(Tn, pfl);
            const float f = qv - dqc - qsn;
            const float fp = -1.f - dqsdT(Tn, esn, pfl) * (L_V / CP);
            dqc -= f / fp;
            dqc = fminf(dqc, qv);
            dqc = fmaxf(dqc, -qc);
        }
        qv -= dqc;
        qc += dqc;
        th += L_V * dqc / (CP * Pi);
        T += (L_V / CP) * dqc;
    }
    // --- autoconversion into the rain grid (asph_h100.cu:389-394)
    float dep = 0.f;   // kg/kg moved from the particle into the rain grid
    if (qc > P.qc_auto) {
        const float dqr = (qc - P.qc_auto) * (1.f - expf(-P.rate_auto * dt));
        qc -= dqr;
        dep += dqr;
    }
    const int cid = (iz * P.ny + iy) * P.nx + ix;
    if (P.accretion || P.rain_evap) {
        // Kessler warm rain: rain is Eulerian per cell, qr = M_rain / (rho V_cell).
        const float qr = fmaxf(A.rain_cur[cid], 0.f) / (r * P.v_cell);
        if (P.accretion && qc > 0.f && qr > 0.f) {
            // accretion  dqc/dt = -k qc qr^0.875
            const float dqa = fminf(qc, dt * P.k_accr * qc * powf(qr, 0.875f));
            qc -= dqa;
            dep += dqa;
        }
        if (P.rain_evap && qr > 0.f) {
            // rain evaporation in sub-saturated air (rho in g/cm^3, p in hPa)
            const float qvs = qsat(T, pfl);
            if (qv < qvs && qvs > 0.f) {
                const float rq = 1e-3f * r * qr;
                const float C = 1.6f + 124.9f * powf(rq, 0.2046f);
                const float er = (1.f - qv / qvs) * C * powf(rq, 0.525f) /
                                 (1e-3f * r * (5.4e5f + 2.55e6f / (0.01f * pfl * qvs)));
                const float dqe = fminf(qr, fminf(dt * er, qvs - qv));
                qv += dqe;
                th -= L_V * dqe / (CP * Pi);
                dep -= dqe;
            }
        }
    }
    if (dep != 0.f) atomicAdd(&A.rain_dep[cid], dep * P.pmass);

    th = fminf(fmaxf(th, 100.0f), P.theta_cap);
    qv = fminf(fmaxf(qv, 0.0f), P.qv_cap);
    qc = fmaxf(qc, 0.0f);
    A.thq[i] = make_float4(th, qv, qc, t.w);
    A.rp[i] = make_float2(rho, ppr);
}

// ---------------------------------------------------------------------------
// Rain sedimentation (asph_h100.cu:577-599) for one cell.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void rain_cell(const Phys& P, int cid, float dt, const float* __restrict__ rin,
                                          const float* __restrict__ delta, float* __restrict__ rout,
                                          float* __restrict__ precip) {
    const int ix = cid % P.nx, iy = (cid / P.nx) % P.ny, iz = cid / P.nxy;
    float cur = rin[cid];
    if (delta) cur = fmaxf(cur + delta[cid], 0.f);
    float frac = P.v_rain * dt * P.inv_dz;
    if (frac > 1.f) frac = 1.f;
    const float outMass = cur * frac;
    float inMass = 0.f;
    if (iz < P.nz - 1) {
        float above = rin[cid + P.nxy];
        if (delta) above = fmaxf(above + delta[cid + P.nxy], 0.f);
        inMass = above * frac;
    }
    rout[cid] = cur - outMass + inMass;
    if (iz == 0) atomicAdd(&precip[iy * P.nx + ix], outMass / (P.dx * P.dy));
}

// ---------------------------------------------------------------------------
// M: momentum (asph_h100.cu:415-511) + theta update (562-571) + kick
// (535-544) + sponge (518-530) + velocity maxima (631-647); appended
// blocks advect rain (577-599); last block: CFL control (1040-1078).
// ---------------------------------------------------------------------------
struct MArgs {
    const float4* pos;     // x, y, z, -
    const float4* vel;     // velocities after the first half kick
    float4* thq;
    const float2* rp;      // rho, p'
    const int2* range;
    float4* acc;
    float* dthdt;
    float4* vel_out;       // velocities after the second half kick
    const float* rain_in;
    const float* rain_delta;
    float* rain_out;
    float* precip;
    DevCtl* ctl;
    int part_blocks;
};

__global__ __launch_bounds__(TPB) void k_momentum(const __grid_constant__ Phys P, const __grid_constant__ MArgs A,
                                                  int mode) {
    DevCtl* ctl = A.ctl;
    const bool aborted = ctl->aborted != 0;
    __shared__ float s_max[3][TPB / 32];
    __shared__ bool s_last;
    const float dt = ctl->dt;
    float mx = 0.f, my = 0.f, mz = 0.f;

    if ((int)blockIdx.x >= A.part_blocks) {
        // rain sedimentation blocks
        if (!aborted) {
            const int cid = (blockIdx.x - A.part_blocks) * blockDim.x + threadIdx.x;
            if (cid < P.ncell) rain_cell(P, cid, dt, A.rain_in, A.rain_delta, A.rain_out, A.precip);
        }
    } else {
        const int i = blockIdx.x * blockDim.x + threadIdx.x;
        if (i < P.N) {
            if (aborted) {
                if (mode & M_INTEGRATE) A.vel_out[i] = A.vel[i];
            } else {
                const float4 pi = A.pos[i], vi = A.vel[i];
                float4 ti = A.thq[i];
                const float2 rpi = A.rp[i];
                const int ix = cell_ix(pi.x, P.inv_dx, P.nx);
                const int iy = cell_ix(pi.y, P.inv_dy, P.ny);
                const int iz = cell_ix(pi.z, P.inv_dz, P.nz);
                const int z0 = max(iz - STENCIL, 0), z1 = min(iz + STENCIL, P.nz - 1);
                const float rhoi = fmaxf(rpi.x, 1e-3f);
                const float pri = rpi.y;
                float ax = 0.f, ay = 0.f, az = 0.f, avx = 0.f, avy = 0.f, avz = 0.f;
                for (int jz = z0; jz <= z1; ++jz) {
                    for (int jy = iy - STENCIL; jy <= iy + STENCIL; ++jy) {
                        const int cy = jy < 0 ? jy + P.ny : (jy >= P.ny ? jy - P.ny : jy);
                        const int2* row = A.range + (size_t)(jz * P.ny + cy) * P.nx;
                        for (int jx = ix - STENCIL; jx <= ix + STENCIL; ++jx) {
                            const int cx = jx < 0 ? jx + P.nx : (jx >= P.nx ? jx - P.nx : jx);
                            const int2 rg = row[cx];
                            for (int j = rg.x; j < rg.y; ++j) {
                                if (j == i) continue;
                                const float4 pj = A.pos[j];
                                const float rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z;
                                const float dxt = rx * P.inv_dx, dyt = ry * P.inv_dy, dzt = rz * P.inv_dz;
                                const float r2t = dxt * dxt + dyt * dyt + dzt * dzt;
                                if (r2t >= 4.0f || r2t < 1e-12f) continue;
                                const float q = sqrtf(r2t);
                                const float k = dw3(q) / q;
                                const float gx = k * dxt * P.inv_dx;
                                const float gy = k * dyt * P.inv_dy;
                                const float gz = k * dzt * P.inv_dz;
                                const float2 rpj = A.rp[j];
                                const float rhoj = fmaxf(rpj.x, 1e-3f);
                                const float dp = (rpj.y - pri) / (rhoi * rhoj);
                                const float4 vj = A.vel[j];
                                const float vdx = vi.x - vj.x, vdy = vi.y - vj.y, vdz = vi.z - vj.z;
                                const float vdotr = vdx * rx + vdy * ry + vdz * rz;
                                float visc = 0.f;
                                if (vdotr < 0.f) {
                                    const float rp = sqrtf(rx * rx + ry * ry + rz * rz);
                                    const float mu = vdotr / (rp * rp + P.eta2);
                                    const float rbar = 0.5f * (rhoi + rhoj);
                                    const float muh = P.h_av * mu;
                                    visc = (-P.alpha * P.cs * muh + P.beta * muh * muh) / (rbar * rbar * rhoj);
                                }
                                const float br = dp + visc;
                                ax -= br * gx; ay -= br * gy; az -= br * gz;
                                avx -= visc * gx; avy -= visc * gy; avz -= visc * gz;
                            }
                        }
                    }
                }
                ax *= P.mm; ay *= P.mm; az *= P.mm;
                avx *= P.mm; avy *= P.mm; avz *= P.mm;
                const float thv = ti.x * (1.0f + 0.608f * ti.y);
                const float thvr = theta_ref(P, pi.z) * (1.0f + 0.608f * qv_ref(P, pi.z));
                az += GRAV * ((thv - thvr) / thvr - ti.z);
                A.acc[i] = make_float4(ax, ay, az, 0.f);
                const float Pi = powf(fmaxf(pres_ref(P, pi.z) + pri, 1.f) / P0, R_D / CP);
                const float dth = -(vi.x * avx + vi.y * avy + vi.z * avz) / (CP * Pi);
                const float dthc = fminf(fmaxf(dth, -P.dthdt_cap), P.dthdt_cap);
                A.dthdt[i] = dthc;
                if (mode & M_INTEGRATE) {
                    ti.x = fminf(fmaxf(ti.x + dthc * dt, 100.0f), P.theta_cap);
                    A.thq[i] = ti;
                    const float hdt = 0.5f * dt;
                    float4 vn = vi;
                    vn.x += ax * hdt; vn.y += ay * hdt; vn.z += az * hdt;
                    const float zs = (1.f - P.sponge_frac) * P.lz;
                    if (pi.z >= zs) {
                        const float tt = (pi.z - zs) / (P.sponge_frac * P.lz);
                        const float sg = P.sponge_sigma * tt * tt;
                        vn.z *= 1.f / (1.f + sg * dt);
                    }
                    A.vel_out[i] = vn;
                    mx = fabsf(vn.x); my = fabsf(vn.y); mz = fabsf(vn.z);
                }
            }
        }
        if (mode & M_INTEGRATE) {
            mx = warp_max(mx); my = warp_max(my); mz = warp_max(mz);
            const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
            if (lane == 0) { s_max[0][warp] = mx; s_max[1][warp] = my; s_max[2][warp] = mz; }
            __syncthreads();
            if (threadIdx.x == 0) {
                float a = 0.f, b = 0.f, c = 0.f;
                for (int w = 0; w < TPB / 32; ++w) {
                    a = fmaxf(a, s_max[0][w]); b = fmaxf(b, s_max[1][w]); c = fmaxf(c, s_max[2][w]);
                }
                atomicMax(&ctl->gmax[0], __float_as_uint(a));
                atomicMax(&ctl->gmax[1], __float_as_uint(b));
                atomicMax(&ctl->gmax[2], __float_as_uint(c));
            }
        }
    }
    if (mode & M_CFL) {
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            const unsigned t = atomicAdd(&ctl->done, 1u);
            s_last = (t == gridDim.x - 1);
        }
        __syncthreads();
        if (s_last && threadIdx.x == 0) {
            __threadfence();
            ctl->done = 0u;
            if (!aborted) cfl_control(P, ctl);
        }
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
// ---------------------------------------------------------------------------
__global__ void k_audit_partial(const __grid_constant__ Phys P, const float4* __restrict__ pos,
                                const float4* __restrict__ vel, const float4* __restrict__ thq,
                                double* __restrict__ partial) {
    double a[5] = {0, 0, 0, 0, 0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.N; i += gridDim.x * blockDim.x) {
        const float4 p = pos[i], v = vel[i], t = thq[i];
        const float Pi = powf(fmaxf(pres_ref(P, p.z), 1.f) / P0, R_D / CP);
        a[0] += 0.5 * ((double)v.x * v.x + (double)v.y * v.y + (double)v.z * v.z);
        a[1] += (double)GRAV * p.z;
        a[2] += (double)CP * t.x * Pi;
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
__global__ void k_audit_final(const __grid_constant__ Phys P, const double* __restrict__ partial, int nblk,
                              double* __restrict__ out) {
    if (threadIdx.x < 5) {
        double acc = 0.0;
        for (int b = 0; b < nblk; ++b) acc += partial[b * 5 + threadIdx.x];
        out[threadIdx.x] = acc * (double)P.pmass;
    }
    if (threadIdx.x == 5) out[5] = (double)P.pmass * (double)P.N;
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
    A.rp = B.rp; A.acc = B.acc; A.perm = B.perm; A.skeys = B.skeys; A.range = B.range;
    A.surf = B.surf; A.kin = B.kin; A.ctl = B.ctl;
    k_gather<<<blocks_for(P.N), TPB, 0, s>>>(P, A, mode);
}

void launch_density(const Phys& P, const Bufs& B, cudaStream_t s) {
    DArgs A;
    A.pos = B.pos[B.pc]; A.range = B.range; A.thq = B.thq[B.qc]; A.rp = B.rp;
    const bool reads = P.accretion || P.rain_evap;
    A.rain_cur = B.rain[B.rc];
    A.rain_dep = reads ? B.rain_delta : B.rain[B.rc];
    A.ctl = B.ctl;
    k_density<<<blocks_for(P.N), TPB, 0, s>>>(P, A);
}

void launch_momentum(const Phys& P, const Bufs& B, int mode, cudaStream_t s) {
    MArgs A;
    A.pos = B.pos[B.pc]; A.vel = B.vel[B.vc]; A.thq = B.thq[B.qc]; A.rp = B.rp; A.range = B.range;
    A.acc = B.acc; A.dthdt = B.dthdt; A.vel_out = B.vel[1 - B.vc];
    A.rain_in = B.rain[B.rc];
    A.rain_delta = (P.accretion || P.rain_evap) ? B.rain_delta : nullptr;
    A.rain_out = B.rain[1 - B.rc];
    A.precip = B.precip; A.ctl = B.ctl;
    A.part_blocks = blocks_for(P.N);
    const int nb = A.part_blocks + ((mode & M_RAIN) ? blocks_for(P.ncell) : 0);
    k_momentum<<<nb, TPB, 0, s>>>(P, A, mode);
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

void launch_audit(const Phys& P, const Bufs& B, double* partial, int nblk, double* out, cudaStream_t s) {
    k_audit_partial<<<nblk, TPB, 0, s>>>(P, B.pos[B.pc], B.vel[B.vc], B.thq[B.qc], partial);
    k_audit_final<<<1, 32, 0, s>>>(P, partial, nblk, out);
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
