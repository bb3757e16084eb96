// asph_device.cuh — device helpers shared by the kernel files: the
// sounding table, the closed-loop CFL control, rain sedimentation of one
// cell, and the per-particle epilogues of the density and momentum passes.
#pragma once
#include "asph_internal.cuh"

namespace asph {

__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// A reference-sounding value as an unevaluated float pair hi + lo with
// |lo| << |hi|.  Node k of a table holds {hi_k, lo_k, c1_k, c2_k}; on
// [k, k+1) m the value is hi_k + (lo_k + t (c1_k + t c2_k)), t = z - k, a
// quadratic fitted in double on the host, accurate to ~1e-11 relative.
// Keeping the pair lets differences such as rho_j - rho_ref(z_i) be formed
// without the float rounding of rho_ref itself.
struct FF {
    float hi, lo;
    __device__ __forceinline__ float v() const { return hi + lo; }
};
__device__ __forceinline__ FF snd_eval(const float4* __restrict__ tab, int nnode, float z) {
    int k = (int)z;
    k = k < 0 ? 0 : (k > nnode - 2 ? nnode - 2 : k);
    const float t = z - (float)k;
    const float4 c = __ldg(&tab[k]);
    FF r;
    r.hi = c.x;
    r.lo = c.y + t * (c.z + t * c.w);
    return r;
}

// Pair distances in cell units.  Every acceptance test (brick and global
// paths, the deferred pass, the momentum fallback, the adjoint) and every
// density weight uses this one function, so all of them accept exactly the
// same pairs: the coordinate differences are taken in metres first and then
// scaled to cell units with one rounded product each, as the reference does
// (asph_h100.cu:315-320), and r^2 is formed with explicit fused
// multiply-adds.  (Scaling each position to cell units before differencing
// would cost the pair ulp(x / dx), ~1.5e-5 cells at 133 cells, i.e. ~1e-5 of
// a neighbour's weight.)  The momentum pair sum forms the same r^2.
__device__ __forceinline__ float r2_pair(const Phys& P, float xi, float yi, float zi, float xj, float yj, float zj) {
    const float dx = __fmul_rn(__fsub_rn(xi, xj), P.inv_dx);
    const float dy = __fmul_rn(__fsub_rn(yi, yj), P.inv_dy);
    const float dz = __fmul_rn(__fsub_rn(zi, zj), P.inv_dz);
    return __fmaf_rn(dx, dx, __fmaf_rn(dy, dy, __fmul_rn(dz, dz)));
}

// Stop the run from inside a kernel: record the reason (first one wins)
// and make every later kernel of the step and of later steps do nothing.
__device__ __forceinline__ void stop_run(DevCtl* ctl, int code) {
    atomicCAS(&ctl->error, 0, code);
    atomicExch(&ctl->aborted, 1);
}

// Surface skin temperature ramp (asph_h100.cu:989-992).
__device__ __forceinline__ void surface_targets(const Phys& P, double simt, float& Ts, float& qs_sfc) {
    float r = fminf(fmaxf((float)simt / P.ramp, 0.f), 1.f);
    float sw = r * r * (3.f - 2.f * r);
    Ts = P.th0 + P.dts_skin * sw;
    qs_sfc = qsat(Ts, snd_eval(P.snd_p, P.snd_n, 0.f).v());
}

// Closed-loop CFL control (asph_h100.cu:1040-1078), run by one thread after
// every block of the step has contributed its velocity maxima.
__device__ __forceinline__ void cfl_control(const Phys& P, DevCtl* ctl) {
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

// Rain sedimentation of one cell (asph_h100.cu:577-599).  `delta` holds
// this step's deposits when the microphysics reads the grid.
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

// Density pair sums of one target, in units of SIGMA_W / 4: S1 = sum W, S2 = sum W/rho_j,
// T = sum W (rho_j - hi) / rho_j with rho_ref(z_i) = hi + lo (T - lo S2 = S1 - rho_ref S2
// without the cancellation).  Self pair included (asph_h100.cu:314-325).
struct DSum {
    float S1, S2, T;
};
__device__ __forceinline__ void dsum_add(DSum& s, float r2, float rho_j, const FF& rr) {
    // accepted pairs only (r2 < 4): the spline of w3 in Horner form with FMAs,
    // scaled by 4 / SIGMA_W (4 - 6 q^2 + 3 q^3 inside, (2 - q)^3 outside): the
    // epilogue uses the sums only as the ratios S1 / S2 and T / S2
    const float q = r2 > 0.f ? r2 * rsqrtf(r2) : 0.f;
    const float t = 2.0f - q;
    const float W = q < 1.0f ? __fmaf_rn(q * q, __fmaf_rn(3.0f, q, -6.0f), 4.0f) : t * t * t;
    const float rj = fmaxf(rho_j, 1e-3f);
    const float iw = __fdividef(W, rj);
    s.S1 += W;
    s.S2 += iw;
    s.T = fmaf(iw, rj - rr.hi, s.T);   // rho_ref's low part enters once, in the epilogue
}

// Density result + EOS + saturation adjustment + autoconversion (+ Kessler
// accretion and rain evaporation) for one particle
// (asph_h100.cu:328-332, 340-402).  Writes thq and rp, deposits rain.
struct DOut {
    float4* thq;
    float2* rp;
    const float* rain_cur;
    float* rain_dep;
    const float4* vel;   // velocities the momentum pass reads (after the first half kick) ...
    float4* ms0;         // ... packed for its neighbour loads: x, y, z, p' ...
    float4* ms1;         // ... and u, v, w, rho
};
__device__ __forceinline__ void density_eos_epilogue(const Phys& P, const DOut& O, int i, float4 pi, const DSum& s,
                                                     const FF& rr, float dt) {
    const float z = pi.z;
    const float rref = rr.v();
    float rho, dd;
    if (s.S2 > 1e-20f) {
        const float raw = s.S1 / s.S2;
        rho = fminf(fmaxf(raw, 0.5f * rref), 2.0f * rref);
        dd = (rho == raw) ? s.T / s.S2 - rr.lo : rho - rref;
    } else {
        rho = fminf(fmaxf(rref, 0.5f * rref), 2.0f * rref);
        dd = 0.f;
    }
    // EOS (asph_h100.cu:352-361)
    if (rho < 1e-3f) dd = 1e-3f - rref;
    const float r = fmaxf(rho, 1e-3f);
    dd = fminf(fmaxf(dd, -0.3f * rref), 0.3f * rref);
    const float ppr = P.cs * P.cs * dd;
    const float pfl = fmaxf(snd_eval(P.snd_p, P.snd_n, z).v() + ppr, 1.0f);
    const float Pi = powf(pfl / P0, R_D / CP);

    const float4 t = O.thq[i];
    float th = t.x, qv = t.y, qc = t.z;
    float T = th * Pi;
    const float qs = qsat(T, pfl);
    // saturation adjustment, 3 Newton iterations (asph_h100.cu:370-385)
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
    // autoconversion into the rain grid (asph_h100.cu:389-394)
    float dep = 0.f;
    if (qc > P.qc_auto) {
        const float dqr = (qc - P.qc_auto) * (1.f - expf(-P.rate_auto * dt));
        qc -= dqr;
        dep += dqr;
    }
    const int ix = cell_ix(pi.x, P.inv_dx, P.nx), iy = cell_ix(pi.y, P.inv_dy, P.ny), iz = cell_ix(z, P.inv_dz, P.nz);
    const int cid = (iz * P.ny + iy) * P.nx + ix;
    if (P.accretion || P.rain_evap) {
        // Kessler warm rain; rain is Eulerian per cell, qr = M_rain / (rho V_cell)
        const float qr = fmaxf(O.rain_cur[cid], 0.f) / (r * P.v_cell);
        if (P.accretion && qc > 0.f && qr > 0.f) {
            const float dqa = fminf(qc, dt * P.k_accr * qc * powf(qr, 0.875f));
            qc -= dqa;
            dep += dqa;
        }
        if (P.rain_evap && qr > 0.f) {
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
    if (dep != 0.f) atomicAdd(&O.rain_dep[cid], dep * P.pmass);
    th = fminf(fmaxf(th, 100.0f), P.theta_cap);
    qv = fminf(fmaxf(qv, 0.0f), P.qv_cap);
    qc = fmaxf(qc, 0.0f);
    O.thq[i] = make_float4(th, qv, qc, t.w);
    O.rp[i] = make_float2(rho, ppr);
    const float4 v = O.vel[i];
    O.ms0[i] = make_float4(pi.x, pi.y, pi.z, ppr);
    O.ms1[i] = make_float4(v.x, v.y, v.z, rho);
}

// Momentum pair accumulation (asph_h100.cu:448-492), arithmetic rearranged
// to one rsqrt and at most one division per pair.
struct MSum {
    float ax, ay, az, vx, vy, vz;
};
struct MTarget {
    float x, y, z, u, v, w, rhoi, irhoi, pri;
};
__device__ __forceinline__ void msum_add(const Phys& P, MSum& s, const MTarget& T, float4 pj, float4 vj) {
    // pj = (x, y, z, p'_j), vj = (u, v, w, rho_j); FMAs and approximate
    // reciprocals throughout (relative error ~1e-7 per pair)
    const float rx = __fsub_rn(T.x, pj.x), ry = __fsub_rn(T.y, pj.y), rz = __fsub_rn(T.z, pj.z);
    const float dxt = __fmul_rn(rx, P.inv_dx), dyt = __fmul_rn(ry, P.inv_dy), dzt = __fmul_rn(rz, P.inv_dz);
    const float r2t = __fmaf_rn(dxt, dxt, __fmaf_rn(dyt, dyt, __fmul_rn(dzt, dzt)));   // = r2_pair
    const float rs = rsqrtf(r2t);
    const float q = r2t * rs;
    const float t2 = 2.0f - q;
    // dW/dq / q in units of -0.75 SIGMA_W: inner 4 - 3 q, outer (2 - q)^2 / q
    const float k = q < 1.0f ? __fmaf_rn(-3.0f, q, 4.0f) : (t2 * t2) * rs;
    const float rhoj = fmaxf(vj.w, 1e-3f);
    const float irj = __fdividef(1.0f, rhoj);
    const float dp = (pj.w - T.pri) * (T.irhoi * irj);
    const float ux = T.u - vj.x, uy = T.v - vj.y, uz = T.w - vj.z;
    const float vdotr = __fmaf_rn(ux, rx, __fmaf_rn(uy, ry, uz * rz));
    float visc = 0.f;
    if (vdotr < 0.f) {
        const float rp2 = __fmaf_rn(rx, rx, __fmaf_rn(ry, ry, rz * rz));
        // (-alpha cs mu + beta mu^2) / (rbar^2 rho_j) with mu = h m, m = vdotr / (r^2 + eta^2),
        // rbar = s / 2: m (4 beta h^2 m - 4 alpha cs h) / (s^2 rho_j)
        const float m = __fdividef(vdotr, rp2 + P.eta2);
        const float is = __fdividef(1.0f, T.rhoi + rhoj);
        visc = (m * __fmaf_rn(P.av_quad, m, P.av_lin)) * (irj * (is * is));
    }
    const float br = dp + visc;
    // grad_i W = k (dxt inv_dx, dyt inv_dy, dzt inv_dz): the sums carry k (dxt, dyt, dzt)
    // and the epilogue applies inv_d once per target (4 products fewer per pair)
    const float ck = -br * k, cv = -visc * k;
    s.ax = __fmaf_rn(ck, dxt, s.ax); s.ay = __fmaf_rn(ck, dyt, s.ay); s.az = __fmaf_rn(ck, dzt, s.az);
    s.vx = __fmaf_rn(cv, dxt, s.vx); s.vy = __fmaf_rn(cv, dyt, s.vy); s.vz = __fmaf_rn(cv, dzt, s.vz);
}

// Momentum epilogue: mass scaling, buoyancy with condensate loading,
// viscous heating (asph_h100.cu:497-510); with integrate also theta update
// (562-571), second half kick (535-544) and sponge (518-530).
struct MOut {
    float4* thq;
    float4* acc;
    float* dthdt;
    float4* vel_out;
    const float4* src_cur;   // source-term tendencies in this step's order (NULL: hook off)
    float4* src_keep;        // where they are kept for the next step
};
__device__ __forceinline__ float3 momentum_epilogue(const Phys& P, const MOut& O, int i, const MTarget& T, MSum s,
                                                    bool integrate, float dt) {
    // mass scaling and the gradient's per-axis factor (msum_add leaves it out)
    const float mk = P.mm * (-0.75f * SIGMA_W);   // msum_add's k is in units of -0.75 SIGMA_W
    const float mx = mk * P.inv_dx, my = mk * P.inv_dy, mz = mk * P.inv_dz;
    s.ax *= mx; s.ay *= my; s.az *= mz;
    s.vx *= mx; s.vy *= my; s.vz *= mz;
    float4 ti = O.thq[i];
    // theta_v - theta_v,ref without cancellation: (th - thvr) + 0.608 th qv
    const FF vr = snd_eval(P.snd_thvr, P.snd_n, T.z);
    const float dth_v = ((ti.x - vr.hi) - vr.lo) + 0.608f * ti.x * ti.y;
    s.az += GRAV * (dth_v / vr.v() - ti.z);
    O.acc[i] = make_float4(s.ax, s.ay, s.az, 0.f);
    const float Pi = powf(fmaxf(snd_eval(P.snd_p, P.snd_n, T.z).v() + T.pri, 1.f) / P0, R_D / CP);
    const float dth = -(T.u * s.vx + T.v * s.vy + T.w * s.vz) / (CP * Pi);
    const float dthc = fminf(fmaxf(dth, -P.dthdt_cap), P.dthdt_cap);
    O.dthdt[i] = dthc;
    float3 m = make_float3(0.f, 0.f, 0.f);
    if (integrate) {
        if (O.src_cur) {
            // source-term hook: additive tendencies before the theta update
            const float4 sv = O.src_cur[i];
            O.src_keep[i] = sv;
            ti.x = fminf(fmaxf(ti.x + (dthc + sv.x) * dt, 100.0f), P.theta_cap);
            ti.y = fminf(fmaxf(ti.y + sv.y * dt, 0.0f), P.qv_cap);
            ti.z = fmaxf(ti.z + sv.z * dt, 0.0f);
        } else {
            ti.x = fminf(fmaxf(ti.x + dthc * dt, 100.0f), P.theta_cap);
        }
        O.thq[i] = ti;
        const float hdt = 0.5f * dt;
        float4 vn = make_float4(T.u + s.ax * hdt, T.v + s.ay * hdt, T.w + s.az * hdt, 0.f);
        const float zs = (1.f - P.sponge_frac) * P.lz;
        if (T.z >= zs) {
            const float tt = (T.z - zs) / (P.sponge_frac * P.lz);
            const float sg = P.sponge_sigma * tt * tt;
            vn.z *= 1.f / (1.f + sg * dt);
        }
        O.vel_out[i] = vn;
        m = make_float3(fabsf(vn.x), fabsf(vn.y), fabsf(vn.z));
    }
    return m;
}

}  // namespace asph
