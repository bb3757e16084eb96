// asph_adjoint.cu — the discrete adjoint of the SPH warm-rain step.
//
// No counterpart in the reference.  The forward it differentiates (the
// "adjoint window step") is the reference's KDK step (asph_h100.cu:958-1078)
// with one change of order: the kick/drift/flux runs first, on the current
// order, and the sort, gather and cell table follow on the drifted
// positions, so the density pass's neighbour lists hold exactly the pairs
// with q < 2 (the cell window of +-2 around a fresh table is exact) and are
// symmetric.  The sort (a permutation) and the lists are held fixed in the
// adjoint: the reverse applies the inverse permutation and walks the same
// lists.  dt is fixed over the window.
//
// Reverse of one step, in the sorted order of that step unless noted:
//   R6 k_adj_rain       rain sedimentation (per cell)
//   R5a k_adj_mom_seed  sponge, second kick, theta update, heating, buoyancy;
//                       per-particle seeds of the momentum pair sums
//   R5b k_adj_mom_pairs momentum pairs: each target gathers the terms of its
//                       own sums and, through the symmetric list, the terms it
//                       contributes to its neighbours' sums (no atomics);
//                       dJ/dalpha, dJ/dbeta
//   R4 k_adj_micro      saturation adjustment (3 unrolled Newton steps),
//                       autoconversion, accretion, evaporation, clamps — the
//                       per-particle Jacobian by forward-mode dual numbers —
//                       and the EOS
//   R3 k_adj_dens_a/b   lagged Shepard density (pair gather)
//   R2 k_adj_unperm     inverse of the sort's gather
//   R1 k_adj_integrate  surface flux, drift with wrap/reflection, first kick
//                       (order before the sort)
// Checkpoints: a device snapshot every `every` steps in the forward; the
// backward restores each segment, recomputes it recording a per-step tape,
// and reverses it.
#include <stdio.h>
#include <string.h>
#include <map>
#include <utility>
#include <vector>
#include "asph_ctx.cuh"
#include "asph_device.cuh"

namespace asph {
namespace {

constexpr int ATPB = 256;
constexpr float KAPPA = R_D / CP;

// ---------------------------------------------------------------------------
// forward-mode dual numbers for per-particle Jacobians
// ---------------------------------------------------------------------------
template <int N>
struct Dn {
    float v;
    float d[N];
};
template <int N>
__device__ __forceinline__ Dn<N> dconst(float a) {
    Dn<N> r;
    r.v = a;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = 0.f;
    return r;
}
template <int N>
__device__ __forceinline__ Dn<N> dvar(float a, int k0) {
    Dn<N> r = dconst<N>(a);
    r.d[k0] = 1.f;
    return r;
}
template <int N>
__device__ __forceinline__ Dn<N> lin(const Dn<N>& a, float va, float ca, const Dn<N>& b, float cb) {
    Dn<N> r;
    r.v = va;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = ca * a.d[k] + cb * b.d[k];
    return r;
}
template <int N>
__device__ __forceinline__ Dn<N> scale(const Dn<N>& a, float va, float c) {
    Dn<N> r;
    r.v = va;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = c * a.d[k];
    return r;
}
template <int N> __device__ __forceinline__ Dn<N> operator+(const Dn<N>& a, const Dn<N>& b) { return lin(a, a.v + b.v, 1.f, b, 1.f); }
template <int N> __device__ __forceinline__ Dn<N> operator-(const Dn<N>& a, const Dn<N>& b) { return lin(a, a.v - b.v, 1.f, b, -1.f); }
template <int N> __device__ __forceinline__ Dn<N> operator*(const Dn<N>& a, const Dn<N>& b) { return lin(a, a.v * b.v, b.v, b, a.v); }
template <int N> __device__ __forceinline__ Dn<N> operator/(const Dn<N>& a, const Dn<N>& b) {
    const float q = a.v / b.v;
    return lin(a, q, 1.f / b.v, b, -q / b.v);
}
template <int N> __device__ __forceinline__ Dn<N> operator-(const Dn<N>& a) { return scale(a, -a.v, -1.f); }
template <int N> __device__ __forceinline__ Dn<N> operator+(const Dn<N>& a, float b) { return scale(a, a.v + b, 1.f); }
template <int N> __device__ __forceinline__ Dn<N> operator+(float b, const Dn<N>& a) { return scale(a, a.v + b, 1.f); }
template <int N> __device__ __forceinline__ Dn<N> operator-(const Dn<N>& a, float b) { return scale(a, a.v - b, 1.f); }
template <int N> __device__ __forceinline__ Dn<N> operator-(float b, const Dn<N>& a) { return scale(a, b - a.v, -1.f); }
template <int N> __device__ __forceinline__ Dn<N> operator*(const Dn<N>& a, float b) { return scale(a, a.v * b, b); }
template <int N> __device__ __forceinline__ Dn<N> operator*(float b, const Dn<N>& a) { return scale(a, a.v * b, b); }
template <int N> __device__ __forceinline__ Dn<N> operator/(const Dn<N>& a, float b) { return scale(a, a.v / b, 1.f / b); }
template <int N> __device__ __forceinline__ Dn<N> operator/(float b, const Dn<N>& a) {
    const float q = b / a.v;
    return scale(a, q, -q / a.v);
}

template <int N> __device__ __forceinline__ float val(const Dn<N>& a) { return a.v; }
template <int N> __device__ __forceinline__ Dn<N> xexp(const Dn<N>& a) {
    const float e = expf(a.v);
    return scale(a, e, e);
}
template <int N> __device__ __forceinline__ Dn<N> xpow(const Dn<N>& a, float c) {
    const float p = powf(a.v, c);
    return scale(a, p, a.v != 0.f ? c * p / a.v : 0.f);
}
template <class S> __device__ __forceinline__ S xmin(const S& a, const S& b) { return val(a) < val(b) ? a : b; }
template <class S> __device__ __forceinline__ S xmax(const S& a, const S& b) { return val(a) > val(b) ? a : b; }
template <int N> __device__ __forceinline__ Dn<N> cst(float a, const Dn<N>&) { return dconst<N>(a); }

// thermodynamics of asph_phys.cuh, generic in the scalar
template <class S>
__device__ __forceinline__ S esat_t(const S& T) {
    const S Tc = T - 273.15f;
    return 611.2f * xexp(17.67f * Tc / (Tc + 243.5f));
}
template <class S>
__device__ __forceinline__ S qsat_t(const S& T, const S& p) {
    const S es = xmin(esat_t(T), 0.5f * p);
    const S den = p - 0.378f * es;
    return val(den) > 1.0f ? 0.622f * es / den : cst(0.f, T);
}
template <class S>
__device__ __forceinline__ S dqsdT_t(const S& T, const S& es, const S& p) {
    const S Tc = T - 273.15f;
    const S d = Tc + 243.5f;
    const S desdT = es * (17.67f * 243.5f) / (d * d);
    const S den = p - 0.378f * es;
    return 0.622f * p * desdT / (den * den);
}

// The microphysics of the density epilogue (saturation adjustment,
// autoconversion, accretion, evaporation, caps) as a function of
// (theta, qv, qc, p_full, rho, rain mass of the cell).
template <class S>
__device__ void micro_t(const Phys& P, float dt, S th, S qv, S qc, const S& pfl, const S& r, const S& R, S& th_o,
                        S& qv_o, S& qc_o, S& dep_o) {
    const S Pi = xpow(pfl / P0, KAPPA);
    S T = th * Pi;
    const S qs = qsat_t(T, pfl);
    if (val(qv) > val(qs) || val(qc) > 0.f) {
        S dqc = cst(0.f, th);
        for (int it = 0; it < 3; ++it) {
            const S Tn = T + (L_V / CP) * dqc;
            const S esn = esat_t(Tn);
            const S qsn = qsat_t(Tn, pfl);
            const S f = qv - dqc - qsn;
            const S fp = -1.f - dqsdT_t(Tn, esn, pfl) * (L_V / CP);
            dqc = dqc - f / fp;
            dqc = xmin(dqc, qv);
            dqc = xmax(dqc, -qc);
        }
        qv = qv - dqc;
        qc = qc + dqc;
        th = th + L_V * dqc / (CP * Pi);
        T = T + (L_V / CP) * dqc;
    }
    S dep = cst(0.f, th);
    if (val(qc) > P.qc_auto) {
        const S dqr = (qc - P.qc_auto) * (1.f - expf(-P.rate_auto * dt));
        qc = qc - dqr;
        dep = dep + dqr;
    }
    if (P.accretion || P.rain_evap) {
        const S qr = xmax(R, cst(0.f, th)) / (r * P.v_cell);
        if (P.accretion && val(qc) > 0.f && val(qr) > 0.f) {
            const S dqa = xmin(qc, dt * P.k_accr * qc * xpow(qr, 0.875f));
            qc = qc - dqa;
            dep = dep + dqa;
        }
        if (P.rain_evap && val(qr) > 0.f) {
            const S qvs = qsat_t(T, pfl);
            if (val(qv) < val(qvs) && val(qvs) > 0.f) {
                const S rq = 1e-3f * r * qr;
                const S C = 1.6f + 124.9f * xpow(rq, 0.2046f);
                const S er = (1.f - qv / qvs) * C * xpow(rq, 0.525f) /
                             (1e-3f * r * (5.4e5f + 2.55e6f / (0.01f * pfl * qvs)));
                const S dqe = xmin(qr, xmin(dt * er, qvs - qv));
                qv = qv + dqe;
                th = th - L_V * dqe / (CP * Pi);
                dep = dep - dqe;
            }
        }
    }
    th_o = xmin(xmax(th, cst(100.0f, th)), cst(P.theta_cap, th));
    qv_o = xmin(xmax(qv, cst(0.0f, th)), cst(P.qv_cap, th));
    qc_o = xmax(qc, cst(0.0f, th));
    dep_o = dep;
}

// slope d/dz of a sounding table (quadratic per metre node)
__device__ __forceinline__ float snd_slope(const float4* __restrict__ tab, int nnode, float z) {
    int k = (int)z;
    k = k < 0 ? 0 : (k > nnode - 2 ? nnode - 2 : k);
    const float t = z - (float)k;
    const float4 c = __ldg(&tab[k]);
    return c.z + 2.f * t * c.w;
}

__device__ __forceinline__ int cell_of(const Phys& P, float x, float y, float z) {
    const int ix = cell_ix(x, P.inv_dx, P.nx), iy = cell_ix(y, P.inv_dy, P.ny), iz = cell_ix(z, P.inv_dz, P.nz);
    return (iz * P.ny + iy) * P.nx + ix;
}


// ---------------------------------------------------------------------------
// tape of one step
// ---------------------------------------------------------------------------
struct StepTape {
    float4 *pos0, *vel0, *thq0, *acc0;   // step start, order before the sort
    uint8_t* surf0;                      // surface flags used by the flux
    uint32_t* perm;                      // the step's sort
    float4 *pos1, *vel1, *thq1;          // after the gather: x1 (w = rho_old), v1, micro inputs
    float2* rp;                          // rho, p'
    float4* thq2;                        // micro outputs
    int *cnt, *lst;                      // neighbour lists, slot-major [NBR_CAP][N]
    float *rain0, *dep;                  // rain grid at the step start, deposits of the step
    float4* acc;                         // acceleration of the step
    float* dthdt;                        // clamped heating tendency
    double simt;                         // simulated time at the step start
};

struct AdjBufs {
    // adjoint of the state at the end of the step being reversed (sorted order)
    float4 *e_pos, *e_vel, *e_thq, *e_acc;
    float* e_rain;
    // intermediates
    float4 *sF, *sV, *lx, *lv, *lq;
    float* lP;
    float2* lS;
    float *l_depc, *l_rain0;
    float4 *px, *pv, *pq;
    double* ab;   // dJ/dalpha, dJ/dbeta
    int* err;
};

// ---------------------------------------------------------------------------
// reverse kernels
// ---------------------------------------------------------------------------

// R6: rain sedimentation of every cell, asph_device.cuh rain_cell.
__global__ void k_adj_rain(const Phys P, float dt, const float* __restrict__ rain0, const float* __restrict__ dep,
                           const float* __restrict__ l_out, float* __restrict__ l_rain0, float* __restrict__ l_depc,
                           int reads) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= P.ncell) return;
    float f = P.v_rain * dt * P.inv_dz;
    if (f > 1.f) f = 1.f;
    const int iz = c / P.nxy;
    float lcur = (1.f - f) * l_out[c];
    if (iz > 0) lcur += f * l_out[c - P.nxy];
    float g = lcur;
    if (reads && !(rain0[c] + dep[c] > 0.f)) g = 0.f;   // cur = max(rain0 + dep, 0)
    l_rain0[c] = g;
    l_depc[c] = g;
}

// R5a: per-particle reverse of the momentum epilogue and the integration.
__global__ void k_adj_mom_seed(const Phys P, float dt, StepTape T, AdjBufs A) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const float4 x1 = T.pos1[i], v1 = T.vel1[i], t2 = T.thq2[i], a = T.acc[i];
    const float2 rp = T.rp[i];
    const float dthdt = T.dthdt[i];
    const float4 ep = A.e_pos[i], ev = A.e_vel[i], eq = A.e_thq[i], ea = A.e_acc[i];
    const float z = x1.z, hdt = 0.5f * dt;
    // sponge on the vertical velocity after the second kick
    float S = 1.f, dS = 0.f;
    const float zs = (1.f - P.sponge_frac) * P.lz;
    if (z >= zs) {
        const float den = P.sponge_frac * P.lz;
        const float tt = (z - zs) / den;
        const float sg = P.sponge_sigma * tt * tt;
        S = 1.f / (1.f + sg * dt);
        dS = -S * S * dt * P.sponge_sigma * 2.f * tt / den;
    }
    float lvx = ev.x, lvy = ev.y, lvz = S * ev.z;
    float lax = hdt * ev.x + ea.x, lay = hdt * ev.y + ea.y, laz = hdt * S * ev.z + ea.z;
    float lz = dS * (v1.z + hdt * a.z) * ev.z;
    // theta update with its clamp
    const float th3 = t2.x + dthdt * dt;
    const float I1 = (th3 > 100.f && th3 < P.theta_cap) ? 1.f : 0.f;
    float lth2 = I1 * eq.x;
    const float ldthdt = I1 * dt * eq.x;
    // heating: dthdt = clamp(-(v1 . Vm) / (cp Pi))
    const float I2 = fabsf(dthdt) < P.dthdt_cap ? 1.f : 0.f;
    const float ldth = I2 * ldthdt;
    const float pref = snd_eval(P.snd_p, P.snd_n, z).v();
    const float pflm_raw = pref + rp.y;
    const float pflm = fmaxf(pflm_raw, 1.f);
    const float Pi = powf(pflm / P0, KAPPA);
    const float cpPi = CP * Pi;
    // lVm = -v1/(cp Pi) ldth ; lPi = (v1.Vm)/(cp Pi^2) ldth = -dthdt/Pi ldth
    const float lPi = -dthdt / Pi * ldth;
    float lP = 0.f;
    if (pflm_raw > 1.f) {
        const float dPi = KAPPA * Pi / pflm;
        lP += dPi * lPi;
        lz += dPi * snd_slope(P.snd_p, P.snd_n, z) * lPi;
    }
    // buoyancy on the vertical acceleration
    const FF vr = snd_eval(P.snd_thvr, P.snd_n, z);
    const float thvr = vr.v();
    const float fac = 1.f + 0.608f * t2.y;
    lth2 += laz * GRAV * fac / thvr;
    const float lqv2 = eq.y + laz * GRAV * 0.608f * t2.x / thvr;
    const float lqc2 = eq.z - GRAV * laz;
    lz += laz * (-GRAV * t2.x * fac * snd_slope(P.snd_thvr, P.snd_n, z) / (thvr * thvr));
    const float cv = -ldth / cpPi;
    A.sF[i] = make_float4(P.mm * lax, P.mm * lay, P.mm * laz, ldth);
    A.sV[i] = make_float4(P.mm * cv * v1.x, P.mm * cv * v1.y, P.mm * cv * v1.z, cpPi);
    // the step's final positions are the drifted x1: their adjoint carries on;
    // w: dJ/drho of this step's density (the next step's rho_old)
    A.lx[i] = make_float4(ep.x, ep.y, ep.z + lz, ep.w);
    A.lv[i] = make_float4(lvx, lvy, lvz, 0.f);
    A.lq[i] = make_float4(lth2, lqv2, lqc2, 0.f);
    A.lP[i] = lP;
}

// R5b: momentum pair sums.  For the pair (i, j) in i's list, the thread of
// i takes the derivative of i's own pair term (seeds of i) and of the term
// i contributes to j's sum (seeds of j) with respect to i's variables.
__global__ __launch_bounds__(ATPB, 4) void k_adj_mom_pairs(const Phys P, StepTape T, AdjBufs A) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float la = 0.f, lb = 0.f;
    if (i < P.N) {
        const float4 xi = T.pos1[i], vi = T.vel1[i], sFi = A.sF[i], sVi = A.sV[i];
        const float2 ri = T.rp[i];
        const float rhoi = fmaxf(ri.x, 1e-3f), iri = __fdividef(1.f, rhoi);
        const float Ii = ri.x > 1e-3f ? 1.f : 0.f;
        const int cnt = T.cnt[i];
        if (cnt < 0) atomicExch(A.err, 1);   // list overflow: the adjoint needs every pair
        float gx = 0.f, gy = 0.f, gz = 0.f, gvx = 0.f, gvy = 0.f, gvz = 0.f, grho = 0.f, gP = 0.f;
        float Vx = 0.f, Vy = 0.f, Vz = 0.f;
        const float Mx = P.inv_dx * P.inv_dx, My = P.inv_dy * P.inv_dy, Mz = P.inv_dz * P.inv_dz;
        for (int q = 0; q < cnt; ++q) {
            const int j = T.lst[(size_t)q * P.N + i];
            const float4 xj = T.pos1[j], vj = T.vel1[j], sFj = A.sF[j], sVj = A.sV[j];
            const float2 rj = T.rp[j];
            // the pair geometry exactly as the forward pass forms it (msum_add)
            const float rx = xi.x - xj.x, ry = xi.y - xj.y, rz = xi.z - xj.z;
            const float dxt = rx * P.inv_dx, dyt = ry * P.inv_dy, dzt = rz * P.inv_dz;
            const float r2t = __fmaf_rn(dxt, dxt, __fmaf_rn(dyt, dyt, dzt * dzt));
            if (r2t < 1e-12f) continue;
            const float rs = rsqrtf(r2t);
            const float qq = r2t * rs;
            const float t2 = 2.f - qq;
            // W'(q)/q and its q-derivative (both branches as in the forward)
            const float kq = qq < 1.f ? SIGMA_W * __fmaf_rn(2.25f, qq, -3.f) : (-0.75f * SIGMA_W) * (t2 * t2) * rs;
            const float kpq = qq < 1.f ? (2.25f * SIGMA_W) * rs : (0.75f * SIGMA_W) * t2 * (qq + 2.f) * (rs * rs * rs);
            const float Mrx = Mx * rx, Mry = My * ry, Mrz = Mz * rz;   // M r
            const float gxx = kq * Mrx, gyy = kq * Mry, gzz = kq * Mrz;   // grad_i W
            const float rhoj = fmaxf(rj.x, 1e-3f), irj = __fdividef(1.f, rhoj);
            const float dp = (rj.y - ri.y) * (iri * irj);   // dp_ij ; dp_ji = -dp
            const float ux = vi.x - vj.x, uy = vi.y - vj.y, uz = vi.z - vj.z;
            const float sdot = __fmaf_rn(ux, rx, __fmaf_rn(uy, ry, uz * rz));
            float mu = 0.f, hd = 0.f, m2 = 0.f, Phi = 0.f, dPhi = 0.f;
            const float rbar = 0.5f * (rhoi + rhoj), irb = __fdividef(1.f, rbar), ir2 = irb * irb;
            const bool vis = sdot < 0.f;
            if (vis) {
                const float iden = __fdividef(1.f, __fmaf_rn(rx, rx, __fmaf_rn(ry, ry, rz * rz)) + P.eta2);
                hd = P.h_av * iden;
                mu = hd * sdot;
                m2 = 2.f * mu * iden;
                Phi = mu * __fmaf_rn(P.beta, mu, -P.alpha * P.cs);
                dPhi = __fmaf_rn(2.f * P.beta, mu, -P.alpha * P.cs);
            }
            const float visc_ij = Phi * (irj * ir2);   // in i's sum
            const float visc_ji = Phi * (iri * ir2);   // in j's sum
            Vx = __fmaf_rn(-visc_ij, gxx, Vx); Vy = __fmaf_rn(-visc_ij, gyy, Vy); Vz = __fmaf_rn(-visc_ij, gzz, Vz);
            // ---- (a) i's own term, seeds of i; (b) the term of j's sum in which i is
            // the neighbour, seeds of j (g_ji = -g_ij, dp_ji = -dp).  Both give
            // dc/dx_i = +-(kq M c + kpq (r.Mc) M r) with c = dc/dg.
            const float Aa = __fmaf_rn(sFi.x, gxx, __fmaf_rn(sFi.y, gyy, sFi.z * gzz));
            const float Ba = __fmaf_rn(sVi.x, gxx, __fmaf_rn(sVi.y, gyy, sVi.z * gzz));
            const float Ab = -__fmaf_rn(sFj.x, gxx, __fmaf_rn(sFj.y, gyy, sFj.z * gzz));
            const float Bb = -__fmaf_rn(sVj.x, gxx, __fmaf_rn(sVj.y, gyy, sVj.z * gzz));
            const float bra = dp + visc_ij, brb = visc_ji - dp;
            // c_a - c_b (the x_i derivative of (b) enters with a minus sign)
            const float cx = -bra * sFi.x - visc_ij * sVi.x + brb * sFj.x + visc_ji * sVj.x;
            const float cy = -bra * sFi.y - visc_ij * sVi.y + brb * sFj.y + visc_ji * sVj.y;
            const float cz = -bra * sFi.z - visc_ij * sVi.z + brb * sFj.z + visc_ji * sVj.z;
            const float rMc = __fmaf_rn(Mrx, cx, __fmaf_rn(Mry, cy, Mrz * cz));
            gx += __fmaf_rn(kq * Mx, cx, kpq * rMc * Mrx);
            gy += __fmaf_rn(kq * My, cy, kpq * rMc * Mry);
            gz += __fmaf_rn(kq * Mz, cz, kpq * rMc * Mrz);
            gP += (Aa - Ab) * (iri * irj);
            grho += Ii * (Aa - Ab) * dp * iri;
            if (vis) {
                const float Psa = -(Aa + Ba), Psb = -(Ab + Bb);
                const float lmu = dPhi * ir2 * (Psa * irj + Psb * iri);
                gvx = __fmaf_rn(lmu * hd, rx, gvx); gvy = __fmaf_rn(lmu * hd, ry, gvy); gvz = __fmaf_rn(lmu * hd, rz, gvz);
                gx = __fmaf_rn(lmu, __fmaf_rn(hd, ux, -m2 * rx), gx);
                gy = __fmaf_rn(lmu, __fmaf_rn(hd, uy, -m2 * ry), gy);
                gz = __fmaf_rn(lmu, __fmaf_rn(hd, uz, -m2 * rz), gz);
                // visc_ij = Phi / (rho_j rbar^2), visc_ji = Phi / (rho_i rbar^2), rbar = (rho_i + rho_j)/2
                grho += Ii * (Psa * (-visc_ij * irb) + Psb * (-visc_ji) * (iri + irb));
                const float wa = Psa * (irj * ir2);
                la = __fmaf_rn(wa, -P.cs * mu, la);
                lb = __fmaf_rn(wa, mu * mu, lb);
            }
        }
        // heating: d dth / d v1 = -Vm / (cp Pi)
        const float ldth = sFi.w, cpPi = sVi.w;
        gvx += -P.mm * Vx / cpPi * ldth;
        gvy += -P.mm * Vy / cpPi * ldth;
        gvz += -P.mm * Vz / cpPi * ldth;
        float4 lx = A.lx[i];
        lx.x += gx; lx.y += gy; lx.z += gz; lx.w += grho;
        A.lx[i] = lx;
        float4 lv = A.lv[i];
        lv.x += gvx; lv.y += gvy; lv.z += gvz;
        A.lv[i] = lv;
        A.lP[i] += gP;
    }
    // dJ/dalpha, dJ/dbeta: warp sums, one double atomic per warp
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        la += __shfl_xor_sync(0xffffffffu, la, o);
        lb += __shfl_xor_sync(0xffffffffu, lb, o);
    }
    if ((threadIdx.x & 31) == 0 && (la != 0.f || lb != 0.f)) {
        atomicAdd(&A.ab[0], (double)la);
        atomicAdd(&A.ab[1], (double)lb);
    }
}

// R4: microphysics (dual numbers) and EOS, per particle.
__global__ void k_adj_micro(const Phys P, float dt, StepTape T, AdjBufs A) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const float4 x1 = T.pos1[i], t1 = T.thq1[i];
    const float2 rp = T.rp[i];
    const float z = x1.z;
    const int cid = cell_of(P, x1.x, x1.y, z);
    const float pref = snd_eval(P.snd_p, P.snd_n, z).v();
    const float pfl_raw = pref + rp.y;
    const float pflv = fmaxf(pfl_raw, 1.0f);
    const float rv = fmaxf(rp.x, 1e-3f);
    const float Rv = (P.accretion || P.rain_evap) ? T.rain0[cid] : 0.f;
    typedef Dn<6> D;
    D th = dvar<6>(t1.x, 0), qv = dvar<6>(t1.y, 1), qc = dvar<6>(t1.z, 2), pfl = dvar<6>(pflv, 3),
      r = dvar<6>(rv, 4), R = dvar<6>(Rv, 5);
    D tho, qvo, qco, dep;
    micro_t<D>(P, dt, th, qv, qc, pfl, r, R, tho, qvo, qco, dep);
    const float4 lq = A.lq[i];
    const float ldep = P.pmass * A.l_depc[cid];
    float lin[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) lin[k] = lq.x * tho.d[k] + lq.y * qvo.d[k] + lq.z * qco.d[k] + ldep * dep.d[k];
    A.lq[i] = make_float4(lin[0], lin[1], lin[2], 0.f);
    float lz = 0.f, lrho = 0.f;
    float lP = A.lP[i];
    if (pfl_raw > 1.0f) {
        lP += lin[3];
        lz += lin[3] * snd_slope(P.snd_p, P.snd_n, z);
    }
    if (rp.x > 1e-3f) lrho += lin[4];
    if (lin[5] != 0.f) atomicAdd(&A.l_rain0[cid], lin[5]);
    // EOS: p' = cs^2 clamp(rho - rho_ref(z), +-0.3 rho_ref)
    const float rref = snd_eval(P.snd_rho, P.snd_n, z).v();
    const float dref = snd_slope(P.snd_rho, P.snd_n, z);
    const float dd = rp.x - rref;
    const float c2 = P.cs * P.cs;
    if (fabsf(dd) < 0.3f * rref) {
        lrho += c2 * lP;
        lz -= c2 * dref * lP;
    } else {
        lz += (dd > 0.f ? 0.3f : -0.3f) * c2 * dref * lP;
    }
    float4 lx = A.lx[i];
    lx.z += lz;
    lx.w += lrho;
    A.lx[i] = lx;
}

// R3a: density sums of the target and the adjoint of rho = clamp(S1/S2).
__global__ void k_adj_dens_a(const Phys P, StepTape T, AdjBufs A) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const float4 xi = T.pos1[i];
    float S1 = w3(0.f), S2 = __fdividef(w3(0.f), fmaxf(xi.w, 1e-3f));   // self pair
    const int cnt = T.cnt[i];
    for (int q = 0; q < cnt; ++q) {
        const int j = T.lst[(size_t)q * P.N + i];
        const float4 xj = T.pos1[j];
        const float r2t = r2_pair(P, xi.x, xi.y, xi.z, xj.x, xj.y, xj.z);   // the density pass's own r^2
        if (r2t >= 4.f || r2t < 1e-12f) continue;
        const float qq = r2t * rsqrtf(r2t), t = 2.f - qq;
        const float W = qq < 1.f ? SIGMA_W * __fmaf_rn(qq * qq, __fmaf_rn(0.75f, qq, -1.5f), 1.f)
                                 : (0.25f * SIGMA_W) * (t * t * t);
        S1 += W;
        S2 += __fdividef(W, fmaxf(xj.w, 1e-3f));
    }
    float4 lx = A.lx[i];
    const float lrho = lx.w;
    const float rref = snd_eval(P.snd_rho, P.snd_n, xi.z).v();
    const float dref = snd_slope(P.snd_rho, P.snd_n, xi.z);
    float lS1 = 0.f, lS2 = 0.f;
    const float raw = S1 / S2;
    if (raw < 0.5f * rref) {
        lx.z += 0.5f * dref * lrho;
    } else if (raw > 2.0f * rref) {
        lx.z += 2.0f * dref * lrho;
    } else {
        lS1 = lrho / S2;
        lS2 = -lrho * raw / S2;
    }
    lx.w = 0.f;   // consumed; R3b writes dJ/drho_old here
    A.lx[i] = lx;
    A.lS[i] = make_float2(lS1, lS2);
}

// R3b: density pairs: positions and the lagged densities rho_old.
__global__ __launch_bounds__(ATPB) void k_adj_dens_b(const Phys P, StepTape T, AdjBufs A) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const float4 xi = T.pos1[i];
    const float2 lSi = A.lS[i];
    const float roi = fmaxf(xi.w, 1e-3f), iroi = __fdividef(1.f, roi);
    const float Mx = P.inv_dx * P.inv_dx, My = P.inv_dy * P.inv_dy, Mz = P.inv_dz * P.inv_dz;
    float gx = 0.f, gy = 0.f, gz = 0.f;
    float lro = lSi.y * (-w3(0.f) * iroi * iroi);   // self pair in S2_i
    const int cnt = T.cnt[i];
    for (int q = 0; q < cnt; ++q) {
        const int j = T.lst[(size_t)q * P.N + i];
        const float4 xj = T.pos1[j];
        const float2 lSj = A.lS[j];
        const float r2t = r2_pair(P, xi.x, xi.y, xi.z, xj.x, xj.y, xj.z);   // the density pass's own r^2
        if (r2t >= 4.f || r2t < 1e-12f) continue;
        const float rx = xi.x - xj.x, ry = xi.y - xj.y, rz = xi.z - xj.z;
        const float rs = rsqrtf(r2t), qq = r2t * rs, t = 2.f - qq;
        const float W = qq < 1.f ? SIGMA_W * __fmaf_rn(qq * qq, __fmaf_rn(0.75f, qq, -1.5f), 1.f)
                                 : (0.25f * SIGMA_W) * (t * t * t);
        const float kq = qq < 1.f ? SIGMA_W * __fmaf_rn(2.25f, qq, -3.f) : (-0.75f * SIGMA_W) * (t * t) * rs;
        const float iroj = __fdividef(1.f, fmaxf(xj.w, 1e-3f));
        const float c = (lSi.x + lSj.x) + lSi.y * iroj + lSj.y * iroi;
        gx += c * kq * Mx * rx;
        gy += c * kq * My * ry;
        gz += c * kq * Mz * rz;
        lro += lSj.y * (-W * iroi * iroi);   // i is a neighbour in S2_j
    }
    if (!(xi.w > 1e-3f)) lro = 0.f;
    float4 lx = A.lx[i];
    lx.x += gx; lx.y += gy; lx.z += gz; lx.w = lro;
    A.lx[i] = lx;
}

// R2: inverse of the gather new[k] = old[perm[k]].
__global__ void k_adj_unperm(const Phys P, const uint32_t* __restrict__ perm, AdjBufs A) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P.N) return;
    const uint32_t i = perm[k];
    A.px[i] = A.lx[k];
    A.pv[i] = A.lv[k];
    A.pq[i] = A.lq[k];
}

// R1: surface flux, drift, first half kick (order before the sort); writes
// the adjoint of the previous step's end state.
__global__ void k_adj_integrate(const Phys P, float dt, float Ts, float qs_sfc, StepTape T, AdjBufs A) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const float4 x0 = T.pos0[i], v0 = T.vel0[i], t0 = T.thq0[i], a0 = T.acc0[i];
    const float4 lx = A.px[i], lv = A.pv[i], lq = A.pq[i];
    const float hdt = 0.5f * dt;
    const float vzp = v0.z + a0.z * hdt;
    const float zp = x0.z + (v0.z + a0.z * hdt) * dt;
    float sz = 1.f, svz = 1.f;
    float z1 = zp;
    if (zp < 0.f) {
        z1 = -zp; sz = -1.f; svz = vzp >= 0.f ? 1.f : -1.f;    // vz = |vz|
    } else if (zp > P.lz) {
        z1 = 2.f * P.lz - zp; sz = -1.f; svz = vzp >= 0.f ? -1.f : 1.f;   // vz = -|vz|
    }
    float lth0 = lq.x, lqv0 = lq.y, lz1 = lx.z;
    const bool surf = T.surf0[i] != 0;
    if (P.surface_flux && surf && z1 < P.dz) {
        const float praw = snd_eval(P.snd_p, P.snd_n, z1).v();
        const float pf = fmaxf(praw, 1.f);
        const float Pi = powf(pf / P0, KAPPA);
        const float kth = P.c_h * P.v_bg * dt / P.dz;
        const float th1 = t0.x + kth * (Ts - t0.x * Pi);
        const float Ith = (th1 > 100.f && th1 < P.theta_cap) ? 1.f : 0.f;
        lth0 = Ith * (1.f - kth * Pi) * lq.x;
        if (praw > 1.f) lz1 += Ith * (-kth * t0.x) * (KAPPA * Pi / pf) * snd_slope(P.snd_p, P.snd_n, z1) * lq.x;
        const float kq = P.beta_moist * P.c_e * P.v_bg * dt / P.dz;
        const float qv1 = t0.y + kq * (qs_sfc - t0.y);
        const float Iq = (qv1 > 0.f && qv1 < P.qv_cap) ? 1.f : 0.f;
        lqv0 = Iq * (1.f - kq) * lq.y;
    }
    // drift x1 = x0 + dt v' (wrap: identity; z: reflection)
    const float lzp = sz * lz1;
    const float lvpx = lv.x + dt * lx.x, lvpy = lv.y + dt * lx.y, lvpz = svz * lv.z + dt * lzp;
    A.e_pos[i] = make_float4(lx.x, lx.y, lzp, lx.w);   // w: dJ/drho of the previous step's density
    A.e_vel[i] = make_float4(lvpx, lvpy, lvpz, 0.f);
    A.e_thq[i] = make_float4(lth0, lqv0, lq.z, 0.f);
    A.e_acc[i] = make_float4(hdt * lvpx, hdt * lvpy, hdt * lvpz, 0.f);
}

}  // namespace
}  // namespace asph

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
// A captured window step: its graph and the ping-pong indices it leaves.
struct AfGraph {
    cudaGraphExec_t exec = nullptr;
    int pc = 0, vc = 0, qc = 0, rc = 0;
    bool lists_valid = false;
};

struct asph_adj {
    asph_ctx* c = nullptr;
    int K = 0, every = 0, nseg = 0;
    float dt = 0.f;
    double simt0 = 0.0;
    float p_sfc = 0.f;                     // reference pressure at the surface
    int trips0 = 0;
    Phys P;                                // window physics: fixed dt, sort every step
    std::vector<asph_snapshot*> ckpt;      // segment starts
    asph_snapshot* last = nullptr;         // state after the forward
    std::vector<StepTape> tape;            // one segment
    AdjBufs A;
    std::vector<void*> mem;
    bool forward_done = false;
    // window steps as CUDA graphs, keyed by (tape slot or -1, ping-pong state); valid for the
    // window physics and the context's option epoch they were captured with
    std::map<std::pair<int, int>, AfGraph> graphs;
    Phys graphs_P;
    unsigned graphs_epoch = 0;
    void drop_graphs() {
        for (auto& kv : graphs) cudaGraphExecDestroy(kv.second.exec);
        graphs.clear();
    }
    ~asph_adj() {
        drop_graphs();
        for (auto* s : ckpt) asph_snapshot_destroy(s);
        if (last) asph_snapshot_destroy(last);
        for (void* p : mem) cudaFree(p);
    }
    template <class T>
    cudaError_t alloc(T** p, size_t bytes) {
        void* q = nullptr;
        cudaError_t e = cudaMalloc(&q, bytes < 256 ? 256 : bytes);
        if (e == cudaSuccess) {
            mem.push_back(q);
            *p = (T*)q;
        }
        return e;
    }
};

namespace {

int blocks(int n) { return (n + ATPB - 1) / ATPB; }

// One window step; with a tape, the pieces the reverse needs are copied out.
int af_step(asph_adj* a, StepTape* t) {
    asph_ctx* c = a->c;
    const Phys& P = a->P;
    Bufs& B = c->B;
    cudaStream_t s = c->stream;
    const size_t N = (size_t)P.N, C = (size_t)P.ncell;
    // the window runs without the source-term hook (its tendencies are not differentiated)
    float4* const src = B.src;
    B.src = nullptr;
#define CP_(dst, src, bytes) CKR(cudaMemcpyAsync((dst), (src), (bytes), cudaMemcpyDeviceToDevice, s))
    if (t) {
        CP_(t->pos0, B.pos[B.pc], N * 16); CP_(t->vel0, B.vel[B.vc], N * 16); CP_(t->thq0, B.thq[B.qc], N * 16);
        CP_(t->acc0, B.acc, N * 16); CP_(t->surf0, B.surf, N); CP_(t->rain0, B.rain[B.rc], C * 4);
    }
    launch_gather(P, B, G_INTEGRATE, s);   // kick, drift, flux, keys (current order)
    B.pc ^= 1; B.vc ^= 1; B.qc ^= 1;
    launch_sort_prep(P, B, 1, reads_rain(P) ? 1 : 0, s);
    launch_sort(P, B, 1, s);
    launch_gather(P, B, G_SORTED | G_FORCE, s);   // reorder, cell table, surface flags
    B.pc ^= 1; B.vc ^= 1; B.qc ^= 1;
    if (t) {
        CP_(t->perm, B.perm, N * 4);
        CP_(t->pos1, B.pos[B.pc], N * 16); CP_(t->vel1, B.vel[B.vc], N * 16); CP_(t->thq1, B.thq[B.qc], N * 16);
    }
    // a recorded step writes its neighbour lists straight into the tape
    int* const nbr = B.nbr;
    int* const nbr_cnt = B.nbr_cnt;
    if (t) { B.nbr = t->lst; B.nbr_cnt = t->cnt; }
    launch_density(P, B, s);
    if (t) {
        CP_(t->rp, B.rp, N * 8); CP_(t->thq2, B.thq[B.qc], N * 16);
        if (reads_rain(P)) CP_(t->dep, B.rain_delta, C * 4);
    }
    launch_momentum(P, B, M_INTEGRATE | M_RAIN | M_CFL, 1, s);
    B.nbr = nbr;
    B.nbr_cnt = nbr_cnt;
    B.src = src;
    B.vc ^= 1; B.rc ^= 1;
    if (t) {
        CP_(t->acc, B.acc, N * 16); CP_(t->dthdt, B.dthdt, N * 4);
        c->lists_valid = false;   // the context's own lists are from an earlier step
    }
#undef CP_
    CKR(cudaGetLastError());
    if (!t) c->lists_valid = true;
    return ASPH_OK;
}

int check_window(asph_adj* a) {
    int st = sync_status(a->c);
    if (st) return st;
    AsphControl ctl;
    st = asph_get_control(a->c, &ctl);
    if (st) return st;
    if (ctl.trips > a->trips0 || ctl.clamp_pending)
        return fail(ASPH_ERR_STATE, "a CFL trip inside the adjoint window (velocity clamp is not differentiated)");
    return ASPH_OK;
}

// One window step through its captured graph (captured on first use).
int af_step_graph(asph_adj* a, int slot) {
    asph_ctx* c = a->c;
    if (memcmp(&a->graphs_P, &a->P, sizeof(Phys)) != 0 || a->graphs_epoch != c->graph_epoch) {
        a->drop_graphs();
        a->graphs_P = a->P;
        a->graphs_epoch = c->graph_epoch;
    }
    const std::pair<int, int> key(slot, graph_slot(c->B));
    auto it = a->graphs.find(key);
    if (it == a->graphs.end()) {
        const Bufs before = c->B;
        cudaGraph_t g = nullptr;
        CKR(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        const int st = af_step(a, slot >= 0 ? &a->tape[slot] : nullptr);
        const cudaError_t e = cudaStreamEndCapture(c->stream, &g);
        AfGraph ag;
        ag.pc = c->B.pc; ag.vc = c->B.vc; ag.qc = c->B.qc; ag.rc = c->B.rc;
        ag.lists_valid = c->lists_valid;
        c->B = before;
        if (st) {
            if (g) cudaGraphDestroy(g);
            return st;
        }
        if (e != cudaSuccess) return fail(ASPH_ERR_CUDA, "adjoint graph capture: %s", cudaGetErrorString(e));
        const cudaError_t ei = cudaGraphInstantiate(&ag.exec, g, 0);
        cudaGraphDestroy(g);
        if (ei != cudaSuccess) return fail(ASPH_ERR_CUDA, "adjoint graph instantiate: %s", cudaGetErrorString(ei));
        it = a->graphs.emplace(key, ag).first;
    }
    CKR(cudaGraphLaunch(it->second.exec, c->stream));
    c->B.pc = it->second.pc; c->B.vc = it->second.vc; c->B.qc = it->second.qc; c->B.rc = it->second.rc;
    c->lists_valid = it->second.lists_valid;
    return ASPH_OK;
}

void reverse_step(asph_adj* a, StepTape& t, cudaStream_t s) {
    const Phys& P = a->P;
    AdjBufs& A = a->A;
    const float dt = a->dt;
    // surface targets of the step (asph_h100.cu:989-992), on the host
    const float rr = fminf(fmaxf((float)t.simt / P.ramp, 0.f), 1.f);
    const float Ts = P.th0 + P.dts_skin * rr * rr * (3.f - 2.f * rr);
    const float qs = qsat(Ts, a->p_sfc);
    k_adj_rain<<<blocks(P.ncell), ATPB, 0, s>>>(P, dt, t.rain0, t.dep, A.e_rain, A.l_rain0, A.l_depc,
                                                reads_rain(P) ? 1 : 0);
    k_adj_mom_seed<<<blocks(P.N), ATPB, 0, s>>>(P, dt, t, A);
    k_adj_mom_pairs<<<blocks(P.N), ATPB, 0, s>>>(P, t, A);
    k_adj_micro<<<blocks(P.N), ATPB, 0, s>>>(P, dt, t, A);
    k_adj_dens_a<<<blocks(P.N), ATPB, 0, s>>>(P, t, A);
    k_adj_dens_b<<<blocks(P.N), ATPB, 0, s>>>(P, t, A);
    k_adj_unperm<<<blocks(P.N), ATPB, 0, s>>>(P, t.perm, A);
    k_adj_integrate<<<blocks(P.N), ATPB, 0, s>>>(P, dt, Ts, qs, t, A);
    // the rain adjoint of the previous step's end
    cudaMemcpyAsync(A.e_rain, A.l_rain0, (size_t)P.ncell * 4, cudaMemcpyDeviceToDevice, s);
}

}  // namespace

extern "C" int asph_adj_create(asph_ctx* c, int nsteps, int every, asph_adj** out) {
    if (!c || !out || nsteps < 1 || every < 1) return fail(ASPH_ERR_ARG, "bad adjoint window arguments");
    *out = nullptr;
    asph_adj* a = new asph_adj();
    a->c = c;
    a->K = nsteps;
    a->every = every < nsteps ? every : nsteps;
    a->nseg = (nsteps + a->every - 1) / a->every;
    const size_t N = (size_t)c->P.N, C = (size_t)c->P.ncell;
    int st = ASPH_OK;
    for (int k = 0; k < a->nseg && !st; ++k) {
        asph_snapshot* s = nullptr;
        st = asph_snapshot_create(c, &s);
        if (!st) a->ckpt.push_back(s);
    }
    if (!st) st = asph_snapshot_create(c, &a->last);
    cudaError_t e = cudaSuccess;
    a->tape.resize(a->every);
#define AL(p, b) if (e == cudaSuccess) e = a->alloc(&(p), (b))
    for (auto& t : a->tape) {
        AL(t.pos0, N * 16); AL(t.vel0, N * 16); AL(t.thq0, N * 16); AL(t.acc0, N * 16); AL(t.surf0, N);
        AL(t.perm, N * 4); AL(t.pos1, N * 16); AL(t.vel1, N * 16); AL(t.thq1, N * 16); AL(t.rp, N * 8);
        AL(t.thq2, N * 16); AL(t.cnt, N * 4); AL(t.lst, (size_t)NBR_CAP * N * 4); AL(t.rain0, C * 4);
        AL(t.dep, C * 4); AL(t.acc, N * 16); AL(t.dthdt, N * 4);
    }
    AdjBufs& A = a->A;
    AL(A.e_pos, N * 16); AL(A.e_vel, N * 16); AL(A.e_thq, N * 16); AL(A.e_acc, N * 16); AL(A.e_rain, C * 4);
    AL(A.sF, N * 16); AL(A.sV, N * 16); AL(A.lx, N * 16); AL(A.lv, N * 16); AL(A.lq, N * 16);
    AL(A.lP, N * 4); AL(A.lS, N * 8); AL(A.l_depc, C * 4); AL(A.l_rain0, C * 4);
    AL(A.px, N * 16); AL(A.pv, N * 16); AL(A.pq, N * 16); AL(A.ab, 16); AL(A.err, 16);
#undef AL
    if (!st && e != cudaSuccess)
        st = fail(e == cudaErrorMemoryAllocation ? ASPH_ERR_NOMEM : ASPH_ERR_CUDA, "adjoint allocation: %s",
                  cudaGetErrorString(e));
    if (st) {
        delete a;
        return st;
    }
    for (auto& t : a->tape)
        if (!reads_rain(c->P)) cudaMemsetAsync(t.dep, 0, C * 4, c->stream);
    *out = a;
    return ASPH_OK;
}

extern "C" int asph_adj_destroy(asph_adj* a) {
    delete a;
    return ASPH_OK;
}

extern "C" int asph_adj_forward(asph_adj* a) {
    if (!a) return fail(ASPH_ERR_ARG, "NULL argument");
    asph_ctx* c = a->c;
    if (!c->initialised) return fail(ASPH_ERR_STATE, "adjoint forward before init/set_state");
    AsphControl ctl;
    int st = asph_get_control(c, &ctl);
    if (st) return st;
    if (ctl.clamp_pending) return fail(ASPH_ERR_STATE, "a velocity clamp is pending; step once before the window");
    a->P = c->P;
    a->P.adaptive_dt = 0;
    a->P.sort_every = 1;
    a->dt = ctl.dt;
    a->simt0 = ctl.simt;
    a->trips0 = ctl.trips;
    a->p_sfc = pres_ref(c->P, 0.f);
    for (int sgm = 0; sgm < a->nseg; ++sgm) {
        if ((st = asph_snapshot_save(c, a->ckpt[sgm]))) return st;
        const int n = (sgm == a->nseg - 1) ? a->K - sgm * a->every : a->every;
        for (int k = 0; k < n; ++k)
            if ((st = af_step_graph(a, -1))) return st;
    }
    if ((st = asph_snapshot_save(c, a->last))) return st;
    if ((st = check_window(a))) return st;
    a->forward_done = true;
    return ASPH_OK;
}

extern "C" int asph_adj_backward(asph_adj* a, const float* dL_dqc, const float* dL_dtheta, const float* dL_dxyz,
                                 float* dL_dtheta0, double* dL_dalpha_beta) {
    if (!a || !dL_dtheta0) return fail(ASPH_ERR_ARG, "NULL argument");
    if (!a->forward_done) return fail(ASPH_ERR_STATE, "adjoint backward before forward");
    asph_ctx* c = a->c;
    cudaStream_t s = c->stream;
    const Phys& P = a->P;
    const size_t N = (size_t)P.N, C = (size_t)P.ncell;
    AdjBufs& A = a->A;
    int st = ASPH_OK;
    // terminal adjoint: dL/dqc and dL/dtheta of the final state (its order)
    std::vector<float> h(N * 4, 0.f);
    for (size_t i = 0; i < N; ++i) {
        h[4 * i + 0] = dL_dtheta ? dL_dtheta[i] : 0.f;
        h[4 * i + 2] = dL_dqc ? dL_dqc[i] : 0.f;
    }
    CKR(cudaMemcpyAsync(A.e_thq, h.data(), N * 16, cudaMemcpyHostToDevice, s));
    std::vector<float> hp(N * 4, 0.f);
    if (dL_dxyz)
        for (size_t i = 0; i < N; ++i) {
            hp[4 * i + 0] = dL_dxyz[i];
            hp[4 * i + 1] = dL_dxyz[N + i];
            hp[4 * i + 2] = dL_dxyz[2 * N + i];
        }
    CKR(cudaMemcpyAsync(A.e_pos, hp.data(), N * 16, cudaMemcpyHostToDevice, s));
    CKR(cudaStreamSynchronize(s));   // the host staging vectors go out of scope below
    CKR(cudaMemsetAsync(A.e_vel, 0, N * 16, s));
    CKR(cudaMemsetAsync(A.e_acc, 0, N * 16, s));
    CKR(cudaMemsetAsync(A.e_rain, 0, C * 4, s));
    CKR(cudaMemsetAsync(A.ab, 0, 16, s));
    CKR(cudaMemsetAsync(A.err, 0, 16, s));
    for (int sgm = a->nseg - 1; sgm >= 0 && !st; --sgm) {
        const int n = (sgm == a->nseg - 1) ? a->K - sgm * a->every : a->every;
        if ((st = asph_snapshot_restore(c, a->ckpt[sgm]))) break;
        for (int k = 0; k < n && !st; ++k) {
            a->tape[k].simt = a->simt0 + (double)a->dt * (double)(sgm * a->every + k);
            st = af_step_graph(a, k);
        }
        for (int k = n - 1; k >= 0 && !st; --k) reverse_step(a, a->tape[k], s);
        CKR(cudaGetLastError());
    }
    if (st) return st;
    int err = 0;
    double ab[2];
    CKR(cudaMemcpyAsync(&err, A.err, sizeof(int), cudaMemcpyDeviceToHost, s));
    CKR(cudaMemcpyAsync(ab, A.ab, sizeof ab, cudaMemcpyDeviceToHost, s));
    CKR(cudaMemcpyAsync(h.data(), A.e_thq, N * 16, cudaMemcpyDeviceToHost, s));
    CKR(cudaStreamSynchronize(s));
    if (err) return fail(ASPH_ERR_STATE, "a neighbour list overflowed inside the adjoint window");
    for (size_t i = 0; i < N; ++i) dL_dtheta0[i] = h[4 * i];
    if (dL_dalpha_beta) {
        dL_dalpha_beta[0] = ab[0];
        dL_dalpha_beta[1] = ab[1];
    }
    // leave the context at the end of the window, as after the forward
    if ((st = asph_snapshot_restore(c, a->last))) return st;
    return sync_status(c);
}

extern "C" int asph_set_viscosity(asph_ctx* c, float alpha, float beta) {
    if (!c) return fail(ASPH_ERR_ARG, "ctx is NULL");
    c->P.alpha = alpha;
    c->P.beta = beta;
    set_viscosity_terms(c->P);
    c->prm.alpha_av = alpha;
    c->prm.beta_av = beta;
    for (auto& g : c->gexec)
        if (g) { cudaGraphExecDestroy(g); g = nullptr; }
    return ASPH_OK;
}
