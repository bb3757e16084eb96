// adjoint_host.cpp — FP64 host reference of the adjoint window.
// TEST INFRASTRUCTURE ONLY: called by the tests as the checker of the CUDA
// adjoint; nothing in the library links or calls it.
//
// The window step (the library's adjoint window, asph_adjoint.cu) written
// once, generic in the scalar type, following the reference kernels it is
// built from: kick/drift (asph_h100.cu:535-561), surface flux (606-626),
// density (286-333), EOS + saturation adjustment + autoconversion
// (340-402), momentum (415-511), theta update (562-571), second kick and
// sponge (518-544), rain sedimentation (577-599); plus the Kessler
// accretion and rain evaporation of the library (no reference code).
// Pairs: every j with q < 2 in cell units (no minimum image), self apart,
// which is exactly the set the window's neighbour lists hold.  Reference
// profiles are the analytic double functions (asph_h100.cu:136-153).
//
//   with S = double: the forward (loss for central finite differences);
//   with S = Rev: reverse-mode automatic differentiation on a tape — the
//   FP64 host adjoint (gradient of the loss with respect to the initial
//   theta of every particle and alpha, beta).
//
// Loss: L = (1/N) sum_i (qc_i - T(x_i))^2 at the end of the window, T a sum
// of Gaussians {cx, cy, cz, s_xy, s_z, amplitude}.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../include/asph.h"

namespace {

// ---------------------------------------------------------------------------
// reverse-mode tape
// ---------------------------------------------------------------------------
struct Tape {
    std::vector<int> pa, pb;
    std::vector<double> da, db;
    int nvars = 0;
    int add(int a, double x, int b, double y) {
        pa.push_back(a); da.push_back(x); pb.push_back(b); db.push_back(y);
        return (int)pa.size() - 1;
    }
};
Tape* g_tape = nullptr;

struct Rev {
    double v = 0.0;
    int id = -1;   // -1: constant
    Rev() = default;
    Rev(double x) : v(x), id(-1) {}
};
inline Rev node(double v, int a, double x, int b = -1, double y = 0.0) {
    Rev r;
    r.v = v;
    if (a < 0 && b < 0) return r;
    if (a < 0) { a = b; x = y; b = -1; y = 0.0; }
    r.id = g_tape->add(a, x, b, y);
    return r;
}
inline Rev var(double v) {
    Rev r;
    r.v = v;
    r.id = g_tape->add(-1, 0.0, -1, 0.0);
    return r;
}
inline Rev operator+(const Rev& a, const Rev& b) { return node(a.v + b.v, a.id, 1.0, b.id, 1.0); }
inline Rev operator-(const Rev& a, const Rev& b) { return node(a.v - b.v, a.id, 1.0, b.id, -1.0); }
inline Rev operator*(const Rev& a, const Rev& b) { return node(a.v * b.v, a.id, b.v, b.id, a.v); }
inline Rev operator/(const Rev& a, const Rev& b) {
    const double q = a.v / b.v;
    return node(q, a.id, 1.0 / b.v, b.id, -q / b.v);
}
inline Rev operator-(const Rev& a) { return node(-a.v, a.id, -1.0); }
inline Rev& operator+=(Rev& a, const Rev& b) { return a = a + b; }
inline Rev& operator-=(Rev& a, const Rev& b) { return a = a - b; }
inline Rev exp(const Rev& a) {
    const double e = std::exp(a.v);
    return node(e, a.id, e);
}
inline Rev pow(const Rev& a, double c) {
    const double p = std::pow(a.v, c);
    return node(p, a.id, a.v != 0.0 ? c * p / a.v : 0.0);
}
inline Rev sqrt(const Rev& a) {
    const double s = std::sqrt(a.v);
    return node(s, a.id, s > 0.0 ? 0.5 / s : 0.0);
}
inline Rev fabs(const Rev& a) { return a.v >= 0.0 ? a : -a; }
inline double val(double a) { return a; }
inline double val(const Rev& a) { return a.v; }
template <class S> inline S smin(const S& a, const S& b) { return val(a) < val(b) ? a : b; }
template <class S> inline S smax(const S& a, const S& b) { return val(a) > val(b) ? a : b; }
inline double exp_(double a) { return std::exp(a); }
inline Rev exp_(const Rev& a) { return exp(a); }
inline double pow_(double a, double c) { return std::pow(a, c); }
inline Rev pow_(const Rev& a, double c) { return pow(a, c); }
inline double sqrt_(double a) { return std::sqrt(a); }
inline Rev sqrt_(const Rev& a) { return sqrt(a); }
inline double abs_(double a) { return std::fabs(a); }
inline Rev abs_(const Rev& a) { return fabs(a); }

constexpr double GRAV = 9.80665, RD = 287.05, CPD = 1004.0, P0 = 100000.0, LV = 2.501e6;
constexpr double SIGMA = 0.31830988618379067, KAPPA = RD / CPD;

// ---------------------------------------------------------------------------
// the window step, generic in S
// ---------------------------------------------------------------------------
template <class S>
struct Window {
    const AsphParams& p;
    int N, nx, ny, nz, nxy, ncell;
    double dx, dy, dz, lx, ly, lz, vcell, pmass, mm, hav, eta2, aex, dt;
    S alpha, beta;
    bool reads;

    Window(const AsphParams& prm, double dt_) : p(prm) {
        N = p.n_particles; nx = p.nx; ny = p.ny; nz = p.nz; nxy = nx * ny; ncell = nxy * nz;
        dx = p.dx; dy = p.dy; dz = p.dz;
        lx = nx * dx; ly = ny * dy; lz = nz * dz;
        vcell = dx * dy * dz;
        const double rho0 = P0 / (RD * p.th0);
        // the library's particle mass rounds through float
        const float base = (float)(100000.0f / (287.05f * p.th0)) * (float)(p.dx * p.dy * p.dz);
        pmass = p.pmass > 0.f ? p.pmass
                              : (N == ncell ? (double)base : (double)(float)((double)base * ncell / N));
        (void)rho0;
        mm = pmass / vcell;
        hav = p.h_av > 0.f ? p.h_av : 2.0 * p.dz;
        eta2 = (0.01 * hav) * (0.01 * hav);
        aex = GRAV * GRAV / (CPD * p.th0 * p.n2);
        dt = dt_;
        reads = p.accretion || p.rain_evap;
    }
    // reference sounding (analytic, double)
    template <class T> T th_ref(const T& z) const { return p.th0 * exp_(z * (p.n2 / GRAV)); }
    template <class T> T ex_ref(const T& z) const { return 1.0 - aex * (1.0 - exp_(z * (-p.n2 / GRAV))); }
    template <class T> T pres_ref(const T& z) const { return P0 * pow_(ex_ref(z), CPD / RD); }
    template <class T> T rho_ref(const T& z) const { return pres_ref(z) / (RD * th_ref(z) * ex_ref(z)); }
    template <class T> static T esat(const T& Tk) {
        const T tc = Tk - 273.15;
        return 611.2 * exp_(17.67 * tc / (tc + 243.5));
    }
    template <class T> static T qsat(const T& Tk, const T& pp) {
        const T es = smin(esat(Tk), 0.5 * pp);
        const T den = pp - 0.378 * es;
        return val(den) > 1.0 ? 0.622 * es / den : T(0.0);
    }
    template <class T> static T dqsdT(const T& Tk, const T& es, const T& pp) {
        const T tc = Tk - 273.15;
        const T d = tc + 243.5;
        const T desdT = es * (17.67 * 243.5) / (d * d);
        const T den = pp - 0.378 * es;
        return 0.622 * pp * desdT / (den * den);
    }
    template <class T> T qv_ref(const T& z) const {
        if (p.qv_mode == ASPH_QV_REFERENCE) {
            const T q = p.qv0 * exp_(z * (-1.0 / 2500.0));
            const T d = smax(z - 5000.0, T(0.0));
            return q * exp_(d * (-1.0 / 1000.0));
        }
        const T pi = ex_ref(z);
        const T Tk = th_ref(z) * pi;
        const T pp = P0 * pow_(pi, CPD / RD);
        const double rh = val(z) < p.z_bl ? p.rh_bl : p.rh;
        return rh * qsat(Tk, pp);
    }
    template <class T> T thvr(const T& z) const { return th_ref(z) * (1.0 + 0.608 * qv_ref(z)); }

    static double w3(double q) {
        if (q >= 2.0) return 0.0;
        if (q < 1.0) return SIGMA * (1.0 - 1.5 * q * q + 0.75 * q * q * q);
        const double t = 2.0 - q;
        return 0.25 * SIGMA * t * t * t;
    }
    static S w3s(const S& q) {
        if (val(q) < 1.0) return SIGMA * (1.0 - 1.5 * q * q + 0.75 * q * q * q);
        const S t = 2.0 - q;
        return 0.25 * SIGMA * t * t * t;
    }
    static S dw3s(const S& q) {
        if (val(q) < 1.0) return SIGMA * (-3.0 * q + 2.25 * q * q);
        const S t = 2.0 - q;
        return -0.75 * SIGMA * t * t;
    }
    int cell(double x, double y, double z) const {
        auto ci = [](double v, double d, int n) {
            int k = (int)std::floor(v / d);
            return k < 0 ? 0 : (k > n - 1 ? n - 1 : k);
        };
        return (ci(z, dz, nz) * ny + ci(y, dy, ny)) * nx + ci(x, dx, nx);
    }

    struct State {
        std::vector<S> x, y, z, u, v, w, th, qv, qc, rho, ax, ay, az, rain;
        double simt;
    };

    // pairs i < j with q < 2 (cell units, raw differences)
    void pairs(const State& s, std::vector<std::pair<int, int>>& out) const {
        out.clear();
        std::vector<std::vector<int>> bins(ncell);
        for (int i = 0; i < N; ++i) bins[cell(val(s.x[i]), val(s.y[i]), val(s.z[i]))].push_back(i);
        for (int i = 0; i < N; ++i) {
            const double xi = val(s.x[i]), yi = val(s.y[i]), zi = val(s.z[i]);
            const int c = cell(xi, yi, zi);
            const int cx = c % nx, cy = (c / nx) % ny, cz = c / nxy;
            for (int kz = std::max(cz - 2, 0); kz <= std::min(cz + 2, nz - 1); ++kz)
                for (int ky = std::max(cy - 2, 0); ky <= std::min(cy + 2, ny - 1); ++ky)
                    for (int kx = std::max(cx - 2, 0); kx <= std::min(cx + 2, nx - 1); ++kx)
                        for (int j : bins[(kz * ny + ky) * nx + kx]) {
                            if (j <= i) continue;
                            const double a = (xi - val(s.x[j])) / dx, b = (yi - val(s.y[j])) / dy,
                                         d = (zi - val(s.z[j])) / dz;
                            const double r2 = a * a + b * b + d * d;
                            if (r2 < 4.0 && r2 >= 1e-12) out.push_back({i, j});
                        }
        }
    }

    // microphysics of one particle (asph_h100.cu:362-402 + Kessler terms)
    void micro(S& th, S& qv, S& qc, const S& pfl, const S& r, const S& R, S& dep) const {
        const S Pi = pow_(pfl / P0, KAPPA);
        S T = th * Pi;
        const S qs = qsat(T, pfl);
        if (val(qv) > val(qs) || val(qc) > 0.0) {
            S dqc(0.0);
            for (int it = 0; it < 3; ++it) {
                const S Tn = T + (LV / CPD) * dqc;
                const S esn = esat(Tn);
                const S qsn = qsat(Tn, pfl);
                const S f = qv - dqc - qsn;
                const S fp = -1.0 - dqsdT(Tn, esn, pfl) * (LV / CPD);
                dqc = dqc - f / fp;
                dqc = smin(dqc, qv);
                dqc = smax(dqc, -qc);
            }
            qv = qv - dqc;
            qc = qc + dqc;
            th = th + LV * dqc / (CPD * Pi);
            T = T + (LV / CPD) * dqc;
        }
        dep = S(0.0);
        if (val(qc) > p.qc_auto) {
            const S dqr = (qc - (double)p.qc_auto) * (1.0 - std::exp(-(double)p.rate_auto * dt));
            qc = qc - dqr;
            dep = dep + dqr;
        }
        if (reads) {
            const S qr = smax(R, S(0.0)) / (r * vcell);
            if (p.accretion && val(qc) > 0.0 && val(qr) > 0.0) {
                const S dqa = smin(qc, dt * p.k_accr * qc * pow_(qr, 0.875));
                qc = qc - dqa;
                dep = dep + dqa;
            }
            if (p.rain_evap && val(qr) > 0.0) {
                const S qvs = qsat(T, pfl);
                if (val(qv) < val(qvs) && val(qvs) > 0.0) {
                    const S rq = 1e-3 * r * qr;
                    const S C = 1.6 + 124.9 * pow_(rq, 0.2046);
                    const S er = (1.0 - qv / qvs) * C * pow_(rq, 0.525) /
                                 (1e-3 * r * (5.4e5 + 2.55e6 / (0.01 * pfl * qvs)));
                    const S dqe = smin(qr, smin(dt * er, qvs - qv));
                    qv = qv + dqe;
                    th = th - LV * dqe / (CPD * Pi);
                    dep = dep - dqe;
                }
            }
        }
        th = smin(smax(th, S(100.0)), S((double)p.theta_cap));
        qv = smin(smax(qv, S(0.0)), S((double)p.qv_cap));
        qc = smax(qc, S(0.0));
    }

    void step(State& s) const {
        const double h = 0.5 * dt;
        // surface flags at the step start (the last sort's lowest layer)
        std::vector<char> surf(N);
        for (int i = 0; i < N; ++i) surf[i] = (int)std::floor(val(s.z[i]) / dz) == 0;
        // kick, drift, flux
        const double rr = std::min(std::max(s.simt / p.ramp, 0.0), 1.0);
        const double Ts = p.th0 + p.dts_skin * rr * rr * (3.0 - 2.0 * rr);
        const double qs_sfc = val(qsat(S(Ts), S(pres_ref(0.0))));
        for (int i = 0; i < N; ++i) {
            S u = s.u[i] + h * s.ax[i], v = s.v[i] + h * s.ay[i], w = s.w[i] + h * s.az[i];
            S x = s.x[i] + dt * u, y = s.y[i] + dt * v, z = s.z[i] + dt * w;
            for (int k = 0; k < 64 && val(x) < 0.0; ++k) x = x + lx;
            for (int k = 0; k < 64 && val(x) >= lx; ++k) x = x - lx;
            for (int k = 0; k < 64 && val(y) < 0.0; ++k) y = y + ly;
            for (int k = 0; k < 64 && val(y) >= ly; ++k) y = y - ly;
            if (val(z) < 0.0) { z = -z; w = abs_(w); }
            if (val(z) > lz) { z = 2.0 * lz - z; w = -abs_(w); }
            if (p.surface_flux && surf[i] && val(z) < dz) {
                const S Pi = pow_(smax(pres_ref(z), S(1.0)) / P0, KAPPA);
                S th = s.th[i] + p.c_h * p.v_bg * (Ts - s.th[i] * Pi) * dt / dz;
                S qv = s.qv[i] + p.beta_moist * p.c_e * p.v_bg * (qs_sfc - s.qv[i]) * dt / dz;
                s.th[i] = smin(smax(th, S(100.0)), S((double)p.theta_cap));
                s.qv[i] = smin(smax(qv, S(0.0)), S((double)p.qv_cap));
            }
            s.x[i] = x; s.y[i] = y; s.z[i] = z; s.u[i] = u; s.v[i] = v; s.w[i] = w;
        }
        std::vector<std::pair<int, int>> pr;
        pairs(s, pr);
        // density (self + pairs), EOS
        std::vector<S> S1(N), S2(N);
        for (int i = 0; i < N; ++i) {
            S1[i] = S(SIGMA);
            S2[i] = SIGMA / smax(s.rho[i], S(1e-3));
        }
        for (auto& e : pr) {
            const int i = e.first, j = e.second;
            const S a = (s.x[i] - s.x[j]) / dx, b = (s.y[i] - s.y[j]) / dy, d = (s.z[i] - s.z[j]) / dz;
            const S W = w3s(sqrt_(a * a + b * b + d * d));
            S1[i] += W; S1[j] += W;
            S2[i] += W / smax(s.rho[j], S(1e-3));
            S2[j] += W / smax(s.rho[i], S(1e-3));
        }
        std::vector<S> rho(N), prs(N), dep(N);
        std::vector<S> delta(reads ? ncell : 0, S(0.0));
        for (int i = 0; i < N; ++i) {
            const S rref = rho_ref(s.z[i]);
            const S raw = S1[i] / S2[i];
            const S rh = smin(smax(raw, 0.5 * rref), 2.0 * rref);
            S dd = rh - rref;
            dd = smin(smax(dd, -0.3 * rref), 0.3 * rref);
            rho[i] = rh;
            prs[i] = p.cs * p.cs * dd;
        }
        for (int i = 0; i < N; ++i) {
            const int c = cell(val(s.x[i]), val(s.y[i]), val(s.z[i]));
            const S pfl = smax(pres_ref(s.z[i]) + prs[i], S(1.0));
            const S r = smax(rho[i], S(1e-3));
            const S R = reads ? s.rain[c] : S(0.0);
            micro(s.th[i], s.qv[i], s.qc[i], pfl, r, R, dep[i]);
            if (reads) delta[c] += dep[i] * pmass;
            else s.rain[c] += dep[i] * pmass;
        }
        // momentum
        std::vector<S> fx(N, S(0.0)), fy(N, S(0.0)), fz(N, S(0.0)), vx(N, S(0.0)), vy(N, S(0.0)), vz(N, S(0.0));
        auto term = [&](int i, int j) {
            const S rx = s.x[i] - s.x[j], ry = s.y[i] - s.y[j], rz = s.z[i] - s.z[j];
            const S a = rx / dx, b = ry / dy, d = rz / dz;
            const S q = sqrt_(a * a + b * b + d * d);
            const S kq = dw3s(q) / q;
            const S gx = kq * a / dx, gy = kq * b / dy, gz = kq * d / dz;
            const S ri = smax(rho[i], S(1e-3)), rj = smax(rho[j], S(1e-3));
            const S dp = (prs[j] - prs[i]) / (ri * rj);
            const S sdot = (s.u[i] - s.u[j]) * rx + (s.v[i] - s.v[j]) * ry + (s.w[i] - s.w[j]) * rz;
            S visc(0.0);
            if (val(sdot) < 0.0) {
                const S den = rx * rx + ry * ry + rz * rz + eta2;
                const S mu = hav * sdot / den;
                const S rbar = 0.5 * (ri + rj);
                visc = (-1.0 * alpha * p.cs * mu + beta * mu * mu) / (rj * rbar * rbar);
            }
            const S br = dp + visc;
            fx[i] -= br * gx; fy[i] -= br * gy; fz[i] -= br * gz;
            vx[i] -= visc * gx; vy[i] -= visc * gy; vz[i] -= visc * gz;
        };
        for (auto& e : pr) {
            term(e.first, e.second);
            term(e.second, e.first);
        }
        const double hcap = p.dthdt_cap;
        const double zs = (1.0 - p.sponge_frac) * lz;
        for (int i = 0; i < N; ++i) {
            const S ax = mm * fx[i], ay = mm * fy[i];
            const S tv = thvr(s.z[i]);
            const S az = mm * fz[i] + GRAV * ((s.th[i] * (1.0 + 0.608 * s.qv[i]) - tv) / tv - s.qc[i]);
            const S Pi = pow_(smax(pres_ref(s.z[i]) + prs[i], S(1.0)) / P0, KAPPA);
            S dth = -1.0 * (s.u[i] * (mm * vx[i]) + s.v[i] * (mm * vy[i]) + s.w[i] * (mm * vz[i])) / (CPD * Pi);
            dth = smin(smax(dth, S(-hcap)), S(hcap));
            s.th[i] = smin(smax(s.th[i] + dth * dt, S(100.0)), S((double)p.theta_cap));
            S un = s.u[i] + ax * h, vn = s.v[i] + ay * h, wn = s.w[i] + az * h;
            if (val(s.z[i]) >= zs) {
                const S tt = (s.z[i] - zs) / (p.sponge_frac * lz);
                const S sg = p.sponge_sigma * tt * tt;
                wn = wn * (1.0 / (1.0 + sg * dt));
            }
            s.u[i] = un; s.v[i] = vn; s.w[i] = wn;
            s.ax[i] = ax; s.ay[i] = ay; s.az[i] = az;
            s.rho[i] = rho[i];
        }
        // rain sedimentation
        double f = p.v_rain * dt / dz;
        if (f > 1.0) f = 1.0;
        std::vector<S> cur(ncell), out(ncell);
        for (int c = 0; c < ncell; ++c) cur[c] = reads ? smax(s.rain[c] + delta[c], S(0.0)) : s.rain[c];
        for (int c = 0; c < ncell; ++c) {
            const int iz = c / nxy;
            out[c] = cur[c] * (1.0 - f);
            if (iz < nz - 1) out[c] += cur[c + nxy] * f;
        }
        s.rain.swap(out);
        s.simt += dt;
    }

    S target(const double* g, int ng, const S& x, const S& y, const S& z) const {
        S t(0.0);
        for (int k = 0; k < ng; ++k) {
            const double* q = g + 6 * k;
            const S ex = ((x - q[0]) * (x - q[0]) + (y - q[1]) * (y - q[1])) / (-2.0 * q[3] * q[3]) +
                         (z - q[2]) * (z - q[2]) / (-2.0 * q[4] * q[4]);
            t += q[5] * exp_(ex);
        }
        return t;
    }

    S loss(const State& s, const double* g, int ng) const {
        S L(0.0);
        for (int i = 0; i < N; ++i) {
            const S d = s.qc[i] - target(g, ng, s.x[i], s.y[i], s.z[i]);
            L += d * d;
        }
        return L / (double)N;
    }
};

template <class S>
typename Window<S>::State load(const Window<S>& W, const double* st, const double* rain, double simt,
                               const double* theta0) {
    typename Window<S>::State s;
    const int N = W.N;
    std::vector<S>* f[13] = {&s.x, &s.y, &s.z, &s.u, &s.v, &s.w, &s.th, &s.qv, &s.qc, &s.rho, &s.ax, &s.ay, &s.az};
    for (int k = 0; k < 13; ++k) {
        f[k]->resize(N);
        for (int i = 0; i < N; ++i) (*f[k])[i] = S(st[(size_t)k * N + i]);
    }
    if (theta0)
        for (int i = 0; i < N; ++i) s.th[i] = S(theta0[i]);
    s.rain.resize(W.ncell);
    for (int c = 0; c < W.ncell; ++c) s.rain[c] = S(rain[c]);
    s.simt = simt;
    return s;
}

}  // namespace

extern "C" {

// Loss after nsteps window steps in FP64.  state: 13 x N SoA (x y z u v w th
// qv qc rho ax ay az), rain: nx*ny*nz.  alpha_beta overrides the viscosity
// coefficients; final (may be NULL) receives the final 13 x N state.
int adj_host_loss(const AsphParams* p, const double* state, const double* rain, double simt, double dt, int nsteps,
                  const double* alpha_beta, const double* gauss, int ngauss, double* L, double* final_state) {
    Window<double> W(*p, dt);
    W.alpha = alpha_beta[0];
    W.beta = alpha_beta[1];
    auto s = load(W, state, rain, simt, nullptr);
    for (int k = 0; k < nsteps; ++k) W.step(s);
    *L = W.loss(s, gauss, ngauss);
    if (final_state) {
        std::vector<double>* f[13] = {&s.x, &s.y, &s.z, &s.u, &s.v, &s.w, &s.th, &s.qv, &s.qc, &s.rho, &s.ax, &s.ay, &s.az};
        for (int k = 0; k < 13; ++k)
            std::memcpy(final_state + (size_t)k * W.N, f[k]->data(), sizeof(double) * W.N);
    }
    return 0;
}

// Gradient of the same loss by reverse-mode differentiation of the FP64
// window: dL/dtheta0[N], dL/dalpha, dL/dbeta.  Returns the tape length.
long adj_host_grad(const AsphParams* p, const double* state, const double* rain, double simt, double dt, int nsteps,
                   const double* alpha_beta, const double* gauss, int ngauss, double* L, double* dtheta0,
                   double* dalpha_beta) {
    Tape tape;
    g_tape = &tape;
    Window<Rev> W(*p, dt);
    const int N = W.N;
    std::vector<double> th0(N);
    for (int i = 0; i < N; ++i) th0[i] = state[(size_t)6 * N + i];
    auto s = load(W, state, rain, simt, nullptr);
    std::vector<int> ids(N);
    for (int i = 0; i < N; ++i) {
        s.th[i] = var(th0[i]);
        ids[i] = s.th[i].id;
    }
    W.alpha = var(alpha_beta[0]);
    W.beta = var(alpha_beta[1]);
    const int ida = W.alpha.id, idb = W.beta.id;
    for (int k = 0; k < nsteps; ++k) W.step(s);
    Rev J = W.loss(s, gauss, ngauss);
    *L = J.v;
    std::vector<double> adj(tape.pa.size(), 0.0);
    if (J.id >= 0) adj[J.id] = 1.0;
    for (long n = (long)tape.pa.size() - 1; n >= 0; --n) {
        const double g = adj[n];
        if (g == 0.0) continue;
        if (tape.pa[n] >= 0) adj[tape.pa[n]] += g * tape.da[n];
        if (tape.pb[n] >= 0) adj[tape.pb[n]] += g * tape.db[n];
    }
    for (int i = 0; i < N; ++i) dtheta0[i] = adj[ids[i]];
    dalpha_beta[0] = adj[ida];
    dalpha_beta[1] = adj[idb];
    g_tape = nullptr;
    return (long)tape.pa.size();
}

}  // extern "C"
