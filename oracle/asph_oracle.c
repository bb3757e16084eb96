/*
 * asph_oracle.c — CPU restatement of the reference algorithm (FP64).
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA path
 * and the timed CPU baseline; the product never links, loads or calls it.
 *
 * It restates, block by block, the hot path of Forbu/sph_cuda
 * asph_h100.cu, with the reference's constexpr parameters taken from an
 * AsphParams struct (include/asph.h).  Arithmetic is double precision,
 * except the integer quantities the reference derives from float32
 * products (cell indices, Morton keys, the surface-layer test), which are
 * computed from the float32 value of the position with one rounded float
 * multiply, exactly as the reference does, so that keys, permutations and
 * cell tables can be compared bit for bit.
 *
 * Stage functions take double arrays (a float32 state converts exactly)
 * and are parallelised with OpenMP over particles; accumulations into
 * cells are done serially in index order so every result is deterministic.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "../include/asph.h"

/* asph_h100.cu:66-70 */
#define GRAV 9.80665
#define R_D 287.05
#define CP 1004.0
#define P0 100000.0
#define L_V 2.501e6
#define SIGMA_W 0.31830988618   /* asph_h100.cu:56 */
#define STENCIL 2               /* asph_h100.cu:54 */

typedef struct {
    int nx, ny, nz, nxy, N, ncell;
    float inv_dx_f, inv_dy_f, inv_dz_f; /* 1.0f/dx rounded in float (asph_h100.cu:49) */
    double dx, dy, dz, lx, ly, lz, v_cell;
    double th0, n2, cs, a_exner;
    int qv_mode;
    double qv0, rh, rh_bl, z_bl;
    double alpha, beta, h_av, eta2, sponge_sigma, sponge_frac, dthdt_cap;
    int surface_flux;
    double c_h, c_e, beta_moist, v_bg, dts_skin, ramp;
    double qc_auto, rate_auto, v_rain, theta_cap, qv_cap;
    int accretion, rain_evap;
    double k_accr;
    double pmass, mm;
    double cfl, dt_cap, dt_floor, dt_static;
    int max_trip, strict_cfl, adaptive_dt, sort_every, permute_acc, key_bits;
} OP;

static int ceil_log2(int n) { int b = 1; while ((1 << b) < n) ++b; return b; } /* asph_h100.cu:865 */

static void derive(const AsphParams* p, OP* o) {
    memset(o, 0, sizeof(*o));
    o->nx = p->nx; o->ny = p->ny; o->nz = p->nz; o->nxy = p->nx * p->ny;
    o->N = p->n_particles; o->ncell = p->nx * p->ny * p->nz;
    o->inv_dx_f = 1.0f / p->dx; o->inv_dy_f = 1.0f / p->dy; o->inv_dz_f = 1.0f / p->dz;
    o->dx = p->dx; o->dy = p->dy; o->dz = p->dz;
    /* the box edges are float products in the reference (asph_h100.cu:792) */
    o->lx = (double)((float)p->nx * p->dx); o->ly = (double)((float)p->ny * p->dy);
    o->lz = (double)((float)p->nz * p->dz);
    o->v_cell = o->dx * o->dy * o->dz;
    o->th0 = p->th0; o->n2 = p->n2; o->cs = p->cs;
    o->a_exner = GRAV * GRAV / (CP * o->th0 * o->n2);       /* asph_h100.cu:140 */
    o->qv_mode = p->qv_mode; o->qv0 = p->qv0; o->rh = p->rh; o->rh_bl = p->rh_bl; o->z_bl = p->z_bl;
    o->alpha = p->alpha_av; o->beta = p->beta_av;
    o->h_av = p->h_av > 0.f ? p->h_av : 2.0 * o->dz;         /* asph_h100.cu:85 */
    o->eta2 = (0.01 * o->h_av) * (0.01 * o->h_av);           /* asph_h100.cu:482 */
    o->sponge_sigma = p->sponge_sigma; o->sponge_frac = p->sponge_frac; o->dthdt_cap = p->dthdt_cap;
    o->surface_flux = p->surface_flux;
    o->c_h = p->c_h; o->c_e = p->c_e; o->beta_moist = p->beta_moist; o->v_bg = p->v_bg;
    o->dts_skin = p->dts_skin; o->ramp = p->ramp;
    o->qc_auto = p->qc_auto; o->rate_auto = p->rate_auto; o->v_rain = p->v_rain;
    o->theta_cap = p->theta_cap; o->qv_cap = p->qv_cap;
    o->accretion = p->accretion; o->rain_evap = p->rain_evap; o->k_accr = p->k_accr;
    {
        double rho0 = P0 / (R_D * o->th0);                   /* asph_h100.cu:75 */
        o->pmass = p->pmass > 0.f ? (double)p->pmass : rho0 * o->lx * o->ly * o->lz / (double)o->N;
        o->mm = o->pmass / o->v_cell;                         /* asph_h100.cu:497 */
    }
    o->cfl = p->cfl;
    o->dt_static = (double)(p->cfl * fminf(fminf(p->dx, p->dy), p->dz) / p->cs);  /* asph_h100.cu:794 */
    o->dt_cap = p->dt_request > 0.f ? fmin((double)p->dt_request, o->dt_static) : o->dt_static;
    o->dt_floor = 0.05 * o->dt_cap;
    o->max_trip = p->max_trip; o->strict_cfl = p->strict_cfl; o->adaptive_dt = p->adaptive_dt;
    o->sort_every = p->sort_every; o->permute_acc = p->permute_acc;
    {
        int m = p->nx > p->ny ? p->nx : p->ny;
        m = m > p->nz ? m : p->nz;
        o->key_bits = 3 * ceil_log2(m);                        /* asph_h100.cu:866-868 */
    }
}

/* ---- SPH kernel, asph_h100.cu:125-134 ------------------------------------ */
static double w3(double q) {
    if (q >= 2.0) return 0.0;
    if (q < 1.0) return SIGMA_W * (1.0 - 1.5 * q * q + 0.75 * q * q * q);
    double t = 2.0 - q;
    return 0.25 * SIGMA_W * t * t * t;
}
static double dw3(double q) {
    if (q >= 2.0) return 0.0;
    if (q < 1.0) return SIGMA_W * (-3.0 * q + 2.25 * q * q);
    double t = 2.0 - q;
    return -0.75 * SIGMA_W * t * t;
}

/* ---- reference state, asph_h100.cu:136-153 -------------------------------- */
static double theta_ref(const OP* o, double z) { return o->th0 * exp(o->n2 * z / GRAV); }
static double exner_ref(const OP* o, double z) { return 1.0 - o->a_exner * (1.0 - exp(-o->n2 * z / GRAV)); }
static double pres_ref(const OP* o, double z) { return P0 * pow(exner_ref(o, z), CP / R_D); }
static double rho_ref(const OP* o, double z) {
    return pres_ref(o, z) / (R_D * theta_ref(o, z) * exner_ref(o, z));
}
/* ---- thermodynamics, asph_h100.cu:155-171 --------------------------------- */
static double esat(double T) { double Tc = T - 273.15; return 611.2 * exp(17.67 * Tc / (Tc + 243.5)); }
static double qsat(double T, double p) {
    double es = fmin(esat(T), 0.5 * p);
    double den = p - 0.378 * es;
    return den > 1.0 ? 0.622 * es / den : 0.0;
}
static double dqsdT(double T, double es, double p) {
    double Tc = T - 273.15, d = Tc + 243.5;
    double desdT = es * (17.67 * 243.5) / (d * d);
    double den = p - 0.378 * es;
    return 0.622 * p * desdT / (den * den);
}
static double qv_ref(const OP* o, double z) {
    if (o->qv_mode == ASPH_QV_REFERENCE) {                     /* asph_h100.cu:149-153 */
        double q = o->qv0 * exp(-z / 2500.0);
        double d = fmax(z - 5000.0, 0.0);
        return q * exp(-d / 1000.0);
    }
    {
        double pi = exner_ref(o, z), T = theta_ref(o, z) * pi, p = P0 * pow(pi, CP / R_D);
        double rh = z < o->z_bl ? o->rh_bl : o->rh;
        return rh * qsat(T, p);
    }
}

/* ---- hashing, asph_h100.cu:176-198 ---------------------------------------- */
static uint32_t part1by2_10(uint32_t n) {
    n &= 0x000003ffu;
    n = (n ^ (n << 16)) & 0xff0000ffu;
    n = (n ^ (n << 8)) & 0x0300f00fu;
    n = (n ^ (n << 4)) & 0x030c30c3u;
    n = (n ^ (n << 2)) & 0x09249249u;
    return n;
}
static uint32_t morton3(uint32_t x, uint32_t y, uint32_t z) {
    return part1by2_10(x) | (part1by2_10(y) << 1) | (part1by2_10(z) << 2);
}
/* (int)(p.x*INV_DX) clamped (asph_h100.cu:236-238): one float multiply of the
 * float32 position; identical to floorf() + clamp of cell_of for x >= 0. */
static int cell1(double x, float inv, int n) {
    float s = (float)x * inv;
    int c;
    if (!(s > -2147483520.0f)) c = INT32_MIN;      /* NaN / huge negative */
    else if (s > 2147483520.0f) c = INT32_MAX;
    else c = (int)s;
    return c < 0 ? 0 : (c > n - 1 ? n - 1 : c);
}
static float hash_noise(int i, int j, int k) {   /* asph_h100.cu:187-192 */
    uint32_t h = (uint32_t)i * 374761393u + (uint32_t)j * 668265263u + (uint32_t)k * 2246822519u;
    h = (h ^ (h >> 13)) * 1274126177u;
    h ^= h >> 16;
    return (float)(h & 0x00ffffffu) * (1.0f / 16777215.0f) - 0.5f;
}
static int wrapi(int i, int n) { i %= n; return i < 0 ? i + n : i; }   /* asph_h100.cu:199-200 */

/* ========================================================================= */
/* exported stages                                                            */
/* ========================================================================= */
int or_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
void or_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int or_key_bits(const AsphParams* p) { OP o; derive(p, &o); return o.key_bits; }

/* Reference init lattice (asph_h100.cu:210-227).  Hash noise is bit exact;
 * the analytic profiles are evaluated in double. */
int or_init_reference(const AsphParams* p, double* x, double* y, double* z, double* th, double* qv, double* rho) {
    OP o; derive(p, &o);
    if (o.N != o.ncell) return ASPH_ERR_CONFIG;
    #pragma omp parallel for schedule(static)
    for (int i = 0; i < o.N; ++i) {
        int ix = i % o.nx, iy = (i / o.nx) % o.ny, iz = i / (o.nx * o.ny);
        double zz = (double)((iz + 0.5f) * (float)o.dz);
        x[i] = (double)((ix + 0.5f) * (float)o.dx);
        y[i] = (double)((iy + 0.5f) * (float)o.dy);
        z[i] = zz;
        th[i] = theta_ref(&o, zz) + (double)p->noise * (double)hash_noise(ix, iy, iz);
        qv[i] = fmax(qv_ref(&o, zz) * (1.0 + 0.02 * (double)hash_noise(ix + 17, iy + 31, iz + 7)), 0.0);
        rho[i] = rho_ref(&o, zz);
    }
    return 0;
}

/* Counter-based generator of the lattice init: splitmix64 finaliser over
 * (seed, particle, stream), 24-bit uniforms (same integer recipe as the
 * CUDA init, so the jitter and noise draws are the same numbers). */
static uint64_t mix64(uint64_t z) {
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
static double uniform24(uint32_t seed, uint32_t i, uint32_t stream) {
    uint64_t h = mix64(((uint64_t)seed << 32) ^ mix64(((uint64_t)stream << 40) ^ (uint64_t)i));
    return (double)(uint32_t)(h >> 40) / 16777216.0;
}
static double normal01(uint32_t seed, uint32_t i, uint32_t stream) {
    double u1 = uniform24(seed, i, 2u * stream) + 0.5 / 16777216.0;
    double u2 = uniform24(seed, i, 2u * stream + 1u);
    return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

/* Jittered-lattice init with Gaussian warm bubbles and Gaussian theta noise
 * (no counterpart in the reference, which only has the cell-centre lattice).
 * Positions are float32 values formed by the float operations the library's
 * init uses, each rounded once (this file is built without FMA contraction),
 * so they, and the keys derived from them, match bit for bit; the profiles
 * are evaluated in double at those positions. */
static double lattice_coord(int i, float jitter, uint32_t seed, uint32_t i_part, uint32_t stream, float s) {
    float j = jitter * (float)(2.0 * uniform24(seed, i_part, stream) - 1.0);   /* 2u - 1 is exact */
    float c = ((float)i + 0.5f) + j;
    return (double)(c * s);
}
int or_init_lattice(const AsphParams* p, double* x, double* y, double* z, double* th, double* qv, double* rho) {
    OP o; derive(p, &o);
    const int lnx = p->lat_nx, lny = p->lat_ny, lnz = p->lat_nz;
    if ((long long)lnx * lny * lnz != o.N) return ASPH_ERR_CONFIG;
    const float sx = (float)o.lx / (float)lnx, sy = (float)o.ly / (float)lny, sz = (float)o.lz / (float)lnz;
    #pragma omp parallel for schedule(static)
    for (int i = 0; i < o.N; ++i) {
        int ix = i % lnx, iy = (i / lnx) % lny, iz = i / (lnx * lny);
        double px = lattice_coord(ix, p->jitter, p->seed, (uint32_t)i, 0u, sx);
        double py = lattice_coord(iy, p->jitter, p->seed, (uint32_t)i, 1u, sy);
        double pz = lattice_coord(iz, p->jitter, p->seed, (uint32_t)i, 2u, sz);
        double t = theta_ref(&o, pz);
        for (int b = 0; b < p->n_bubbles; ++b) {
            double dx = px - p->bubble_x[b], dy = py - p->bubble_y[b], dz = pz - p->bubble_z[b];
            double r = p->bubble_r[b];
            t += p->bubble_amp[b] * exp(-(dx * dx + dy * dy + dz * dz) / (r * r));
        }
        if (p->noise > 0.f) t += p->noise * normal01(p->seed, (uint32_t)i, 3u);
        x[i] = px; y[i] = py; z[i] = pz; th[i] = t; qv[i] = qv_ref(&o, pz); rho[i] = rho_ref(&o, pz);
    }
    return 0;
}

/* Morton keys of the current order (asph_h100.cu:229-240). */
int or_keys(const AsphParams* p, const double* x, const double* y, const double* z, uint32_t* keys) {
    OP o; derive(p, &o);
    #pragma omp parallel for schedule(static)
    for (int i = 0; i < o.N; ++i)
        keys[i] = morton3((uint32_t)cell1(x[i], o.inv_dx_f, o.nx), (uint32_t)cell1(y[i], o.inv_dy_f, o.ny),
                          (uint32_t)cell1(z[i], o.inv_dz_f, o.nz));
    return 0;
}

/* Stable sort of (key, i) over bits [0, key_bits): the result of
 * cub::DeviceRadixSort::SortPairs(keys, iota) (asph_h100.cu:869, 903, 966),
 * restated as an LSD counting sort with 8-bit digits. */
int or_stable_sort(int N, int key_bits, const uint32_t* keys, uint32_t* perm, uint32_t* sorted) {
    uint32_t *k0 = (uint32_t*)malloc((size_t)N * 4), *v0 = (uint32_t*)malloc((size_t)N * 4);
    uint32_t *k1 = (uint32_t*)malloc((size_t)N * 4), *v1 = (uint32_t*)malloc((size_t)N * 4);
    if (!k0 || !v0 || !k1 || !v1) { free(k0); free(v0); free(k1); free(v1); return ASPH_ERR_NOMEM; }
    for (int i = 0; i < N; ++i) { k0[i] = keys[i]; v0[i] = (uint32_t)i; }
    for (int shift = 0; shift < key_bits; shift += 8) {
        size_t cnt[257];
        memset(cnt, 0, sizeof(cnt));
        for (int i = 0; i < N; ++i) cnt[((k0[i] >> shift) & 255u) + 1]++;
        for (int d = 0; d < 256; ++d) cnt[d + 1] += cnt[d];
        for (int i = 0; i < N; ++i) {
            size_t o = cnt[(k0[i] >> shift) & 255u]++;
            k1[o] = k0[i]; v1[o] = v0[i];
        }
        { uint32_t* t = k0; k0 = k1; k1 = t; t = v0; v0 = v1; v1 = t; }
    }
    memcpy(perm, v0, (size_t)N * 4);
    if (sorted) memcpy(sorted, k0, (size_t)N * 4);
    free(k0); free(v0); free(k1); free(v1);
    return 0;
}

/* Cell table from the sorted order (asph_h100.cu:258-272 after the memset
 * at asph_h100.cu:971): range[2c] = start, range[2c+1] = end, {0,0} empty. */
int or_cell_table(const AsphParams* p, const double* x, const double* y, const double* z, int32_t* range) {
    OP o; derive(p, &o);
    memset(range, 0, (size_t)o.ncell * 8);
    int pc = -1;
    for (int i = 0; i < o.N; ++i) {
        int c = (cell1(z[i], o.inv_dz_f, o.nz) * o.ny + cell1(y[i], o.inv_dy_f, o.ny)) * o.nx +
                cell1(x[i], o.inv_dx_f, o.nx);
        if (i == 0) range[2 * c] = 0;
        else if (c != pc) { range[2 * c] = i; range[2 * pc + 1] = i; }
        if (i == o.N - 1) range[2 * c + 1] = o.N;
        pc = c;
    }
    return 0;
}

/* Surface-layer membership (asph_h100.cu:274-277): (int)(z*INV_DZ) == 0. */
int or_surface(const AsphParams* p, const double* z, uint8_t* flags) {
    OP o; derive(p, &o);
    for (int i = 0; i < o.N; ++i) {
        float s = (float)z[i] * o.inv_dz_f;
        flags[i] = (s > -1.0f && s < 1.0f) ? 1 : 0;
    }
    return 0;
}

/* Half kick (asph_h100.cu:535-544), drift with periodic x/y and reflective
 * z (545-561), surface flux for listed particles (606-626; Ts ramp
 * 989-992).  clamp != 0 applies the emergency clamp first (669-675). */
int or_kick_drift_flux(const AsphParams* p, double simt, double dt, int clamp, const uint8_t* surf,
                       double* x, double* y, double* z, double* u, double* v, double* w,
                       double* th, double* qv, const double* ax, const double* ay, const double* az) {
    OP o; derive(p, &o);
    double r = fmin(fmax(simt / o.ramp, 0.0), 1.0);
    double sw = r * r * (3.0 - 2.0 * r);
    double Ts = o.th0 + o.dts_skin * sw;
    double qs_sfc = qsat(Ts, pres_ref(&o, 0.0));
    #pragma omp parallel for schedule(static)
    for (int i = 0; i < o.N; ++i) {
        double vx = u[i], vy = v[i], vz = w[i];
        if (clamp) {
            double vmax = 0.5 * o.cs, s2 = vx * vx + vy * vy + vz * vz;
            if (s2 > vmax * vmax) { double f = vmax / sqrt(s2); vx *= f; vy *= f; vz *= f; }
        }
        double h = 0.5 * dt;
        vx += ax[i] * h; vy += ay[i] * h; vz += az[i] * h;
        double px = x[i] + vx * dt, py = y[i] + vy * dt, pz = z[i] + vz * dt;
        while (px < 0.0) px += o.lx;
        while (px >= o.lx) px -= o.lx;
        while (py < 0.0) py += o.ly;
        while (py >= o.ly) py -= o.ly;
        if (pz < 0.0) { pz = -pz; vz = fabs(vz); }
        if (pz > o.lz) { pz = 2.0 * o.lz - pz; vz = -fabs(vz); }
        x[i] = px; y[i] = py; z[i] = pz; u[i] = vx; v[i] = vy; w[i] = vz;
        if (o.surface_flux && surf[i] && pz < o.dz) {
            double Pi = pow(fmax(pres_ref(&o, pz), 1.0) / P0, R_D / CP);
            double Ta = th[i] * Pi;
            double t1 = th[i] + o.c_h * o.v_bg * (Ts - Ta) * dt / o.dz;
            double q1 = qv[i] + o.beta_moist * o.c_e * o.v_bg * (qs_sfc - qv[i]) * dt / o.dz;
            th[i] = fmin(fmax(t1, 100.0), o.theta_cap);
            qv[i] = fmin(fmax(q1, 0.0), o.qv_cap);
        }
    }
    return 0;
}

/* Window iteration of the pair loops (asph_h100.cu:296-313, 429-446):
 * own cell by truncation + clamp of the current position, z clipped at
 * the walls, x/y cells wrapped, no minimum image on the distances. */
#define FOR_WINDOW(o, range, xi, yi, zi, J, ...)                                            \
    do {                                                                                     \
        int ix_ = cell1(xi, (o)->inv_dx_f, (o)->nx), iy_ = cell1(yi, (o)->inv_dy_f, (o)->ny); \
        int iz_ = cell1(zi, (o)->inv_dz_f, (o)->nz);                                         \
        int z0_ = iz_ - STENCIL < 0 ? 0 : iz_ - STENCIL;                                     \
        int z1_ = iz_ + STENCIL > (o)->nz - 1 ? (o)->nz - 1 : iz_ + STENCIL;                 \
        for (int jz_ = z0_; jz_ <= z1_; ++jz_)                                               \
            for (int jy_ = iy_ - STENCIL; jy_ <= iy_ + STENCIL; ++jy_) {                     \
                int cy_ = wrapi(jy_, (o)->ny);                                               \
                const int32_t* row_ = (range) + 2 * (size_t)((jz_ * (o)->ny + cy_) * (o)->nx); \
                for (int jx_ = ix_ - STENCIL; jx_ <= ix_ + STENCIL; ++jx_) {                 \
                    int cx_ = wrapi(jx_, (o)->nx);                                           \
                    for (int J = row_[2 * cx_]; J < row_[2 * cx_ + 1]; ++J) { __VA_ARGS__ }  \
                }                                                                            \
            }                                                                                \
    } while (0)

/* Density (asph_h100.cu:286-333) + EOS / saturation adjustment /
 * autoconversion (340-402) + Kessler accretion and rain evaporation.
 * rain_dep[c] receives this call's net deposit [kg] per cell. */
int or_density_eos(const AsphParams* p, double dt, const double* x, const double* y, const double* z,
                   const double* rho_old, const int32_t* range, const double* rain_cur,
                   double* th, double* qv, double* qc, double* rho, double* prs, double* rain_dep) {
    OP o; derive(p, &o);
    double* dep = (double*)calloc((size_t)o.N, sizeof(double));
    int* dcell = (int*)calloc((size_t)o.N, sizeof(int));
    if (!dep || !dcell) { free(dep); free(dcell); return ASPH_ERR_NOMEM; }
    #pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < o.N; ++i) {
        double xi = x[i], yi = y[i], zi = z[i], S1 = 0.0, S2 = 0.0;
        FOR_WINDOW(&o, range, xi, yi, zi, j, {
            double dx = (xi - x[j]) / o.dx, dy = (yi - y[j]) / o.dy, dz = (zi - z[j]) / o.dz;
            double r2 = dx * dx + dy * dy + dz * dz;
            if (r2 < 4.0) {
                double W = w3(sqrt(r2));
                S1 += W;
                S2 += W / fmax(rho_old[j], 1e-3);
            }
        });
        double rref = rho_ref(&o, zi);
        double rr = S2 > 1e-20 ? S1 / S2 : rref;
        double rh = fmin(fmax(rr, 0.5 * rref), 2.0 * rref);
        /* EOS, asph_h100.cu:352-361 */
        double r = fmax(rh, 1e-3);
        double dd = fmin(fmax(r - rref, -0.3 * rref), 0.3 * rref);
        double ppr = o.cs * o.cs * dd;
        double pfl = fmax(pres_ref(&o, zi) + ppr, 1.0);
        double Pi = pow(pfl / P0, R_D / CP);
        double t = th[i], v = qv[i], c = qc[i], T = t * Pi;
        double qs = qsat(T, pfl);
        if (v > qs || c > 0.0) {                                  /* asph_h100.cu:370-385 */
            double dqc = 0.0;
            for (int it = 0; it < 3; ++it) {
                double Tn = T + (L_V / CP) * dqc;
                double esn = esat(Tn), qsn = qsat(Tn, pfl);
                double f = v - dqc - qsn;
                double fp = -1.0 - dqsdT(Tn, esn, pfl) * (L_V / CP);
                dqc -= f / fp;
                dqc = fmin(dqc, v);
                dqc = fmax(dqc, -c);
            }
            v -= dqc; c += dqc; t += L_V * dqc / (CP * Pi); T += (L_V / CP) * dqc;
        }
        double d = 0.0;
        if (c > o.qc_auto) {                                      /* asph_h100.cu:389-394 */
            double dqr = (c - o.qc_auto) * (1.0 - exp(-o.rate_auto * dt));
            c -= dqr; d += dqr;
        }
        int ix = cell1(xi, o.inv_dx_f, o.nx), iy = cell1(yi, o.inv_dy_f, o.ny), iz = cell1(zi, o.inv_dz_f, o.nz);
        int cid = (iz * o.ny + iy) * o.nx + ix;
        if (o.accretion || o.rain_evap) {
            /* Kessler (1969) warm rain in the Klemp & Wilhelmson (1978) forms;
             * rain is Eulerian per cell: qr = M_rain / (rho V_cell). */
            double qr = fmax(rain_cur[cid], 0.0) / (r * o.v_cell);
            if (o.accretion && c > 0.0 && qr > 0.0) {
                double dqa = fmin(c, dt * o.k_accr * c * pow(qr, 0.875));
                c -= dqa; d += dqa;
            }
            if (o.rain_evap && qr > 0.0) {
                double qvs = qsat(T, pfl);
                if (v < qvs && qvs > 0.0) {
                    double rq = 1e-3 * r * qr;
                    double C = 1.6 + 124.9 * pow(rq, 0.2046);
                    double er = (1.0 - v / qvs) * C * pow(rq, 0.525) /
                                (1e-3 * r * (5.4e5 + 2.55e6 / (0.01 * pfl * qvs)));
                    double dqe = fmin(qr, fmin(dt * er, qvs - v));
                    v += dqe; t -= L_V * dqe / (CP * Pi); d -= dqe;
                }
            }
        }
        dep[i] = d; dcell[i] = cid;
        th[i] = fmin(fmax(t, 100.0), o.theta_cap);
        qv[i] = fmin(fmax(v, 0.0), o.qv_cap);
        qc[i] = fmax(c, 0.0);
        rho[i] = rh;
        prs[i] = ppr;
    }
    if (rain_dep) {
        memset(rain_dep, 0, (size_t)o.ncell * sizeof(double));
        for (int i = 0; i < o.N; ++i) rain_dep[dcell[i]] += dep[i] * o.pmass;
    }
    free(dep); free(dcell);
    return 0;
}

/* Momentum (asph_h100.cu:415-511); integrate != 0 adds the theta update
 * (562-571), the second half kick (535-544) and the sponge (518-530). */
int or_momentum(const AsphParams* p, double dt, int integrate, const double* x, const double* y, const double* z,
                double* u, double* v, double* w, double* th, const double* qv, const double* qc,
                const double* rho, const double* prs, const int32_t* range,
                double* ax, double* ay, double* az, double* dthdt) {
    OP o; derive(p, &o);
    double* un = (double*)malloc((size_t)o.N * 3 * sizeof(double));
    if (!un) return ASPH_ERR_NOMEM;
    #pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < o.N; ++i) {
        double xi = x[i], yi = y[i], zi = z[i], ui = u[i], vi = v[i], wi = w[i];
        double rhoi = fmax(rho[i], 1e-3), pri = prs[i];
        double sx = 0, sy = 0, sz = 0, vx = 0, vy = 0, vz = 0;
        FOR_WINDOW(&o, range, xi, yi, zi, j, {
            if (j == i) continue;
            double rx = xi - x[j], ry = yi - y[j], rz = zi - z[j];
            double dxt = rx / o.dx, dyt = ry / o.dy, dzt = rz / o.dz;
            double r2t = dxt * dxt + dyt * dyt + dzt * dzt;
            if (r2t >= 4.0 || r2t < 1e-12) continue;
            double q = sqrt(r2t), k = dw3(q) / q;
            double gx = k * dxt / o.dx, gy = k * dyt / o.dy, gz = k * dzt / o.dz;
            double rhoj = fmax(rho[j], 1e-3);
            double dp = (prs[j] - pri) / (rhoi * rhoj);
            double vdx = ui - u[j], vdy = vi - v[j], vdz = wi - w[j];
            double vdotr = vdx * rx + vdy * ry + vdz * rz;
            double visc = 0.0;
            if (vdotr < 0.0) {
                double rp2 = rx * rx + ry * ry + rz * rz;
                double mu = vdotr / (rp2 + o.eta2);
                double rbar = 0.5 * (rhoi + rhoj);
                double muh = o.h_av * mu;
                visc = (-o.alpha * o.cs * muh + o.beta * muh * muh) / (rbar * rbar * rhoj);
            }
            double br = dp + visc;
            sx -= br * gx; sy -= br * gy; sz -= br * gz;
            vx -= visc * gx; vy -= visc * gy; vz -= visc * gz;
        });
        sx *= o.mm; sy *= o.mm; sz *= o.mm;
        vx *= o.mm; vy *= o.mm; vz *= o.mm;
        double thv = th[i] * (1.0 + 0.608 * qv[i]);
        double thvr = theta_ref(&o, zi) * (1.0 + 0.608 * qv_ref(&o, zi));
        sz += GRAV * ((thv - thvr) / thvr - qc[i]);
        ax[i] = sx; ay[i] = sy; az[i] = sz;
        double Pi = pow(fmax(pres_ref(&o, zi) + pri, 1.0) / P0, R_D / CP);
        double dth = -(ui * vx + vi * vy + wi * vz) / (CP * Pi);
        dth = fmin(fmax(dth, -o.dthdt_cap), o.dthdt_cap);
        dthdt[i] = dth;
        un[3 * i] = ui; un[3 * i + 1] = vi; un[3 * i + 2] = wi;
        if (integrate) {
            double h = 0.5 * dt;
            double nw = wi + sz * h;
            double zs = (1.0 - o.sponge_frac) * o.lz;
            if (zi >= zs) {
                double tt = (zi - zs) / (o.sponge_frac * o.lz);
                nw *= 1.0 / (1.0 + o.sponge_sigma * tt * tt * dt);
            }
            un[3 * i] = ui + sx * h; un[3 * i + 1] = vi + sy * h; un[3 * i + 2] = nw;
        }
    }
    if (integrate) {
        #pragma omp parallel for schedule(static)
        for (int i = 0; i < o.N; ++i) {
            u[i] = un[3 * i]; v[i] = un[3 * i + 1]; w[i] = un[3 * i + 2];
            th[i] = fmin(fmax(th[i] + dthdt[i] * dt, 100.0), o.theta_cap);
        }
    }
    free(un);
    return 0;
}

/* Rain sedimentation (asph_h100.cu:577-599).  delta (nullable) is added to
 * the grid first (and clipped at zero), as the accretion/evaporation path
 * does; precip accumulates [kg/m^2]. */
int or_rain(const AsphParams* p, double dt, const double* rin, const double* delta, double* rout, double* precip) {
    OP o; derive(p, &o);
    double frac = fmin(o.v_rain * dt / o.dz, 1.0);
    for (int c = 0; c < o.ncell; ++c) {
        int ix = c % o.nx, iy = (c / o.nx) % o.ny, iz = c / o.nxy;
        double cur = rin[c];
        if (delta) cur = fmax(cur + delta[c], 0.0);
        double outm = cur * frac, inm = 0.0;
        if (iz < o.nz - 1) {
            double ab = rin[c + o.nxy];
            if (delta) ab = fmax(ab + delta[c + o.nxy], 0.0);
            inm = ab * frac;
        }
        rout[c] = cur - outm + inm;
        if (iz == 0) precip[iy * o.nx + ix] += outm / (o.dx * o.dy);
    }
    return 0;
}

/* Closed-loop CFL control (asph_h100.cu:1040-1078).  ctl[] in/out:
 * 0 dt, 1 trips, 2 clamp (out), 3 abort (out), 4 sort_dt (out),
 * 5 dt_required (out); umax[3] = |u|,|v|,|w| maxima. */
int or_cfl(const AsphParams* p, const double umax[3], double ctl[6]) {
    OP o; derive(p, &o);
    double ux = umax[0], uy = umax[1], uz = umax[2];
    double dt = ctl[0];
    int trips = (int)ctl[1];
    ctl[2] = 0; ctl[3] = 0;
    double req = o.cfl * fmin(fmin(o.dx / (o.cs + ux), o.dy / (o.cs + uy)), o.dz / (o.cs + uz)) * 0.90;
    double adopt = fmin(o.dt_cap, req);
    ctl[5] = req;
    if (adopt < o.dt_floor) {
        ++trips;
        if (o.strict_cfl || trips > o.max_trip) { ctl[1] = trips; ctl[3] = 1; return ASPH_ERR_CFL_ABORT; }
        ctl[2] = 1;
        adopt = fmax(o.dt_floor, o.cfl * fmin(fmin(o.dx, o.dy), o.dz) / (1.5 * o.cs) * 0.90);
    } else if (adopt < 0.98 * dt) {
        trips = 0;
    }
    if (o.adaptive_dt) dt = adopt;
    {
        double dzm = 0.3 * o.dz / fmax(uz, 0.5), dhm = 0.3 * o.dx / fmax(fmax(ux, uy), 0.5);
        ctl[4] = fmin(fmax(fmin(dzm, dhm), dt), 15.0);
    }
    ctl[0] = dt; ctl[1] = trips;
    return 0;
}

/* FP64 audit (asph_h100.cu:650-668): KE, PE, IE, water, p_z, mass. */
int or_audit(const AsphParams* p, const double* z, const double* u, const double* v, const double* w,
             const double* th, const double* qv, const double* qc, double out[6]) {
    OP o; derive(p, &o);
    double a0 = 0, a1 = 0, a2 = 0, a3 = 0, a4 = 0;
    #pragma omp parallel for reduction(+ : a0, a1, a2, a3, a4) schedule(static)
    for (int i = 0; i < o.N; ++i) {
        double Pi = pow(fmax(pres_ref(&o, z[i]), 1.0) / P0, R_D / CP);
        a0 += 0.5 * (u[i] * u[i] + v[i] * v[i] + w[i] * w[i]);
        a1 += GRAV * z[i];
        a2 += CP * th[i] * Pi;
        a3 += qv[i] + qc[i];
        a4 += w[i];
    }
    out[0] = a0 * o.pmass; out[1] = a1 * o.pmass; out[2] = a2 * o.pmass;
    out[3] = a3 * o.pmass; out[4] = a4 * o.pmass; out[5] = o.pmass * o.N;
    return 0;
}

/* Reference helper values for the pinning test (asph_h100.cu:125-171).
 * in: n rows of (z, T, p, q); out: n rows of theta_ref(z), exner_ref(z),
 * pres_ref(z), rho_ref(z), qv_ref(z), esat(T), qsat(T,p), dqsdT(T,esat(T),p),
 * w3(q), dw3(q). */
int or_helpers(const AsphParams* p, int n, const double* arg, double* out) {
    OP o; derive(p, &o);
    for (int i = 0; i < n; ++i) {
        double z = arg[4 * i], T = arg[4 * i + 1], pr = arg[4 * i + 2], q = arg[4 * i + 3];
        out[10 * i + 0] = theta_ref(&o, z);
        out[10 * i + 1] = exner_ref(&o, z);
        out[10 * i + 2] = pres_ref(&o, z);
        out[10 * i + 3] = rho_ref(&o, z);
        out[10 * i + 4] = qv_ref(&o, z);
        out[10 * i + 5] = esat(T);
        out[10 * i + 6] = qsat(T, pr);
        out[10 * i + 7] = dqsdT(T, esat(T), pr);
        out[10 * i + 8] = w3(q);
        out[10 * i + 9] = dw3(q);
    }
    return 0;
}
int or_hash_noise(int n, const int* ijk, float* out) {
    for (int i = 0; i < n; ++i) out[i] = hash_noise(ijk[3 * i], ijk[3 * i + 1], ijk[3 * i + 2]);
    return 0;
}
/* ========================================================================= */
/* Parameter presets, restated on the oracle side so that the CPU legs of    */
/* the benchmark never load the CUDA library.  Same float expressions as the */
/* library's table (include/asph.h ASPH_PRESET_*); a CPU test holds the two  */
/* equal field by field.  The reference physics are asph_h100.cu:48-120.    */
/* ========================================================================= */
static float preset_uniform(uint32_t i, uint32_t stream) {
    uint64_t h = mix64(((uint64_t)1u << 32) ^ mix64(((uint64_t)stream << 40) ^ (uint64_t)i));
    return (float)(uint32_t)(h >> 40) * (1.0f / 16777216.0f);
}
static void preset_reference_physics(AsphParams* p) {
    p->dx = 1000.0f; p->dy = 1000.0f; p->dz = 100.0f;            /* asph_h100.cu:48 */
    p->th0 = 300.0f; p->n2 = 6.0e-5f; p->cs = 80.0f;              /* asph_h100.cu:71-73 */
    p->qv_mode = ASPH_QV_REFERENCE; p->qv0 = 0.016f; p->rh = 0.8f; p->rh_bl = 0.8f; p->z_bl = 0.f;
    p->alpha_av = 0.2f; p->beta_av = 0.0f; p->h_av = 0.f;         /* asph_h100.cu:84-85 */
    p->sponge_sigma = 0.05f; p->sponge_frac = 0.15f; p->dthdt_cap = 1.0f;   /* asph_h100.cu:89-91 */
    p->surface_flux = 1;
    p->c_h = 1.2e-3f; p->c_e = 1.2e-3f; p->beta_moist = 0.20f; p->v_bg = 7.0f; p->dts_skin = 3.15f;
    p->ramp = 3600.0f;                                             /* asph_h100.cu:100-105 */
    p->qc_auto = 1.0e-3f; p->rate_auto = 1.0e-3f; p->v_rain = 9.0f; p->theta_cap = 500.0f;
    p->qv_cap = 0.060f;                                            /* asph_h100.cu:111-120 */
    p->accretion = 0; p->rain_evap = 0; p->k_accr = 2.2f;
    p->dt_request = 0.f; p->cfl = 0.40f; p->max_trip = 20; p->strict_cfl = 0; p->adaptive_dt = 1;
    p->sort_every = 0; p->permute_acc = 0; p->pmass = 0.f;
    p->dump_sx = 10; p->dump_sy = 10; p->dump_sz = 3;             /* asph_h100.cu:737 */
    p->init_mode = ASPH_INIT_REFERENCE; p->noise = 0.1f; p->seed = 0; p->jitter = 0.f;
}
static void preset_config_physics(AsphParams* p, float Lx, float Ly, float Lz, float hxy, float hz, int lnx,
                                  int lny, int lnz) {
    preset_reference_physics(p);
    p->nx = (int)floorf(Lx / hxy); p->ny = (int)floorf(Ly / hxy); p->nz = (int)floorf(Lz / hz);
    p->dx = Lx / p->nx; p->dy = Ly / p->ny; p->dz = Lz / p->nz;
    p->n2 = 9.80665f * 4.0e-3f / 300.0f;                           /* 4 K/km at the surface */
    p->qv_mode = ASPH_QV_RH; p->rh = 0.8f; p->rh_bl = 0.8f; p->z_bl = 0.f;
    p->accretion = 1; p->rain_evap = 1;
    p->permute_acc = 1;
    p->init_mode = ASPH_INIT_LATTICE;
    p->lat_nx = lnx; p->lat_ny = lny; p->lat_nz = lnz;
    p->n_particles = lnx * lny * lnz;
    p->jitter = 0.25f; p->seed = 0; p->noise = 0.f;
}
int or_params_preset(AsphParams* p, int preset, int nx, int ny, int nz) {
    memset(p, 0, sizeof(*p));
    switch (preset) {
        case ASPH_PRESET_REFERENCE:
            preset_reference_physics(p);
            p->nx = 1000; p->ny = 1000; p->nz = 150;              /* asph_h100.cu:729 */
            if (nx > 0) p->nx = nx;
            if (ny > 0) p->ny = ny;
            if (nz > 0) p->nz = nz;
            p->n_particles = p->nx * p->ny * p->nz;
            return 0;
        case ASPH_PRESET_SMALL_65K:
        case ASPH_PRESET_ADJOINT_262K: {
            const int n = preset == ASPH_PRESET_SMALL_65K ? 32 : 64;
            preset_config_physics(p, 10000.f, 10000.f, 5000.f, 200.f, 50.f, n, n, 64);
            p->n_bubbles = 1;
            p->bubble_x[0] = 5000.f; p->bubble_y[0] = 5000.f; p->bubble_z[0] = 1000.f;
            p->bubble_r[0] = 1000.f; p->bubble_amp[0] = 2.0f;
            p->dt_request = 0.5f;
            p->sort_every = 0;
            break;
        }
        case ASPH_PRESET_BUBBLE_2M:
            preset_config_physics(p, 20000.f, 20000.f, 8000.f, 150.f, 40.f, 128, 128, 128);
            p->n_bubbles = 3;
            for (int b = 0; b < 3; ++b) {
                p->bubble_x[b] = 20000.f * (0.2f + 0.6f * preset_uniform((uint32_t)b, 10u));
                p->bubble_y[b] = 20000.f * (0.2f + 0.6f * preset_uniform((uint32_t)b, 11u));
                p->bubble_z[b] = 800.f + 800.f * preset_uniform((uint32_t)b, 12u);
                p->bubble_r[b] = 800.f + 700.f * preset_uniform((uint32_t)b, 13u);
                p->bubble_amp[b] = 1.5f + 1.5f * preset_uniform((uint32_t)b, 14u);
            }
            p->dt_request = 0.25f;
            p->sort_every = 1;
            break;
        case ASPH_PRESET_LARGE_16M:
            preset_config_physics(p, 40000.f, 40000.f, 10000.f, 160.f, 20.f, 256, 256, 256);
            p->rh_bl = 0.95f; p->z_bl = 1000.f;
            p->noise = 0.2f;
            p->dt_request = 0.f;
            p->sort_every = 1;
            break;
        default:
            return ASPH_ERR_ARG;
    }
    if (nx > 0) p->nx = nx;
    if (ny > 0) p->ny = ny;
    if (nz > 0) p->nz = nz;
    return 0;
}

int or_derived(const AsphParams* p, double out[12]) {
    OP o; derive(p, &o);
    out[0] = o.pmass; out[1] = o.mm; out[2] = o.dt_static; out[3] = o.dt_cap; out[4] = o.dt_floor;
    out[5] = o.lx; out[6] = o.ly; out[7] = o.lz; out[8] = o.key_bits; out[9] = o.h_av;
    out[10] = o.a_exner; out[11] = o.v_cell;
    return 0;
}

/* ========================================================================= */
/* Full steps (asph_h100.cu:958-1078) on an FP64 state, for the CPU baseline. */
/* fields: x y z u v w th qv qc rho ax ay az prs dthdt (N each).              */
/* ctl in/out: 0 simt, 1 dt, 2 since_sort, 3 sort_dt, 4 trips, 5 step,       */
/*             6 do_sort, 7 aborted, 8 clamp_pending.                         */
/* The cell table and surface list live only inside one call, so the first   */
/* step of a call always sorts.                                               */
/* ========================================================================= */
int or_run(const AsphParams* p, int nsteps, double** f, double* rain, double* precip, double* ctl) {
    OP o; derive(p, &o);
    const int N = o.N;
    uint32_t* keys = (uint32_t*)malloc((size_t)N * 4);
    uint32_t* perm = (uint32_t*)malloc((size_t)N * 4);
    int32_t* range = (int32_t*)malloc((size_t)o.ncell * 8);
    uint8_t* surf = (uint8_t*)malloc((size_t)N);
    double* tmp = (double*)malloc((size_t)N * sizeof(double));
    double* dep = (double*)malloc((size_t)o.ncell * sizeof(double));
    double* rnext = (double*)malloc((size_t)o.ncell * sizeof(double));
    int rc = 0;
    if (!keys || !perm || !range || !surf || !tmp || !dep || !rnext) { rc = ASPH_ERR_NOMEM; goto done; }
    for (int s = 0; s < nsteps && !ctl[7]; ++s) {
        int sorted = (s == 0) || ctl[6] != 0.0;
        double dt = ctl[1];
        if (sorted) {
            or_keys(p, f[0], f[1], f[2], keys);
            or_stable_sort(N, o.key_bits, keys, perm, NULL);
            int nf = o.permute_acc ? 13 : 10;
            for (int k = 0; k < nf; ++k) {
                double* a = f[k];
                #pragma omp parallel for schedule(static)
                for (int i = 0; i < N; ++i) tmp[i] = a[perm[i]];
                memcpy(a, tmp, (size_t)N * sizeof(double));
            }
            or_cell_table(p, f[0], f[1], f[2], range);
            or_surface(p, f[2], surf);
        }
        or_kick_drift_flux(p, ctl[0], dt, (int)ctl[8], surf, f[0], f[1], f[2], f[3], f[4], f[5], f[6], f[7],
                           f[10], f[11], f[12]);
        memcpy(tmp, f[9], (size_t)N * sizeof(double));
        or_density_eos(p, dt, f[0], f[1], f[2], tmp, range, rain, f[6], f[7], f[8], f[9], f[13], dep);
        if (!(o.accretion || o.rain_evap))
            for (int c = 0; c < o.ncell; ++c) rain[c] += dep[c];
        or_momentum(p, dt, 1, f[0], f[1], f[2], f[3], f[4], f[5], f[6], f[7], f[8], f[9], f[13], range,
                    f[10], f[11], f[12], f[14]);
        or_rain(p, dt, rain, (o.accretion || o.rain_evap) ? dep : NULL, rnext, precip);
        memcpy(rain, rnext, (size_t)o.ncell * sizeof(double));
        {
            double um[3] = {0, 0, 0};
            for (int i = 0; i < N; ++i) {
                um[0] = fmax(um[0], fabs(f[3][i])); um[1] = fmax(um[1], fabs(f[4][i]));
                um[2] = fmax(um[2], fabs(f[5][i]));
            }
            double c6[6] = {dt, ctl[4], 0, 0, 0, 0};
            ctl[0] += dt;
            ctl[2] = (sorted ? 0.0 : ctl[2]) + dt;
            ctl[5] += 1;
            int st = or_cfl(p, um, c6);
            ctl[4] = c6[1];
            ctl[8] = c6[2];
            if (st) { ctl[7] = 1; rc = st; break; }
            ctl[1] = c6[0];
            ctl[3] = c6[4];
            if (o.sort_every > 0) ctl[6] = ((int)ctl[5] % o.sort_every) == 0;
            else ctl[6] = ctl[2] >= ctl[3];
        }
    }
done:
    free(keys); free(perm); free(range); free(surf); free(tmp); free(dep); free(rnext);
    return rc;
}
