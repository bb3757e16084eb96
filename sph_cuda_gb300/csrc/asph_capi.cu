// asph_capi.cu — the extern "C" boundary (include/asph.h): parameters,
// context and device memory, the granular calls that mirror the blocks of
// the reference host loop, and the CUDA-graph step.
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <string>
#include <vector>
#include <sys/stat.h>
#include "asph_ctx.cuh"

using namespace asph;

namespace {

thread_local std::string g_err;

int ceil_log2(int n) {   // asph_h100.cu:865
    int b = 1;
    while ((1 << b) < n) ++b;
    return b;
}

}  // namespace

int asph::fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

int asph::set_error(int code, const char* msg) { return fail(code, "%s", msg); }

// ---------------------------------------------------------------------------
// parameters
// ---------------------------------------------------------------------------
extern "C" int asph_abi_version(void) { return ASPH_ABI_VERSION; }
extern "C" int asph_params_size(void) { return (int)sizeof(AsphParams); }
extern "C" const char* asph_last_error(void) { return g_err.c_str(); }
extern "C" const char* asph_status_string(int s) {
    switch (s) {
        case ASPH_OK: return "ok";
        case ASPH_ERR_CUDA: return "CUDA error";
        case ASPH_ERR_CONFIG: return "invalid configuration";
        case ASPH_ERR_CFL_ABORT: return "CFL trip limit exceeded";
        case ASPH_ERR_TIMEOUT: return "device wait timed out";
        case ASPH_ERR_ARG: return "bad argument";
        case ASPH_ERR_NOMEM: return "out of memory";
        case ASPH_ERR_IO: return "I/O error";
        case ASPH_ERR_STATE: return "call out of order";
        case ASPH_ERR_NONFINITE: return "non-finite particle state, run stopped";
        case ASPH_ERR_DENSE: return "search window above ASPH_MAX_CANDIDATES, run stopped";
        default: return "unknown status";
    }
}

static void reference_physics(AsphParams* p) {
    // asph_h100.cu:48-120
    p->dx = 1000.0f; p->dy = 1000.0f; p->dz = 100.0f;
    p->th0 = 300.0f; p->n2 = 6.0e-5f; p->cs = 80.0f;
    p->qv_mode = ASPH_QV_REFERENCE; p->qv0 = 0.016f; p->rh = 0.8f; p->rh_bl = 0.8f; p->z_bl = 0.f;
    p->alpha_av = 0.2f; p->beta_av = 0.0f; p->h_av = 0.f;  // 0: 2*dz
    p->sponge_sigma = 0.05f; p->sponge_frac = 0.15f; p->dthdt_cap = 1.0f;
    p->surface_flux = 1;
    p->c_h = 1.2e-3f; p->c_e = 1.2e-3f; p->beta_moist = 0.20f; p->v_bg = 7.0f; p->dts_skin = 3.15f;
    p->ramp = 3600.0f;
    p->qc_auto = 1.0e-3f; p->rate_auto = 1.0e-3f; p->v_rain = 9.0f; p->theta_cap = 500.0f; p->qv_cap = 0.060f;
    p->accretion = 0; p->rain_evap = 0; p->k_accr = 2.2f;
    p->dt_request = 0.f; p->cfl = 0.40f; p->max_trip = 20; p->strict_cfl = 0; p->adaptive_dt = 1;
    p->sort_every = 0; p->permute_acc = 0; p->pmass = 0.f;
    p->dump_sx = 10; p->dump_sy = 10; p->dump_sz = 3;
    p->init_mode = ASPH_INIT_REFERENCE; p->noise = 0.1f; p->seed = 0; p->jitter = 0.f;
}

// Config-mode atmosphere: theta = 300 K + 4 K/km as a constant-N^2 profile
// (N^2 = g * 4e-3 / 300), vapour at a relative humidity, warm rain with
// accretion and evaporation, jittered lattice.
static void config_physics(AsphParams* p, float Lx, float Ly, float Lz, float hxy, float hz, int lnx, int lny,
                           int lnz) {
    reference_physics(p);
    p->nx = (int)floorf(Lx / hxy); p->ny = (int)floorf(Ly / hxy); p->nz = (int)floorf(Lz / hz);
    p->dx = Lx / p->nx; p->dy = Ly / p->ny; p->dz = Lz / p->nz;
    p->n2 = asph::GRAV * 4.0e-3f / 300.0f;
    p->qv_mode = ASPH_QV_RH; p->rh = 0.8f; p->rh_bl = 0.8f; p->z_bl = 0.f;
    p->accretion = 1; p->rain_evap = 1;
    p->permute_acc = 1;
    p->init_mode = ASPH_INIT_LATTICE;
    p->lat_nx = lnx; p->lat_ny = lny; p->lat_nz = lnz;
    p->n_particles = lnx * lny * lnz;
    p->jitter = 0.25f; p->seed = 0; p->noise = 0.f;
}

extern "C" int asph_params_preset(AsphParams* p, int preset, int nx, int ny, int nz) {
    if (!p) return fail(ASPH_ERR_ARG, "params is NULL");
    memset(p, 0, sizeof(*p));
    switch (preset) {
        case ASPH_PRESET_REFERENCE:
            reference_physics(p);
            p->nx = 1000; p->ny = 1000; p->nz = 150;   // Config defaults, asph_h100.cu:729
            if (nx > 0) p->nx = nx;
            if (ny > 0) p->ny = ny;
            if (nz > 0) p->nz = nz;
            p->n_particles = p->nx * p->ny * p->nz;
            break;
        case ASPH_PRESET_SMALL_65K:
        case ASPH_PRESET_ADJOINT_262K: {
            const int n = preset == ASPH_PRESET_SMALL_65K ? 32 : 64;
            config_physics(p, 10000.f, 10000.f, 5000.f, 200.f, 50.f, n, n, preset == ASPH_PRESET_SMALL_65K ? 64 : 64);
            p->n_bubbles = 1;
            p->bubble_x[0] = 5000.f; p->bubble_y[0] = 5000.f; p->bubble_z[0] = 1000.f;
            p->bubble_r[0] = 1000.f; p->bubble_amp[0] = 2.0f;
            p->dt_request = 0.5f;
            p->sort_every = 0;
            break;
        }
        case ASPH_PRESET_BUBBLE_2M: {
            config_physics(p, 20000.f, 20000.f, 8000.f, 150.f, 40.f, 128, 128, 128);
            p->n_bubbles = 3;
            for (int b = 0; b < 3; ++b) {
                p->bubble_x[b] = 20000.f * (0.2f + 0.6f * uniform24(1u, (uint32_t)b, 10u));
                p->bubble_y[b] = 20000.f * (0.2f + 0.6f * uniform24(1u, (uint32_t)b, 11u));
                p->bubble_z[b] = 800.f + 800.f * uniform24(1u, (uint32_t)b, 12u);
                p->bubble_r[b] = 800.f + 700.f * uniform24(1u, (uint32_t)b, 13u);
                p->bubble_amp[b] = 1.5f + 1.5f * uniform24(1u, (uint32_t)b, 14u);
            }
            p->dt_request = 0.25f;
            p->sort_every = 1;
            break;
        }
        case ASPH_PRESET_LARGE_16M:
            config_physics(p, 40000.f, 40000.f, 10000.f, 160.f, 20.f, 256, 256, 256);
            p->rh_bl = 0.95f; p->z_bl = 1000.f;
            p->noise = 0.2f;
            p->dt_request = 0.f;
            p->sort_every = 1;
            break;
        default:
            return fail(ASPH_ERR_ARG, "unknown preset %d", preset);
    }
    if (preset != ASPH_PRESET_REFERENCE) {
        if (nx > 0) p->nx = nx;
        if (ny > 0) p->ny = ny;
        if (nz > 0) p->nz = nz;
    }
    return ASPH_OK;
}

extern "C" int asph_params_check(const AsphParams* p) {
    if (!p) return fail(ASPH_ERR_ARG, "params is NULL");
    if (p->nx > 1024 || p->ny > 1024 || p->nz > 1024)
        return fail(ASPH_ERR_CONFIG, "30-bit Morton key addresses 1024 cells/axis");
    if (p->nx < 3 || p->ny < 3 || p->nz < 1)
        return fail(ASPH_ERR_CONFIG, "grid must have nx, ny >= 3 and nz >= 1 (got %d %d %d)", p->nx, p->ny, p->nz);
    if (!(p->dx > 0.f && p->dy > 0.f && p->dz > 0.f)) return fail(ASPH_ERR_CONFIG, "cell sizes must be positive");
    if (p->n_particles < 1 || p->n_particles >= (1 << 30))
        return fail(ASPH_ERR_CONFIG, "n_particles must be in [1, 2^30)");
    if (p->init_mode == ASPH_INIT_REFERENCE && p->n_particles != p->nx * p->ny * p->nz)
        return fail(ASPH_ERR_CONFIG, "reference init needs n_particles == nx*ny*nz");
    if (p->init_mode == ASPH_INIT_LATTICE &&
        (long long)p->lat_nx * p->lat_ny * p->lat_nz != (long long)p->n_particles)
        return fail(ASPH_ERR_CONFIG, "lattice counts must multiply to n_particles");
    if (p->init_mode != ASPH_INIT_REFERENCE && p->init_mode != ASPH_INIT_LATTICE)
        return fail(ASPH_ERR_CONFIG, "unknown init_mode %d", p->init_mode);
    if (p->n_bubbles < 0 || p->n_bubbles > ASPH_MAX_BUBBLES) return fail(ASPH_ERR_CONFIG, "n_bubbles out of range");
    if (!(p->cs > 0.f) || !(p->cfl > 0.f)) return fail(ASPH_ERR_CONFIG, "cs and cfl must be positive");
    if (p->dump_sx < 1 || p->dump_sy < 1 || p->dump_sz < 1) return fail(ASPH_ERR_CONFIG, "dump strides must be >= 1");
    if (p->qv_mode == ASPH_QV_RH && p->z_bl != floorf(p->z_bl))
        return fail(ASPH_ERR_CONFIG, "z_bl must be a whole number of metres (sounding table node spacing)");
    if (!(p->nz * p->dz < 60000.f)) return fail(ASPH_ERR_CONFIG, "domain top must be below 60 km");
    return ASPH_OK;
}

AuditConst asph::audit_constants(const AsphParams& p) {
    AuditConst A;
    A.th0 = p.th0;
    A.n2 = p.n2;
    A.a_exner = 9.80665 * 9.80665 / (1004.0 * A.th0 * A.n2);
    const double lx = (double)((float)p.nx * p.dx), ly = (double)((float)p.ny * p.dy),
                 lz = (double)((float)p.nz * p.dz);
    A.pmass = p.pmass > 0.f ? (double)p.pmass : 100000.0 / (287.05 * A.th0) * lx * ly * lz / (double)p.n_particles;
    A.N = p.n_particles;
    return A;
}

static void derive(const AsphParams& p, Phys& P) {
    memset(&P, 0, sizeof(P));
    P.nx = p.nx; P.ny = p.ny; P.nz = p.nz; P.nxy = p.nx * p.ny;
    P.N = p.n_particles; P.ncell = p.nx * p.ny * p.nz;
    P.dx = p.dx; P.dy = p.dy; P.dz = p.dz;
    P.inv_dx = 1.0f / p.dx; P.inv_dy = 1.0f / p.dy; P.inv_dz = 1.0f / p.dz;
    P.lx = p.nx * p.dx; P.ly = p.ny * p.dy; P.lz = p.nz * p.dz;
    P.v_cell = p.dx * p.dy * p.dz;
    P.th0 = p.th0; P.n2 = p.n2; P.cs = p.cs;
    P.a_exner = asph::GRAV * asph::GRAV / (asph::CP * p.th0 * p.n2);
    P.qv_mode = p.qv_mode; P.qv0 = p.qv0; P.rh = p.rh; P.rh_bl = p.rh_bl; P.z_bl = p.z_bl;
    P.alpha = p.alpha_av; P.beta = p.beta_av;
    P.h_av = p.h_av > 0.f ? p.h_av : 2.0f * p.dz;
    P.eta2 = (0.01f * P.h_av) * (0.01f * P.h_av);
    asph::set_viscosity_terms(P);
    P.sponge_sigma = p.sponge_sigma; P.sponge_frac = p.sponge_frac; P.dthdt_cap = p.dthdt_cap;
    P.surface_flux = p.surface_flux;
    P.c_h = p.c_h; P.c_e = p.c_e; P.beta_moist = p.beta_moist; P.v_bg = p.v_bg; P.dts_skin = p.dts_skin;
    P.ramp = p.ramp;
    P.qc_auto = p.qc_auto; P.rate_auto = p.rate_auto; P.v_rain = p.v_rain; P.theta_cap = p.theta_cap;
    P.qv_cap = p.qv_cap; P.accretion = p.accretion; P.rain_evap = p.rain_evap; P.k_accr = p.k_accr;
    const float rho0 = asph::P0 / (asph::R_D * p.th0);   // asph_h100.cu:75
    const float base = rho0 * P.v_cell;                   // asph_h100.cu:76
    if (p.pmass > 0.f)
        P.pmass = p.pmass;
    else
        P.pmass = (P.N == P.ncell) ? base : (float)((double)base * (double)P.ncell / (double)P.N);
    P.mm = P.pmass / P.v_cell;                            // asph_h100.cu:497
    P.cfl = p.cfl;
    P.dt_static = p.cfl * fminf(fminf(p.dx, p.dy), p.dz) / p.cs;   // asph_h100.cu:794
    P.dt_cap = p.dt_request > 0.f ? fminf(p.dt_request, P.dt_static) : P.dt_static;
    P.dt_floor = 0.05f * P.dt_cap;
    P.max_trip = p.max_trip; P.strict_cfl = p.strict_cfl; P.adaptive_dt = p.adaptive_dt;
    P.sort_every = p.sort_every; P.permute_acc = p.permute_acc;
    const int nmax = p.nx > p.ny ? (p.nx > p.nz ? p.nx : p.nz) : (p.ny > p.nz ? p.ny : p.nz);
    P.key_bits = 3 * ceil_log2(nmax);
}

// Reference sounding in double (asph_h100.cu:136-153, 155-163) for the
// device tables.  One node per metre of height; on [k, k+1) the value is a
// quadratic through the values at k, k+1/2 and k+1 (left limit), stored as
// {hi, lo, c1, c2} so that the device recovers the value as the pair
// hi + (lo + t (c1 + t c2)) to ~1e-11 relative.
namespace {
struct SndD {
    double th0, n2, a;
    int qv_mode;
    double qv0, rh, rh_bl, z_bl;
};
constexpr double G_D = 9.80665, RD_D = 287.05, CP_D = 1004.0, P0_D = 100000.0;
double th_ref_d(const SndD& s, double z) { return s.th0 * exp(s.n2 * z / G_D); }
double ex_ref_d(const SndD& s, double z) { return 1.0 - s.a * (1.0 - exp(-s.n2 * z / G_D)); }
double p_ref_d(const SndD& s, double z) { return P0_D * pow(ex_ref_d(s, z), CP_D / RD_D); }
double rho_ref_d(const SndD& s, double z) { return p_ref_d(s, z) / (RD_D * th_ref_d(s, z) * ex_ref_d(s, z)); }
double esat_d(double T) {
    const double Tc = T - 273.15;
    return 611.2 * exp(17.67 * Tc / (Tc + 243.5));
}
double qsat_d(double T, double p) {
    const double es = fmin(esat_d(T), 0.5 * p);
    const double den = p - 0.378 * es;
    return den > 1.0 ? 0.622 * es / den : 0.0;
}
double qv_ref_d(const SndD& s, double z) {
    if (s.qv_mode == ASPH_QV_REFERENCE) return s.qv0 * exp(-z / 2500.0) * exp(-fmax(z - 5000.0, 0.0) / 1000.0);
    const double ex = ex_ref_d(s, z);
    return (z < s.z_bl ? s.rh_bl : s.rh) * qsat_d(th_ref_d(s, z) * ex, P0_D * pow(ex, CP_D / RD_D));
}
double thvr_d(const SndD& s, double z) { return th_ref_d(s, z) * (1.0 + 0.608 * qv_ref_d(s, z)); }

template <class F>
void fill_table(float4* out, int n, F&& f) {
    for (int k = 0; k < n; ++k) {
        const double f0 = f((double)k), fm = f(k + 0.5), f1 = f(k + 1.0 - 1e-9);
        const float hi = (float)f0;
        out[k] = make_float4(hi, (float)(f0 - (double)hi), (float)(-3.0 * f0 + 4.0 * fm - f1),
                             (float)(2.0 * f0 - 4.0 * fm + 2.0 * f1));
    }
}
}  // namespace

static int build_sounding(asph_ctx* c) {
    const AsphParams& p = c->prm;
    SndD s;
    s.th0 = p.th0; s.n2 = p.n2;
    s.a = G_D * G_D / (CP_D * s.th0 * s.n2);
    s.qv_mode = p.qv_mode; s.qv0 = p.qv0; s.rh = p.rh; s.rh_bl = p.rh_bl; s.z_bl = p.z_bl;
    const int n = (int)ceil((double)c->P.lz) + 2;
    std::vector<float4> h((size_t)3 * n);
    fill_table(h.data(), n, [&](double z) { return rho_ref_d(s, z); });
    fill_table(h.data() + n, n, [&](double z) { return p_ref_d(s, z); });
    fill_table(h.data() + 2 * n, n, [&](double z) { return thvr_d(s, z); });
    CKR(c->alloc(&c->B.snd, h.size() * sizeof(float4)));
    CKR(cudaMemcpyAsync(c->B.snd, h.data(), h.size() * sizeof(float4), cudaMemcpyHostToDevice, c->stream));
    CKR(cudaStreamSynchronize(c->stream));
    c->P.snd_rho = c->B.snd;
    c->P.snd_p = c->B.snd + n;
    c->P.snd_thvr = c->B.snd + 2 * n;
    c->P.snd_n = n;
    return ASPH_OK;
}

int asph::reset_control(asph_ctx* c) {
    DevCtl h;
    memset(&h, 0, sizeof(h));
    h.simt = 0.0;
    h.since_sort = 1e9;
    h.dt = (!c->P.adaptive_dt && c->prm.dt_request > 0.f) ? c->prm.dt_request : c->P.dt_cap;
    h.sort_dt = 0.5f;
    h.dt_required = h.dt;
    h.do_sort = 1;
    // The radix look-back epoch is left as it is: status words written by
    // earlier sorts of this context carry epochs up to the current one, so
    // the epoch must only ever grow (it starts at 0 from asph_create).
    CKR(cudaMemcpyAsync(c->B.ctl, &h, offsetof(DevCtl, epoch), cudaMemcpyHostToDevice, c->stream));
    return ASPH_OK;
}

extern "C" int asph_create(const AsphParams* p, void* stream, asph_ctx** out) {
    if (!p || !out) return fail(ASPH_ERR_ARG, "NULL argument");
    *out = nullptr;
    int st = asph_params_check(p);
    if (st) return st;
    asph_ctx* c = new asph_ctx();
    c->prm = *p;
    derive(*p, c->P);
    if (stream) {
        c->stream = (cudaStream_t)stream;
    } else {
        cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            delete c;
            return fail(ASPH_ERR_CUDA, "stream create: %s", cudaGetErrorString(e));
        }
        c->own_stream = true;
    }
    const Phys& P = c->P;
    Bufs& B = c->B;
    memset(&B, 0, sizeof(B));
    {
        cudaError_t e = cudaStreamCreateWithFlags(&B.aux, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&B.ev_fork, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&B.ev_join, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&B.aux2, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&B.ev_fork2, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&B.ev_join2, cudaEventDisableTiming);
        if (e != cudaSuccess) {
            delete c;
            return fail(ASPH_ERR_CUDA, "stream create: %s", cudaGetErrorString(e));
        }
    }
    const size_t N = (size_t)P.N, C = (size_t)P.ncell;
    B.npasses = (P.key_bits + 7) / 8;
    B.ntiles = (int)((N + SORT_TILE - 1) / SORT_TILE);
    cudaError_t e = cudaSuccess;
#define AL(ptr, bytes) \
    if (e == cudaSuccess) e = c->alloc(&(ptr), (bytes))
    for (int k = 0; k < 2; ++k) {
        AL(B.pos[k], N * 16); AL(B.vel[k], N * 16); AL(B.thq[k], N * 16);
        AL(B.kbuf[k], N * 4); AL(B.vbuf[k], N * 4); AL(B.rain[k], C * 4);
    }
    AL(B.skeys_ahead, N * 4); AL(B.perm_ahead, N * 4);
    AL(B.rp, N * 8); AL(B.acc, N * 16); AL(B.ms[0], N * 16); AL(B.ms[1], N * 16); AL(B.dthdt, N * 4); AL(B.kin, N * 4);
    AL(B.status, (size_t)B.npasses * B.ntiles * 256 * 8);
    AL(B.range, C * 8); AL(B.surf, N); AL(B.rain_delta, C * 4); AL(B.precip, (size_t)P.nxy * 4);
    AL(B.ctl, sizeof(DevCtl));
    AL(B.spans, pair_span_slots(P) * 8);
    AL(B.nbr, (size_t)NBR_CAP * N * 4);
    AL(B.nbr_cnt, N * 4);
    AL(B.defer, N * 4);
    sort_inc_sizes(P.N, &B.inc_max, &B.inc_tiles, &B.inc_blocks);
    AL(B.inc_u, N * 4);
    AL(B.inc_uk, N * 4);
    for (int k = 0; k < 2; ++k) {
        AL(B.inc_k[k], (size_t)B.inc_max * 4);
        AL(B.inc_i[k], (size_t)B.inc_max * 4);
    }
    AL(B.inc_cnt, (size_t)B.inc_blocks * 4);
    AL(B.inc_status, (size_t)B.npasses * B.inc_tiles * 256 * 8);
#undef AL
    if (e != cudaSuccess) {
        delete c;
        return fail(e == cudaErrorMemoryAllocation ? ASPH_ERR_NOMEM : ASPH_ERR_CUDA, "allocation: %s",
                    cudaGetErrorString(e));
    }
    B.skeys = B.kbuf[(B.npasses - 1) & 1];
    B.perm = B.vbuf[(B.npasses - 1) & 1];
    B.pc = B.vc = B.qc = B.rc = 0;
    B.shape = -1;
    B.m_tpt = 0;
    cudaStream_t s = c->stream;
    e = cudaMemsetAsync(B.status, 0, (size_t)B.npasses * B.ntiles * 256 * 8, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(B.inc_status, 0, (size_t)B.npasses * B.inc_tiles * 256 * 8, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(B.range, 0, C * 8, s);
    for (int k = 0; k < 2 && e == cudaSuccess; ++k) e = cudaMemsetAsync(B.rain[k], 0, C * 4, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(B.rain_delta, 0, C * 4, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(B.precip, 0, (size_t)P.nxy * 4, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(B.acc, 0, N * 16, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(B.dthdt, 0, N * 4, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(B.rp, 0, N * 8, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(B.surf, 0, N, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(B.perm, 0, N * 4, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(B.skeys, 0, N * 4, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(B.nbr_cnt, 0xff, N * 4, s);   // -1: no list yet
    if (e == cudaSuccess) e = cudaMemsetAsync(B.ctl, 0, sizeof(DevCtl), s);
    if (e != cudaSuccess) {
        delete c;
        return fail(ASPH_ERR_CUDA, "memset: %s", cudaGetErrorString(e));
    }
    st = build_sounding(c);
    if (!st) st = reset_control(c);
    if (st) {
        delete c;
        return st;
    }
    *out = c;
    return ASPH_OK;
}

extern "C" int asph_destroy(asph_ctx* c) {
    if (!c) return ASPH_OK;
    cudaStreamSynchronize(c->stream);
    delete c;
    return ASPH_OK;
}

// Collect the stream status and the device error word.
int asph::sync_status(asph_ctx* c) {
    CKR(cudaStreamSynchronize(c->stream));
    CKR(cudaGetLastError());
    int words[2];
    CKR(cudaMemcpy(words, &c->B.ctl->aborted, sizeof(int), cudaMemcpyDeviceToHost));
    CKR(cudaMemcpy(words + 1, &c->B.ctl->error, sizeof(int), cudaMemcpyDeviceToHost));
    if (words[1]) return fail(words[1], "%s", asph_status_string(words[1]));
    if (words[0]) return fail(ASPH_ERR_CFL_ABORT, "CFL abort: the scheme is outside its stability envelope");
    return ASPH_OK;
}

extern "C" int asph_set_option(asph_ctx* c, int option, int value) {
    if (!c) return fail(ASPH_ERR_ARG, "ctx is NULL");
    if (option == ASPH_OPT_PAIR_PATH) {
        if (value < 0 || value > 2)
            return fail(ASPH_ERR_ARG, "pair path must be 0 (auto), 1 (global) or 2 (warp per target)");
        c->B.force_global = value;
    } else if (option == ASPH_OPT_PAIR_SHAPE) {
        if (value != -1 && !pair_shape_fits(c->P, value))
            return fail(ASPH_ERR_ARG, "brick shape %d does not suit this grid and density", value);
        c->B.shape = value;
    } else if (option == ASPH_OPT_SORT_EVERY) {
        if (value < 0) return fail(ASPH_ERR_ARG, "sort cadence must be >= 0");
        c->P.sort_every = value;
        c->prm.sort_every = value;
    } else if (option == ASPH_OPT_TARGETS_PER_THREAD) {
        if (value != 0 && value != 1 && value != 2 && value != 4)
            return fail(ASPH_ERR_ARG, "momentum targets per thread must be 1, 2 or 4 (0: default)");
        c->B.m_tpt = value;
    } else if (option == ASPH_OPT_SORT_AHEAD) {
        if (value != 0 && value != 1) return fail(ASPH_ERR_ARG, "sort ahead must be 0 or 1");
        c->sort_ahead = value != 0;
    } else {
        return fail(ASPH_ERR_ARG, "unknown option %d", option);
    }
    for (auto& g : c->gexec)   // captured graphs hold the old kernels and parameters
        if (g) { cudaGraphExecDestroy(g); g = nullptr; }
    ++c->graph_epoch;
    if (option == ASPH_OPT_PAIR_PATH || option == ASPH_OPT_PAIR_SHAPE)
        c->spans_valid = false;   // spans are per brick shape
    return ASPH_OK;
}

extern "C" int asph_get_option(asph_ctx* c, int option, int* value) {
    if (!c || !value) return fail(ASPH_ERR_ARG, "NULL argument");
    if (option == ASPH_OPT_PAIR_PATH) {
        *value = c->B.force_global;
        return ASPH_OK;
    }
    if (option == ASPH_OPT_PAIR_SHAPE) {
        *value = pair_shape(c->P, c->B);
        return ASPH_OK;
    }
    if (option == ASPH_OPT_SORT_EVERY) {
        *value = c->P.sort_every;
        return ASPH_OK;
    }
    if (option == ASPH_OPT_TARGETS_PER_THREAD) {
        *value = momentum_tpt(c->B);
        return ASPH_OK;
    }
    if (option == ASPH_OPT_SORT_AHEAD) {
        *value = c->sort_ahead ? 1 : 0;
        return ASPH_OK;
    }
    return fail(ASPH_ERR_ARG, "unknown option %d", option);
}

// ---------------------------------------------------------------------------
// source-term hook
// ---------------------------------------------------------------------------
static void drop_graphs(asph_ctx* c) {
    for (auto& g : c->gexec)
        if (g) { cudaGraphExecDestroy(g); g = nullptr; }
}

extern "C" int asph_source_enable(asph_ctx* c, int on) {
    if (!c) return fail(ASPH_ERR_ARG, "ctx is NULL");
    const size_t N = (size_t)c->P.N;
    if (on && !c->src_mem) {
        CKR(c->alloc(&c->src_mem, N * 32));
        CKR(cudaMemsetAsync(c->src_mem, 0, N * 32, c->stream));
    }
    c->B.src = on ? c->src_mem : nullptr;
    c->B.src_tmp = on ? c->src_mem + N : nullptr;
    drop_graphs(c);   // the captured steps hold the buffer pointers
    return ASPH_OK;
}

extern "C" int asph_source_set(asph_ctx* c, const float* dth, const float* dqv, const float* dqc) {
    if (!c) return fail(ASPH_ERR_ARG, "ctx is NULL");
    if (!c->B.src) return fail(ASPH_ERR_STATE, "source-term hook is off (asph_source_enable)");
    const size_t N = (size_t)c->P.N;
    std::vector<float4> h(N);
    for (size_t i = 0; i < N; ++i)
        h[i] = make_float4(dth ? dth[i] : 0.f, dqv ? dqv[i] : 0.f, dqc ? dqc[i] : 0.f, 0.f);
    CKR(cudaMemcpyAsync(c->B.src, h.data(), N * 16, cudaMemcpyHostToDevice, c->stream));
    CKR(cudaStreamSynchronize(c->stream));
    return ASPH_OK;
}

extern "C" int asph_source_set_device(asph_ctx* c, const void* tendencies) {
    if (!c || !tendencies) return fail(ASPH_ERR_ARG, "NULL argument");
    if (!c->B.src) return fail(ASPH_ERR_STATE, "source-term hook is off (asph_source_enable)");
    CKR(cudaMemcpyAsync(c->B.src, tendencies, (size_t)c->P.N * 16, cudaMemcpyDeviceToDevice, c->stream));
    return ASPH_OK;
}

extern "C" int asph_state_device(asph_ctx* c, void* pos, void* vel, void* thq) {
    if (!c) return fail(ASPH_ERR_ARG, "ctx is NULL");
    if (!c->initialised) return fail(ASPH_ERR_STATE, "no state yet (init/set_state)");
    apply_pending_clamp(c);
    const size_t n = (size_t)c->P.N * 16;
    Bufs& B = c->B;
    if (pos) CKR(cudaMemcpyAsync(pos, B.pos[B.pc], n, cudaMemcpyDeviceToDevice, c->stream));
    if (vel) CKR(cudaMemcpyAsync(vel, B.vel[B.vc], n, cudaMemcpyDeviceToDevice, c->stream));
    if (thq) CKR(cudaMemcpyAsync(thq, B.thq[B.qc], n, cudaMemcpyDeviceToDevice, c->stream));
    return ASPH_OK;
}

extern "C" int asph_sync(asph_ctx* c) {
    if (!c) return fail(ASPH_ERR_ARG, "ctx is NULL");
    return sync_status(c);
}

// ---------------------------------------------------------------------------
// granular blocks of the reference step
// ---------------------------------------------------------------------------
bool asph::reads_rain(const Phys& P) { return P.accretion || P.rain_evap; }

static void do_sort_build(asph_ctx* c, int force) {
    launch_sort_prep(c->P, c->B, force, 0, c->stream);
    launch_sort(c->P, c->B, force, c->stream);
    launch_gather(c->P, c->B, G_SORTED | (force ? G_FORCE : 0), c->stream);
    c->B.pc ^= 1; c->B.vc ^= 1; c->B.qc ^= 1;
    if (force) c->spans_valid = true;   // the gather of a sort writes the brick spans
    // source-term tendencies follow their particles (a step keeps them in its momentum pass)
    if (c->B.src)
        cudaMemcpyAsync(c->B.src, c->B.src_tmp, (size_t)c->P.N * 16, cudaMemcpyDeviceToDevice, c->stream);
}

extern "C" int asph_init(asph_ctx* c) {
    if (!c) return fail(ASPH_ERR_ARG, "ctx is NULL");
    const AsphParams& p = c->prm;
    float bub[5 * ASPH_MAX_BUBBLES];
    for (int b = 0; b < p.n_bubbles; ++b) {
        bub[5 * b + 0] = p.bubble_x[b]; bub[5 * b + 1] = p.bubble_y[b]; bub[5 * b + 2] = p.bubble_z[b];
        bub[5 * b + 3] = p.bubble_r[b]; bub[5 * b + 4] = p.bubble_amp[b];
    }
    int st = reset_control(c);
    if (st) return st;
    CKR(cudaMemsetAsync(c->B.rain[0], 0, (size_t)c->P.ncell * 4, c->stream));
    CKR(cudaMemsetAsync(c->B.rain[1], 0, (size_t)c->P.ncell * 4, c->stream));
    CKR(cudaMemsetAsync(c->B.rain_delta, 0, (size_t)c->P.ncell * 4, c->stream));
    CKR(cudaMemsetAsync(c->B.precip, 0, (size_t)c->P.nxy * 4, c->stream));
    launch_init(c->P, c->B, bub, p.n_bubbles, p.init_mode, p.lat_nx, p.lat_ny, p.lat_nz, p.jitter, p.seed, p.noise,
                c->stream);
    launch_keys(c->P, c->B, c->stream);
    do_sort_build(c, 1);
    launch_density(c->P, c->B, c->stream);
    launch_momentum(c->P, c->B, 0, 1, c->stream);
    c->lists_valid = true;
    CKR(cudaGetLastError());
    c->initialised = true;
    return sync_status(c);
}

static int ensure_stage(asph_ctx* c) {
    if (!c->stage) CKR(c->alloc(&c->stage, (size_t)c->P.N * 16 * sizeof(float)));
    return ASPH_OK;
}

namespace asph {
__global__ void k_pack(Phys P, const float* __restrict__ st, unsigned mask, float4* pos, float4* vel, float4* thq,
                       float2* rp, float4* acc, float* dthdt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const size_t N = (size_t)P.N;
    auto f = [&](int k) { return (mask >> k) & 1u ? st[k * N + i] : 0.f; };
    const float rho = f(9);
    pos[i] = make_float4(f(0), f(1), f(2), rho);
    vel[i] = make_float4(f(3), f(4), f(5), 0.f);
    thq[i] = make_float4(f(6), f(7), f(8), 0.f);
    rp[i] = make_float2(rho, f(13));
    acc[i] = make_float4(f(10), f(11), f(12), 0.f);
    dthdt[i] = f(14);
}
__global__ void k_unpack(Phys P, float* __restrict__ st, const float4* pos, const float4* vel, const float4* thq,
                         const float2* rp, const float4* acc, const float* dthdt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const size_t N = (size_t)P.N;
    const float4 p = pos[i], v = vel[i], t = thq[i], a = acc[i];
    const float2 r = rp[i];
    st[0 * N + i] = p.x; st[1 * N + i] = p.y; st[2 * N + i] = p.z;
    st[3 * N + i] = v.x; st[4 * N + i] = v.y; st[5 * N + i] = v.z;
    st[6 * N + i] = t.x; st[7 * N + i] = t.y; st[8 * N + i] = t.z;
    st[9 * N + i] = r.x;
    st[10 * N + i] = a.x; st[11 * N + i] = a.y; st[12 * N + i] = a.z;
    st[13 * N + i] = r.y; st[14 * N + i] = dthdt[i];
}
// The same packing straight from / into pinned host arrays: the kernel
// reads and writes host memory over the host link, so the fields need no
// staging copy (one pass each way instead of a copy plus a pass).
struct HostFields {
    float* f[15];   // device-usable addresses of the caller's pinned arrays, NULL = absent
};
__global__ void k_pack_host(Phys P, HostFields H, float4* pos, float4* vel, float4* thq, float2* rp, float4* acc,
                            float* dthdt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    auto f = [&](int k) { return H.f[k] ? H.f[k][i] : 0.f; };
    const float rho = f(9);
    pos[i] = make_float4(f(0), f(1), f(2), rho);
    vel[i] = make_float4(f(3), f(4), f(5), 0.f);
    thq[i] = make_float4(f(6), f(7), f(8), 0.f);
    rp[i] = make_float2(rho, f(13));
    acc[i] = make_float4(f(10), f(11), f(12), 0.f);
    dthdt[i] = f(14);
}
__global__ void k_unpack_host(Phys P, HostFields H, const float4* pos, const float4* vel, const float4* thq,
                              const float2* rp, const float4* acc, const float* dthdt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const float4 p = pos[i], v = vel[i], t = thq[i], a = acc[i];
    const float2 r = rp[i];
    const float val[15] = {p.x, p.y, p.z, v.x, v.y, v.z, t.x, t.y, t.z, r.x, a.x, a.y, a.z, r.y, dthdt[i]};
#pragma unroll
    for (int k = 0; k < 15; ++k)
        if (H.f[k]) H.f[k][i] = val[k];
}
}  // namespace asph

// Device-usable addresses of the non-NULL fields when every one of them is
// pinned (page-locked) host memory; false otherwise (pageable arrays take
// the staged path).
static bool pinned_fields(float* const f[15], HostFields* H) {
    for (int k = 0; k < 15; ++k) {
        H->f[k] = nullptr;
        if (!f[k]) continue;
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, f[k]) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        if (a.type != cudaMemoryTypeHost || !a.devicePointer) return false;
        H->f[k] = (float*)a.devicePointer;
    }
    return true;
}

static float* const* state_fields(const AsphHostState* s, float* out[15]) {
    float* f[15] = {s->x, s->y, s->z, s->u, s->v, s->w, s->th, s->qv, s->qc, s->rho, s->ax, s->ay, s->az, s->prs, s->dthdt};
    for (int k = 0; k < 15; ++k) out[k] = f[k];
    return out;
}

extern "C" int asph_set_state(asph_ctx* c, const AsphHostState* s) {
    if (!c || !s) return fail(ASPH_ERR_ARG, "NULL argument");
    float* f[15];
    state_fields(s, f);
    for (int k = 0; k < 10; ++k)
        if (!f[k]) return fail(ASPH_ERR_ARG, "set_state: field %d (x..rho) is required", k);
    Bufs& B = c->B;
    HostFields H;
    if (pinned_fields(f, &H)) {
        k_pack_host<<<(c->P.N + TPB - 1) / TPB, TPB, 0, c->stream>>>(c->P, H, B.pos[B.pc], B.vel[B.vc], B.thq[B.qc],
                                                                     B.rp, B.acc, B.dthdt);
    } else {
        int st = ensure_stage(c);
        if (st) return st;
        const size_t N = (size_t)c->P.N;
        unsigned mask = 0;
        for (int k = 0; k < 15; ++k) {
            if (!f[k]) continue;
            mask |= 1u << k;
            CKR(cudaMemcpyAsync(c->stage + k * N, f[k], N * 4, cudaMemcpyHostToDevice, c->stream));
        }
        k_pack<<<(c->P.N + TPB - 1) / TPB, TPB, 0, c->stream>>>(c->P, c->stage, mask, B.pos[B.pc], B.vel[B.vc],
                                                                B.thq[B.qc], B.rp, B.acc, B.dthdt);
    }
    launch_keys(c->P, B, c->stream);
    CKR(cudaGetLastError());
    c->initialised = true;
    c->lists_valid = false;
    return sync_status(c);
}

void asph::apply_pending_clamp(asph_ctx* c) { launch_clamp(c->P, c->B, c->stream); }

extern "C" int asph_get_state(asph_ctx* c, AsphHostState* s) {
    if (!c || !s) return fail(ASPH_ERR_ARG, "NULL argument");
    apply_pending_clamp(c);
    Bufs& B = c->B;
    float* f[15];
    state_fields(s, f);
    HostFields H;
    if (pinned_fields(f, &H)) {
        k_unpack_host<<<(c->P.N + TPB - 1) / TPB, TPB, 0, c->stream>>>(c->P, H, B.pos[B.pc], B.vel[B.vc],
                                                                       B.thq[B.qc], B.rp, B.acc, B.dthdt);
        CKR(cudaGetLastError());
        CKR(cudaStreamSynchronize(c->stream));
        return ASPH_OK;
    }
    int st = ensure_stage(c);
    if (st) return st;
    k_unpack<<<(c->P.N + TPB - 1) / TPB, TPB, 0, c->stream>>>(c->P, c->stage, B.pos[B.pc], B.vel[B.vc], B.thq[B.qc],
                                                              B.rp, B.acc, B.dthdt);
    CKR(cudaGetLastError());
    const size_t N = (size_t)c->P.N;
    for (int k = 0; k < 15; ++k)
        if (f[k]) CKR(cudaMemcpyAsync(f[k], c->stage + k * N, N * 4, cudaMemcpyDeviceToHost, c->stream));
    CKR(cudaStreamSynchronize(c->stream));
    return ASPH_OK;
}

extern "C" int asph_get_rain(asph_ctx* c, float* rain, float* precip) {
    if (!c) return fail(ASPH_ERR_ARG, "ctx is NULL");
    if (rain)
        CKR(cudaMemcpyAsync(rain, c->B.rain[c->B.rc], (size_t)c->P.ncell * 4, cudaMemcpyDeviceToHost, c->stream));
    if (precip) CKR(cudaMemcpyAsync(precip, c->B.precip, (size_t)c->P.nxy * 4, cudaMemcpyDeviceToHost, c->stream));
    CKR(cudaStreamSynchronize(c->stream));
    return ASPH_OK;
}

extern "C" int asph_set_rain(asph_ctx* c, const float* rain, const float* precip) {
    if (!c) return fail(ASPH_ERR_ARG, "ctx is NULL");
    if (rain)
        CKR(cudaMemcpyAsync(c->B.rain[c->B.rc], rain, (size_t)c->P.ncell * 4, cudaMemcpyHostToDevice, c->stream));
    if (precip) CKR(cudaMemcpyAsync(c->B.precip, precip, (size_t)c->P.nxy * 4, cudaMemcpyHostToDevice, c->stream));
    CKR(cudaStreamSynchronize(c->stream));
    return ASPH_OK;
}

extern "C" int asph_get_control(asph_ctx* c, AsphControl* o) {
    if (!c || !o) return fail(ASPH_ERR_ARG, "NULL argument");
    DevCtl h;
    CKR(cudaMemcpyAsync(&h, c->B.ctl, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    CKR(cudaStreamSynchronize(c->stream));
    o->simt = h.simt; o->since_sort = h.since_sort; o->dt = h.dt;
    o->dt_cap = c->P.dt_cap; o->dt_floor = c->P.dt_floor; o->dt_static = c->P.dt_static;
    o->dt_required = h.dt_required; o->sort_dt = h.sort_dt;
    o->umax = h.umax; o->vmax = h.vmax; o->wmax = h.wmax;
    o->step = h.step; o->trips = h.trips; o->sort_count = h.sort_count; o->aborted = h.aborted;
    o->clamp_pending = h.clamp_pending; o->do_sort = h.do_sort; o->error = h.error; o->surf_count = h.surf_count;
    o->deferred = (int32_t)h.defer_last;
    o->split_regions = (int32_t)h.split_last;
    return ASPH_OK;
}

extern "C" int asph_set_time(asph_ctx* c, double simt, float dt, int do_sort) {
    if (!c) return fail(ASPH_ERR_ARG, "ctx is NULL");
    DevCtl h;
    CKR(cudaMemcpyAsync(&h, c->B.ctl, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    CKR(cudaStreamSynchronize(c->stream));
    h.simt = simt;
    if (dt > 0.f) h.dt = dt;
    h.do_sort = do_sort ? 1 : 0;
    CKR(cudaMemcpyAsync(c->B.ctl, &h, sizeof(h), cudaMemcpyHostToDevice, c->stream));
    CKR(cudaStreamSynchronize(c->stream));
    return ASPH_OK;
}

namespace asph {
// After a standalone sort the single-buffered outputs of the last density
// and momentum passes (rho, p', acc) are still in the pre-sort order; put
// them in the new order (acc only when it follows its particle).
__global__ void k_sort_fixup_a(Phys P, const uint32_t* __restrict__ perm, const float2* __restrict__ rp,
                               const float4* __restrict__ acc, float4* __restrict__ tmp, int move_acc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const uint32_t s = perm[i];
    const float4 a = move_acc ? acc[s] : acc[i];
    tmp[i] = make_float4(a.x, a.y, a.z, rp[s].y);
}
__global__ void k_sort_fixup_b(Phys P, const float4* __restrict__ pos, const float4* __restrict__ tmp,
                               float2* __restrict__ rp, float4* __restrict__ acc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const float4 t = tmp[i];
    rp[i] = make_float2(pos[i].w, t.w);
    acc[i] = make_float4(t.x, t.y, t.z, 0.f);
}
}  // namespace asph

extern "C" int asph_sort_build(asph_ctx* c) {
    if (!c) return fail(ASPH_ERR_ARG, "ctx is NULL");
    if (!c->initialised) return fail(ASPH_ERR_STATE, "sort before init/set_state");
    int st = ensure_stage(c);
    if (st) return st;
    do_sort_build(c, 1);
    c->lists_valid = false;
    Bufs& B = c->B;
    const int nb = (c->P.N + TPB - 1) / TPB;
    float4* tmp = reinterpret_cast<float4*>(c->stage);
    k_sort_fixup_a<<<nb, TPB, 0, c->stream>>>(c->P, B.perm, B.rp, B.acc, tmp, c->P.permute_acc);
    k_sort_fixup_b<<<nb, TPB, 0, c->stream>>>(c->P, B.pos[B.pc], tmp, B.rp, B.acc);
    CKR(cudaGetLastError());
    return sync_status(c);
}

extern "C" int asph_get_sort(asph_ctx* c, uint32_t* keys_in, uint32_t* keys_sorted, uint32_t* perm,
                             int32_t* cell_range, int32_t* surf_list, int32_t* surf_count) {
    if (!c) return fail(ASPH_ERR_ARG, "ctx is NULL");
    const size_t N = (size_t)c->P.N;
    cudaStream_t s = c->stream;
    if (keys_in) CKR(cudaMemcpyAsync(keys_in, c->B.kin, N * 4, cudaMemcpyDeviceToHost, s));
    if (keys_sorted) CKR(cudaMemcpyAsync(keys_sorted, c->B.skeys, N * 4, cudaMemcpyDeviceToHost, s));
    if (perm) CKR(cudaMemcpyAsync(perm, c->B.perm, N * 4, cudaMemcpyDeviceToHost, s));
    if (cell_range)
        CKR(cudaMemcpyAsync(cell_range, c->B.range, (size_t)c->P.ncell * 8, cudaMemcpyDeviceToHost, s));
    if (surf_list || surf_count) {
        std::vector<uint8_t> fl(N);
        CKR(cudaMemcpyAsync(fl.data(), c->B.surf, N, cudaMemcpyDeviceToHost, s));
        CKR(cudaStreamSynchronize(s));
        int32_t n = 0;
        for (size_t i = 0; i < N; ++i)
            if (fl[i]) {
                if (surf_list) surf_list[n] = (int32_t)i;
                ++n;
            }
        if (surf_count) *surf_count = n;
    }
    CKR(cudaStreamSynchronize(s));
    return ASPH_OK;
}

extern "C" int asph_get_neighbours(asph_ctx* c, int32_t* count, int32_t* list) {
    if (!c) return fail(ASPH_ERR_ARG, "ctx is NULL");
    if (!c->lists_valid) return fail(ASPH_ERR_STATE, "no neighbour lists for the current positions");
    const size_t N = (size_t)c->P.N;
    if (count) CKR(cudaMemcpyAsync(count, c->B.nbr_cnt, N * 4, cudaMemcpyDeviceToHost, c->stream));
    if (list) CKR(cudaMemcpyAsync(list, c->B.nbr, N * NBR_CAP * 4, cudaMemcpyDeviceToHost, c->stream));
    CKR(cudaStreamSynchronize(c->stream));
    return ASPH_OK;
}

extern "C" int asph_kick_drift_flux(asph_ctx* c) {
    if (!c) return fail(ASPH_ERR_ARG, "ctx is NULL");
    launch_gather(c->P, c->B, G_INTEGRATE, c->stream);
    c->B.pc ^= 1; c->B.vc ^= 1; c->B.qc ^= 1;
    c->lists_valid = false;
    CKR(cudaGetLastError());
    return sync_status(c);
}

void asph::ensure_spans(asph_ctx* c) {
    if (c->spans_valid) return;
    launch_brick_spans(c->P, c->B, c->stream);
    c->spans_valid = true;
}

extern "C" int asph_density_eos(asph_ctx* c) {
    if (!c) return fail(ASPH_ERR_ARG, "ctx is NULL");
    ensure_spans(c);
    launch_density(c->P, c->B, c->stream);
    c->lists_valid = true;
    CKR(cudaGetLastError());
    return sync_status(c);
}

extern "C" int asph_momentum(asph_ctx* c, int integrate) {
    if (!c) return fail(ASPH_ERR_ARG, "ctx is NULL");
    launch_momentum(c->P, c->B, integrate ? M_INTEGRATE : 0, c->lists_valid ? 1 : 0, c->stream);
    if (integrate) c->B.vc ^= 1;
    CKR(cudaGetLastError());
    return sync_status(c);
}

extern "C" int asph_rain(asph_ctx* c) {
    if (!c) return fail(ASPH_ERR_ARG, "ctx is NULL");
    launch_rain(c->P, c->B, c->stream);
    c->B.rc ^= 1;
    if (reads_rain(c->P)) CKR(cudaMemsetAsync(c->B.rain_delta, 0, (size_t)c->P.ncell * 4, c->stream));
    CKR(cudaGetLastError());
    return sync_status(c);
}

extern "C" int asph_cfl(asph_ctx* c) {
    if (!c) return fail(ASPH_ERR_ARG, "ctx is NULL");
    launch_cfl(c->P, c->B, c->stream);
    CKR(cudaGetLastError());
    return sync_status(c);
}

// One full step: sort (gated on the device) -> G -> D -> M(+rain,+CFL).
// In a run of steps with a sort every step, the next step's sort is forked
// off after G (it needs G's keys of the drifted positions and the last
// applied sort, and writes only its own buffers) and joined after M, so it
// runs beside D and M; the next step's G applies it (StepKind).
void asph::enqueue_step(asph_ctx* c, int kind) {
    const Phys& P = c->P;
    launch_sort_prep(P, c->B, 0, reads_rain(P) ? 1 : 0, c->stream);
    if (kind == STEP_PLAIN || kind == STEP_FIRST) launch_sort(P, c->B, 0, c->stream);
    launch_gather(P, c->B, G_SORTED | G_INTEGRATE | ((kind == STEP_MID || kind == STEP_LAST) ? G_AHEAD : 0),
                  c->stream);
    c->B.pc ^= 1; c->B.vc ^= 1; c->B.qc ^= 1;
    const bool ahead = kind == STEP_FIRST || kind == STEP_MID;
    if (ahead) launch_sort_ahead(P, c->B, c->stream);
    launch_density(P, c->B, c->stream);
    launch_momentum(P, c->B, M_INTEGRATE | M_RAIN | M_CFL, 1, c->stream);
    if (ahead) cudaStreamWaitEvent(c->stream, c->B.ev_join2, 0);
    c->B.vc ^= 1; c->B.rc ^= 1;
    c->lists_valid = true;
}

extern "C" int asph_step_profiled(asph_ctx* c, int nsteps, float* phase_ms) {
    if (!c || !phase_ms) return fail(ASPH_ERR_ARG, "NULL argument");
    if (!c->initialised) return fail(ASPH_ERR_STATE, "step before init/set_state");
    ensure_spans(c);
    const Phys& P = c->P;
    cudaEvent_t ev[7];
    for (auto& e : ev) CKR(cudaEventCreate(&e));
    double acc[ASPH_NPHASES] = {0, 0, 0, 0, 0, 0};
    int st = ASPH_OK;
    for (int k = 0; k < nsteps && st == ASPH_OK; ++k) {
        cudaStream_t s = c->stream;
        cudaEventRecord(ev[0], s);
        launch_sort_prep(P, c->B, 0, reads_rain(P) ? 1 : 0, s);
        cudaEventRecord(ev[1], s);
        launch_sort(P, c->B, 0, s);   // histogram + radix passes
        cudaEventRecord(ev[2], s);
        launch_gather(P, c->B, G_SORTED | G_INTEGRATE, s);
        c->B.pc ^= 1; c->B.vc ^= 1; c->B.qc ^= 1;
        cudaEventRecord(ev[3], s);
        launch_density(P, c->B, s);
        cudaEventRecord(ev[4], s);
        launch_momentum(P, c->B, M_INTEGRATE | M_RAIN | M_CFL, 1, s);
        c->B.vc ^= 1; c->B.rc ^= 1;
        cudaEventRecord(ev[5], s);
        cudaError_t e = cudaEventSynchronize(ev[5]);
        if (e != cudaSuccess) { st = fail(ASPH_ERR_CUDA, "profiled step: %s", cudaGetErrorString(e)); break; }
        float ms;
        for (int ph = 0; ph < 5; ++ph) {
            cudaEventElapsedTime(&ms, ev[ph], ev[ph + 1]);
            acc[ph] += ms;
        }
        cudaEventElapsedTime(&ms, ev[0], ev[5]);
        acc[5] += ms;
    }
    for (auto& e : ev) cudaEventDestroy(e);
    for (int ph = 0; ph < ASPH_NPHASES; ++ph) phase_ms[ph] = (float)acc[ph];
    if (st) return st;
    return sync_status(c);
}

int asph::graph_slot(const Bufs& B) { return B.pc | (B.vc << 1) | (B.qc << 2) | (B.rc << 3); }

// Capture the step of `kind` that starts from the current ping-pong state
// into its graph (the indices are left as they were); counts the graph's
// kernels.
static int capture_step_graph(asph_ctx* c, int kind) {
    const int slot = kind * 16 + graph_slot(c->B);
    const Bufs saved = c->B;
    cudaGraph_t g = nullptr;
    CKR(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    if (kind == STEP_MID2) {   // two middle steps in one graph
        enqueue_step(c, STEP_MID);
        enqueue_step(c, STEP_MID);
    } else {
        enqueue_step(c, kind);
    }
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    c->B = saved;
    if (e != cudaSuccess) return fail(ASPH_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
    size_t nn = 0;
    e = cudaGraphGetNodes(g, nullptr, &nn);
    std::vector<cudaGraphNode_t> nodes(nn);
    if (e == cudaSuccess && nn) e = cudaGraphGetNodes(g, nodes.data(), &nn);
    int kernels = 0;
    for (size_t k = 0; e == cudaSuccess && k < nn; ++k) {
        cudaGraphNodeType t;
        e = cudaGraphNodeGetType(nodes[k], &t);
        kernels += (e == cudaSuccess && t == cudaGraphNodeTypeKernel) ? 1 : 0;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&c->gexec[slot], g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(ASPH_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
    c->graph_kernels[kind] = kernels;
    return ASPH_OK;
}

// Whether a run of nsteps steps sorts ahead (a sort every step, the option
// on, at least two steps).
static bool runs_ahead(const asph_ctx* c, int nsteps) {
    return c->sort_ahead && c->P.sort_every == 1 && nsteps >= 2;
}

static int step_kind(const asph_ctx* c, int k, int nsteps) {
    if (!runs_ahead(c, nsteps)) return STEP_PLAIN;
    return k == 0 ? STEP_FIRST : (k == nsteps - 1 ? STEP_LAST : STEP_MID);
}

// Kernel nodes per step of a long run: the middle steps' graph when the run
// sorts ahead, else the plain step's.
extern "C" int asph_step_kernels(asph_ctx* c, int* n) {
    if (!c || !n) return fail(ASPH_ERR_ARG, "NULL argument");
    if (!c->initialised) return fail(ASPH_ERR_STATE, "step_kernels before init/set_state");
    const int kind = step_kind(c, 1, 3);
    if (!c->gexec[kind * 16 + graph_slot(c->B)]) {
        const int st = capture_step_graph(c, kind);
        if (st) return st;
    }
    *n = c->graph_kernels[kind];
    return ASPH_OK;
}

extern "C" int asph_step_async(asph_ctx* c, int nsteps) {
    if (!c) return fail(ASPH_ERR_ARG, "ctx is NULL");
    if (!c->initialised) return fail(ASPH_ERR_STATE, "step before init/set_state");
    ensure_spans(c);
    for (int k = 0; k < nsteps;) {
        int kind = step_kind(c, k, nsteps), adv = 1;
        // two middle steps per graph launch: one inter-graph gap fewer per pair
        // (524k: 0.270 -> 0.267 ms per step)
        if (kind == STEP_MID && k + 2 <= nsteps - 1) { kind = STEP_MID2; adv = 2; }
        const int slot = kind * 16 + graph_slot(c->B);
        if (!c->gexec[slot]) {
            const int st = capture_step_graph(c, kind);
            if (st) return st;
        }
        CKR(cudaGraphLaunch(c->gexec[slot], c->stream));
        for (int a = 0; a < adv; ++a) { c->B.pc ^= 1; c->B.qc ^= 1; c->B.rc ^= 1; }   // vel flips twice per step
        c->lists_valid = true;
        k += adv;
    }
    return ASPH_OK;
}

extern "C" int asph_step(asph_ctx* c, int nsteps) {
    int st = asph_step_async(c, nsteps);
    if (st) return st;
    return sync_status(c);
}

// ---------------------------------------------------------------------------
// diagnostics and dumps
// ---------------------------------------------------------------------------
extern "C" int asph_audit(asph_ctx* c, double out[6]) {
    if (!c || !out) return fail(ASPH_ERR_ARG, "NULL argument");
    if (!c->audit_part) {
        CKR(c->alloc(&c->audit_part, (size_t)c->audit_blocks * 5 * sizeof(double)));
        CKR(c->alloc(&c->audit_out, 6 * sizeof(double)));
    }
    apply_pending_clamp(c);
    launch_audit(c->P, audit_constants(c->prm), c->B, c->audit_part, c->audit_blocks, c->audit_out, c->stream);
    CKR(cudaGetLastError());
    CKR(cudaMemcpyAsync(out, c->audit_out, 6 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CKR(cudaStreamSynchronize(c->stream));
    return ASPH_OK;
}

static int ensure_dump(asph_ctx* c) {
    const AsphParams& p = c->prm;
    c->cx = (p.nx + p.dump_sx - 1) / p.dump_sx;
    c->cy = (p.ny + p.dump_sy - 1) / p.dump_sy;
    c->cz = (p.nz + p.dump_sz - 1) / p.dump_sz;
    if (!c->coarse) {
        CKR(c->alloc(&c->coarse, (size_t)c->cx * c->cy * c->cz * 6 * sizeof(float)));
        CKR(c->alloc(&c->coldiag, (size_t)c->P.nxy * sizeof(float4)));
    }
    return ASPH_OK;
}

// Dump header (asph_h100.cu:743-747), 68 bytes little-endian.
struct DumpHeader {
    uint32_t magic, version;
    int32_t nx, ny, nz, cx, cy, cz, sx, sy, sz, nfields;
    float t_sim, dt, lx, ly, lz;
};
static_assert(sizeof(DumpHeader) == 68, "dump header is 68 bytes");

extern "C" int asph_dump(asph_ctx* c, const char* outdir, char* path, int path_len) {
    if (!c || !outdir) return fail(ASPH_ERR_ARG, "NULL argument");
    int st = ensure_dump(c);
    if (st) return st;
    apply_pending_clamp(c);
    const AsphParams& p = c->prm;
    launch_coarse(c->P, c->B, c->coarse, p.dump_sx, p.dump_sy, p.dump_sz, c->cx, c->cy, c->cz, c->coldiag, c->stream);
    CKR(cudaGetLastError());
    const size_t n = (size_t)c->cx * c->cy * c->cz * 6;
    std::vector<float> h(n);
    CKR(cudaMemcpyAsync(h.data(), c->coarse, n * 4, cudaMemcpyDeviceToHost, c->stream));
    DevCtl ctl;
    CKR(cudaMemcpyAsync(&ctl, c->B.ctl, sizeof(ctl), cudaMemcpyDeviceToHost, c->stream));
    CKR(cudaStreamSynchronize(c->stream));
    mkdir(outdir, 0775);
    char fn[1024];
    snprintf(fn, sizeof(fn), "%s/asph_t%06.0fs.bin", outdir, ctl.simt);   // asph_h100.cu:1107
    FILE* f = fopen(fn, "wb");
    if (!f) return fail(ASPH_ERR_IO, "cannot open %s", fn);
    DumpHeader hh{};
    hh.magic = 0x41535048u; hh.version = 3;
    hh.nx = p.nx; hh.ny = p.ny; hh.nz = p.nz;
    hh.cx = c->cx; hh.cy = c->cy; hh.cz = c->cz;
    hh.sx = p.dump_sx; hh.sy = p.dump_sy; hh.sz = p.dump_sz;
    hh.nfields = 6; hh.t_sim = (float)ctl.simt; hh.dt = ctl.dt;
    hh.lx = c->P.lx; hh.ly = c->P.ly; hh.lz = c->P.lz;
    const bool ok = fwrite(&hh, sizeof(hh), 1, f) == 1 && fwrite(h.data(), 4, n, f) == n;
    fclose(f);
    if (!ok) return fail(ASPH_ERR_IO, "short write to %s", fn);
    if (path && path_len > 0) snprintf(path, (size_t)path_len, "%s", fn);
    return ASPH_OK;
}

// Asynchronous dump: the coarse fields, the column diagnostics, the surface
// precipitation and the control block are copied into pinned host memory on
// the context's stream; steps queued afterwards run while the copy completes
// and the file is written.
extern "C" int asph_dump_begin(asph_ctx* c) {
    if (!c) return fail(ASPH_ERR_ARG, "ctx is NULL");
    if (c->dump_pending) return fail(ASPH_ERR_STATE, "a dump is already in flight (asph_dump_finish)");
    int st = ensure_dump(c);
    if (st) return st;
    const size_t n = (size_t)c->cx * c->cy * c->cz * 6, ncol = (size_t)c->P.nxy;
    if (!c->h_dump) {
        CKR(cudaMallocHost(&c->h_dump, n * 4 + ncol * 20 + sizeof(DevCtl)));
        CKR(cudaEventCreateWithFlags(&c->dump_ev, cudaEventDisableTiming));
    }
    apply_pending_clamp(c);
    const AsphParams& p = c->prm;
    launch_coarse(c->P, c->B, c->coarse, p.dump_sx, p.dump_sy, p.dump_sz, c->cx, c->cy, c->cz, c->coldiag, c->stream);
    CKR(cudaGetLastError());
    char* h = (char*)c->h_dump;
    CKR(cudaMemcpyAsync(h, c->coarse, n * 4, cudaMemcpyDeviceToHost, c->stream));
    CKR(cudaMemcpyAsync(h + n * 4, c->coldiag, ncol * 16, cudaMemcpyDeviceToHost, c->stream));
    CKR(cudaMemcpyAsync(h + n * 4 + ncol * 16, c->B.precip, ncol * 4, cudaMemcpyDeviceToHost, c->stream));
    CKR(cudaMemcpyAsync(h + n * 4 + ncol * 20, c->B.ctl, sizeof(DevCtl), cudaMemcpyDeviceToHost, c->stream));
    // the precipitation accumulator restarts at every dump (asph_h100.cu:1105)
    CKR(cudaMemsetAsync(c->B.precip, 0, ncol * 4, c->stream));
    CKR(cudaEventRecord(c->dump_ev, c->stream));
    c->dump_pending = true;
    return ASPH_OK;
}

extern "C" int asph_dump_finish(asph_ctx* c, const char* outdir, char* path, int path_len, float diag[4]) {
    if (!c || !outdir) return fail(ASPH_ERR_ARG, "NULL argument");
    if (!c->dump_pending) return fail(ASPH_ERR_STATE, "no dump in flight (asph_dump_begin)");
    c->dump_pending = false;
    CKR(cudaEventSynchronize(c->dump_ev));
    const AsphParams& p = c->prm;
    const size_t n = (size_t)c->cx * c->cy * c->cz * 6, ncol = (size_t)c->P.nxy;
    const char* h = (const char*)c->h_dump;
    const float* coarse = (const float*)h;
    const float4* cd = (const float4*)(h + n * 4);
    const float* pr = (const float*)(h + n * 4 + ncol * 16);
    DevCtl ctl;
    memcpy(&ctl, h + n * 4 + ncol * 20, sizeof ctl);
    if (diag) {
        int ncloud = 0;
        float qlmax = 0.f, wmax = 0.f, psum = 0.f;
        for (size_t k = 0; k < ncol; ++k) {   // asph_h100.cu:1095-1102
            if (cd[k].z > 1e-4f) ++ncloud;
            qlmax = fmaxf(qlmax, cd[k].z);
            wmax = fmaxf(wmax, cd[k].w);
            psum += pr[k];
        }
        diag[0] = ncol ? 100.f * (float)ncloud / ncol : 0.f;
        diag[1] = qlmax;
        diag[2] = wmax;
        diag[3] = ncol ? psum / ncol : 0.f;
    }
    mkdir(outdir, 0775);
    char fn[1024];
    snprintf(fn, sizeof(fn), "%s/asph_t%06.0fs.bin", outdir, ctl.simt);   // asph_h100.cu:1107
    FILE* f = fopen(fn, "wb");
    if (!f) return fail(ASPH_ERR_IO, "cannot open %s", fn);
    DumpHeader hh{};
    hh.magic = 0x41535048u; hh.version = 3;
    hh.nx = p.nx; hh.ny = p.ny; hh.nz = p.nz;
    hh.cx = c->cx; hh.cy = c->cy; hh.cz = c->cz;
    hh.sx = p.dump_sx; hh.sy = p.dump_sy; hh.sz = p.dump_sz;
    hh.nfields = 6; hh.t_sim = (float)ctl.simt; hh.dt = ctl.dt;
    hh.lx = c->P.lx; hh.ly = c->P.ly; hh.lz = c->P.lz;
    const bool ok = fwrite(&hh, sizeof(hh), 1, f) == 1 && fwrite(coarse, 4, n, f) == n;
    fclose(f);
    if (!ok) return fail(ASPH_ERR_IO, "short write to %s", fn);
    if (path && path_len > 0) snprintf(path, (size_t)path_len, "%s", fn);
    return ASPH_OK;
}

extern "C" int asph_column_diag(asph_ctx* c, float out[4]) {
    if (!c || !out) return fail(ASPH_ERR_ARG, "NULL argument");
    int st = ensure_dump(c);
    if (st) return st;
    apply_pending_clamp(c);
    const AsphParams& p = c->prm;
    launch_coarse(c->P, c->B, c->coarse, p.dump_sx, p.dump_sy, p.dump_sz, c->cx, c->cy, c->cz, c->coldiag, c->stream);
    CKR(cudaGetLastError());
    const int ncol = c->P.nxy;
    std::vector<float4> cd(ncol);
    std::vector<float> pr(ncol);
    CKR(cudaMemcpyAsync(cd.data(), c->coldiag, (size_t)ncol * sizeof(float4), cudaMemcpyDeviceToHost, c->stream));
    CKR(cudaMemcpyAsync(pr.data(), c->B.precip, (size_t)ncol * 4, cudaMemcpyDeviceToHost, c->stream));
    CKR(cudaStreamSynchronize(c->stream));
    int ncloud = 0;
    float qlmax = 0.f, wmax = 0.f, psum = 0.f;
    for (int k = 0; k < ncol; ++k) {   // asph_h100.cu:1095-1102
        if (cd[k].z > 1e-4f) ++ncloud;
        qlmax = fmaxf(qlmax, cd[k].z);
        wmax = fmaxf(wmax, cd[k].w);
        psum += pr[k];
    }
    out[0] = ncol ? 100.f * (float)ncloud / ncol : 0.f;
    out[1] = qlmax;
    out[2] = wmax;
    out[3] = (float)(psum / ncol);
    CKR(cudaMemsetAsync(c->B.precip, 0, (size_t)ncol * 4, c->stream));
    CKR(cudaStreamSynchronize(c->stream));
    return ASPH_OK;
}
