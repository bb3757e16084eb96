// asph_phys.cuh — physical constants, derived run constants and the point
// functions of the anisotropic-SPH warm-rain model.  Usable from device
// code and from host code (the context fills `Phys` on the host).
//
// Each function follows the reference helper named beside it
// (asph_h100.cu:125-204); the constexpr parameters of the reference
// (asph_h100.cu:48-120) are fields of `Phys` here.
#pragma once
#include <stdint.h>
#include <math.h>

#if defined(__CUDACC__)
#define AHD __host__ __device__ __forceinline__
#else
#define AHD inline
#endif

namespace asph {

// Universal constants (asph_h100.cu:66-70).
constexpr float GRAV = 9.80665f;
constexpr float R_D  = 287.05f;
constexpr float CP   = 1004.0f;
constexpr float P0   = 100000.0f;
constexpr float L_V  = 2.501e6f;
constexpr float SIGMA_W = 0.31830988618f;  // 1/pi, 3-D cubic spline (asph_h100.cu:56)
constexpr int   STENCIL = 2;               // support radius in cells (asph_h100.cu:54)

// Run constants handed to every kernel by value.
struct Phys {
    int   nx, ny, nz, nxy;
    int   N;           // particles
    int   ncell;       // nx*ny*nz
    float dx, dy, dz;
    float inv_dx, inv_dy, inv_dz;   // 1.0f/dx etc., rounded once (asph_h100.cu:49)
    float lx, ly, lz;
    float v_cell;
    // sounding
    float th0, n2, cs, a_exner;     // a_exner = g^2/(cp th0 N^2) (asph_h100.cu:140)
    int   qv_mode;
    float qv0, rh, rh_bl, z_bl;
    // dissipation
    float alpha, beta, h_av, eta2;  // eta2 = (0.01 h_av)^2 (asph_h100.cu:482)
    float av_lin, av_quad;          // -4 alpha cs h_av and 4 beta h_av^2 (set_viscosity_terms)
    float sponge_sigma, sponge_frac, dthdt_cap;
    // surface
    int   surface_flux;
    float c_h, c_e, beta_moist, v_bg, dts_skin, ramp;
    // microphysics
    float qc_auto, rate_auto, v_rain, theta_cap, qv_cap;
    int   accretion, rain_evap;
    float k_accr;
    // mass
    float pmass;       // kg per particle
    float mm;          // pmass / v_cell (asph_h100.cu:497)
    // time control
    float cfl, dt_cap, dt_floor, dt_static;
    int   max_trip, strict_cfl, adaptive_dt, sort_every, permute_acc;
    int   key_bits;    // 3*ceil_log2(max n) (asph_h100.cu:866-868)
    // reference-sounding tables, one node per metre of height (device)
    const float4* snd_rho;    // rho_ref
    const float4* snd_p;      // pres_ref
    const float4* snd_thvr;   // theta_ref * (1 + 0.608 qv_ref)
    int   snd_n;              // nodes
};

// Viscosity constants of the momentum pair term, from alpha, beta, cs, h_av.
inline void set_viscosity_terms(Phys& P) {
    P.av_lin = -4.0f * P.alpha * P.cs * P.h_av;
    P.av_quad = 4.0f * P.beta * P.h_av * P.h_av;
}

// ---- SPH kernel (asph_h100.cu:125-134) -----------------------------------
AHD float w3(float q) {
    if (q >= 2.0f) return 0.0f;
    if (q < 1.0f) return SIGMA_W * (1.0f - 1.5f * q * q + 0.75f * q * q * q);
    float t = 2.0f - q;
    return 0.25f * SIGMA_W * t * t * t;
}
AHD float dw3(float q) {
    if (q >= 2.0f) return 0.0f;
    if (q < 1.0f) return SIGMA_W * (-3.0f * q + 2.25f * q * q);
    float t = 2.0f - q;
    return -0.75f * SIGMA_W * t * t;
}

// ---- analytic reference state (asph_h100.cu:136-153) ----------------------
AHD float theta_ref(const Phys& P, float z) { return P.th0 * expf(P.n2 * z / GRAV); }
AHD float exner_ref(const Phys& P, float z) {
    return 1.0f - P.a_exner * (1.0f - expf(-P.n2 * z / GRAV));
}
AHD float pres_ref(const Phys& P, float z) { return P0 * powf(exner_ref(P, z), CP / R_D); }
AHD float rho_ref(const Phys& P, float z) {
    return pres_ref(P, z) / (R_D * theta_ref(P, z) * exner_ref(P, z));
}

// ---- thermodynamics (asph_h100.cu:155-171) --------------------------------
AHD float esat(float T) {
    float Tc = T - 273.15f;
    return 611.2f * expf(17.67f * Tc / (Tc + 243.5f));
}
AHD float qsat(float T, float p) {
    float es = fminf(esat(T), 0.5f * p);
    float den = p - 0.378f * es;
    return den > 1.0f ? 0.622f * es / den : 0.0f;
}
AHD float dqsdT(float T, float es, float p) {
    float Tc = T - 273.15f;
    float d = Tc + 243.5f;
    float desdT = es * (17.67f * 243.5f) / (d * d);
    float den = p - 0.378f * es;
    return 0.622f * p * desdT / (den * den);
}

AHD float qv_ref(const Phys& P, float z) {
    if (P.qv_mode == 0) {   // asph_h100.cu:149-153
        float q = P.qv0 * expf(-z / 2500.0f);
        float d = fmaxf(z - 5000.0f, 0.0f);
        return q * expf(-d / 1000.0f);
    }
    // relative-humidity profile about the reference sounding
    float pi = exner_ref(P, z);
    float T = theta_ref(P, z) * pi;
    float p = P0 * powf(pi, CP / R_D);
    float rh = (z < P.z_bl) ? P.rh_bl : P.rh;
    return rh * qsat(T, p);
}

// ---- spatial hashing (asph_h100.cu:176-198) -------------------------------
AHD uint32_t part1by2_10(uint32_t n) {
    n &= 0x000003ffu;
    n = (n ^ (n << 16)) & 0xff0000ffu;
    n = (n ^ (n << 8)) & 0x0300f00fu;
    n = (n ^ (n << 4)) & 0x030c30c3u;
    n = (n ^ (n << 2)) & 0x09249249u;
    return n;
}
AHD uint32_t compact1by2_10(uint32_t n) {   // inverse of part1by2_10
    n &= 0x09249249u;
    n = (n ^ (n >> 2)) & 0x030c30c3u;
    n = (n ^ (n >> 4)) & 0x0300f00fu;
    n = (n ^ (n >> 8)) & 0xff0000ffu;
    n = (n ^ (n >> 16)) & 0x000003ffu;
    return n;
}
AHD uint32_t morton3(uint32_t x, uint32_t y, uint32_t z) {
    return part1by2_10(x) | (part1by2_10(y) << 1) | (part1by2_10(z) << 2);
}
AHD int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// Cell coordinate by truncation then clamp (asph_h100.cu:236-238, 297-299).
// The multiply is a single rounded float product, so the integer cell is
// identical on every device and on the host.
AHD int cell_ix(float x, float inv, int n) {
#if defined(__CUDA_ARCH__)
    float s = __fmul_rn(x, inv);
#else
    float s = x * inv;
#endif
    return clampi((int)s, 0, n - 1);
}
AHD uint32_t key_of(const Phys& P, float x, float y, float z) {
    return morton3((uint32_t)cell_ix(x, P.inv_dx, P.nx), (uint32_t)cell_ix(y, P.inv_dy, P.ny),
                   (uint32_t)cell_ix(z, P.inv_dz, P.nz));
}
AHD int cid_of_key(const Phys& P, uint32_t k) {
    int ix = (int)compact1by2_10(k), iy = (int)compact1by2_10(k >> 1), iz = (int)compact1by2_10(k >> 2);
    return (iz * P.ny + iy) * P.nx + ix;
}
AHD int wrapi(int i, int n) { i %= n; return i < 0 ? i + n : i; }

// Reference noise hash (asph_h100.cu:187-192).
AHD float hash_noise(int i, int j, int k) {
    uint32_t h = (uint32_t)i * 374761393u + (uint32_t)j * 668265263u + (uint32_t)k * 2246822519u;
    h = (h ^ (h >> 13)) * 1274126177u;
    h ^= h >> 16;
    return (float)(h & 0x00ffffffu) * (1.0f / 16777215.0f) - 0.5f;
}

// Counter-based generator for the lattice init (splitmix64 finaliser over
// (seed, particle, stream)); 24-bit uniforms in [0,1).
AHD uint64_t mix64(uint64_t z) {
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
AHD float uniform24(uint32_t seed, uint32_t i, uint32_t stream) {
    uint64_t h = mix64(((uint64_t)seed << 32) ^ mix64(((uint64_t)stream << 40) ^ (uint64_t)i));
    return (float)(uint32_t)(h >> 40) * (1.0f / 16777216.0f);
}
// Box-Muller normal deviate from two uniforms of streams 2s and 2s+1.
AHD float normal01(uint32_t seed, uint32_t i, uint32_t stream) {
    float u1 = uniform24(seed, i, 2u * stream) + (0.5f / 16777216.0f);
    float u2 = uniform24(seed, i, 2u * stream + 1u);
    return sqrtf(-2.0f * logf(u1)) * cosf(6.283185307f * u2);
}

}  // namespace asph
