// refgpu.cu — TEST INFRASTRUCTURE ONLY: runs the reference's own kernels.
//
// The reference's device code (asph_h100.cu, compiled unmodified into
// oracle/_ref/asph_ref.cubin by oracle/build_oracle.py) is loaded through the
// CUDA driver API, and this program replays the blocks of the reference's
// host step loop (asph_h100.cu:958-1078) around those kernels, with the
// reference's own library sort, cub::DeviceRadixSort::SortPairs
// (asph_h100.cu:866-871, 966-967), compiled from the CUDA toolkit's CUB.
// It writes every intermediate array so that the CUDA path and the CPU
// oracle can be compared against the reference itself (golden fixtures),
// and it times the reference step loop on the GPU.
//
// usage:
//   refgpu <cubin> stages <in.bin> <outdir>   one step, every stage saved
//   refgpu <cubin> init <nx> <ny> <nz> <noise> <outdir>
//   refgpu <cubin> run <nx> <ny> <nz> <steps> <dt> <sort_every>
//          sort_every 0 = the reference's displacement-gated cadence
//   refgpu <cubin> runstate <in.bin> <steps> <warmup> <dx> <dy> <dz>
#include <cuda.h>
#include <cuda_runtime.h>
#include <cub/cub.cuh>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#define CK(x)                                                                              \
    do {                                                                                   \
        cudaError_t e_ = (x);                                                              \
        if (e_ != cudaSuccess) {                                                           \
            fprintf(stderr, "CUDA %s:%d %s\n", __FILE__, __LINE__, cudaGetErrorString(e_)); \
            exit(1);                                                                       \
        }                                                                                  \
    } while (0)
#define CU(x)                                                                  \
    do {                                                                       \
        CUresult r_ = (x);                                                     \
        if (r_ != CUDA_SUCCESS) {                                              \
            const char* s_ = nullptr;                                          \
            cuGetErrorString(r_, &s_);                                         \
            fprintf(stderr, "CU %s:%d %s (%s)\n", __FILE__, __LINE__, s_, #x); \
            exit(1);                                                           \
        }                                                                      \
    } while (0)

// Reference constants needed on the host (asph_h100.cu:48-105).
static const float DX = 1000.0f, DY = 1000.0f, DZ = 100.0f, CS = 80.0f, TH0 = 300.0f, N2 = 6.0e-5f;
static const float GRAV = 9.80665f, R_D = 287.05f, CP = 1004.0f, P0 = 100000.0f;
static const float DTS_SKIN = 3.15f, RAMP = 3600.0f;

// Host restatement of the two helpers the reference evaluates on the host
// for the surface forcing (asph_h100.cu:139-163, 989-992).
static float h_exner(float z) {
    const float A = GRAV * GRAV / (CP * TH0 * N2);
    return 1.0f - A * (1.0f - expf(-N2 * z / GRAV));
}
static float h_pres(float z) { return P0 * powf(h_exner(z), CP / R_D); }
static float h_esat(float T) {
    float Tc = T - 273.15f;
    return 611.2f * expf(17.67f * Tc / (Tc + 243.5f));
}
static float h_qsat(float T, float p) {
    float es = fminf(h_esat(T), 0.5f * p);
    float den = p - 0.378f * es;
    return den > 1.0f ? 0.622f * es / den : 0.0f;
}

struct Ref {
    CUmodule mod;
    CUfunction init, keys, iota, gather, build, density, eos, momentum, sponge, kick, drift, theta, rain, flux,
        maxvel, audit, clampv;
};

static CUfunction getf(CUmodule m, const char* name) {
    CUfunction f;
    CU(cuModuleGetFunction(&f, m, name));
    return f;
}

static void load(Ref& R, const char* cubin) {
    CK(cudaFree(0));   // create the primary context
    CU(cuModuleLoad(&R.mod, cubin));
    // Itanium-mangled names of the reference kernels (asph_h100.cu:210-675).
    R.init = getf(R.mod, "_Z11kernel_initP6float4S0_S0_Pfiiif");
    R.keys = getf(R.mod, "_Z18kernel_morton_keysPK6float4Pjiiii");
    R.iota = getf(R.mod, "_Z11kernel_iotaPji");
    R.gather = getf(R.mod, "_Z13kernel_gatherPKjPK6float4PS1_S3_S4_S3_S4_PKfPfi");
    R.build = getf(R.mod, "_Z18kernel_build_pairsPK6float4P4int2PiS4_iiiii");
    R.density = getf(R.mod, "_Z14kernel_densityPK6float4PKfPK4int2Pfiiii");
    R.eos = getf(R.mod, "_Z16kernel_eos_microP6float4PKS_PKfPfS5_iiiif");
    R.momentum = getf(R.mod, "_Z15kernel_momentumPK6float4S1_S1_PKfS3_PK4int2PS_Pfiiii");
    R.sponge = getf(R.mod, "_Z13kernel_spongeP6float4S0_iff");
    R.kick = getf(R.mod, "_Z11kernel_kickP6float4PKS_if");
    R.drift = getf(R.mod, "_Z12kernel_driftP6float4S0_iffff");
    R.theta = getf(R.mod, "_Z19kernel_theta_updateP6float4PKfif");
    R.rain = getf(R.mod, "_Z15kernel_rain_advPKfPfS1_iiif");
    R.flux = getf(R.mod, "_Z19kernel_surface_fluxP6float4PKS_PKiS4_ifff");
    R.maxvel = getf(R.mod, "_Z14kernel_max_velPK6float4iPf");
    R.audit = getf(R.mod, "_Z12kernel_auditPK6float4S1_S1_Pdi");
    R.clampv = getf(R.mod, "_Z16kernel_clamp_velP6float4if");
    // asph_h100.cu:877-880
    CU(cuFuncSetAttribute(R.density, CU_FUNC_ATTRIBUTE_PREFERRED_SHARED_MEMORY_CARVEOUT, 0));
    CU(cuFuncSetAttribute(R.momentum, CU_FUNC_ATTRIBUTE_PREFERRED_SHARED_MEMORY_CARVEOUT, 0));
}

template <typename... A>
static void launch(CUfunction f, int grid, int block, A... args) {
    void* p[] = {(void*)&args...};
    CU(cuLaunchKernel(f, grid, 1, 1, block, 1, 1, 0, 0, p, nullptr));
}

struct Dev {
    int nx, ny, nz, N, C, surfCap, endbit;
    float4 *pos, *vel, *thq, *pos2, *vel2, *thq2, *acc;
    float *rho, *rho2, *prs, *dthdt, *rainA, *rainB, *precip, *gmax;
    uint32_t *keysIn, *keysOut, *valsIn, *perm;
    int2* cellRange;
    int *surfList, *surfCount;
    void* sortTmp;
    size_t sortTmpBytes;
    double* tot;
};

static void alloc(Dev& d, int nx, int ny, int nz, int N) {
    d.nx = nx; d.ny = ny; d.nz = nz; d.N = N; d.C = nx * ny * nz;
    const size_t n = (size_t)N, c = (size_t)d.C;
    CK(cudaMalloc(&d.pos, n * 16)); CK(cudaMalloc(&d.vel, n * 16)); CK(cudaMalloc(&d.thq, n * 16));
    CK(cudaMalloc(&d.pos2, n * 16)); CK(cudaMalloc(&d.vel2, n * 16)); CK(cudaMalloc(&d.thq2, n * 16));
    CK(cudaMalloc(&d.acc, n * 16));
    CK(cudaMalloc(&d.rho, n * 4)); CK(cudaMalloc(&d.rho2, n * 4)); CK(cudaMalloc(&d.prs, n * 4));
    CK(cudaMalloc(&d.dthdt, n * 4));
    CK(cudaMalloc(&d.rainA, c * 4)); CK(cudaMalloc(&d.rainB, c * 4));
    CK(cudaMalloc(&d.precip, (size_t)nx * ny * 4)); CK(cudaMalloc(&d.gmax, 16));
    CK(cudaMalloc(&d.keysIn, n * 4)); CK(cudaMalloc(&d.keysOut, n * 4));
    CK(cudaMalloc(&d.valsIn, n * 4)); CK(cudaMalloc(&d.perm, n * 4));
    CK(cudaMalloc(&d.cellRange, c * 8));
    d.surfCap = nx * ny * 2;
    CK(cudaMalloc(&d.surfList, (size_t)d.surfCap * 4)); CK(cudaMalloc(&d.surfCount, 4));
    CK(cudaMalloc(&d.tot, 6 * 8));
    auto ceil_log2 = [](int v) { int b = 1; while ((1 << b) < v) ++b; return b; };
    int bits = std::max(ceil_log2(nx), std::max(ceil_log2(ny), ceil_log2(nz)));
    d.endbit = 3 * bits;
    d.sortTmp = nullptr;
    d.sortTmpBytes = 0;
    CK(cub::DeviceRadixSort::SortPairs(nullptr, d.sortTmpBytes, d.keysIn, d.keysOut, d.valsIn, d.perm, N, 0, d.endbit));
    CK(cudaMalloc(&d.sortTmp, d.sortTmpBytes));
    CK(cudaMemset(d.cellRange, 0, c * 8));
    CK(cudaMemset(d.rainA, 0, c * 4)); CK(cudaMemset(d.rainB, 0, c * 4));
    CK(cudaMemset(d.precip, 0, (size_t)nx * ny * 4));
    CK(cudaMemset(d.acc, 0, n * 16)); CK(cudaMemset(d.dthdt, 0, n * 4));
    CK(cudaMemset(d.surfCount, 0, 4));
}

static const int TPB = 256;
static int bpb(int n) { return (n + TPB - 1) / TPB; }

// The sort block of the reference step (asph_h100.cu:963-977).
static void sort_block(const Ref& R, Dev& d) {
    launch(R.keys, bpb(d.N), TPB, (const float4*)d.pos, d.keysIn, d.nx, d.ny, d.nz, d.N);
    CK(cub::DeviceRadixSort::SortPairs(d.sortTmp, d.sortTmpBytes, d.keysIn, d.keysOut, d.valsIn, d.perm, d.N, 0,
                                       d.endbit));
    launch(R.gather, bpb(d.N), TPB, (const uint32_t*)d.perm, (const float4*)d.pos, d.pos2, (const float4*)d.vel, d.vel2,
           (const float4*)d.thq, d.thq2, (const float*)d.rho, d.rho2, d.N);
    std::swap(d.pos, d.pos2); std::swap(d.vel, d.vel2); std::swap(d.thq, d.thq2); std::swap(d.rho, d.rho2);
    CK(cudaMemsetAsync(d.cellRange, 0, (size_t)d.C * 8));
    CK(cudaMemsetAsync(d.surfCount, 0, 4));
    launch(R.build, bpb(d.N), TPB, (const float4*)d.pos, d.cellRange, d.surfList, d.surfCount, d.nx, d.ny, d.nz, d.N,
           d.surfCap);
}

static void flux_targets(double simt, float& Ts, float& qs) {
    float r = fminf(fmaxf((float)simt / RAMP, 0.f), 1.f);
    float sw = r * r * (3.f - 2.f * r);
    Ts = TH0 + DTS_SKIN * sw;
    qs = h_qsat(Ts, h_pres(0.f));
}

template <class T>
static void save(const std::string& dir, const char* name, const T* dptr, size_t count) {
    std::vector<T> h(count);
    CK(cudaMemcpy(h.data(), dptr, count * sizeof(T), cudaMemcpyDeviceToHost));
    std::string fn = dir + "/" + name + ".bin";
    FILE* f = fopen(fn.c_str(), "wb");
    if (!f) { fprintf(stderr, "cannot write %s\n", fn.c_str()); exit(1); }
    fwrite(h.data(), sizeof(T), count, f);
    fclose(f);
}

template <class T>
static void read_into(FILE* f, T* dptr, size_t count) {
    std::vector<T> h(count);
    if (fread(h.data(), sizeof(T), count, f) != count) { fprintf(stderr, "short input\n"); exit(1); }
    CK(cudaMemcpy(dptr, h.data(), count * sizeof(T), cudaMemcpyHostToDevice));
}

// One reference step on a given state, saving every stage.
static int cmd_stages(const Ref& R, const char* in, const std::string& out) {
    FILE* f = fopen(in, "rb");
    if (!f) { fprintf(stderr, "cannot open %s\n", in); return 1; }
    int32_t hdr[8];
    double simt;
    float dt;
    if (fread(hdr, 4, 8, f) != 8 || fread(&simt, 8, 1, f) != 1 || fread(&dt, 4, 1, f) != 1) return 1;
    // hdr: magic, nx, ny, nz, N, do_sort, clamp, reserved
    Dev d;
    alloc(d, hdr[1], hdr[2], hdr[3], hdr[4]);
    read_into(f, d.pos, (size_t)d.N); read_into(f, d.vel, (size_t)d.N); read_into(f, d.thq, (size_t)d.N);
    read_into(f, d.rho, (size_t)d.N); read_into(f, d.acc, (size_t)d.N);
    read_into(f, d.rainA, (size_t)d.C); read_into(f, d.precip, (size_t)d.nx * d.ny);
    fclose(f);
    launch(R.iota, bpb(d.N), TPB, d.valsIn, d.N);
    const int do_sort = hdr[5], clamp = hdr[6];
    const float Lx = d.nx * DX, Ly = d.ny * DY, Lz = d.nz * DZ;
    if (clamp) launch(R.clampv, 1024, TPB, d.vel, d.N, 0.5f * CS);   // asph_h100.cu:1067
    if (do_sort) {
        sort_block(R, d);
        save(out, "keys_in", d.keysIn, d.N); save(out, "keys_sorted", d.keysOut, d.N);
        save(out, "perm", d.perm, d.N);
        save(out, "g_pos", d.pos, d.N); save(out, "g_vel", d.vel, d.N); save(out, "g_thq", d.thq, d.N);
        save(out, "g_rho", d.rho, d.N);
        save(out, "cell_range", d.cellRange, d.C);
        save(out, "surf_count", d.surfCount, 1);
        save(out, "surf_list", d.surfList, d.surfCap);
    } else {
        // the cell table and surface list of the input state's own sort
        launch(R.build, bpb(d.N), TPB, (const float4*)d.pos, d.cellRange, d.surfList, d.surfCount, d.nx, d.ny, d.nz, d.N,
               d.surfCap);
    }
    launch(R.kick, bpb(d.N), TPB, d.vel, (const float4*)d.acc, d.N, 0.5f * dt);
    launch(R.drift, bpb(d.N), TPB, d.pos, d.vel, d.N, dt, Lx, Ly, Lz);
    save(out, "kd_pos", d.pos, d.N); save(out, "kd_vel", d.vel, d.N);
    float Ts, qs;
    flux_targets(simt, Ts, qs);
    launch(R.flux, bpb(d.surfCap), TPB, d.thq, (const float4*)d.pos, (const int*)d.surfList, (const int*)d.surfCount,
           d.surfCap, dt, Ts, qs);
    save(out, "flux_thq", d.thq, d.N);
    launch(R.density, bpb(d.N), TPB, (const float4*)d.pos, (const float*)d.rho, (const int2*)d.cellRange, d.rho2, d.nx,
           d.ny, d.nz, d.N);
    std::swap(d.rho, d.rho2);
    save(out, "d_rho", d.rho, d.N);
    launch(R.eos, bpb(d.N), TPB, d.thq, (const float4*)d.pos, (const float*)d.rho, d.prs, d.rainA, d.nx, d.ny, d.nz,
           d.N, dt);
    save(out, "e_thq", d.thq, d.N); save(out, "e_prs", d.prs, d.N); save(out, "e_rain", d.rainA, d.C);
    launch(R.momentum, bpb(d.N), TPB, (const float4*)d.pos, (const float4*)d.vel, (const float4*)d.thq,
           (const float*)d.rho, (const float*)d.prs, (const int2*)d.cellRange, d.acc, d.dthdt, d.nx, d.ny, d.nz, d.N);
    save(out, "m_acc", d.acc, d.N); save(out, "m_dthdt", d.dthdt, d.N);
    launch(R.theta, bpb(d.N), TPB, d.thq, (const float*)d.dthdt, d.N, dt);
    launch(R.kick, bpb(d.N), TPB, d.vel, (const float4*)d.acc, d.N, 0.5f * dt);
    launch(R.sponge, bpb(d.N), TPB, d.pos, d.vel, d.N, dt, Lz);
    save(out, "i_thq", d.thq, d.N); save(out, "i_vel", d.vel, d.N);
    launch(R.rain, bpb(d.C), TPB, (const float*)d.rainA, d.rainB, d.precip, d.nx, d.ny, d.nz, dt);
    save(out, "r_rain", d.rainB, d.C); save(out, "r_precip", d.precip, (size_t)d.nx * d.ny);
    CK(cudaMemset(d.gmax, 0, 12));
    launch(R.maxvel, 1024, TPB, (const float4*)d.vel, d.N, d.gmax);
    save(out, "gmax", d.gmax, 3);
    CK(cudaMemset(d.tot, 0, 48));
    launch(R.audit, 1024, TPB, (const float4*)d.pos, (const float4*)d.vel, (const float4*)d.thq, d.tot, d.N);
    save(out, "audit", d.tot, 6);
    CK(cudaDeviceSynchronize());
    return 0;
}

// Reference initial state + initial sort + initial forces (asph_h100.cu:885-921).
static void init_state(const Ref& R, Dev& d, float noise, float dt) {
    launch(R.init, bpb(d.N), TPB, d.pos, d.vel, d.thq, d.rho, d.nx, d.ny, d.nz, noise);
    launch(R.iota, bpb(d.N), TPB, d.valsIn, d.N);
    CK(cudaMemsetAsync(d.cellRange, 0, (size_t)d.C * 8));
    CK(cudaMemsetAsync(d.surfCount, 0, 4));
    sort_block(R, d);
    launch(R.density, bpb(d.N), TPB, (const float4*)d.pos, (const float*)d.rho, (const int2*)d.cellRange, d.rho2, d.nx,
           d.ny, d.nz, d.N);
    std::swap(d.rho, d.rho2);
    launch(R.eos, bpb(d.N), TPB, d.thq, (const float4*)d.pos, (const float*)d.rho, d.prs, d.rainA, d.nx, d.ny, d.nz,
           d.N, dt);
    launch(R.momentum, bpb(d.N), TPB, (const float4*)d.pos, (const float4*)d.vel, (const float4*)d.thq,
           (const float*)d.rho, (const float*)d.prs, (const int2*)d.cellRange, d.acc, d.dthdt, d.nx, d.ny, d.nz, d.N);
    CK(cudaDeviceSynchronize());
}

static int cmd_init(const Ref& R, int nx, int ny, int nz, float noise, const std::string& out) {
    Dev d;
    alloc(d, nx, ny, nz, nx * ny * nz);
    const float dt = 0.40f * fminf(fminf(DX, DY), DZ) / CS;   // asph_h100.cu:794-797, no --dt
    init_state(R, d, noise, dt);
    save(out, "pos", d.pos, d.N); save(out, "vel", d.vel, d.N); save(out, "thq", d.thq, d.N);
    save(out, "rho", d.rho, d.N); save(out, "prs", d.prs, d.N); save(out, "acc", d.acc, d.N);
    save(out, "dthdt", d.dthdt, d.N); save(out, "rain", d.rainA, d.C);
    save(out, "cell_range", d.cellRange, d.C); save(out, "perm", d.perm, d.N);
    return 0;
}

// The reference step loop (asph_h100.cu:958-1078) for timing: kick, drift,
// flux, density, eos, momentum, theta, kick, sponge, rain, CFL with its
// per-step host synchronisation; sorts displacement-gated (sort_every 0)
// or every k steps.
static int cmd_run(const Ref& R, int nx, int ny, int nz, int steps, float dt_req, int sort_every) {
    Dev d;
    alloc(d, nx, ny, nz, nx * ny * nz);
    const float Lx = nx * DX, Ly = ny * DY, Lz = nz * DZ;
    const float dt_static = 0.40f * fminf(fminf(DX, DY), DZ) / CS;
    const float dt_cap = dt_req > 0.f ? fminf(dt_req, dt_static) : dt_static;
    const float dt_floor = 0.05f * dt_cap;
    float dt = dt_cap, sort_dt = 0.5f;
    double simt = 0.0, since_sort = 1e9;
    int sorts = 0, trips = 0;
    init_state(R, d, 0.1f, dt);
    float hg[3];
    auto now = [] { return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count(); };
    CK(cudaDeviceSynchronize());
    const double t0 = now();
    for (int step = 1; step <= steps; ++step) {
        const bool srt = sort_every > 0 ? ((step - 1) % sort_every == 0) : (since_sort >= sort_dt);
        if (srt) { sort_block(R, d); since_sort = 0.0; ++sorts; }
        launch(R.kick, bpb(d.N), TPB, d.vel, (const float4*)d.acc, d.N, 0.5f * dt);
        launch(R.drift, bpb(d.N), TPB, d.pos, d.vel, d.N, dt, Lx, Ly, Lz);
        float Ts, qs;
        flux_targets(simt, Ts, qs);
        launch(R.flux, bpb(d.surfCap), TPB, d.thq, (const float4*)d.pos, (const int*)d.surfList,
               (const int*)d.surfCount, d.surfCap, dt, Ts, qs);
        launch(R.density, bpb(d.N), TPB, (const float4*)d.pos, (const float*)d.rho, (const int2*)d.cellRange, d.rho2,
               d.nx, d.ny, d.nz, d.N);
        std::swap(d.rho, d.rho2);
        launch(R.eos, bpb(d.N), TPB, d.thq, (const float4*)d.pos, (const float*)d.rho, d.prs, d.rainA, d.nx, d.ny,
               d.nz, d.N, dt);
        launch(R.momentum, bpb(d.N), TPB, (const float4*)d.pos, (const float4*)d.vel, (const float4*)d.thq,
               (const float*)d.rho, (const float*)d.prs, (const int2*)d.cellRange, d.acc, d.dthdt, d.nx, d.ny, d.nz,
               d.N);
        launch(R.theta, bpb(d.N), TPB, d.thq, (const float*)d.dthdt, d.N, dt);
        launch(R.kick, bpb(d.N), TPB, d.vel, (const float4*)d.acc, d.N, 0.5f * dt);
        launch(R.sponge, bpb(d.N), TPB, d.pos, d.vel, d.N, dt, Lz);
        launch(R.rain, bpb(d.C), TPB, (const float*)d.rainA, d.rainB, d.precip, d.nx, d.ny, d.nz, dt);
        std::swap(d.rainA, d.rainB);
        simt += dt;
        since_sort += dt;
        CK(cudaMemsetAsync(d.gmax, 0, 12));
        launch(R.maxvel, 1024, TPB, (const float4*)d.vel, d.N, d.gmax);
        CK(cudaMemcpy(hg, d.gmax, 12, cudaMemcpyDeviceToHost));
        const float ux = hg[0], uy = hg[1], uz = hg[2];
        const float req = 0.40f * fminf(fminf(DX / (CS + ux), DY / (CS + uy)), DZ / (CS + uz)) * 0.90f;
        float adopt = fminf(dt_cap, req);
        if (adopt < dt_floor) {
            if (++trips > 20) { fprintf(stderr, "CFL abort at step %d\n", step); return 2; }
            launch(R.clampv, 1024, TPB, d.vel, d.N, 0.5f * CS);
            adopt = fmaxf(dt_floor, 0.40f * fminf(fminf(DX, DY), DZ) / (1.5f * CS) * 0.90f);
        } else if (adopt < 0.98f * dt) {
            trips = 0;
        }
        dt = adopt;
        const float dzm = 0.3f * DZ / fmaxf(uz, 0.5f), dhm = 0.3f * DX / fmaxf(fmaxf(ux, uy), 0.5f);
        sort_dt = fminf(fmaxf(fminf(dzm, dhm), dt), 15.0f);
    }
    CK(cudaDeviceSynchronize());
    const double wall = now() - t0;
    printf("{\"impl\": \"reference-gpu\", \"N\": %d, \"steps\": %d, \"wall_s\": %.6f, \"particle_steps_per_s\": %.6e, "
           "\"ms_per_step\": %.6f, \"sorts\": %d, \"final_dt\": %.6f, \"sim_s\": %.3f}\n",
           d.N, steps, wall, (double)d.N * steps / wall, 1e3 * wall / steps, sorts, dt, simt);
    return 0;
}

// The reference step loop on a given state (cmd_stages input format), a sort
// every step, for timing: `warmup` untimed steps, then K timed steps, each
// with the reference's per-step velocity maxima read back to the host and
// its closed-loop dt control (asph_h100.cu:1040-1073), starting from the
// state's dt.  Cell sizes are passed because the cubin may carry other
// constexprs.
static int cmd_runstate(const Ref& R, const char* in, int steps, int warmup, float dx, float dy, float dz) {
    FILE* f = fopen(in, "rb");
    if (!f) { fprintf(stderr, "cannot open %s\n", in); return 1; }
    int32_t hdr[8];
    double simt;
    float dt;
    if (fread(hdr, 4, 8, f) != 8 || fread(&simt, 8, 1, f) != 1 || fread(&dt, 4, 1, f) != 1) return 1;
    Dev d;
    alloc(d, hdr[1], hdr[2], hdr[3], hdr[4]);
    read_into(f, d.pos, (size_t)d.N); read_into(f, d.vel, (size_t)d.N); read_into(f, d.thq, (size_t)d.N);
    read_into(f, d.rho, (size_t)d.N); read_into(f, d.acc, (size_t)d.N);
    read_into(f, d.rainA, (size_t)d.C); read_into(f, d.precip, (size_t)d.nx * d.ny);
    fclose(f);
    launch(R.iota, bpb(d.N), TPB, d.valsIn, d.N);
    const float Lx = d.nx * dx, Ly = d.ny * dy, Lz = d.nz * dz;
    const float dt_cap = dt, dt_floor = 0.05f * dt_cap;
    int trips = 0;
    float hg[3];
    auto now = [] { return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count(); };
    auto one = [&]() {
        sort_block(R, d);
        launch(R.kick, bpb(d.N), TPB, d.vel, (const float4*)d.acc, d.N, 0.5f * dt);
        launch(R.drift, bpb(d.N), TPB, d.pos, d.vel, d.N, dt, Lx, Ly, Lz);
        float Ts, qs;
        flux_targets(simt, Ts, qs);
        launch(R.flux, bpb(d.surfCap), TPB, d.thq, (const float4*)d.pos, (const int*)d.surfList,
               (const int*)d.surfCount, d.surfCap, dt, Ts, qs);
        launch(R.density, bpb(d.N), TPB, (const float4*)d.pos, (const float*)d.rho, (const int2*)d.cellRange, d.rho2,
               d.nx, d.ny, d.nz, d.N);
        std::swap(d.rho, d.rho2);
        launch(R.eos, bpb(d.N), TPB, d.thq, (const float4*)d.pos, (const float*)d.rho, d.prs, d.rainA, d.nx, d.ny,
               d.nz, d.N, dt);
        launch(R.momentum, bpb(d.N), TPB, (const float4*)d.pos, (const float4*)d.vel, (const float4*)d.thq,
               (const float*)d.rho, (const float*)d.prs, (const int2*)d.cellRange, d.acc, d.dthdt, d.nx, d.ny, d.nz,
               d.N);
        launch(R.theta, bpb(d.N), TPB, d.thq, (const float*)d.dthdt, d.N, dt);
        launch(R.kick, bpb(d.N), TPB, d.vel, (const float4*)d.acc, d.N, 0.5f * dt);
        launch(R.sponge, bpb(d.N), TPB, d.pos, d.vel, d.N, dt, Lz);
        launch(R.rain, bpb(d.C), TPB, (const float*)d.rainA, d.rainB, d.precip, d.nx, d.ny, d.nz, dt);
        std::swap(d.rainA, d.rainB);
        simt += dt;
        CK(cudaMemsetAsync(d.gmax, 0, 12));
        launch(R.maxvel, 1024, TPB, (const float4*)d.vel, d.N, d.gmax);
        CK(cudaMemcpy(hg, d.gmax, 12, cudaMemcpyDeviceToHost));
        const float req = 0.40f * fminf(fminf(dx / (CS + hg[0]), dy / (CS + hg[1])), dz / (CS + hg[2])) * 0.90f;
        float adopt = fminf(dt_cap, req);
        if (adopt < dt_floor) {
            ++trips;
            launch(R.clampv, 1024, TPB, d.vel, d.N, 0.5f * CS);
            adopt = fmaxf(dt_floor, 0.40f * fminf(fminf(dx, dy), dz) / (1.5f * CS) * 0.90f);
        } else if (adopt < 0.98f * dt) {
            trips = 0;
        }
        dt = adopt;
    };
    for (int k = 0; k < warmup; ++k) one();
    CK(cudaDeviceSynchronize());
    const double t0 = now();
    for (int k = 0; k < steps; ++k) one();
    CK(cudaDeviceSynchronize());
    const double wall = now() - t0;
    printf("{\"impl\": \"reference-gpu\", \"N\": %d, \"cells\": %d, \"steps\": %d, \"warmup\": %d, "
           "\"wall_s\": %.6f, \"particle_steps_per_s\": %.6e, \"ms_per_step\": %.6f, \"wmax\": %.4f, "
           "\"final_dt\": %.6f, \"trips\": %d}\n",
           d.N, d.C, steps, warmup, wall, (double)d.N * steps / wall, 1e3 * wall / steps, hg[2], dt, trips);
    return 0;
}

int main(int argc, char** argv) {
    if (argc < 3) {
        fprintf(stderr, "usage: refgpu <cubin> stages|init|run ...\n");
        return 1;
    }
    Ref R;
    load(R, argv[1]);
    const std::string cmd = argv[2];
    if (cmd == "stages" && argc == 5) return cmd_stages(R, argv[3], argv[4]);
    if (cmd == "init" && argc == 8)
        return cmd_init(R, atoi(argv[3]), atoi(argv[4]), atoi(argv[5]), (float)atof(argv[6]), argv[7]);
    if (cmd == "run" && argc == 9)
        return cmd_run(R, atoi(argv[3]), atoi(argv[4]), atoi(argv[5]), atoi(argv[6]), (float)atof(argv[7]),
                       atoi(argv[8]));
    if (cmd == "runstate" && argc == 9)
        return cmd_runstate(R, argv[3], atoi(argv[4]), atoi(argv[5]), (float)atof(argv[6]), (float)atof(argv[7]),
                            (float)atof(argv[8]));
    fprintf(stderr, "bad arguments\n");
    return 1;
}
