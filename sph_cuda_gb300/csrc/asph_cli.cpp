// asph_cli.cpp — command-line driver of the SPH warm-rain model over the C ABI.
//
// The reference's user-facing boundary is its executable: the flags of
// main() (asph_h100.cu:753-784), the banner (asph_h100.cu:799-824), the
// step loop with its dump line, audit printout and periodic report
// (asph_h100.cu:944-1161), the closing summary (asph_h100.cu:1163-1175) and
// its exit codes (0 done, 1 bad grid or CUDA error, 2 CFL abort).  This
// driver keeps all of that and runs every step through libasph.so, in
// chunks of graph-launched steps between the points where the reference
// talks to the host (dumps, reports, the end time).
//
// Additions: --preset selects one of the library presets (default: the
// reference physics at --nx/--ny/--nz), --steps caps the step count,
// --report sets the report interval (200 in the reference, fixed),
// --sort-every forces a sort cadence, --seed the initial-state seed.
#include <cuda_runtime.h>
#include <sys/stat.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "asph.h"

namespace {

constexpr float kP0 = 100000.0f;   // asph_h100.cu:69
constexpr float kRd = 287.05f;     // asph_h100.cu:67

struct Cli {
    std::string preset = "reference";
    int nx = 0, ny = 0, nz = 0;
    float dt_cap = 0.f;
    float cfl = -1.f;
    int cfl_interval = 8;
    int max_trip = -1;
    bool strict_cfl = false;
    double dump_every = 900.0;
    double sim_hours = 3.0;
    int dump_sx = -1, dump_sz = -1;
    std::string outdir = "dumps";
    int report = 200;
    bool validate = false;
    float noise = -1.f;
    long long max_steps = -1;
    int sort_every = -1;
    long long seed = -1;
};

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

void usage() {
    std::printf(
        "asph [--nx N --ny N --nz N --dt cap --cfl c\n"
        "      --cfl-interval k --max-trip n --strict-cfl\n"
        "      --dump-every s --sim-hours h --dump-stride sx sz\n"
        "      --outdir dir --noise a --validate --quick]\n"
        "     [--preset reference|small65k|bubble2m|large16m|adjoint262k]\n"
        "     [--steps n --report k --sort-every k --seed s]\n");
}

int preset_id(const std::string& s) {
    if (s == "reference") return ASPH_PRESET_REFERENCE;
    if (s == "small65k") return ASPH_PRESET_SMALL_65K;
    if (s == "bubble2m") return ASPH_PRESET_BUBBLE_2M;
    if (s == "large16m") return ASPH_PRESET_LARGE_16M;
    if (s == "adjoint262k") return ASPH_PRESET_ADJOINT_262K;
    return -1;
}

// 1 = parsed, 0 = --help printed, -1 = bad flag
int parse(int argc, char** argv, Cli& c) {
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        auto need = [&](int k) {
            if (i + k >= argc) {
                std::fprintf(stderr, "ERROR: %s needs %d value(s)\n", a.c_str(), k);
                return false;
            }
            return true;
        };
        auto next = [&]() { return std::string(argv[++i]); };
        if (a == "--help") { usage(); return 0; }
        else if (a == "--strict-cfl") c.strict_cfl = true;
        else if (a == "--validate") c.validate = true;
        else if (a == "--quick") { c.nx = 128; c.ny = 128; c.nz = 64; c.sim_hours = 0.25; c.dump_every = 300.0; }
        else if (a == "--dump-stride") {
            if (!need(2)) return -1;
            c.dump_sx = std::atoi(next().c_str());
            c.dump_sz = std::atoi(next().c_str());
        } else {
            if (a.rfind("--", 0) != 0) { std::fprintf(stderr, "ERROR: unexpected argument %s\n", a.c_str()); return -1; }
            if (!need(1)) return -1;
            const std::string v = next();
            if (a == "--nx") c.nx = std::atoi(v.c_str());
            else if (a == "--ny") c.ny = std::atoi(v.c_str());
            else if (a == "--nz") c.nz = std::atoi(v.c_str());
            else if (a == "--dt") c.dt_cap = (float)std::atof(v.c_str());
            else if (a == "--cfl") c.cfl = (float)std::atof(v.c_str());
            else if (a == "--cfl-interval") c.cfl_interval = std::atoi(v.c_str());
            else if (a == "--max-trip") c.max_trip = std::atoi(v.c_str());
            else if (a == "--dump-every") c.dump_every = std::atof(v.c_str());
            else if (a == "--sim-hours") c.sim_hours = std::atof(v.c_str());
            else if (a == "--outdir") c.outdir = v;
            else if (a == "--noise") c.noise = (float)std::atof(v.c_str());
            else if (a == "--preset") c.preset = v;
            else if (a == "--steps") c.max_steps = std::atoll(v.c_str());
            else if (a == "--report") c.report = std::atoi(v.c_str());
            else if (a == "--sort-every") c.sort_every = std::atoi(v.c_str());
            else if (a == "--seed") c.seed = std::atoll(v.c_str());
            else { std::fprintf(stderr, "ERROR: unknown flag %s\n", a.c_str()); return -1; }
        }
    }
    return 1;
}

struct Run {
    asph_ctx* ctx = nullptr;
    ~Run() { if (ctx) asph_destroy(ctx); }
};

int fail(const char* what, int st) {
    std::fprintf(stderr, "ERROR: %s: %s (%s)\n", what, asph_status_string(st), asph_last_error());
    return st == ASPH_ERR_CFL_ABORT ? 2 : 1;
}

}  // namespace

int main(int argc, char** argv) {
    Cli cli;
    const int pr = parse(argc, argv, cli);
    if (pr <= 0) return pr == 0 ? 0 : 1;
    const int pid = preset_id(cli.preset);
    if (pid < 0) { std::fprintf(stderr, "ERROR: unknown preset %s\n", cli.preset.c_str()); return 1; }
    if (cli.nx > 1024 || cli.ny > 1024 || cli.nz > 1024) {
        std::fprintf(stderr, "ERROR: 30-bit Morton key addresses 1024 cells/axis.\n");
        return 1;
    }

    AsphParams p;
    int st = asph_params_preset(&p, pid, cli.nx, cli.ny, cli.nz);
    if (st) return fail("preset", st);
    if (cli.dt_cap > 0.f) p.dt_request = cli.dt_cap;
    if (cli.cfl > 0.f) p.cfl = cli.cfl;
    if (cli.max_trip >= 0) p.max_trip = cli.max_trip;
    if (cli.strict_cfl) p.strict_cfl = 1;
    if (cli.dump_sx > 0) { p.dump_sx = cli.dump_sx; p.dump_sy = cli.dump_sx; }
    if (cli.dump_sz > 0) p.dump_sz = cli.dump_sz;
    if (cli.noise >= 0.f) p.noise = cli.noise;
    if (cli.sort_every >= 0) p.sort_every = cli.sort_every;
    if (cli.seed >= 0) p.seed = (uint32_t)cli.seed;
    if (cli.report < 1) cli.report = 1;
    st = asph_params_check(&p);
    if (st) return fail("parameters", st);

    const int N = p.n_particles;
    const float Lx = p.nx * p.dx, Ly = p.ny * p.dy, Lz = p.nz * p.dz;
    const double pmass = p.pmass > 0.f ? p.pmass : (double)kP0 / (kRd * p.th0) * Lx * Ly * Lz / N;

    Run run;
    st = asph_create(&p, nullptr, &run.ctx);
    if (st) return fail("create", st);
    AsphControl c0;
    asph_get_control(run.ctx, &c0);

    cudaDeviceProp prop;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaGetDeviceProperties(&prop, dev);
    std::printf("=== ASPH (GB300) ==================================================\n");
    std::printf("device        : %s (%d SM, %.1f GB)\n", prop.name, prop.multiProcessorCount,
                prop.totalGlobalMem / 1e9);
    std::printf("preset        : %s\n", cli.preset.c_str());
    std::printf("domain        : %.0f x %.0f x %.0f km  periodic xy, reflective z\n", Lx / 1e3, Ly / 1e3,
                Lz / 1e3);
    std::printf("grid          : %d x %d x %d cells of %.1f x %.1f x %.1f m\n", p.nx, p.ny, p.nz, p.dx, p.dy, p.dz);
    std::printf("parcels       : %d  (mass %.3e kg each)\n", N, pmass);
    std::printf("sounding      : theta0=%.0f K, N^2=%.1e /s^2, c_s=%.0f m/s\n", p.th0, p.n2, p.cs);
    std::printf("--- CFL -----------------------------------------------------------\n");
    std::printf("  static bound : dt <= %.4f s  (CFL %.2f * min(dx,dy,dz)/c_s)\n", c0.dt_static, p.cfl);
    std::printf("  closed loop  : dt <= CFL*Daxis/(c_s+|v|max)*0.9 every step (on the device)\n");
    std::printf("  floor %.4f s ; abort after %d violations%s\n", c0.dt_floor, p.max_trip,
                p.strict_cfl ? " (STRICT)" : "");
    std::printf("--- FORCING -------------------------------------------------------\n");
    std::printf("  bulk flux    : C_H=C_E=%.1e |V|=%.0f m/s beta=%.2f dTs=%.2f K\n", p.c_h, p.v_bg, p.beta_moist,
                p.dts_skin);
    std::printf("  dtheta/dt    : %.2e K/s peak (= %.2f K/h in lowest %.0f m)\n", p.c_h * p.v_bg * p.dts_skin / p.dz,
                p.c_h * p.v_bg * p.dts_skin / p.dz * 3600.0f, p.dz);
    std::printf("  microphysics : autoconversion%s%s\n", p.accretion ? " + accretion" : "",
                p.rain_evap ? " + rain evaporation" : "");
    std::printf("  run          : %.2f sim h, dump every %.0f sim s\n", cli.sim_hours, cli.dump_every);
    std::printf("===================================================================\n");
    size_t freeB = 0, totB = 0;
    cudaMemGetInfo(&freeB, &totB);
    std::printf("VRAM          : %.2f GB used of %.2f GB\n", (totB - freeB) / 1e9, totB / 1e9);
    mkdir(cli.outdir.c_str(), 0775);

    st = asph_init(run.ctx);
    if (st) return fail("init", st);
    double tot0[6] = {0}, tot[6] = {0};
    if ((st = asph_audit(run.ctx, tot0))) return fail("audit", st);

    const double sim_end = cli.sim_hours * 3600.0;
    double next_dump = cli.dump_every;
    long long step = 0;
    int dumps = 0;
    const double wall0 = now_s();
    double wall_report = wall0, sim_report = 0.0;
    float phase_acc[ASPH_NPHASES] = {0};
    static const char* phase_names[ASPH_NPHASES] = {"clear", "sort", "gather+kick+drift+flux", "density+eos+micro",
                                                    "momentum+integrate+rain+cfl", "step"};
    AsphControl ctl;
    asph_get_control(run.ctx, &ctl);
    struct {
        bool on = false;
        long long step = 0;
        AsphControl ctl;
    } pending;
    auto print_dump = [&](long long at_step, const AsphControl& c, const float* cd) {
        std::printf("%-8lld +%-8.0fs %-8.1f %-9.4f CFL %.2f | cloud %5.2f%% ql_max %.3f g/kg | w_max %5.2f m/s | "
                    "precip %.3f mm\n",
                    at_step, c.simt, now_s() - wall0, c.dt, c.dt_required > 0 ? c.dt / c.dt_required : 0.f, cd[0],
                    cd[1] * 1e3f, cd[2], cd[3]);
    };

    std::printf("\n%-8s %-9s %-8s %-9s %s\n", "step", "sim time", "wall s", "dt s", "CFL / cloud / precip");
    while (ctl.simt < sim_end && (cli.max_steps < 0 || step < cli.max_steps)) {
        // Steps that certainly stay before the next host event: a step never
        // advances time by more than dt_cap, so n steps of at most dt_cap end
        // short of the event; the last approach goes one step at a time.
        const double horizon = std::fmin(sim_end, next_dump) - ctl.simt;
        long long n = (long long)std::ceil(horizon / (double)ctl.dt_cap) - 1;
        if (n < 1) n = 1;
        const long long to_report = cli.report - (step % cli.report);
        if (n > to_report) n = to_report;
        const long long to_prof = 50 - (step % 50);   // one profiled step in 50 (asph_h100.cu:961)
        if (n > to_prof) n = to_prof;
        if (cli.max_steps >= 0 && n > cli.max_steps - step) n = cli.max_steps - step;
        if (n > 1 << 20) n = 1 << 20;
        const bool profiled = (step + n) % 50 == 0;
        if (profiled) {
            if (n > 1 && (st = asph_step_async(run.ctx, (int)(n - 1)))) break;
        } else if ((st = asph_step_async(run.ctx, (int)n))) {
            break;
        }
        // a dump begun after the previous chunk is written while this chunk runs
        if (pending.on) {
            char fn[1024];
            float cd[4];
            pending.on = false;
            if ((st = asph_dump_finish(run.ctx, cli.outdir.c_str(), fn, sizeof fn, cd))) break;
            ++dumps;
            print_dump(pending.step, pending.ctl, cd);
        }
        if ((st = asph_sync(run.ctx))) break;
        if (profiled) {
            float ph[ASPH_NPHASES];
            if ((st = asph_step_profiled(run.ctx, 1, ph))) break;
            for (int k = 0; k < ASPH_NPHASES; ++k) phase_acc[k] += ph[k];
        }
        step += n;
        asph_get_control(run.ctx, &ctl);

        if (ctl.simt >= next_dump) {
            if (cli.validate) {
                // the audit reads the state of the dump: dump synchronously
                char fn[1024];
                float cd[4];
                if ((st = asph_dump(run.ctx, cli.outdir.c_str(), fn, sizeof fn))) break;
                ++dumps;
                if ((st = asph_column_diag(run.ctx, cd))) break;
                print_dump(step, ctl, cd);
                if ((st = asph_audit(run.ctx, tot))) break;
                const double e0 = tot0[0] + tot0[1] + tot0[2], e1 = tot[0] + tot[1] + tot[2];
                std::printf("  AUDIT  KE %.4e  PE %.4e  IE %.4e  E_tot %.4e  water %.4e  pz %.4e\n", tot[0], tot[1],
                            tot[2], e1, tot[3], tot[4]);
                std::printf("  DRIFT  dKE %.2e  dE %.2e (%.3f%%/h)  dwater %.2e\n", tot[0] - tot0[0], e1 - e0,
                            100.0 * (e1 - e0) / std::fmax(1.0, std::fabs(e0)) * 3600.0 / std::fmax(1.0, ctl.simt),
                            tot[3] - tot0[3]);
            } else {
                if ((st = asph_dump_begin(run.ctx))) break;
                pending.on = true;
                pending.step = step;
                pending.ctl = ctl;
            }
            next_dump += cli.dump_every;
        }
        if (step % cli.report == 0) {
            const double wall = now_s();
            const double dw = wall - wall_report, ds = ctl.simt - sim_report;
            std::printf("  [step %lld] sim-s/wall-s=%.2f  dt=%.4f  req=%.4f  sorts=%d  trips=%d | ", step,
                        dw > 0 ? ds / dw : 0.0, ctl.dt, ctl.dt_required, ctl.sort_count, ctl.trips);
            for (int k = 0; k < ASPH_NPHASES; ++k) {
                if (phase_acc[k] > 0) std::printf("%s %.2f  ", phase_names[k], phase_acc[k]);
                phase_acc[k] = 0;
            }
            std::printf("\n");
            wall_report = wall;
            sim_report = ctl.simt;
        }
    }
    if (pending.on && st == ASPH_OK) {
        char fn[1024];
        float cd[4];
        pending.on = false;
        st = asph_dump_finish(run.ctx, cli.outdir.c_str(), fn, sizeof fn, cd);
        if (st == ASPH_OK) {
            ++dumps;
            print_dump(pending.step, pending.ctl, cd);
        }
    }
    asph_get_control(run.ctx, &ctl);
    if (st == ASPH_ERR_CFL_ABORT) {
        std::fprintf(stderr, "[CFL] step %d t=%.1fs : |u|=%.1f |v|=%.1f |w|=%.1f\n", ctl.step, ctl.simt, ctl.umax,
                     ctl.vmax, ctl.wmax);
        std::fprintf(stderr, "[CFL] ABORT after %d violation(s). The scheme is outside its stability envelope.\n",
                     ctl.trips);
        return 2;
    }
    if (st) return fail("step", st);

    const double wall = now_s() - wall0, rate = ctl.simt / wall;
    std::printf("\n=== DONE ==========================================================\n");
    std::printf("wall clock   : %.1f s\n", wall);
    std::printf("simulated    : %.2f sim h\n", ctl.simt / 3600.0);
    std::printf("throughput   : %.2f sim-s per wall-s (%.2fx real time)\n", rate, rate);
    std::printf("24 h forecast: %.2f wall-h\n", rate > 0 ? 24.0 / rate : 0.0);
    std::printf("parcel-steps : %.2f G/s\n", (double)N * (double)ctl.step / wall / 1e9);
    std::printf("sorts %d, dumps %d -> %s/\n", ctl.sort_count, dumps, cli.outdir.c_str());
    std::printf("CFL trips %d (tolerated %d)\n", ctl.trips, p.max_trip);
    std::printf("final dt %.4f s (required %.4f, static %.4f)\n", ctl.dt, ctl.dt_required, ctl.dt_static);
    std::printf("===================================================================\n");
    return 0;
}
