// asph_ensemble.cu — device-resident state snapshots, restart files, and the
// batched ensemble with its autotuner.  None of these has a counterpart in
// the reference (asph_h100.cu runs one simulation per process and cannot
// restart); they wrap its step (asph_h100.cu:958-1078) without changing it.
//
// Snapshot: everything a context needs to continue a run bit for bit — the
// particle field groups, the stale cell table and surface flags of the last
// sort (the next steps may search with them), the rain grid, the surface
// precipitation and the device control block — copied device to device into
// one allocation.
//
// Ensemble: M member contexts, each with its own stream, parameters and
// control block (dt, CFL, sort cadence).  One ensemble step is one CUDA
// graph: a fork from the caller's stream into every member stream, each
// member's full step, and a join.  The members' kernels are independent
// graph branches, so small members fill the SMs that large members leave
// idle and no kernel launch is issued per member from the host.
#include <stdio.h>
#include <string.h>
#include <stddef.h>
#include <map>
#include <vector>
#include "asph_ctx.cuh"

// ---------------------------------------------------------------------------
// snapshots
// ---------------------------------------------------------------------------
struct asph_snapshot {
    int N = 0, ncell = 0, nxy = 0;
    void* mem = nullptr;
    float4 *pos = nullptr, *vel = nullptr, *thq = nullptr, *acc = nullptr;
    float2* rp = nullptr;
    float *dthdt = nullptr, *rain = nullptr, *precip = nullptr;
    uint32_t* kin = nullptr;
    uint32_t* skeys = nullptr;
    uint8_t* surf = nullptr;
    int2* range = nullptr;
    DevCtl* ctl = nullptr;
    ~asph_snapshot() {
        if (mem) cudaFree(mem);
    }
};

namespace {

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// One copy per field group, in a fixed order shared by save, restore and
// the restart file.  Besides the particle and grid state this holds what the
// last sort left for the next step: the cell table, the surface flags and the
// sorted keys (the next incremental sort takes the particles whose key still
// equals its sorted key as an already sorted subsequence, and the density
// pass finds its bricks' spans in them).
struct Part {
    void* dev;      // context buffer
    void* snap;     // snapshot buffer
    size_t bytes;
};
constexpr int NPARTS = 12;

int parts(asph_ctx* c, const asph_snapshot* s, Part out[NPARTS]) {
    const Bufs& B = c->B;
    const size_t N = (size_t)c->P.N, C = (size_t)c->P.ncell;
    Part p[NPARTS] = {
        {B.pos[B.pc], s->pos, N * 16},  {B.vel[B.vc], s->vel, N * 16}, {B.thq[B.qc], s->thq, N * 16},
        {B.acc, s->acc, N * 16},        {B.rp, s->rp, N * 8},         {B.dthdt, s->dthdt, N * 4},
        {B.kin, s->kin, N * 4},         {B.skeys, s->skeys, N * 4},   {B.surf, s->surf, N},
        {B.range, s->range, C * 8},     {B.rain[B.rc], s->rain, C * 4},
        {B.precip, s->precip, (size_t)c->P.nxy * 4},
    };
    memcpy(out, p, sizeof(p));
    return NPARTS;
}

bool same_shape(const asph_ctx* c, const asph_snapshot* s) {
    return s->N == c->P.N && s->ncell == c->P.ncell && s->nxy == c->P.nxy;
}

}  // namespace

extern "C" int asph_snapshot_create(asph_ctx* c, asph_snapshot** out) {
    if (!c || !out) return fail(ASPH_ERR_ARG, "NULL argument");
    *out = nullptr;
    asph_snapshot* s = new asph_snapshot();
    s->N = c->P.N; s->ncell = c->P.ncell; s->nxy = c->P.nxy;
    const size_t N = (size_t)s->N, C = (size_t)s->ncell;
    const size_t sizes[NPARTS + 1] = {N * 16, N * 16, N * 16, N * 16, N * 8, N * 4, N * 4, N * 4, N, C * 8,
                                      C * 4, (size_t)s->nxy * 4, sizeof(DevCtl)};
    size_t total = 0;
    for (size_t b : sizes) total += align256(b);
    cudaError_t e = cudaMalloc(&s->mem, total);
    if (e != cudaSuccess) {
        delete s;
        return fail(e == cudaErrorMemoryAllocation ? ASPH_ERR_NOMEM : ASPH_ERR_CUDA, "snapshot allocation: %s",
                    cudaGetErrorString(e));
    }
    char* q = (char*)s->mem;
    void** dst[NPARTS + 1] = {(void**)&s->pos,   (void**)&s->vel,   (void**)&s->thq,   (void**)&s->acc,
                              (void**)&s->rp,    (void**)&s->dthdt, (void**)&s->kin,   (void**)&s->skeys,
                              (void**)&s->surf,  (void**)&s->range, (void**)&s->rain,  (void**)&s->precip,
                              (void**)&s->ctl};
    for (int k = 0; k < NPARTS + 1; ++k) {
        *dst[k] = q;
        q += align256(sizes[k]);
    }
    *out = s;
    return ASPH_OK;
}

extern "C" int asph_snapshot_destroy(asph_snapshot* s) {
    delete s;
    return ASPH_OK;
}

extern "C" int asph_snapshot_save(asph_ctx* c, asph_snapshot* s) {
    if (!c || !s) return fail(ASPH_ERR_ARG, "NULL argument");
    if (!same_shape(c, s)) return fail(ASPH_ERR_ARG, "snapshot was made for another particle count or grid");
    if (!c->initialised) return fail(ASPH_ERR_STATE, "snapshot before init/set_state");
    Part p[NPARTS];
    const int n = parts(c, s, p);
    for (int k = 0; k < n; ++k) CKR(cudaMemcpyAsync(p[k].snap, p[k].dev, p[k].bytes, cudaMemcpyDeviceToDevice, c->stream));
    CKR(cudaMemcpyAsync(s->ctl, c->B.ctl, sizeof(DevCtl), cudaMemcpyDeviceToDevice, c->stream));
    return ASPH_OK;
}

extern "C" int asph_snapshot_restore(asph_ctx* c, const asph_snapshot* s) {
    if (!c || !s) return fail(ASPH_ERR_ARG, "NULL argument");
    if (!same_shape(c, s)) return fail(ASPH_ERR_ARG, "snapshot was made for another particle count or grid");
    Part p[NPARTS];
    const int n = parts(c, s, p);
    for (int k = 0; k < n; ++k) CKR(cudaMemcpyAsync(p[k].dev, p[k].snap, p[k].bytes, cudaMemcpyDeviceToDevice, c->stream));
    // the radix look-back epoch keeps growing (status words of later sorts carry larger epochs)
    CKR(cudaMemcpyAsync(c->B.ctl, s->ctl, offsetof(DevCtl, epoch), cudaMemcpyDeviceToDevice, c->stream));
    c->initialised = true;
    c->lists_valid = false;
    c->spans_valid = false;   // the restored sorted keys' brick spans are rebuilt before the next pass
    return ASPH_OK;
}

// ---------------------------------------------------------------------------
// restart files: header, parameters, control block, field groups
// ---------------------------------------------------------------------------
namespace {

struct RestartHeader {
    uint32_t magic, version;
    int32_t n_particles, nx, ny, nz, params_size, ctl_bytes;
};
constexpr uint32_t RESTART_MAGIC = 0x41535052u;   // "RPSA" little-endian: ASPH restart
constexpr uint32_t RESTART_VERSION = 2;   // 2: the sorted keys of the last sort are saved

}  // namespace

extern "C" int asph_checkpoint_write(asph_ctx* c, const char* path) {
    if (!c || !path) return fail(ASPH_ERR_ARG, "NULL argument");
    asph_snapshot* s = nullptr;
    int st = asph_snapshot_create(c, &s);
    if (st) return st;
    st = asph_snapshot_save(c, s);
    FILE* f = nullptr;
    std::vector<char> host;
    if (!st) {
        cudaError_t e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) st = fail(ASPH_ERR_CUDA, "checkpoint: %s", cudaGetErrorString(e));
    }
    if (!st && !(f = fopen(path, "wb"))) st = fail(ASPH_ERR_IO, "cannot open %s", path);
    if (!st) {
        RestartHeader h{RESTART_MAGIC, RESTART_VERSION, c->P.N, c->P.nx, c->P.ny, c->P.nz, (int)sizeof(AsphParams),
                        (int)offsetof(DevCtl, epoch)};
        bool ok = fwrite(&h, sizeof h, 1, f) == 1 && fwrite(&c->prm, sizeof(AsphParams), 1, f) == 1;
        Part p[NPARTS + 1];
        const int n = parts(c, s, p);
        p[n] = Part{nullptr, s->ctl, (size_t)offsetof(DevCtl, epoch)};
        for (int k = 0; k <= n && ok; ++k) {
            host.resize(p[k].bytes);
            cudaError_t e = cudaMemcpy(host.data(), p[k].snap, p[k].bytes, cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) { st = fail(ASPH_ERR_CUDA, "checkpoint copy: %s", cudaGetErrorString(e)); break; }
            ok = fwrite(host.data(), 1, p[k].bytes, f) == p[k].bytes;
        }
        if (fclose(f) != 0) ok = false;
        if (!st && !ok) st = fail(ASPH_ERR_IO, "short write to %s", path);
    }
    asph_snapshot_destroy(s);
    return st;
}

extern "C" int asph_checkpoint_read(asph_ctx* c, const char* path) {
    if (!c || !path) return fail(ASPH_ERR_ARG, "NULL argument");
    FILE* f = fopen(path, "rb");
    if (!f) return fail(ASPH_ERR_IO, "cannot open %s", path);
    RestartHeader h;
    AsphParams prm;
    int st = ASPH_OK;
    if (fread(&h, sizeof h, 1, f) != 1 || h.magic != RESTART_MAGIC || h.version != RESTART_VERSION)
        st = fail(ASPH_ERR_IO, "%s is not an ASPH restart file", path);
    else if (h.params_size != (int)sizeof(AsphParams) || h.ctl_bytes != (int)offsetof(DevCtl, epoch))
        st = fail(ASPH_ERR_IO, "%s was written by an incompatible library build", path);
    else if (h.n_particles != c->P.N || h.nx != c->P.nx || h.ny != c->P.ny || h.nz != c->P.nz)
        st = fail(ASPH_ERR_CONFIG, "%s holds %d particles on %dx%dx%d cells, the context %d on %dx%dx%d", path,
                  h.n_particles, h.nx, h.ny, h.nz, c->P.N, c->P.nx, c->P.ny, c->P.nz);
    else if (fread(&prm, sizeof prm, 1, f) != 1)
        st = fail(ASPH_ERR_IO, "%s is truncated", path);
    asph_snapshot* s = nullptr;
    if (!st) st = asph_snapshot_create(c, &s);
    if (!st) {
        Part p[NPARTS + 1];
        const int n = parts(c, s, p);
        p[n] = Part{nullptr, s->ctl, (size_t)offsetof(DevCtl, epoch)};
        std::vector<char> host;
        for (int k = 0; k <= n && !st; ++k) {
            host.resize(p[k].bytes);
            if (fread(host.data(), 1, p[k].bytes, f) != p[k].bytes) {
                st = fail(ASPH_ERR_IO, "%s is truncated", path);
                break;
            }
            cudaError_t e = cudaMemcpy(p[k].snap, host.data(), p[k].bytes, cudaMemcpyHostToDevice);
            if (e != cudaSuccess) st = fail(ASPH_ERR_CUDA, "restart copy: %s", cudaGetErrorString(e));
        }
        if (!st) st = asph_snapshot_restore(c, s);
        if (!st) st = sync_status(c);
    }
    fclose(f);
    if (s) asph_snapshot_destroy(s);
    return st;
}

// ---------------------------------------------------------------------------
// ensemble
// ---------------------------------------------------------------------------
struct asph_ens {
    std::vector<asph_ctx*> m;
    cudaStream_t origin = nullptr;
    bool own_origin = false;
    cudaEvent_t fork = nullptr, done = nullptr;
    std::vector<cudaEvent_t> join, ready;
    std::map<std::vector<int>, cudaGraphExec_t> graphs;   // keyed by every member's ping-pong state
    ~asph_ens() {
        if (origin) cudaStreamSynchronize(origin);
        for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
        for (asph_ctx* c : m) asph_destroy(c);
        for (cudaEvent_t e : join) cudaEventDestroy(e);
        for (cudaEvent_t e : ready) cudaEventDestroy(e);
        if (fork) cudaEventDestroy(fork);
        if (done) cudaEventDestroy(done);
        if (own_origin && origin) cudaStreamDestroy(origin);
    }
};

namespace {

void drop_ens_graphs(asph_ens* e) {
    for (auto& kv : e->graphs) cudaGraphExecDestroy(kv.second);
    e->graphs.clear();
}

// Work queued by the caller on a member stream (a borrowed context) comes
// before the next ensemble step.
int origin_after_members(asph_ens* e) {
    for (size_t k = 0; k < e->m.size(); ++k) {
        CKR(cudaEventRecord(e->ready[k], e->m[k]->stream));
        CKR(cudaStreamWaitEvent(e->origin, e->ready[k], 0));
    }
    return ASPH_OK;
}

int capture_step(asph_ens* e, cudaGraphExec_t* out) {
    std::vector<Bufs> saved;
    for (asph_ctx* c : e->m) saved.push_back(c->B);
    CKR(cudaStreamBeginCapture(e->origin, cudaStreamCaptureModeThreadLocal));
    cudaError_t err = cudaEventRecord(e->fork, e->origin);
    for (size_t k = 0; k < e->m.size() && err == cudaSuccess; ++k) {
        asph_ctx* c = e->m[k];
        err = cudaStreamWaitEvent(c->stream, e->fork, 0);
        if (err == cudaSuccess) enqueue_step(c);
        if (err == cudaSuccess) err = cudaEventRecord(e->join[k], c->stream);
        if (err == cudaSuccess) err = cudaStreamWaitEvent(e->origin, e->join[k], 0);
    }
    cudaGraph_t g = nullptr;
    cudaError_t err2 = cudaStreamEndCapture(e->origin, &g);
    for (size_t k = 0; k < e->m.size(); ++k) e->m[k]->B = saved[k];
    if (err != cudaSuccess || err2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return fail(ASPH_ERR_CUDA, "ensemble capture: %s",
                    cudaGetErrorString(err != cudaSuccess ? err : err2));
    }
    err = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (err != cudaSuccess) return fail(ASPH_ERR_CUDA, "ensemble instantiate: %s", cudaGetErrorString(err));
    return ASPH_OK;
}

}  // namespace

extern "C" int asph_ens_create(const AsphParams* members, int n_members, void* stream, asph_ens** out) {
    if (!members || !out || n_members < 1) return fail(ASPH_ERR_ARG, "need at least one member");
    *out = nullptr;
    asph_ens* e = new asph_ens();
    int st = ASPH_OK;
    for (int k = 0; k < n_members && !st; ++k) {
        asph_ctx* c = nullptr;
        st = asph_create(&members[k], nullptr, &c);
        if (st) {
            fail(st, "member %d: %s", k, asph_last_error());
            break;
        }
        e->m.push_back(c);
    }
    cudaError_t err = cudaSuccess;
    if (!st) {
        if (stream) {
            e->origin = (cudaStream_t)stream;
        } else {
            err = cudaStreamCreateWithFlags(&e->origin, cudaStreamNonBlocking);
            e->own_origin = err == cudaSuccess;
        }
    }
    if (!st && err == cudaSuccess) err = cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming);
    if (!st && err == cudaSuccess) err = cudaEventCreateWithFlags(&e->done, cudaEventDisableTiming);
    for (int k = 0; k < n_members && !st && err == cudaSuccess; ++k) {
        cudaEvent_t a = nullptr, b = nullptr;
        err = cudaEventCreateWithFlags(&a, cudaEventDisableTiming);
        if (err == cudaSuccess) err = cudaEventCreateWithFlags(&b, cudaEventDisableTiming);
        if (a) e->join.push_back(a);
        if (b) e->ready.push_back(b);
    }
    if (!st && err != cudaSuccess) st = fail(ASPH_ERR_CUDA, "ensemble streams/events: %s", cudaGetErrorString(err));
    if (st) {
        delete e;
        return st;
    }
    *out = e;
    return ASPH_OK;
}

extern "C" int asph_ens_destroy(asph_ens* e) {
    delete e;
    return ASPH_OK;
}

extern "C" int asph_ens_size(asph_ens* e) { return e ? (int)e->m.size() : 0; }

extern "C" int asph_ens_member(asph_ens* e, int k, asph_ctx** ctx) {
    if (!e || !ctx) return fail(ASPH_ERR_ARG, "NULL argument");
    if (k < 0 || k >= (int)e->m.size()) return fail(ASPH_ERR_ARG, "member %d out of range", k);
    // calls on the borrowed context come after the ensemble steps queued so far
    CKR(cudaEventRecord(e->done, e->origin));
    CKR(cudaStreamWaitEvent(e->m[k]->stream, e->done, 0));
    *ctx = e->m[k];
    return ASPH_OK;
}

extern "C" int asph_ens_init(asph_ens* e) {
    if (!e) return fail(ASPH_ERR_ARG, "NULL argument");
    for (size_t k = 0; k < e->m.size(); ++k) {
        int st = asph_init(e->m[k]);
        if (st) return fail(st, "member %zu: %s", k, asph_last_error());
    }
    return ASPH_OK;
}

extern "C" int asph_ens_step_async(asph_ens* e, int nsteps) {
    if (!e) return fail(ASPH_ERR_ARG, "NULL argument");
    for (asph_ctx* c : e->m)
        if (!c->initialised) return fail(ASPH_ERR_STATE, "ensemble step before init");
    for (asph_ctx* c : e->m) ensure_spans(c);   // on each member's stream, before the origin waits on it
    int st = origin_after_members(e);
    if (st) return st;
    std::vector<int> key(e->m.size());
    for (int s = 0; s < nsteps; ++s) {
        for (size_t k = 0; k < e->m.size(); ++k) key[k] = graph_slot(e->m[k]->B);
        auto it = e->graphs.find(key);
        if (it == e->graphs.end()) {
            cudaGraphExec_t g = nullptr;
            st = capture_step(e, &g);
            if (st) return st;
            it = e->graphs.emplace(key, g).first;
        }
        CKR(cudaGraphLaunch(it->second, e->origin));
        for (asph_ctx* c : e->m) {
            c->B.pc ^= 1; c->B.qc ^= 1; c->B.rc ^= 1;   // vel flips twice per step
            c->lists_valid = true;
        }
    }
    CKR(cudaEventRecord(e->done, e->origin));
    for (asph_ctx* c : e->m) CKR(cudaStreamWaitEvent(c->stream, e->done, 0));
    return ASPH_OK;
}

extern "C" int asph_ens_sync(asph_ens* e) {
    if (!e) return fail(ASPH_ERR_ARG, "NULL argument");
    CKR(cudaStreamSynchronize(e->origin));
    for (size_t k = 0; k < e->m.size(); ++k) {
        int st = sync_status(e->m[k]);
        if (st) return fail(st, "member %zu: %s", k, asph_last_error());
    }
    return ASPH_OK;
}

extern "C" int asph_ens_step(asph_ens* e, int nsteps) {
    int st = asph_ens_step_async(e, nsteps);
    if (st) return st;
    return asph_ens_sync(e);
}

// Autotuner: per member, every brick shape that suits its grid plus the
// per-target path (the cells each density block covers), crossed with the
// momentum pass's targets per thread (1, 2, 4: the cells each warp covers)
// and the allowed sort cadences, each timed over trial_steps graph-launched
// steps (after one untimed step) from the same snapshot; the member keeps
// the fastest and its state is put back.
extern "C" int asph_ens_tune(asph_ens* e, int trial_steps, const int* sort_choices, int n_sort_choices,
                             int* chosen) {
    if (!e || trial_steps < 1 || n_sort_choices < 0 || (n_sort_choices > 0 && !sort_choices))
        return fail(ASPH_ERR_ARG, "bad tuner arguments");
    int st = asph_ens_sync(e);
    if (st) return st;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    CKR(cudaEventCreate(&t0));
    if (cudaEventCreate(&t1) != cudaSuccess) {
        cudaEventDestroy(t0);
        return fail(ASPH_ERR_CUDA, "tuner events");
    }
    for (size_t k = 0; k < e->m.size() && !st; ++k) {
        asph_ctx* c = e->m[k];
        asph_snapshot* snap = nullptr;
        if ((st = asph_snapshot_create(c, &snap))) break;
        if ((st = asph_snapshot_save(c, snap))) { asph_snapshot_destroy(snap); break; }
        std::vector<int> cadences;
        if (n_sort_choices == 0) cadences.push_back(c->P.sort_every);
        for (int q = 0; q < n_sort_choices; ++q) cadences.push_back(sort_choices[q]);
        std::vector<int> shapes{-2};   // -2: per-target global path
        for (int s = 0; s < pair_shape_count(); ++s)
            if (pair_shape_fits(c->P, s)) shapes.push_back(s);
        float best = 1e30f;
        int best_shape = -1, best_sort = c->P.sort_every, best_tpt = 2;
        const int tpts[3] = {1, 2, 4};
        for (int sh : shapes) {
            for (int cad : cadences) {
              for (int tpt : tpts) {
                if ((st = asph_set_option(c, ASPH_OPT_PAIR_PATH, sh == -2 ? 1 : 0))) break;
                if ((st = asph_set_option(c, ASPH_OPT_PAIR_SHAPE, sh == -2 ? -1 : sh))) break;
                if ((st = asph_set_option(c, ASPH_OPT_SORT_EVERY, cad))) break;
                if ((st = asph_set_option(c, ASPH_OPT_TARGETS_PER_THREAD, tpt))) break;
                if ((st = asph_snapshot_restore(c, snap))) break;
                if ((st = asph_step(c, 1))) break;   // capture + warm
                cudaError_t err = cudaEventRecord(t0, c->stream);
                if (err == cudaSuccess && (st = asph_step_async(c, trial_steps))) break;
                if (err == cudaSuccess) err = cudaEventRecord(t1, c->stream);
                if (err != cudaSuccess) { st = fail(ASPH_ERR_CUDA, "tuner timing: %s", cudaGetErrorString(err)); break; }
                if ((st = sync_status(c))) break;
                float ms = 0.f;
                cudaEventElapsedTime(&ms, t0, t1);
                if (ms < best) { best = ms; best_shape = sh; best_sort = cad; best_tpt = tpt; }
              }
              if (st) break;
            }
            if (st) break;
        }
        if (!st) st = asph_set_option(c, ASPH_OPT_PAIR_PATH, best_shape == -2 ? 1 : 0);
        if (!st) st = asph_set_option(c, ASPH_OPT_PAIR_SHAPE, best_shape == -2 ? -1 : best_shape);
        if (!st) st = asph_set_option(c, ASPH_OPT_SORT_EVERY, best_sort);
        if (!st) st = asph_set_option(c, ASPH_OPT_TARGETS_PER_THREAD, best_tpt);
        if (!st) st = asph_snapshot_restore(c, snap);
        if (!st) st = sync_status(c);
        asph_snapshot_destroy(snap);
        if (!st && chosen) {
            chosen[3 * k] = best_shape == -2 ? -1 : best_shape;
            chosen[3 * k + 1] = best_sort;
            chosen[3 * k + 2] = best_tpt;
        }
        if (st) fail(st, "tuning member %zu: %s", k, asph_last_error());
    }
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    drop_ens_graphs(e);   // member kernels and parameters may have changed
    return st;
}
