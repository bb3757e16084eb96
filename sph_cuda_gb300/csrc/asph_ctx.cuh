// asph_ctx.cuh — the context behind the opaque asph_ctx handle, shared by
// the C-ABI translation units (asph_capi.cu, asph_ensemble.cu).
#pragma once
#include <cuda_runtime.h>
#include <vector>
#include "asph_internal.cuh"
#include "../../include/asph.h"

using namespace asph;

struct asph_ctx {
    AsphParams prm;
    Phys P;
    Bufs B{};
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    bool initialised = false;
    bool lists_valid = false;   // neighbour lists match the current positions
    bool spans_valid = false;   // brick spans match the sorted keys and the brick shape in use
    // step graphs keyed by kind (StepKind) x the ping-pong state at the start of the step
    cudaGraphExec_t gexec[5 * 16] = {};
    int graph_kernels[5] = {};  // kernel nodes of a captured step graph of each kind
    bool sort_ahead = true;     // ASPH_OPT_SORT_AHEAD
    unsigned graph_epoch = 0;   // bumped whenever an option change drops the captured graphs
    // staging for host <-> device SoA copies (16 floats per particle)
    float* stage = nullptr;
    // audit
    double* audit_part = nullptr;
    double* audit_out = nullptr;
    int audit_blocks = 152 * 4;
    // dumps
    float* coarse = nullptr;
    float4* coldiag = nullptr;
    int cx = 0, cy = 0, cz = 0;
    uint8_t* flags = nullptr;
    // source-term hook: tendencies and their per-step copy (2 x float4[N])
    float4* src_mem = nullptr;
    // asynchronous dump: pinned host copy and its completion event
    void* h_dump = nullptr;
    cudaEvent_t dump_ev = nullptr;
    bool dump_pending = false;
    std::vector<void*> allocs;

    template <class T>
    cudaError_t alloc(T** p, size_t bytes) {
        void* q = nullptr;
        cudaError_t e = cudaMalloc(&q, bytes < 256 ? 256 : bytes);
        if (e == cudaSuccess) {
            allocs.push_back(q);
            *p = (T*)q;
        }
        return e;
    }
    ~asph_ctx() {
        if (h_dump) cudaFreeHost(h_dump);
        if (dump_ev) cudaEventDestroy(dump_ev);
        for (auto& g : gexec)
            if (g) cudaGraphExecDestroy(g);
        for (void* q : allocs) cudaFree(q);
        if (B.ev_fork) cudaEventDestroy(B.ev_fork);
        if (B.ev_join) cudaEventDestroy(B.ev_join);
        if (B.aux) cudaStreamDestroy(B.aux);
        if (B.ev_fork2) cudaEventDestroy(B.ev_fork2);
        if (B.ev_join2) cudaEventDestroy(B.ev_join2);
        if (B.aux2) cudaStreamDestroy(B.aux2);
        if (own_stream && stream) cudaStreamDestroy(stream);
    }
};

namespace asph {
// Record a failure for asph_last_error(); returns `code`.
int fail(int code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
// Wait for the context's stream and turn the device error word / CFL abort
// flag into a status.
int sync_status(asph_ctx* c);
// Kinds of captured step.  STEP_PLAIN sorts at its start.  In a run of
// several steps with a sort every step, the first step (STEP_FIRST) sorts at
// its start and also sorts the next step's keys beside its pair passes, the
// middle steps (STEP_MID) apply the sort run ahead and run the next one, and
// the last (STEP_LAST) applies the sort run ahead and runs none, so that
// between calls the context holds the last applied sort.  STEP_MID2 is two
// middle steps captured in one graph.
enum StepKind : int { STEP_PLAIN = 0, STEP_FIRST = 1, STEP_MID = 2, STEP_LAST = 3, STEP_MID2 = 4 };
// Enqueue one full step (sort, gather/kick/drift/flux, density, momentum)
// on the context's stream and advance the ping-pong indices.
void enqueue_step(asph_ctx* c, int kind = STEP_PLAIN);
// Graph key of the ping-pong state at the start of a step.
int graph_slot(const Bufs& B);
void apply_pending_clamp(asph_ctx* c);
bool reads_rain(const Phys& P);
int reset_control(asph_ctx* c);
// Recompute the brick spans from the sorted keys when no sort's gather wrote
// them for the current keys and brick shape (outside any graph capture).
void ensure_spans(asph_ctx* c);
}  // namespace asph

#define CKR(x)                                                                                  \
    do {                                                                                        \
        cudaError_t e_ = (x);                                                                   \
        if (e_ != cudaSuccess)                                                                  \
            return fail(ASPH_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__, #x, cudaGetErrorString(e_)); \
    } while (0)
