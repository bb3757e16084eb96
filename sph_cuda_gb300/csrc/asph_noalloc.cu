// asph_noalloc.cu — stable key sort that allocates no memory.
//
// Some callers cannot call cudaMalloc or cudaFree: a host driving a
// latency-critical time-step loop where cudaFree would synchronise the whole
// device, a host callback or foreign-language runtime (cgo, JNI) that must
// not block on the driver's allocator, or an application whose memory pool
// owns all device memory.  asph_sort_keys_noalloc() gives them the Morton-key
// sort of the step (the same kernels as asph_sort_build) with its scratch
// in a file-scope device array instead of an allocation.  The caller passes
// the input keys and the two outputs as device pointers.
//
// Scratch: one static __device__ array, ASPH_NOALLOC_MAX_KEYS keys at most,
// held by every GPU that loads the library until the process exits.  All
// calls share it and it keeps the last call's contents, so each call resets
// the counters it needs; calls that overlap on the GPU (two streams, or two
// host threads) race on it and must be serialised by the caller.
//
// Set-up: host code only sees a host-side stand-in for the array, so the
// first call in a CUDA context looks up the array's device address with
// cudaGetSymbolAddress, with that context current, and caches it for that
// context.  The cache is keyed by the context itself (from the driver's
// cuCtxGetCurrent), so a context created later on the same device, by a
// device reset or by a foreign runtime with its own context, gets its own
// look-up.
//
// Every call waits for its stream and reads the device error word back, so
// the function must never be called while any stream on the device is
// being captured into a CUDA graph.
#include <cuda.h>
#include <cuda_runtime.h>
#include <mutex>
#include "asph_internal.cuh"
#include "../../include/asph.h"

namespace asph {

// Kernels of asph_sort.cu, launched unchanged.
__global__ void k_hist(const uint32_t* __restrict__ keys, int N, int npasses, DevCtl* __restrict__ ctl, int force,
                       int lane);
__global__ void k_radix_pass(const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin,
                             uint32_t* __restrict__ kout, uint32_t* __restrict__ vout, uint64_t* __restrict__ status,
                             int N, int ntiles, int pass, DevCtl* __restrict__ ctl, int force, int lane);

namespace {

constexpr int NA_MAX_KEYS = ASPH_NOALLOC_MAX_KEYS;
constexpr int NA_MAX_TILES = (NA_MAX_KEYS + SORT_TILE - 1) / SORT_TILE;
constexpr size_t NA_CTL_BYTES = (sizeof(DevCtl) + 255) / 256 * 256;
constexpr size_t NA_KEYS_OFF = NA_CTL_BYTES;
constexpr size_t NA_VALS_OFF = NA_KEYS_OFF + (size_t)NA_MAX_KEYS * 4;
constexpr size_t NA_STATUS_OFF = NA_VALS_OFF + (size_t)NA_MAX_KEYS * 4;
constexpr size_t NA_BYTES = NA_STATUS_OFF + (size_t)MAX_PASSES * NA_MAX_TILES * 256 * 8;

// The scratch: control block, ping-pong keys and values, look-back words.
static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

// Device addresses of the array, one per CUDA context that called.
constexpr int NA_MAX_CONTEXTS = 64;
struct NaEntry {
    CUcontext ctx;
    unsigned char* ptr;
};
NaEntry g_scratch[NA_MAX_CONTEXTS] = {};
int g_scratch_n = 0;
std::mutex g_scratch_mu;

// The calling thread's current driver context, through the runtime's
// driver entry point (the library links the runtime only); NULL when the
// runtime has not made a context current yet.
CUcontext current_context() {
    typedef CUresult (*GetCurrent)(CUcontext*);
    static GetCurrent fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 4000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (GetCurrent)f;
    });
    CUcontext c = nullptr;
    if (!fn || fn(&c) != CUDA_SUCCESS) return nullptr;
    return c;
}

// The array's device address in the calling thread's current context,
// looked up on the first call in that context.
unsigned char* scratch_address() {
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    CUcontext ctx = current_context();
    if (ctx)
        for (int k = 0; k < g_scratch_n; ++k)
            if (g_scratch[k].ctx == ctx) return g_scratch[k].ptr;
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return nullptr;
    ctx = current_context();   // the look-up makes the device's context current if none was
    if (ctx) {
        int slot = -1;
        for (int k = 0; k < g_scratch_n; ++k)
            if (g_scratch[k].ctx == ctx) slot = k;
        if (slot < 0) slot = g_scratch_n < NA_MAX_CONTEXTS ? g_scratch_n++ : NA_MAX_CONTEXTS - 1;
        g_scratch[slot] = NaEntry{ctx, (unsigned char*)p};
    }
    return (unsigned char*)p;
}

__global__ void k_noalloc_prep(DevCtl* ctl) {
    for (int i = threadIdx.x; i < MAX_PASSES * 256; i += blockDim.x) (&ctl->hist[0][0])[i] = 0u;
    if (threadIdx.x < MAX_PASSES) ctl->tile_ctr[threadIdx.x] = 0u;
    if (threadIdx.x == 0) {
        ctl->epoch += 1u;   // status words of earlier calls carry older epochs
        ctl->error = 0;
        ctl->aborted = 0;
    }
}

int na_fail(int code, const char* msg) { return set_error(code, msg); }

}  // namespace

}  // namespace asph

using namespace asph;

extern "C" int asph_sort_keys_noalloc(const uint32_t* keys, uint32_t* keys_sorted, uint32_t* perm, int n,
                                      int key_bits, void* stream) {
    if (n < 0 || n > NA_MAX_KEYS) return na_fail(ASPH_ERR_ARG, "asph_sort_keys_noalloc: n outside [0, ASPH_NOALLOC_MAX_KEYS]");
    if (key_bits < 1 || key_bits > 8 * MAX_PASSES) return na_fail(ASPH_ERR_ARG, "asph_sort_keys_noalloc: key_bits outside [1, 32]");
    if (n == 0) return ASPH_OK;
    if (!keys || !keys_sorted || !perm) return na_fail(ASPH_ERR_ARG, "asph_sort_keys_noalloc: NULL pointer");
    unsigned char* base = scratch_address();
    if (!base) return na_fail(ASPH_ERR_CUDA, "asph_sort_keys_noalloc: cudaGetSymbolAddress failed");
    DevCtl* ctl = reinterpret_cast<DevCtl*>(base);
    uint32_t* sk = reinterpret_cast<uint32_t*>(base + NA_KEYS_OFF);
    uint32_t* sv = reinterpret_cast<uint32_t*>(base + NA_VALS_OFF);
    uint64_t* status = reinterpret_cast<uint64_t*>(base + NA_STATUS_OFF);
    cudaStream_t s = (cudaStream_t)stream;
    const int npasses = (key_bits + 7) / 8;
    const int ntiles = (n + SORT_TILE - 1) / SORT_TILE;
    k_noalloc_prep<<<1, 256, 0, s>>>(ctl);
    int hb = (n + TPB * 8 - 1) / (TPB * 8);
    hb = hb > 152 * 8 ? 152 * 8 : hb;
    k_hist<<<hb, SORT_TPB, 0, s>>>(keys, n, npasses, ctl, 1, 0);
    const uint32_t* ki = keys;
    const uint32_t* vi = nullptr;
    for (int p = 0; p < npasses; ++p) {
        // the last pass lands in the caller's outputs
        const bool to_out = ((npasses - 1 - p) % 2) == 0;
        uint32_t* ko = to_out ? keys_sorted : sk;
        uint32_t* vo = to_out ? perm : sv;
        k_radix_pass<<<ntiles, SORT_TPB, 0, s>>>(ki, vi, ko, vo, status, n, ntiles, p, ctl, 1, 0);
        ki = ko;
        vi = vo;
    }
    if (cudaGetLastError() != cudaSuccess) return na_fail(ASPH_ERR_CUDA, "asph_sort_keys_noalloc: launch failed");
    // read the error word on the caller's stream only (no device-wide wait)
    int err = 0;
    if (cudaMemcpyAsync(&err, &ctl->error, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return na_fail(ASPH_ERR_CUDA, "asph_sort_keys_noalloc: cannot read the error word");
    if (cudaStreamSynchronize(s) != cudaSuccess) return na_fail(ASPH_ERR_CUDA, "asph_sort_keys_noalloc: kernel failed");
    if (err) return na_fail(ASPH_ERR_TIMEOUT, "asph_sort_keys_noalloc: a bounded look-back wait gave up");
    return ASPH_OK;
}
