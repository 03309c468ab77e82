// static_scratch.cu — issm_resampling_cdf_static: the reference-compatible
// resampling CDF (_resampling_cdf!, src/resampling.jl:199-225) run on a fixed
// device scratch array instead of a caller-provided workspace, for callers that
// cannot allocate device memory.
//
// The scratch is one file-scope __device__ array with the same layout as the
// workspace of issm_resampling_cdf (reduce.cu):
//   [0, 4)      completion counter of the summary kernel — must be zero when a
//               call's first kernel starts; every call zeroes it with
//               cudaMemsetAsync on its stream, and the kernel leaves it at zero
//   [128, 152)  the log-weight summary (max, sum, sum of squares)
//   [256, ...)  per-block summary partials, then the scan's tile sums
// Nothing else needs to start at zero: every word is written before it is read.
//
// One array per device means calls that overlap in time on the same device
// (different streams, or host threads) race on it and corrupt each other's
// results; callers serialise them.
#include <cuda.h>

#include <mutex>

#include "issm_device.cuh"
#include "issm_internal.h"
#include "scan.cuh"

namespace issm {

constexpr int64_t kStaticCdfMaxN = (int64_t)1 << 27;    // 134,217,728 log weights
constexpr size_t kStaticCdfScratchBytes = 270336;        // 264 KiB

// the reduce.cu layout at the largest accepted size must fit
static_assert(256 + sizeof(double) * (size_t)((kStaticCdfMaxN + kScanTile - 1) / kScanTile + 1) <=
                  kStaticCdfScratchBytes,
              "scan tile sums of the largest accepted input exceed the static scratch");
static_assert(256 + 3 * sizeof(double) * (size_t)(kSMs * 8) <= kStaticCdfScratchBytes,
              "summary partials exceed the static scratch");

static __device__ __align__(256) unsigned char g_cdf_scratch[kStaticCdfScratchBytes];

// The array's address belongs to a CUDA context, not to a device: a device
// reset (cudaDeviceReset) destroys the primary context and the next one maps
// the module elsewhere, and a host that creates its own contexts (CUDA.jl can)
// has several per device. Addresses are therefore cached by the unique id of
// the context current at the call (cuCtxGetId; ids are never reused within a
// process), and a context seen for the first time is looked up afresh.
constexpr int kMaxContexts = 64;
static unsigned long long g_ctx_id[kMaxContexts];
static void *g_scratch_address[kMaxContexts];
static int g_contexts = 0;
static std::mutex g_scratch_mutex;

static int driver_status(CUresult r) { return r == CUDA_SUCCESS ? ISSM_OK : (int)cudaErrorUnknown; }

// The two driver calls are resolved through the runtime (the library does not
// link libcuda, so it still loads on a machine without a driver).
typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long *);
static CtxGetCurrentFn g_ctx_get_current = nullptr;
static CtxGetIdFn g_ctx_get_id = nullptr;

static int resolve_driver_calls() {
    if (g_ctx_get_current && g_ctx_get_id) return ISSM_OK;
    void *a = nullptr, *b = nullptr;
    cudaDriverEntryPointQueryResult qa = cudaDriverEntryPointSymbolNotFound, qb = cudaDriverEntryPointSymbolNotFound;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa);
    if (e != cudaSuccess) return (int)e;
    e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb);
    if (e != cudaSuccess) return (int)e;
    if (qa != cudaDriverEntryPointSuccess || qb != cudaDriverEntryPointSuccess || !a || !b)
        return (int)cudaErrorSymbolNotFound;
    g_ctx_get_current = (CtxGetCurrentFn)a;
    g_ctx_get_id = (CtxGetIdFn)b;
    return ISSM_OK;
}

// Device address of g_cdf_scratch in the current context. The first call in a
// context makes that context current if the runtime had not yet done so, may
// load the module, and looks the symbol up.
static int scratch_address(void **out) {
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    int st = resolve_driver_calls();
    if (st) return st;
    CUcontext ctx = nullptr;
    st = driver_status(g_ctx_get_current(&ctx));
    if (st) return st;
    void *fresh = nullptr;
    if (!ctx) {  // no context yet: the runtime creates the device's primary context
        cudaError_t e = cudaGetSymbolAddress(&fresh, g_cdf_scratch);
        if (e != cudaSuccess) return (int)e;
        st = driver_status(g_ctx_get_current(&ctx));
        if (st) return st;
        if (!ctx) return (int)cudaErrorNoDevice;
    }
    unsigned long long id = 0;
    st = driver_status(g_ctx_get_id(ctx, &id));
    if (st) return st;
    for (int i = 0; i < g_contexts; ++i) {
        if (g_ctx_id[i] == id) {
            *out = g_scratch_address[i];
            return ISSM_OK;
        }
    }
    if (!fresh) {
        cudaError_t e = cudaGetSymbolAddress(&fresh, g_cdf_scratch);
        if (e != cudaSuccess) return (int)e;
    }
    if (g_contexts < kMaxContexts) {  // beyond the table the lookup simply repeats every call
        g_ctx_id[g_contexts] = id;
        g_scratch_address[g_contexts] = fresh;
        ++g_contexts;
    }
    *out = fresh;
    return ISSM_OK;
}

}  // namespace issm

extern "C" int64_t issm_resampling_cdf_static_max(void) { return issm::kStaticCdfMaxN; }

extern "C" int issm_resampling_cdf_static(const void *logweights, int64_t n, int32_t dtype, void *cdf,
                                          issm_stream_t stream) {
    if (n < 1) return ISSM_E_SIZE;
    if (n > issm::kStaticCdfMaxN) return ISSM_E_SCRATCH_LIMIT;
    if (!logweights || !cdf) return ISSM_E_NULL;
    if (dtype != ISSM_F32 && dtype != ISSM_F64) return ISSM_E_DTYPE;
    void *ws = nullptr;
    const int st = issm::scratch_address(&ws);
    if (st) return st;
    return issm::resampling_cdf(logweights, n, dtype, cdf, ws, issm::kStaticCdfScratchBytes,
                                (cudaStream_t)stream);
}
