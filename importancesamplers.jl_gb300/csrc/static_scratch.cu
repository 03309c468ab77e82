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

constexpr int kMaxDevices = 64;
static void *g_scratch_address[kMaxDevices];
static std::mutex g_scratch_mutex;

// Device address of g_cdf_scratch on the current device, looked up once per
// device (the first lookup may load the module on that device).
static int scratch_address(void **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return (int)e;
    if (dev < 0 || dev >= kMaxDevices) return ISSM_E_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_address[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_cdf_scratch);
        if (e != cudaSuccess) return (int)e;
        g_scratch_address[dev] = p;
    }
    *out = g_scratch_address[dev];
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
