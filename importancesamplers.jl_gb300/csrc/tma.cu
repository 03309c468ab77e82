// tma.cu — host side of the tensor copies that stage sample tiles: the tensor
// map of an n x d FP32 sample array (row-major, sample i contiguous) with
// 32-float x 128-row boxes, 128-byte swizzle and zero fill beyond the last
// row. cuTensorMapEncodeTiled is a driver call; it is resolved through the
// runtime so the library does not link libcuda.
#include <mutex>

#include "issm_device.cuh"
#include "issm_internal.h"

namespace issm {

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
    static std::mutex mu;
    static EncodeTiledFn fn = nullptr;
    std::lock_guard<std::mutex> lock(mu);
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
    }
    return fn;
}

bool row_tiles_supported(const void *x, int d, int64_t n) {
    return (d == 32 || d == 64) && n >= 1 && n < (int64_t)1 << 31 && ((reinterpret_cast<uintptr_t>(x) & 15) == 0);
}

int encode_row_tiles(CUtensorMap *map, const void *x, int d, int64_t n) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return ISSM_E_UNSUPPORTED;
    const cuuint64_t dims[2] = {(cuuint64_t)d, (cuuint64_t)n};
    const cuuint64_t strides[1] = {(cuuint64_t)d * 4};
    const cuuint32_t box[2] = {32, 128};
    const cuuint32_t elem[2] = {1, 1};
    const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void *>(x), dims, strides, box, elem,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? ISSM_OK : ISSM_E_UNSUPPORTED;
}

}  // namespace issm
