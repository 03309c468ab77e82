// tc_selftest.cu — a one-CTA tcgen05 GEMM, C[128 x n] = A[128 x k] B[n x k]^T,
// used by the test suite to pin the descriptor encodings (tcgen05.cuh) that
// every tensor-core kernel of this library relies on. Inputs are FP32 and are
// rounded to bf16 or tf32 while staged into shared memory.
#include "issm_device.cuh"
#include "issm_internal.h"
#include "tcgen05.cuh"

namespace issm {

// layout 0: K-major, core matrices K-group-major within 8-row groups (tc::kmajor_offset);
// layout 1: K-major, row-contiguous per K group (tc::rowgroup_offset);
// layout 2: MN-major (bf16 only): for each group of 8 rows (M or N) the K
// elements are stored consecutively, 16 bytes (8 rows) each (tc::mn_offset);
// the leading byte offset is the K-group stride (128 bytes) and the stride
// byte offset the row-group stride, as for the K-major layouts.
__global__ void __launch_bounds__(128) tc_gemm_selftest_kernel(const float *__restrict__ A, const float *__restrict__ B,
                                                               float *__restrict__ C, int n, int k, int kind,
                                                               int layout, int *status) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tmem_base;
    const int eb = kind == tc::kBF16 ? 2 : 4;
    const int kg = k * eb / 16;
    unsigned char *sa = smem;
    unsigned char *sb = smem + (size_t)128 * k * eb;
    const uint32_t ncols = n <= 32 ? 32 : n <= 64 ? 64 : n <= 128 ? 128 : 256;
    if (threadIdx.x < 32) tc::tmem_alloc(&tmem_base, ncols);
    if (threadIdx.x == 0) {
        tc::mbar_init(&bar, 1);
        tc::fence_mbar_init();
    }
    for (int e = threadIdx.x; e < 128 * k; e += blockDim.x) {
        const int r = e / k, c = e % k;
        const uint32_t off = layout >= 2 ? tc::mn_offset(r, c, k) : layout ? tc::rowgroup_offset(r, c, 128, eb)
                                                                          : tc::kmajor_offset(r, c, kg, eb);
        if (eb == 2) *reinterpret_cast<uint16_t *>(sa + off) = tc::bf16_bits(A[e]);
        else *reinterpret_cast<float *>(sa + off) = A[e];
    }
    for (int e = threadIdx.x; e < n * k; e += blockDim.x) {
        const int r = e / k, c = e % k;
        const uint32_t off = layout >= 2 ? tc::mn_offset(r, c, k) : layout ? tc::rowgroup_offset(r, c, n, eb)
                                                                          : tc::kmajor_offset(r, c, kg, eb);
        if (eb == 2) *reinterpret_cast<uint16_t *>(sb + off) = tc::bf16_bits(B[e]);
        else *reinterpret_cast<float *>(sb + off) = B[e];
    }
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = tmem_base;
    if (threadIdx.x == 0) {
        const uint32_t idesc = tc::instr_desc(kind, 128, n) | (layout >= 2 ? tc::kMajorMN : 0u);
        const int steps = k * eb / 32;
        for (int s = 0; s < steps; ++s) {
            uint64_t da, db;
            if (layout >= 2) {
                // one K slice (16 bf16) = two 8-element K groups of 128 bytes
                da = tc::smem_desc(tc::smem_u32(sa) + s * 256, 128, (uint32_t)k * 16);
                db = tc::smem_desc(tc::smem_u32(sb) + s * 256, 128, (uint32_t)k * 16);
            } else if (layout == 1) {
                da = tc::smem_desc(tc::smem_u32(sa) + s * 2 * 128 * 16, 128 * 16, 128);
                db = tc::smem_desc(tc::smem_u32(sb) + s * 2 * n * 16, n * 16, 128);
            } else {
                da = tc::smem_desc(tc::smem_u32(sa) + s * 256, 128, kg * 128);
                db = tc::smem_desc(tc::smem_u32(sb) + s * 256, 128, kg * 128);
            }
            if (kind == tc::kBF16) tc::mma(tbase, da, db, idesc, s > 0);
            else tc::mma_tf32(tbase, da, db, idesc, s > 0);
        }
        tc::commit(&bar);
    }
    const bool ok = tc::mbar_wait(&bar, 0);
    if (!ok && threadIdx.x == 0) atomicExch(status, 1);
    tc::fence_after_sync();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (ok) {
        for (int c0 = 0; c0 < n; c0 += 16) {
            float v[16];
            tc::tmem_ld16(tbase + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, v);
            const int row = 32 * warp + lane;
#pragma unroll
            for (int j = 0; j < 16; ++j) C[(size_t)row * n + c0 + j] = v[j];
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (threadIdx.x < 32) tc::tmem_dealloc(tbase, ncols);
}

int tc_gemm_selftest(const float *a, const float *b, float *c, int n, int k, int kind, int *status,
                     cudaStream_t stream) {
    const int layout = (kind >> 8) & 3;
    if (layout == 3) return ISSM_E_KIND;
    kind &= 0xff;
    const int eb = kind == tc::kBF16 ? 2 : 4;
    const size_t smem = (size_t)(128 + n) * k * eb;
    auto kern = tc_gemm_selftest_kernel;
    if (smem > 48 * 1024) {
        const int e = allow_dynamic_smem((const void *)kern);
        if (e) return e;
    }
    { kern<<<1, 128, smem, stream>>>(a, b, c, n, k, kind, layout, status); note_launch(); }
    return (int)cudaGetLastError();
}

}  // namespace issm
