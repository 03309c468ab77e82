// trinv.cuh — FP32 inverse of a lower-triangular factor in shared memory,
// shared by the factor inversion and the moment-fit kernels.
#pragma once

#include <cuda_runtime.h>

namespace issm {

// W = L^-1 for d <= 64, both row-major in shared memory with leading dimension
// ld: the 8 x 8 diagonal blocks are inverted one column per thread, then block
// row i (i = 1..) is W_ij = -W_ii sum_{k=j..i-1} L_ik W_kj, four threads per
// column splitting the k-sum. Needs every thread of the block.
__device__ __forceinline__ void invert_lower_f32(const float *L, float *W, int d, int ld) {
    const int nb = (d + 7) >> 3;
    for (int e = threadIdx.x; e < d * ld; e += blockDim.x) W[e] = 0.f;
    __syncthreads();
    for (int t = threadIdx.x; t < nb * 8; t += blockDim.x) {
        const int b = t >> 3, c = t & 7, col = 8 * b + c, r0 = 8 * b;
        if (col >= d) continue;
        float w[8];
#pragma unroll
        for (int r = 0; r < 8; ++r) {
            const int row = r0 + r;
            float v = 0.f;
            if (row < d && r >= c) {
                v = (r == c) ? 1.f : 0.f;
#pragma unroll
                for (int q = 0; q < r; ++q)
                    if (q >= c) v -= L[row * ld + r0 + q] * w[q];
                v /= L[row * ld + row];
            }
            w[r] = v;
        }
#pragma unroll
        for (int r = 0; r < 8; ++r)
            if (r0 + r < d) W[(r0 + r) * ld + col] = w[r];
    }
    __syncthreads();
    for (int i = 1; i < nb; ++i) {
        const int r0 = 8 * i;
        const int t = threadIdx.x, col = t >> 2, part = t & 3;
        // all four threads of a column sit in one warp; columns beyond the block row idle
        const bool act = col < r0 && col < d;
        float T[8];
#pragma unroll
        for (int s = 0; s < 8; ++s) T[s] = 0.f;
        if (act) {
            const int jb = col & ~7;
            for (int k = jb + part; k < r0; k += 4) {
                const float wk = W[k * ld + col];
#pragma unroll
                for (int s = 0; s < 8; ++s)
                    if (r0 + s < d) T[s] = fmaf(L[(r0 + s) * ld + k], wk, T[s]);
            }
        }
        if (t < 256) {
#pragma unroll
            for (int s = 0; s < 8; ++s) {
                T[s] += __shfl_xor_sync(0xffffffffu, T[s], 1);
                T[s] += __shfl_xor_sync(0xffffffffu, T[s], 2);
            }
        }
        if (act) {
#pragma unroll
            for (int rr = 0; rr < 2; ++rr) {
                const int r = 2 * part + rr, row = r0 + r;
                if (row < d) {
                    float v = 0.f;
#pragma unroll
                    for (int s = 0; s < 8; ++s)
                        if (s <= r) v = fmaf(W[row * ld + r0 + s], T[s], v);
                    W[row * ld + col] = -v;
                }
            }
        }
        __syncthreads();
    }
}

}  // namespace issm
