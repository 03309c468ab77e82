// rng.cu — counter-based normal and uniform streams (Philox-4x32-10; the
// per-block arithmetic is in rng.cuh). Element e of a stream depends only on
// (seed, offset + e). Uniform streams: FP64 takes 53 bits of each 64-bit half
// of a block, FP32 24 bits of each 32-bit word.
#include "issm_device.cuh"
#include "issm_internal.h"
#include "rng.cuh"

namespace issm {

// Each thread evaluates one Philox block and writes every element of the
// requested range that the block covers (4 per block in FP32, 2 in FP64).
template <typename T>
__global__ void normals_kernel(uint64_t seed, const uint64_t *base, uint64_t offset, int64_t n, T *out) {
    using NB = NormalBlock<T>;
    if (base) offset += *base;
    const uint64_t b0 = offset >> NB::kShift, b1 = (offset + (uint64_t)n - 1) >> NB::kShift;
    const int64_t nb = (int64_t)(b1 - b0 + 1);
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < nb; j += stride) {
        const uint64_t blk = b0 + (uint64_t)j;
        T v[NB::kPer];
        NB::eval(blk, seed, v);
        const uint64_t e0 = blk << NB::kShift;
#pragma unroll
        for (int l = 0; l < NB::kPer; ++l) {
            const uint64_t e = e0 + l;
            if (e >= offset && e < offset + (uint64_t)n) out[e - offset] = v[l];
        }
    }
}

__global__ void uniforms_f64_kernel(uint64_t seed, const uint64_t *base, uint64_t offset, int64_t n, double *out) {
    if (base) offset += *base;
    const uint64_t b0 = offset >> 1, b1 = (offset + (uint64_t)n - 1) >> 1;
    const int64_t nb = (int64_t)(b1 - b0 + 1);
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < nb; j += stride) {
        const uint64_t blk = b0 + (uint64_t)j;
        const uint4 o = philox4x32_10(blk, seed);
        const uint64_t e0 = blk << 1;
        const uint64_t q0 = ((uint64_t)o.y << 32) | o.x, q1 = ((uint64_t)o.w << 32) | o.z;
        if (e0 >= offset && e0 < offset + (uint64_t)n) out[e0 - offset] = (double)(q0 >> 11) * 0x1.0p-53;
        if (e0 + 1 >= offset && e0 + 1 < offset + (uint64_t)n) out[e0 + 1 - offset] = (double)(q1 >> 11) * 0x1.0p-53;
    }
}

__global__ void uniforms_f32_kernel(uint64_t seed, const uint64_t *base, uint64_t offset, int64_t n, float *out) {
    if (base) offset += *base;
    const uint64_t b0 = offset >> 2, b1 = (offset + (uint64_t)n - 1) >> 2;
    const int64_t nb = (int64_t)(b1 - b0 + 1);
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < nb; j += stride) {
        const uint64_t blk = b0 + (uint64_t)j;
        const uint4 o = philox4x32_10(blk, seed);
        const uint64_t e0 = blk << 2;
        const uint32_t v[4] = {o.x, o.y, o.z, o.w};
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            const uint64_t e = e0 + l;
            if (e >= offset && e < offset + (uint64_t)n) out[e - offset] = (float)(v[l] >> 8) * 0x1.0p-24f;
        }
    }
}

int fill_normals(uint64_t seed, const uint64_t *base, uint64_t offset, int64_t n, void *out, int dtype,
                 cudaStream_t stream) {
    if (n <= 0) return 0;
    const int blocks = grid_for(n / (dtype == ISSM_F32 ? 4 : 2) + 2, 256, 8);
    if (dtype == ISSM_F32) { normals_kernel<float><<<blocks, 256, 0, stream>>>(seed, base, offset, n, (float *)out); note_launch(); }
    else { normals_kernel<double><<<blocks, 256, 0, stream>>>(seed, base, offset, n, (double *)out); note_launch(); }
    return (int)cudaGetLastError();
}

int fill_uniforms(uint64_t seed, const uint64_t *base, uint64_t offset, int64_t n, void *out, int dtype,
                  cudaStream_t stream) {
    if (n <= 0) return 0;
    const int blocks = grid_for(n / (dtype == ISSM_F32 ? 4 : 2) + 2, 256, 8);
    if (dtype == ISSM_F32) { uniforms_f32_kernel<<<blocks, 256, 0, stream>>>(seed, base, offset, n, (float *)out); note_launch(); }
    else { uniforms_f64_kernel<<<blocks, 256, 0, stream>>>(seed, base, offset, n, (double *)out); note_launch(); }
    return (int)cudaGetLastError();
}

__global__ void counter_advance_kernel(uint64_t *counter, uint64_t inc) { *counter += inc; }

int counter_advance(uint64_t *counter, uint64_t inc, cudaStream_t stream) {
    { counter_advance_kernel<<<1, 1, 0, stream>>>(counter, inc); note_launch(); }
    return (int)cudaGetLastError();
}

}  // namespace issm
