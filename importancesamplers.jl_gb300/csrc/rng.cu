// rng.cu — counter-based normal and uniform streams.
//
// Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC'11): element e of a stream depends only on
// (seed, offset + e). FP64 streams take two 53-bit uniforms per block and
// produce two normals by Box-Muller; FP32 streams take four 24-bit uniforms
// per block (two normal pairs).
#include "issm_device.cuh"
#include "issm_internal.h"

namespace issm {

__device__ __forceinline__ uint4 philox4x32_10(uint64_t counter, uint64_t seed) {
    uint32_t c0 = (uint32_t)counter, c1 = (uint32_t)(counter >> 32), c2 = 0u, c3 = 0u;
    uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t h0 = __umulhi(0xD2511F53u, c0), l0 = 0xD2511F53u * c0;
        const uint32_t h1 = __umulhi(0xCD9E8D57u, c2), l1 = 0xCD9E8D57u * c2;
        const uint32_t n0 = h1 ^ c1 ^ k0, n2 = h0 ^ c3 ^ k1;
        c0 = n0; c1 = l1; c2 = n2; c3 = l0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    return make_uint4(c0, c1, c2, c3);
}

// Each thread evaluates one Philox block and writes every element of the
// requested range that the block covers (4 per block in FP32, 2 in FP64).
__global__ void normals_f64_kernel(uint64_t seed, const uint64_t *base, uint64_t offset, int64_t n, double *out) {
    if (base) offset += *base;
    const uint64_t b0 = offset >> 1, b1 = (offset + (uint64_t)n - 1) >> 1;
    const int64_t nb = (int64_t)(b1 - b0 + 1);
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < nb; j += stride) {
        const uint64_t blk = b0 + (uint64_t)j;
        const uint4 o = philox4x32_10(blk, seed);
        const uint64_t q1 = ((uint64_t)o.y << 32) | o.x, q2 = ((uint64_t)o.w << 32) | o.z;
        const double u1 = ((double)(q1 >> 11) + 1.0) * 0x1.0p-53;
        const double u2 = (double)(q2 >> 11) * 0x1.0p-53;
        const double r = sqrt(-2.0 * log(u1));
        double sn, cs;
        sincospi(2.0 * u2, &sn, &cs);
        const uint64_t e0 = blk << 1;
        if (e0 >= offset && e0 < offset + (uint64_t)n) out[e0 - offset] = r * cs;
        if (e0 + 1 >= offset && e0 + 1 < offset + (uint64_t)n) out[e0 + 1 - offset] = r * sn;
    }
}

__global__ void normals_f32_kernel(uint64_t seed, const uint64_t *base, uint64_t offset, int64_t n, float *out) {
    if (base) offset += *base;
    const uint64_t b0 = offset >> 2, b1 = (offset + (uint64_t)n - 1) >> 2;
    const int64_t nb = (int64_t)(b1 - b0 + 1);
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < nb; j += stride) {
        const uint64_t blk = b0 + (uint64_t)j;
        const uint4 o = philox4x32_10(blk, seed);
        const uint64_t e0 = blk << 2;
#pragma unroll
        for (int pair = 0; pair < 2; ++pair) {
            const uint32_t a = pair == 0 ? o.x : o.z, b = pair == 0 ? o.y : o.w;
            const float u1 = ((float)(a >> 8) + 1.0f) * 0x1.0p-24f;
            const float u2 = (float)(b >> 8) * 0x1.0p-24f;
            const float r = sqrtf(-2.0f * logf(u1));
            float sn, cs;
            sincospif(2.0f * u2, &sn, &cs);
            const uint64_t e = e0 + 2 * pair;
            if (e >= offset && e < offset + (uint64_t)n) out[e - offset] = r * cs;
            if (e + 1 >= offset && e + 1 < offset + (uint64_t)n) out[e + 1 - offset] = r * sn;
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
    if (dtype == ISSM_F32) { normals_f32_kernel<<<blocks, 256, 0, stream>>>(seed, base, offset, n, (float *)out); note_launch(); }
    else { normals_f64_kernel<<<blocks, 256, 0, stream>>>(seed, base, offset, n, (double *)out); note_launch(); }
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
