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

__global__ void normals_f64_kernel(uint64_t seed, uint64_t offset, int64_t n, double *out) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint64_t e = offset + (uint64_t)i;
        const uint4 o = philox4x32_10(e >> 1, seed);
        const uint64_t b1 = ((uint64_t)o.y << 32) | o.x, b2 = ((uint64_t)o.w << 32) | o.z;
        const double u1 = ((double)(b1 >> 11) + 1.0) * 0x1.0p-53;
        const double u2 = (double)(b2 >> 11) * 0x1.0p-53;
        const double r = sqrt(-2.0 * log(u1));
        double s, c;
        sincospi(2.0 * u2, &s, &c);
        out[i] = (e & 1) ? r * s : r * c;
    }
}

__global__ void normals_f32_kernel(uint64_t seed, uint64_t offset, int64_t n, float *out) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint64_t e = offset + (uint64_t)i;
        const uint4 o = philox4x32_10(e >> 2, seed);
        const int lane = (int)(e & 3);
        const uint32_t a = lane < 2 ? o.x : o.z, b = lane < 2 ? o.y : o.w;
        const float u1 = ((float)(a >> 8) + 1.0f) * 0x1.0p-24f;
        const float u2 = (float)(b >> 8) * 0x1.0p-24f;
        const float r = sqrtf(-2.0f * logf(u1));
        float s, c;
        sincospif(2.0f * u2, &s, &c);
        out[i] = (lane & 1) ? r * s : r * c;
    }
}

__global__ void uniforms_f64_kernel(uint64_t seed, uint64_t offset, int64_t n, double *out) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint64_t e = offset + (uint64_t)i;
        const uint4 o = philox4x32_10(e >> 1, seed);
        const uint64_t bits = (e & 1) ? (((uint64_t)o.w << 32) | o.z) : (((uint64_t)o.y << 32) | o.x);
        out[i] = (double)(bits >> 11) * 0x1.0p-53;
    }
}

__global__ void uniforms_f32_kernel(uint64_t seed, uint64_t offset, int64_t n, float *out) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint64_t e = offset + (uint64_t)i;
        const uint4 o = philox4x32_10(e >> 2, seed);
        const int lane = (int)(e & 3);
        const uint32_t v = lane == 0 ? o.x : lane == 1 ? o.y : lane == 2 ? o.z : o.w;
        out[i] = (float)(v >> 8) * 0x1.0p-24f;
    }
}

int fill_normals(uint64_t seed, uint64_t offset, int64_t n, void *out, int dtype, cudaStream_t stream) {
    if (n <= 0) return 0;
    const int blocks = grid_for(n, 256, 8);
    if (dtype == ISSM_F32) { normals_f32_kernel<<<blocks, 256, 0, stream>>>(seed, offset, n, (float *)out); note_launch(); }
    else { normals_f64_kernel<<<blocks, 256, 0, stream>>>(seed, offset, n, (double *)out); note_launch(); }
    return (int)cudaGetLastError();
}

int fill_uniforms(uint64_t seed, uint64_t offset, int64_t n, void *out, int dtype, cudaStream_t stream) {
    if (n <= 0) return 0;
    const int blocks = grid_for(n, 256, 8);
    if (dtype == ISSM_F32) { uniforms_f32_kernel<<<blocks, 256, 0, stream>>>(seed, offset, n, (float *)out); note_launch(); }
    else { uniforms_f64_kernel<<<blocks, 256, 0, stream>>>(seed, offset, n, (double *)out); note_launch(); }
    return (int)cudaGetLastError();
}

}  // namespace issm
