// rng.cuh — the counter-based streams' per-block arithmetic, shared by the
// fill kernels (rng.cu) and the fused-normal draw (mixture_simt.cu) so both
// produce bitwise the same values.
//
// Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC'11): element e of a stream depends only on
// (seed, offset + e). FP32 normal streams take four 24-bit uniforms per block
// (two Box-Muller pairs, elements 4b..4b+3); FP64 streams take two 53-bit
// uniforms per block (one pair, elements 2b, 2b+1).
#pragma once
#include <cstdint>

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

template <typename T> struct NormalBlock;

// elements 4 blk .. 4 blk + 3 of an FP32 normal stream
template <> struct NormalBlock<float> {
    static constexpr int kPer = 4;
    static constexpr int kShift = 2;
    __device__ __forceinline__ static void eval(uint64_t blk, uint64_t seed, float v[4]) {
        const uint4 o = philox4x32_10(blk, seed);
#pragma unroll
        for (int pair = 0; pair < 2; ++pair) {
            const uint32_t a = pair == 0 ? o.x : o.z, b = pair == 0 ? o.y : o.w;
            const float u1 = ((float)(a >> 8) + 1.0f) * 0x1.0p-24f;
            const float u2 = (float)(b >> 8) * 0x1.0p-24f;
            const float r = sqrtf(-2.0f * logf(u1));
            float sn, cs;
            sincospif(2.0f * u2, &sn, &cs);
            v[2 * pair] = r * cs;
            v[2 * pair + 1] = r * sn;
        }
    }
};

// elements 2 blk, 2 blk + 1 of an FP64 normal stream
template <> struct NormalBlock<double> {
    static constexpr int kPer = 2;
    static constexpr int kShift = 1;
    __device__ __forceinline__ static void eval(uint64_t blk, uint64_t seed, double v[2]) {
        const uint4 o = philox4x32_10(blk, seed);
        const uint64_t q1 = ((uint64_t)o.y << 32) | o.x, q2 = ((uint64_t)o.w << 32) | o.z;
        const double u1 = ((double)(q1 >> 11) + 1.0) * 0x1.0p-53;
        const double u2 = (double)(q2 >> 11) * 0x1.0p-53;
        const double r = sqrt(-2.0 * log(u1));
        double sn, cs;
        sincospi(2.0 * u2, &sn, &cs);
        v[0] = r * cs;
        v[1] = r * sn;
    }
};

}  // namespace issm
