// moments_tc.cu — tensor-core form of the weighted moments that drive AMIS /
// N-PMC adaptation (_weighted_moments!, src/adaptive_gaussian_execution.jl:268-273).
//
// One streaming pass over the retained samples. For a tile of 128 samples the
// operand A is 128 rows x 128 samples: rows 0..d-1 hold sqrt(w) (x - c)
// (c = previous proposal mean), row 64 holds sqrt(w), with the samples along
// K; A A^T then holds S2 = sum w z z^T (rows/cols 0..63), S1 = sum w z
// (row 64) and S0 = sum w (D[64][64]). A is split A = Ah + Al in bf16 and
// A A^T ~ Ah Ah^T + X + X^T with X = Al Ah^T, so two accumulators in tensor
// memory (H += Ah Ah^T + Al Al^T, X += Al Ah^T) give the four products with
// three MMAs per K slice; the transpose of X is added when the sums are
// finished. With Al Al^T included, S = (Ah + Al)(Ah + Al)^T is the Gram matrix
// of the split operand, positive semidefinite up to FP32 accumulation, so the
// covariance of a low-ESS sample stays semidefinite (the regularising ridge
// then keeps the fit positive definite).
//
// A is stored MN-major: each sample's 8-coordinate groups are 16-byte chunks,
// so a thread converts its own sample row straight from the staged tile. Warp
// roles: warp 0 issues the MMAs; warps 1..8 stage tiles with cp.async into a
// three-deep ring of padded stages and build A (double-buffered), handing
// buffers over through mbarriers. Per-CTA partials are summed across CTAs
// (compensated FP32, FP64 across lanes) and mean = c + S1/S0,
// cov = S2/S0 - (S1/S0)(S1/S0)^T in FP64.
#include "issm_device.cuh"
#include "issm_internal.h"
#include "tcgen05.cuh"

namespace issm {

constexpr int kMtConvWarps = 8;
constexpr int kMtConvThreads = 32 * kMtConvWarps;
constexpr int kMtThreads = 32 * (1 + kMtConvWarps);
constexpr int kMtTile = 128;   // samples per tile = MMA K extent per tile
constexpr int kMtCols = 80;    // MMA N (64 coordinates + sqrt(w) + padding)
constexpr int kMtStages = 3;   // staged sample tiles in flight
constexpr int kMtRS = 68;      // padded row of a staged tile (floats)
constexpr int kMtRawBytes = kMtTile * kMtRS * 4 + kMtTile * 4;  // rows, then the tile's log weights
// Rows 0..71 (9 row groups: 64 coordinates, sqrt(w), zeros) are stored; the
// MMA's M = 128 also reads row groups 9..15, which land in the next buffer or
// the staged tiles after A: those D rows and the matching columns >= 72 are
// never read, so their content does not matter.
constexpr int kMtGroups = 9;
constexpr int kMtPart = kMtGroups * kMtTile * 16;
constexpr size_t kMtSmem = (size_t)2 * 2 * kMtPart + (size_t)kMtStages * kMtRawBytes + 256;
static_assert((size_t)3 * kMtPart + (size_t)16 * kMtTile * 16 <= kMtSmem, "M = 128 reads stay inside the CTA's shared memory");
constexpr int kMtPartial = 2 * 65 * kMtCols;  // H and X sums of one CTA

__global__ void __launch_bounds__(kMtThreads, 1) moments_tc_kernel(const float *__restrict__ x, int d, int64_t n,
                                                                    const float *__restrict__ lw,
                                                                    const double *__restrict__ summary,
                                                                    const double *__restrict__ center,
                                                                    float *__restrict__ partial, int *error,
                                                                    const int *__restrict__ gate) {
    if (gate != nullptr && *gate == 0) return;  // refinement pass not needed
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *s_a = smem;                                    // [buf][part] x kMtPart
    unsigned char *s_raw = smem + (size_t)2 * 2 * kMtPart;
    float *s_c = reinterpret_cast<float *>(s_raw + (size_t)kMtStages * kMtRawBytes);
    __shared__ __align__(8) uint64_t a_full[2], a_empty[2];
    __shared__ uint32_t tmem_base;
    __shared__ volatile int abort_flag;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (warp == 0) tc::tmem_alloc(&tmem_base, 256);
    if (tid == 0) {
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(&a_full[b], kMtConvWarps);
            tc::mbar_init(&a_empty[b], 1);
        }
        tc::fence_mbar_init();
        abort_flag = 0;
    }
    for (int c = tid; c < 64; c += kMtThreads) s_c[c] = c < d ? (float)center[c] : 0.f;
    const float m = (float)summary[0];
    const float inv_sqrt_s = (float)(1.0 / sqrt(summary[1]));
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = tmem_base;  // H at columns 0..79, X at 128..207
    const int64_t ntiles = (n + kMtTile - 1) / kMtTile;
    const int my_tiles = (int)((ntiles - (int64_t)blockIdx.x + gridDim.x - 1) / gridDim.x);
    auto tile_of = [&](int it) -> int64_t { return (int64_t)blockIdx.x + (int64_t)it * gridDim.x; };
    auto wait = [&](uint64_t *bar, uint32_t parity) -> bool {
        if (abort_flag) return false;
        if (tc::mbar_wait(bar, parity)) return true;
        atomicExch(error, 1);
        abort_flag = 1;
        return false;
    };

    if (warp == 0) {
        // ---- issuer: H += Ah Ah^T + Al Al^T, X += Al Ah^T per K slice ----
        const uint32_t idesc = tc::instr_desc(tc::kBF16, 128, kMtCols) | tc::kMajorMN;
        constexpr uint32_t LBO = 128, SBO = kMtTile * 16;  // K-group stride, row-group stride
        for (int it = 0; it < my_tiles; ++it) {
            const int buf = it & 1;
            if (lane == 0) {
                const bool ok = wait(&a_full[buf], (uint32_t)((it >> 1) & 1));
                tc::fence_after_sync();
                if (ok) {
                    const uint32_t a0 = tc::smem_u32(s_a + (size_t)buf * 2 * kMtPart), a1 = a0 + kMtPart;
#pragma unroll
                    for (int s = 0; s < kMtTile / 16; ++s) {
                        const uint64_t dh = tc::smem_desc(a0 + s * 256, LBO, SBO);
                        const uint64_t dl = tc::smem_desc(a1 + s * 256, LBO, SBO);
                        tc::mma(tbase, dh, dh, idesc, it > 0 || s > 0);
                        tc::mma(tbase + 128, dl, dh, idesc, it > 0 || s > 0);
                        tc::mma(tbase, dl, dl, idesc, true);
                    }
                }
                tc::commit(&a_empty[buf]);
            }
            __syncwarp();
        }
    } else {
        // ---- converters: stage tiles and build A = sqrt(w) (x - c) ----
        const int ctid = tid - 32;
        const bool vec = (d % 4 == 0) && ((reinterpret_cast<uintptr_t>(x) & 15) == 0) &&
                         ((reinterpret_cast<uintptr_t>(lw) & 15) == 0);
        auto issue_raw = [&](int it) {
            if (it < my_tiles) {
                const int64_t row0 = tile_of(it) * kMtTile;
                const int rows = (int)min((int64_t)kMtTile, n - row0);
                float *dst = reinterpret_cast<float *>(s_raw + (size_t)(it % kMtStages) * kMtRawBytes);
                float *dlw = dst + kMtTile * kMtRS;
                const float *src = x + row0 * d;
                if (vec && d == 64) {
                    const int total = rows * 16;
                    for (int e = ctid; e < total; e += kMtConvThreads)
                        tc::cp_async16(dst + (e >> 4) * kMtRS + (e & 15) * 4, src + (size_t)e * 4);
                    if (rows == kMtTile) {
                        if (ctid < kMtTile / 4) tc::cp_async16(dlw + ctid * 4, lw + row0 + ctid * 4);
                    } else {
                        for (int r = ctid; r < rows; r += kMtConvThreads) tc::cp_async4(dlw + r, lw + row0 + r);
                    }
                } else if (vec) {
                    const int q4 = d >> 2, total = rows * q4;
                    for (int e = ctid; e < total; e += kMtConvThreads) {
                        const int r = e / q4, c4 = e - r * q4;
                        tc::cp_async16(dst + r * kMtRS + c4 * 4, src + (size_t)e * 4);
                    }
                    if (rows == kMtTile) {
                        if (ctid < kMtTile / 4) tc::cp_async16(dlw + ctid * 4, lw + row0 + ctid * 4);
                    } else {
                        for (int r = ctid; r < rows; r += kMtConvThreads) tc::cp_async4(dlw + r, lw + row0 + r);
                    }
                } else {
                    for (int e = ctid; e < rows * d; e += kMtConvThreads) {
                        const int r = e / d, c = e - r * d;
                        tc::cp_async4(dst + r * kMtRS + c, src + (size_t)r * d + c);
                    }
                    for (int r = ctid; r < rows; r += kMtConvThreads) tc::cp_async4(dlw + r, lw + row0 + r);
                }
            }
            tc::cp_async_commit();
        };
        for (int s = 0; s < kMtStages; ++s) issue_raw(s);
        const int k = ctid & (kMtTile - 1), half = ctid >> 7;
        for (int it = 0; it < my_tiles; ++it) {
            const int buf = it & 1;
            tc::cp_async_wait<kMtStages - 1>();
            tc::named_sync(1, kMtConvThreads);
            bool ok = true;
            if (it >= 2) {
                if (lane == 0) ok = wait(&a_empty[buf], (uint32_t)(((it - 2) >> 1) & 1));
                ok = __shfl_sync(0xffffffffu, (int)ok, 0) != 0;
            }
            if (ok) {
                const float *raw = reinterpret_cast<const float *>(s_raw + (size_t)(it % kMtStages) * kMtRawBytes);
                unsigned char *ah = s_a + (size_t)buf * 2 * kMtPart;
                unsigned char *al = ah + kMtPart;
                const int64_t i = tile_of(it) * kMtTile + k;
                const bool active = i < n;
                const float l = active ? raw[kMtTile * kMtRS + k] : -INFINITY;
                const float sw = l == -INFINITY ? 0.f : expf(0.5f * (l - m)) * inv_sqrt_s;
                const bool full = active && d == 64;
#pragma unroll
                for (int gg = 0; gg < 4; ++gg) {
                    const int g = half * 4 + gg, c = g * 8;
                    float v[8];
                    const float4 c0 = *reinterpret_cast<const float4 *>(s_c + c),
                                 c1 = *reinterpret_cast<const float4 *>(s_c + c + 4);
                    if (full) {
                        const float4 f0 = *reinterpret_cast<const float4 *>(raw + k * kMtRS + c);
                        const float4 f1 = *reinterpret_cast<const float4 *>(raw + k * kMtRS + c + 4);
                        v[0] = sw * (f0.x - c0.x);
                        v[1] = sw * (f0.y - c0.y);
                        v[2] = sw * (f0.z - c0.z);
                        v[3] = sw * (f0.w - c0.w);
                        v[4] = sw * (f1.x - c1.x);
                        v[5] = sw * (f1.y - c1.y);
                        v[6] = sw * (f1.z - c1.z);
                        v[7] = sw * (f1.w - c1.w);
                    } else {
                        float4 f0 = make_float4(0.f, 0.f, 0.f, 0.f), f1 = f0;
                        if (active) {
                            f0 = *reinterpret_cast<const float4 *>(raw + k * kMtRS + c);
                            f1 = *reinterpret_cast<const float4 *>(raw + k * kMtRS + c + 4);
                        }
                        v[0] = (active && c < d) ? sw * (f0.x - c0.x) : 0.f;
                        v[1] = (active && c + 1 < d) ? sw * (f0.y - c0.y) : 0.f;
                        v[2] = (active && c + 2 < d) ? sw * (f0.z - c0.z) : 0.f;
                        v[3] = (active && c + 3 < d) ? sw * (f0.w - c0.w) : 0.f;
                        v[4] = (active && c + 4 < d) ? sw * (f1.x - c1.x) : 0.f;
                        v[5] = (active && c + 5 < d) ? sw * (f1.y - c1.y) : 0.f;
                        v[6] = (active && c + 6 < d) ? sw * (f1.z - c1.z) : 0.f;
                        v[7] = (active && c + 7 < d) ? sw * (f1.w - c1.w) : 0.f;
                    }
                    const uint4 hi = make_uint4(tc::pack_bf16x2(v[0], v[1]), tc::pack_bf16x2(v[2], v[3]),
                                                tc::pack_bf16x2(v[4], v[5]), tc::pack_bf16x2(v[6], v[7]));
                    auto lo2 = [](float a, float b, uint32_t h) {
                        return tc::pack_bf16x2(a - __uint_as_float(h << 16), b - __uint_as_float(h & 0xffff0000u));
                    };
                    const uint4 lo = make_uint4(lo2(v[0], v[1], hi.x), lo2(v[2], v[3], hi.y), lo2(v[4], v[5], hi.z),
                                                lo2(v[6], v[7], hi.w));
                    *reinterpret_cast<uint4 *>(ah + (size_t)g * kMtTile * 16 + k * 16) = hi;
                    *reinterpret_cast<uint4 *>(al + (size_t)g * kMtTile * 16 + k * 16) = lo;
                }
                if (half == 1) {
                    // row group 8: sqrt(w) in row 64
                    const uint32_t h = tc::pack_bf16x2(sw, 0.f);
                    const uint32_t lo = tc::pack_bf16x2(sw - __uint_as_float(h << 16), 0.f);
                    *reinterpret_cast<uint4 *>(ah + (size_t)8 * kMtTile * 16 + k * 16) = make_uint4(h, 0u, 0u, 0u);
                    *reinterpret_cast<uint4 *>(al + (size_t)8 * kMtTile * 16 + k * 16) = make_uint4(lo, 0u, 0u, 0u);
                }
            }
            tc::fence_proxy_async();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&a_full[buf]);
            tc::named_sync(1, kMtConvThreads);  // the stage is consumed: refill it
            issue_raw(it + kMtStages);
        }
        tc::cp_async_wait_all();
    }
    // ---- the last commit tracks every MMA of the CTA ----
    tc::fence_before_sync();
    __syncthreads();
    if (my_tiles > 0) {
        const int last = my_tiles - 1;
        if (!tc::mbar_wait(&a_empty[last & 1], (uint32_t)((last >> 1) & 1)) && tid == 0) {
            atomicExch(error, 1);
            abort_flag = 1;
        }
    }
    __syncthreads();
    tc::fence_after_sync();
    float *out = partial + (size_t)blockIdx.x * kMtPartial;
    // warps 1..4 read TMEM lane quadrants 1, 2, 3, 0 (a warp reads quadrant warp % 4)
    if (!abort_flag && warp >= 1 && warp <= 4) {
        const int q = warp & 3, row = 32 * q + lane;
#pragma unroll
        for (int acc = 0; acc < 2; ++acc) {
#pragma unroll
            for (int c0 = 0; c0 < kMtCols; c0 += 16) {
                float v[16];
                if (my_tiles > 0) {
                    tc::tmem_ld16(tbase + ((uint32_t)(32 * q) << 16) + (uint32_t)(acc * 128 + c0), v);
                } else {
                    for (int j = 0; j < 16; ++j) v[j] = 0.f;
                }
                if (row <= 64) {
                    for (int j = 0; j < 16; ++j) out[acc * 65 * kMtCols + row * kMtCols + c0 + j] = v[j];
                }
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tbase, 256);
}

// Partials are [block][2][65][80] FP32 (H, X); stage 1 sums them over blocks
// (32 entries x 8 block-strided lanes per CTA, coalesced), stage 2 forms
// S = H + X + X^T and from it the mean and covariance.
__global__ void moments_tc_reduce_kernel(const float *__restrict__ partial, int blocks, double *__restrict__ sums,
                                         const int *__restrict__ gate) {
    if (gate != nullptr && *gate == 0) return;
    __shared__ double acc_s[8][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int e = blockIdx.x * 32 + tx;
    // compensated FP32 over this lane's blocks (no serial FP64 chain), FP64 across lanes
    float s = 0.f, cmp = 0.f;
    if (e < kMtPartial)
        for (int b = ty; b < blocks; b += 8) {
            const float y = partial[(size_t)b * kMtPartial + e] - cmp;
            const float t = s + y;
            cmp = (t - s) - y;
            s = t;
        }
    const double acc = (double)s - (double)cmp;
    acc_s[ty][tx] = acc;
    __syncthreads();
    if (ty == 0 && e < kMtPartial) {
        double t = 0.0;
        for (int r = 0; r < 8; ++r) t += acc_s[r][tx];
        sums[e] = t;
    }
}

// mean = c + S1/S0, cov = S2/S0 - (S1/S0)(S1/S0)^T with S = H + X + X^T (c as
// the FP32 value the pass subtracted; `center` and `mean` may be the same
// array, each entry read before it is written). When
// the new mean lies far from the centre c relative to the spread, S2/S0 and
// the mean's outer product nearly cancel and the bf16-split sums lose their
// accuracy: a diagonal variance below 2^-6 of its second moment about c (six
// bits or more cancelled) sets *refine, and a second pass centred at the new
// mean (gated on that flag) replaces the result.
__global__ void moments_tc_finish_kernel(const double *__restrict__ sums, int d, const double *center,
                                         double *mean, double *__restrict__ cov,
                                         const int *__restrict__ gate, int *__restrict__ refine) {
    if (gate != nullptr && *gate == 0) return;
    const double *H = sums, *X = sums + 65 * kMtCols;
    auto S = [&](int r, int c) { return H[r * kMtCols + c] + X[r * kMtCols + c] + X[c * kMtCols + r]; };
    const double inv = 1.0 / S(64, 64);
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < d * d; e += gridDim.x * blockDim.x) {
        const int r = e % d, c = e / d;
        const double mr = S(64, r) * inv, mc = S(64, c) * inv;
        const double s2 = S(r, c) * inv, v = s2 - mr * mc;
        cov[e] = v;
        if (refine != nullptr && r == c && !(v > s2 * 0.015625)) atomicExch(refine, 1);
    }
    // the mean last: the refinement pass reads this call's mean as its centre
    __syncthreads();
    if (blockIdx.x == 0)
        for (int j = threadIdx.x; j < d; j += blockDim.x) mean[j] = (double)(float)center[j] + S(64, j) * inv;
}

static int moments_tc_blocks(int64_t n) {
    const int64_t t = (n + kMtTile - 1) / kMtTile;
    return (int)(t < kSMs ? (t < 1 ? 1 : t) : kSMs);
}

size_t moments_tc_workspace_bytes(int64_t n) {
    (void)n;
    return sizeof(float) * (size_t)kSMs * kMtPartial + sizeof(double) * kMtPartial + 256;
}

int moments_tc(const void *x, int d, int64_t n, const void *lw, const double *summary, const double *shift,
               double *mean, double *cov, int precision, void *ws, size_t ws_bytes, int *error, cudaStream_t stream) {
    (void)precision;  // both tensor-core forms use the bf16 split contraction
    if (d > 64) return ISSM_E_UNSUPPORTED;
    if (ws_bytes < moments_tc_workspace_bytes(n)) return ISSM_E_WORKSPACE;
    const int blocks = moments_tc_blocks(n);
    float *partial = (float *)ws;
    const int e = allow_dynamic_smem((const void *)moments_tc_kernel);
    if (e) return e;
    double *sums = reinterpret_cast<double *>(partial + (size_t)kSMs * kMtPartial);
    int *refine = reinterpret_cast<int *>(sums + kMtPartial);
    cudaError_t ce = cudaMemsetAsync(refine, 0, sizeof(int), stream);
    if (ce != cudaSuccess) return (int)ce;
    // pass 1 about `shift`
    { moments_tc_kernel<<<blocks, kMtThreads, kMtSmem, stream>>>((const float *)x, d, n, (const float *)lw, summary,
                                                                shift, partial, error, nullptr); note_launch(); }
    { moments_tc_reduce_kernel<<<(kMtPartial + 31) / 32, 256, 0, stream>>>(partial, blocks, sums, nullptr);
      note_launch(); }
    { moments_tc_finish_kernel<<<1, 256, 0, stream>>>(sums, d, shift, mean, cov, nullptr, refine); note_launch(); }
    // pass 2 about the new mean, only when pass 1 cancelled too many bits (kernels exit on the flag)
    { moments_tc_kernel<<<blocks, kMtThreads, kMtSmem, stream>>>((const float *)x, d, n, (const float *)lw, summary,
                                                                mean, partial, error, refine); note_launch(); }
    { moments_tc_reduce_kernel<<<(kMtPartial + 31) / 32, 256, 0, stream>>>(partial, blocks, sums, refine);
      note_launch(); }
    { moments_tc_finish_kernel<<<1, 256, 0, stream>>>(sums, d, mean, mean, cov, refine, nullptr); note_launch(); }
    return (int)cudaGetLastError();
}

}  // namespace issm
