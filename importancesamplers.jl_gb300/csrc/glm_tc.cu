// glm_tc.cu — the regression likelihoods of the batch targets (X beta over
// every observation for every sample; the user batch callback of
// src/batched_targets.jl:54-214, examples/batched_linear_regression.jl:18-37)
// as a tcgen05 GEMM with the log-likelihood reduced in the epilogue.
//
// For a tile of 128 samples (rows, M) and 256 observations (columns, N):
//   D[i, o] = beta_i . x_o         (K = d, padded to DP = 16 / 32 / 64)
// accumulates in tensor memory (FP32), and the epilogue turns each entry into
//   Bernoulli-logit: y_o eta - log(1 + e^eta)
//   Gaussian:        (y_o - eta)^2            (scaled by -1 / (2 sigma^2) at the end)
// summed over the observations in registers: the samples sit on the TMEM
// lanes, so a thread owns one sample and no cross-thread reduction is needed.
// The prior N(0, prior_var I) and the constants are added once per sample.
//
// Precision forms (FP32 accumulation in all):
//   BF16     one kind::f16 MMA per K slice on bf16-rounded operands;
//   BF16x3   operands split v = hi + lo in bf16, D = Bh Xh + Bl Xh + Bh Xl;
//   TF32     one kind::tf32 MMA per K slice, operands rounded to tf32.
//
// The observations' operand form (bf16 hi/lo or tf32, row-contiguous
// canonical K-major layout, 256 observations per tile, zero-padded) is built
// once per target by glm_prepare_kernel. glm_tc_kernel is one CTA per sample
// tile: the 8 epilogue warps first convert the tile's samples into the A
// operand; then warp 0 streams the observation tiles through a ring of bulk
// copies and issues each tile's MMAs into one of two TMEM accumulators while
// the epilogue warps (two per TMEM lane quadrant, 128 columns each) reduce
// the other. Every wait is bounded; a timeout sets the sticky error word.
#include "issm_device.cuh"
#include "issm_internal.h"
#include "tcgen05.cuh"

namespace issm {

constexpr int kGlmRows = 128;      // samples per CTA (MMA M)
constexpr int kGlmCols = 256;      // observations per tile (MMA N)
constexpr int kGlmEpiWarps = 8;    // two per TMEM lane quadrant
constexpr int kGlmThreads = 32 * (1 + kGlmEpiWarps);
constexpr size_t kGlmMaxSmem = 232448 - 1024;
constexpr double kGlmLog2Pi = 1.8378770664093454835606594728112;

template <int KIND> __device__ __forceinline__ uint4 glm_pack(const float *v) {
    if (KIND == tc::kTF32) return make_uint4(tc::tf32_rn(v[0]), tc::tf32_rn(v[1]), tc::tf32_rn(v[2]), tc::tf32_rn(v[3]));
    return make_uint4(tc::pack_bf16x2(v[0], v[1]), tc::pack_bf16x2(v[2], v[3]), tc::pack_bf16x2(v[4], v[5]),
                      tc::pack_bf16x2(v[6], v[7]));
}
__device__ __forceinline__ uint32_t glm_lo_pair(float a, float b, uint32_t hi) {
    return tc::pack_bf16x2(a - __uint_as_float(hi << 16), b - __uint_as_float(hi & 0xffff0000u));
}
__device__ __forceinline__ uint4 glm_pack_lo(const float *v, uint4 hi) {
    return make_uint4(glm_lo_pair(v[0], v[1], hi.x), glm_lo_pair(v[2], v[3], hi.y), glm_lo_pair(v[4], v[5], hi.z),
                      glm_lo_pair(v[6], v[7], hi.w));
}

template <int KIND, int SPLIT, int DP> struct GlmShape {
    static constexpr int EB = KIND == tc::kBF16 ? 2 : 4;
    static constexpr int PER = 16 / EB;          // elements per 16-byte K group
    static constexpr int KG = DP / PER;          // K groups
    static constexpr int NPART = SPLIT == 3 ? 2 : 1;
    static constexpr int KSTEPS = KG / 2;        // MMA K slices of 32 bytes
    static constexpr size_t A_PART = (size_t)KG * kGlmRows * 16;
    static constexpr size_t B_PART = (size_t)KG * kGlmCols * 16;
    static constexpr size_t TILE = NPART * B_PART;  // one observation tile of the operand form
};

// Operand form of the observations: tile t, part p, K group q, row j at
//   t * TILE + p * B_PART + q * 256 * 16 + j * 16.
template <int KIND, int SPLIT, int DP>
__global__ void __launch_bounds__(256) glm_prepare_kernel(const float *__restrict__ X, int nobs, int d, int tiles,
                                                          unsigned char *__restrict__ ops) {
    using S = GlmShape<KIND, SPLIT, DP>;
    const int64_t total = (int64_t)tiles * S::KG * kGlmCols;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int j = (int)(e % kGlmCols), q = (int)((e / kGlmCols) % S::KG), t = (int)(e / ((int64_t)kGlmCols * S::KG));
        const int o = t * kGlmCols + j;
        float v[S::PER];
#pragma unroll
        for (int m = 0; m < S::PER; ++m) {
            const int c = q * S::PER + m;
            v[m] = (o < nobs && c < d) ? X[o + (size_t)c * nobs] : 0.f;  // X column-major, nobs x d
        }
        unsigned char *base = ops + (size_t)t * S::TILE + (size_t)q * kGlmCols * 16 + (size_t)j * 16;
        const uint4 hi = glm_pack<KIND>(v);
        *reinterpret_cast<uint4 *>(base) = hi;
        if (S::NPART == 2) *reinterpret_cast<uint4 *>(base + S::B_PART) = glm_pack_lo(v, hi);
    }
}

struct GlmParams {
    int d, nobs, kind, tiles, ring;
    int64_t n;
    const float *x;              // samples, n x d
    const float *y;              // observations' responses, nobs
    const unsigned char *ops;    // operand form of X
    float *out;
    float sigma, prior_var;
    int *error;
};

template <int KIND, int SPLIT, int DP>
__global__ void __launch_bounds__(kGlmThreads, 1) glm_tc_kernel(GlmParams p) {
    using S = GlmShape<KIND, SPLIT, DP>;
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *s_a = smem;                                   // NPART x A_PART
    unsigned char *s_b = smem + (size_t)S::NPART * S::A_PART;    // ring x TILE
    __shared__ __align__(8) uint64_t a_full, b_full[4], b_empty[4], d_full[2], d_empty[2];
    __shared__ uint32_t tmem_base;
    __shared__ volatile int abort_flag;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int R = p.ring;
    if (warp == 0) tc::tmem_alloc(&tmem_base, 512);
    if (tid == 0) {
        tc::mbar_init(&a_full, kGlmEpiWarps);
        for (int b = 0; b < 4; ++b) {
            tc::mbar_init(&b_full[b], 1);
            tc::mbar_init(&b_empty[b], 1);
        }
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(&d_full[b], 1);
            tc::mbar_init(&d_empty[b], kGlmEpiWarps);
        }
        tc::fence_mbar_init();
        abort_flag = 0;
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = tmem_base;
    const int64_t row0 = (int64_t)blockIdx.x * kGlmRows;
    auto wait = [&](uint64_t *bar, uint32_t parity) -> bool {
        if (abort_flag) return false;
        if (tc::mbar_wait(bar, parity)) return true;
        atomicExch(p.error, 1);
        abort_flag = 1;
        return false;
    };
    const int T = p.tiles;

    if (warp == 0) {
        // ================= issuer: observation tiles in, MMAs out =================
        int issued = 0, waited = 0;
        auto load = [&](int t) {
            if (lane == 0) {
                unsigned char *dst = s_b + (size_t)(t % R) * S::TILE;
                tc::mbar_arrive_expect_tx(&b_full[t % R], (uint32_t)S::TILE);
                tc::bulk_copy_g2s(dst, p.ops + (size_t)t * S::TILE, (uint32_t)S::TILE, &b_full[t % R]);
            }
            __syncwarp();
            ++issued;
        };
        for (int t = 0; t < R && t < T; ++t) load(t);
        int ok = 1;
        if (lane == 0) ok = wait(&a_full, 0u);
        ok = __shfl_sync(0xffffffffu, ok, 0);
        const uint32_t idesc = tc::instr_desc(KIND, kGlmRows, kGlmCols);
        constexpr uint32_t LBO_A = kGlmRows * 16, LBO_B = kGlmCols * 16;
        for (int t = 0; t < T && ok; ++t) {
            const int b = t % R;
            if (lane == 0) {
                int fine = wait(&b_full[b], (uint32_t)((t / R) & 1));
                if (fine) waited = t + 1;
                if (fine && t >= 2) fine = wait(&d_empty[t & 1], (uint32_t)(((t - 2) >> 1) & 1));
                tc::fence_after_sync();
                if (fine) {
                    const uint32_t dt = tbase + (uint32_t)((t & 1) * kGlmCols);
                    const uint32_t a0 = tc::smem_u32(s_a), b0 = tc::smem_u32(s_b + (size_t)b * S::TILE);
#pragma unroll
                    for (int s = 0; s < S::KSTEPS; ++s) {
                        const uint64_t da = tc::smem_desc(a0 + s * 2 * LBO_A, LBO_A, 128);
                        const uint64_t db = tc::smem_desc(b0 + s * 2 * LBO_B, LBO_B, 128);
                        if (KIND == tc::kTF32) {
                            tc::mma_tf32(dt, da, db, idesc, s > 0);
                        } else {
                            tc::mma(dt, da, db, idesc, s > 0);
                            if (SPLIT == 3) {
                                const uint64_t dal = tc::smem_desc(a0 + (uint32_t)S::A_PART + s * 2 * LBO_A, LBO_A, 128);
                                const uint64_t dbl = tc::smem_desc(b0 + (uint32_t)S::B_PART + s * 2 * LBO_B, LBO_B, 128);
                                tc::mma(dt, dal, db, idesc, true);
                                tc::mma(dt, da, dbl, idesc, true);
                            }
                        }
                    }
                }
                tc::commit(&d_full[t & 1]);  // arrives when this tile's MMAs (issued or not) are done
                tc::commit(&b_empty[b]);
                if (!fine) ok = 0;
            }
            ok = __shfl_sync(0xffffffffu, ok, 0);
            // refill the buffer the previous tile's MMAs have finished with
            const int tn = t + R - 1;
            if (ok && t >= 1 && tn < T) {
                int fine = 1;
                if (lane == 0) fine = wait(&b_empty[(t - 1) % R], (uint32_t)(((t - 1) / R) & 1));
                if (__shfl_sync(0xffffffffu, fine, 0)) load(tn);
            }
        }
        // drain: every requested copy lands before the CTA exits
        if (lane == 0)
            for (int q = waited; q < issued; ++q) tc::mbar_wait(&b_full[q % R], (uint32_t)((q / R) & 1));
    } else {
        // ================= epilogue warps =================
        const int et = tid - 32;              // 0..255
        // 1) this CTA's samples -> A operand (two threads per sample row)
        {
            const int r = et & (kGlmRows - 1), half = et >> 7;
            const int64_t i = row0 + r;
            const bool active = i < p.n;
            constexpr int QH = S::KG / 2;
            for (int qq = 0; qq < QH; ++qq) {
                const int q = half * QH + qq;
                float v[S::PER];
#pragma unroll
                for (int m = 0; m < S::PER; ++m) {
                    const int c = q * S::PER + m;
                    v[m] = (active && c < p.d) ? p.x[i * p.d + c] : 0.f;
                }
                const uint4 hi = glm_pack<KIND>(v);
                *reinterpret_cast<uint4 *>(s_a + (size_t)q * kGlmRows * 16 + r * 16) = hi;
                if (S::NPART == 2)
                    *reinterpret_cast<uint4 *>(s_a + S::A_PART + (size_t)q * kGlmRows * 16 + r * 16) =
                        glm_pack_lo(v, hi);
            }
            tc::fence_proxy_async();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&a_full);
        }
        // 2) reduce the accumulators: warp w reads lane quadrant w % 4, columns half (w - 1) / 4
        const int qd = warp & 3, half = (warp - 1) >> 2;
        const int64_t i = row0 + 32 * qd + lane;
        double acc = 0.0;
        const bool logistic = p.kind == ISSM_TARGET_LOGISTIC;
        for (int t = 0; t < T; ++t) {
            const bool ok = __all_sync(0xffffffffu, wait(&d_full[t & 1], (uint32_t)((t >> 1) & 1)));
            tc::fence_after_sync();
            if (!ok) break;
            float part = 0.f;
#pragma unroll 1
            for (int c = 0; c < kGlmCols / 2; c += 32) {
                float v[32];
                tc::tmem_ld32(tbase + ((uint32_t)(32 * qd) << 16) + (uint32_t)((t & 1) * kGlmCols + half * 128 + c), v);
                const int o0 = t * kGlmCols + half * 128 + c;
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    const int o = o0 + j;
                    if (o < p.nobs) {
                        const float eta = v[j], y = __ldg(p.y + o);
                        if (logistic) {
                            // y eta - log(1 + e^eta) = y eta - max(eta, 0) - log1p(e^-|eta|)
                            part += y * eta - fmaxf(eta, 0.f) - log1pf(expf(-fabsf(eta)));
                        } else {
                            const float r = y - eta;
                            part = fmaf(r, r, part);
                        }
                    }
                }
            }
            acc += (double)part;
            tc::fence_before_sync();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&d_empty[t & 1]);
        }
        // the two column halves of a row meet in shared memory
        __shared__ double s_half[kGlmRows];
        if (half == 1) s_half[32 * qd + lane] = acc;
        asm volatile("bar.sync 1, %0;" ::"r"(32 * kGlmEpiWarps) : "memory");
        if (half == 0 && i < p.n && !abort_flag) {
            acc += s_half[32 * qd + lane];
            double bb = 0.0;
            for (int c = 0; c < p.d; ++c) {
                const double b = (double)p.x[i * p.d + c];
                bb += b * b;
            }
            const double pv = (double)p.prior_var;
            const double prior = -0.5 * p.d * (kGlmLog2Pi + log(pv)) - bb / (2.0 * pv);
            double lt;
            if (logistic) {
                lt = acc + prior;
            } else {
                const double sg = (double)p.sigma;
                lt = -0.5 * p.nobs * (kGlmLog2Pi + 2.0 * log(sg)) - acc / (2.0 * sg * sg) + prior;
            }
            p.out[i] = (float)lt;
        }
    }
    // ---- every role is done; in-flight MMAs have completed before TMEM is freed ----
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (tid == 0 && abort_flag && T > 0) tc::mbar_wait(&d_full[(T - 1) & 1], (uint32_t)(((T - 1) >> 1) & 1));
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tbase, 512);
}

static int glm_dp(int d) { return d <= 16 ? 16 : d <= 32 ? 32 : 64; }

size_t glm_operand_bytes(int nobs, int d, int precision) {
    const int DP = glm_dp(d);
    const int tiles = (nobs + kGlmCols - 1) / kGlmCols;
    const size_t eb = precision == ISSM_PREC_TF32 ? 4 : 2;
    const size_t parts = precision == ISSM_PREC_BF16 ? 2 : 1;
    return (size_t)tiles * parts * (size_t)DP * eb * kGlmCols;
}

template <int KIND, int SPLIT, int DP>
static int glm_prepare_t(const float *X, int nobs, int d, unsigned char *ops, cudaStream_t stream) {
    using S = GlmShape<KIND, SPLIT, DP>;
    const int tiles = (nobs + kGlmCols - 1) / kGlmCols;
    const int64_t total = (int64_t)tiles * S::KG * kGlmCols;
    glm_prepare_kernel<KIND, SPLIT, DP><<<grid_for(total, 256, 4), 256, 0, stream>>>(X, nobs, d, tiles, ops);
    note_launch();
    return (int)cudaGetLastError();
}

template <int KIND, int SPLIT, int DP>
static int glm_run_t(GlmParams p, cudaStream_t stream) {
    using S = GlmShape<KIND, SPLIT, DP>;
    const size_t base = S::NPART * S::A_PART;
    int ring = (int)((kGlmMaxSmem - base) / S::TILE);
    ring = ring > 3 ? 3 : ring;
    if (ring < 2) return ISSM_E_UNSUPPORTED;
    p.ring = ring;
    // at least half an SM's shared memory, so one CTA (and its 512 TMEM
    // columns) per SM: the allocation never waits for another CTA's columns
    size_t smem = base + (size_t)ring * S::TILE;
    if (smem < 120 * 1024) smem = 120 * 1024;
    auto kern = glm_tc_kernel<KIND, SPLIT, DP>;
    const int st = allow_dynamic_smem((const void *)kern);
    if (st) return st;
    const int blocks = (int)((p.n + kGlmRows - 1) / kGlmRows);
    { kern<<<blocks, kGlmThreads, smem, stream>>>(p); note_launch(); }
    return (int)cudaGetLastError();
}

#define ISSM_GLM_DISPATCH(FN, ...)                                                           \
    do {                                                                                     \
        const int DP_ = glm_dp(d);                                                           \
        if (precision == ISSM_PREC_TF32) {                                                   \
            if (DP_ == 16) return FN<tc::kTF32, 1, 16>(__VA_ARGS__);                         \
            if (DP_ == 32) return FN<tc::kTF32, 1, 32>(__VA_ARGS__);                         \
            return FN<tc::kTF32, 1, 64>(__VA_ARGS__);                                        \
        }                                                                                    \
        if (precision == ISSM_PREC_BF16) {                                                   \
            if (DP_ == 16) return FN<tc::kBF16, 3, 16>(__VA_ARGS__);                         \
            if (DP_ == 32) return FN<tc::kBF16, 3, 32>(__VA_ARGS__);                         \
            return FN<tc::kBF16, 3, 64>(__VA_ARGS__);                                        \
        }                                                                                    \
        if (DP_ == 16) return FN<tc::kBF16, 1, 16>(__VA_ARGS__);                             \
        if (DP_ == 32) return FN<tc::kBF16, 1, 32>(__VA_ARGS__);                             \
        return FN<tc::kBF16, 1, 64>(__VA_ARGS__);                                            \
    } while (0)

int glm_prepare(const issm_target *t, int precision, void *ops, cudaStream_t stream) {
    const int d = t->dim;
    ISSM_GLM_DISPATCH(glm_prepare_t, (const float *)t->a, t->count, d, (unsigned char *)ops, stream);
}

int glm_logdensity(const issm_target *t, int precision, const void *ops, const float *x, int64_t n, float *out,
                   int *error, cudaStream_t stream) {
    const int d = t->dim;
    GlmParams p{};
    p.d = d;
    p.nobs = t->count;
    p.kind = t->kind;
    p.tiles = (t->count + kGlmCols - 1) / kGlmCols;
    p.n = n;
    p.x = x;
    p.y = (const float *)t->b;
    p.ops = (const unsigned char *)ops;
    p.out = out;
    p.sigma = (float)t->p0;
    p.prior_var = (float)t->p1;
    p.error = error;
    ISSM_GLM_DISPATCH(glm_run_t, p, stream);
}

}  // namespace issm
