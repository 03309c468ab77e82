// mixture_tc.cu — tensor-core (tcgen05) form of the factor-bank mixture
// density for FP32 samples: the Mahalanobis contraction runs as an MMA and
// the radial density plus the balance-heuristic log-sum-exp run in the
// epilogue straight out of tensor memory.
//
// For every component k the reference solves L_k z = x - mu_k by forward
// substitution (_packed_gaussian_logdensity!, src/native_execution.jl:346-384).
// Here W_k = L_k^-1 is formed in FP64 once per slot (invert_factors_kernel;
// cached by the caller in issm_bank.inverse_factors) and the samples are
// centred on one shift c (the generating / appended slot's mean):
//   z_k = W_k (x - c) - b_k,   b_k = W_k (mu_k - c)   (b_k formed per CTA),
// so each 128-sample tile is one GEMM  D[128 x K*DP] = X'[128 x DP] W^T.
// Precision forms (FP32 accumulation in TMEM in both):
//   TF32    one kind::tf32 MMA per K slice, operands rounded to tf32 (RNE);
//   BF16x3  operands split v = hi + lo in bf16, D = Xh Wh + Xl Wh + Xh Wl,
//           about 16 significant bits per product.
// One CTA = 4 warps; warp w owns TMEM lanes 32w..32w+31, i.e. samples
// 32w..32w+31 of the tile, for every component, so the per-sample log-sum-exp
// state stays in registers across component chunks.
#include "issm_device.cuh"
#include "issm_internal.h"
#include "tcgen05.cuh"

namespace issm {

constexpr int kTcThreads = 128;
constexpr int kTcTile = 128;

struct TcParams {
    int d, k, family, mode;       // mode: 0 denominator, 1 append
    int first_slot, last_slot, chunk, ntile_total;
    int den_kind;
    int64_t n;
    const float *x;
    const float *w;               // K x DP x DP, row j holds W_k[j, :]
    const float *loc;             // d x K bank locations
    const float *lognorm, *coef, *dofs;
    const int32_t *slots, *group;
    int fixed_slot;
    const float *center;          // DP
    float *out_logden, *out_generating, *lognum;
    uint64_t *failures;
    int64_t index_base;
    int *error;
};

__device__ __forceinline__ uint32_t tf32_bits(float f) {
    uint32_t u = __float_as_uint(f);
    if ((u & 0x7f800000u) == 0x7f800000u) return u;
    u += 0xFFFu + ((u >> 13) & 1u);
    return u & ~0x1FFFu;
}

// write one 16-byte core-matrix row chunk of operand values (elements e..e+per)
template <int KIND>
__device__ __forceinline__ void put_chunk(unsigned char *tile, int row, int kgrp, int KG, const float *v,
                                          bool lo_part) {
    const uint32_t off = (uint32_t)((((row >> 3) * KG + kgrp) << 7) + ((row & 7) << 4));
    if (KIND == tc::kTF32) {
        uint4 q;
        q.x = tf32_bits(v[0]);
        q.y = tf32_bits(v[1]);
        q.z = tf32_bits(v[2]);
        q.w = tf32_bits(v[3]);
        *reinterpret_cast<uint4 *>(tile + off) = q;
    } else {
        uint32_t h[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            float a = v[2 * i], c = v[2 * i + 1];
            uint16_t ha = tc::bf16_bits(a), hc = tc::bf16_bits(c);
            if (lo_part) {
                ha = tc::bf16_bits(a - __uint_as_float((uint32_t)ha << 16));
                hc = tc::bf16_bits(c - __uint_as_float((uint32_t)hc << 16));
            }
            h[i] = (uint32_t)ha | ((uint32_t)hc << 16);
        }
        *reinterpret_cast<uint4 *>(tile + off) = make_uint4(h[0], h[1], h[2], h[3]);
    }
}

template <int KIND, int SPLIT, int DP>
__global__ void __launch_bounds__(kTcThreads) mixture_tc_kernel(TcParams p) {
    constexpr int EB = KIND == tc::kBF16 ? 2 : 4;
    constexpr int PER = 16 / EB;          // elements per core-matrix row
    constexpr int KG = DP / PER;          // K groups of the DP-long rows
    constexpr int A_BYTES = kTcTile * DP * EB;
    constexpr int B_BYTES = DP * DP * EB;  // one component
    constexpr int NPART = SPLIT == 3 ? 2 : 1;
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *sa = smem;                                  // NPART x A
    unsigned char *sb = smem + NPART * A_BYTES;                // NPART x chunk x B
    float *sbv = reinterpret_cast<float *>(sb + (size_t)NPART * p.chunk * B_BYTES);  // chunk x DP
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tmem_base;
    __shared__ int abort_flag;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t ncols_raw = (uint32_t)(p.chunk * DP);
    const uint32_t ncols = ncols_raw <= 32 ? 32 : ncols_raw <= 64 ? 64 : ncols_raw <= 128 ? 128 : ncols_raw <= 256 ? 256 : 512;
    if (warp == 0) tc::tmem_alloc(&tmem_base, ncols);
    if (tid == 0) {
        tc::mbar_init(&bar, 1);
        tc::fence_mbar_init();
        abort_flag = 0;
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = tmem_base;
    const uint32_t lane_base = tbase + ((uint32_t)(32 * warp) << 16);
    uint32_t phase = 0;
    const int nslots = p.last_slot - p.first_slot + 1;
    const int nchunks = (nslots + p.chunk - 1) / p.chunk;
    int staged_chunk = -1;
    const uint32_t idesc = tc::instr_desc(KIND, kTcTile, DP);
    // rows are loaded with 16-byte vectors when the layout allows it
    const bool vec = (p.d % 4 == 0) && ((reinterpret_cast<uintptr_t>(p.x) & 15) == 0);
    float xs[DP], xn[DP];
    auto load_row = [&](int tile, float (&dst)[DP]) {
        const int64_t r = (int64_t)tile * kTcTile + tid;
#pragma unroll
        for (int c = 0; c < DP; ++c) dst[c] = 0.f;
        if (tile < p.ntile_total && r < p.n) {
            const float *xi = p.x + r * p.d;
            if (vec) {
#pragma unroll
                for (int c = 0; c < DP; c += 4)
                    if (c < p.d) {
                        const float4 q = __ldg(reinterpret_cast<const float4 *>(xi + c));
                        dst[c] = q.x; dst[c + 1] = q.y; dst[c + 2] = q.z; dst[c + 3] = q.w;
                    }
            } else {
#pragma unroll
                for (int c = 0; c < DP; ++c)
                    if (c < p.d) dst[c] = __ldg(xi + c);
            }
        }
    };
    load_row(blockIdx.x, xn);

    for (int tile = blockIdx.x; tile < p.ntile_total; tile += gridDim.x) {
        const int64_t i = (int64_t)tile * kTcTile + tid;
        const bool active = i < p.n;
        // ---- stage A (shifted samples) from the prefetched row ----
#pragma unroll
        for (int c = 0; c < DP; ++c) xs[c] = (c < p.d && active) ? xn[c] - p.center[c] : 0.f;
        // the next tile's row is in flight while this tile's MMAs and epilogue run
        load_row(tile + gridDim.x, xn);
#pragma unroll
        for (int q = 0; q < KG; ++q) {
            put_chunk<KIND>(sa, tid, q, KG, xs + q * PER, false);
            if (NPART == 2) put_chunk<KIND>(sa + A_BYTES, tid, q, KG, xs + q * PER, true);
        }
        const int gen = active ? (p.slots ? p.slots[i] : p.fixed_slot) : 0;
        const int ggen = (p.den_kind == ISSM_DENOM_PARTIAL && active) ? p.group[gen] : 0;
        LseState<float> lse;
        float gen_lq = 0.f, last_lq = 0.f;
        for (int ch = 0; ch < nchunks; ++ch) {
            const int k0 = p.first_slot + ch * p.chunk;
            const int cnt = min(p.chunk, p.last_slot - k0 + 1);
            if (staged_chunk != ch) {
                // ---- stage B (inverse factors) and the shift vectors ----
                for (int e = tid; e < cnt * DP * KG; e += kTcThreads) {
                    const int kk = e / (DP * KG), rem = e - kk * DP * KG, row = rem / KG, q = rem - row * KG;
                    const float *src = p.w + ((size_t)(k0 + kk) * DP + row) * DP + q * PER;
                    float v[PER];
#pragma unroll
                    for (int j = 0; j < PER; ++j) v[j] = src[j];
                    put_chunk<KIND>(sb + (size_t)kk * B_BYTES, row, q, KG, v, false);
                    if (NPART == 2)
                        put_chunk<KIND>(sb + (size_t)(p.chunk + kk) * B_BYTES, row, q, KG, v, true);
                }
                // b_k = W_k (mu_k - c), accumulated in FP32 from the cached inverse
                for (int e = tid; e < cnt * DP; e += kTcThreads) {
                    const int kk = e / DP, j = e - kk * DP, k = k0 + kk;
                    const float *wr = p.w + ((size_t)k * DP + j) * DP;
                    float acc = 0.f;
                    for (int c = 0; c < p.d; ++c) acc = fmaf(wr[c], p.loc[(size_t)k * p.d + c] - p.center[c], acc);
                    sbv[e] = acc;
                }
                staged_chunk = ch;
            }
            tc::fence_proxy_async();
            tc::fence_before_sync();
            __syncthreads();
            tc::fence_after_sync();
            if (abort_flag) break;
            if (tid == 0) {
                const uint32_t a0 = tc::smem_u32(sa), b0 = tc::smem_u32(sb);
                for (int kk = 0; kk < cnt; ++kk) {
                    const uint32_t dcol = tbase + (uint32_t)(kk * DP);
                    for (int s = 0; s < DP * EB / 32; ++s) {
                        const uint64_t da = tc::smem_desc(a0 + s * 256, 128, KG * 128);
                        const uint64_t db = tc::smem_desc(b0 + kk * B_BYTES + s * 256, 128, KG * 128);
                        if (KIND == tc::kTF32) {
                            tc::mma_tf32(dcol, da, db, idesc, s > 0);
                        } else {
                            tc::mma(dcol, da, db, idesc, s > 0);
                            if (SPLIT == 3) {
                                const uint64_t dal = tc::smem_desc(a0 + A_BYTES + s * 256, 128, KG * 128);
                                const uint64_t dbl =
                                    tc::smem_desc(b0 + (p.chunk + kk) * B_BYTES + s * 256, 128, KG * 128);
                                tc::mma(dcol, dal, db, idesc, true);
                                tc::mma(dcol, da, dbl, idesc, true);
                            }
                        }
                    }
                }
                tc::commit(&bar);
                // one thread observes completion; the barrier below publishes it
                if (!tc::mbar_wait(&bar, phase)) {
                    atomicExch(p.error, 1);
                    abort_flag = 1;
                }
            }
            phase ^= 1u;
            tc::fence_before_sync();
            __syncthreads();
            tc::fence_after_sync();
            const bool ok = abort_flag == 0;  // block-uniform
            if (ok) {
                // ---- epilogue: radial density and log-sum-exp per component ----
                for (int kk = 0; kk < cnt; ++kk) {
                    const int k = k0 + kk;
                    float r2 = 0.f;
#pragma unroll
                    for (int c0 = 0; c0 < DP; c0 += 16) {
                        float v[16];
                        tc::tmem_ld16(lane_base + (uint32_t)(kk * DP + c0), v);
#pragma unroll
                        for (int j = 0; j < 16; ++j) {
                            const float z = v[j] - sbv[kk * DP + c0 + j];
                            r2 = fmaf(z, z, r2);
                        }
                    }
                    float lq;
                    if (p.family == ISSM_GAUSSIAN) {
                        lq = p.lognorm[k] - 0.5f * r2;
                    } else {
                        const float nu = p.dofs[k];
                        lq = p.lognorm[k] - (nu + (float)p.d) * 0.5f * log1pf(r2 / nu);
                    }
                    bool member = true;
                    if (p.den_kind == ISSM_DENOM_GENERATING) member = (k == gen);
                    else if (p.den_kind == ISSM_DENOM_PARTIAL) member = (p.group[k] == ggen);
                    if (k == gen) gen_lq = lq;
                    last_lq = lq;
                    if (member) lse.add((p.coef ? p.coef[k] : 0.f) + lq);
                }
            }
            tc::fence_before_sync();
            __syncthreads();
        }
        if (abort_flag) break;
        if (!active) continue;
        if (p.mode == 1) {
            uint16_t reason = isnan(last_lq) ? ISSM_REASON_PROPOSAL_INVALID : 0;
            if (!reason) {
                const float v = logaddexp(p.lognum[i], p.coef[p.first_slot] + last_lq);
                if (isnan(v) || v == -INFINITY) reason = ISSM_REASON_PROPOSAL_INVALID;
                else p.lognum[i] = v;
            }
            if (reason) record_failure(p.failures, p.index_base + i + 1, 0, reason);
        } else {
            float den = lse.value();
            bool bad = isnan(gen_lq) || gen_lq == -INFINITY || isnan(den) || den == -INFINITY;
            if (bad) {
                record_failure(p.failures, p.index_base + i + 1, 0, ISSM_REASON_PROPOSAL_INVALID);
                den = -INFINITY;
            }
            p.out_logden[i] = den;
            if (p.out_generating) p.out_generating[i] = bad ? -INFINITY : gen_lq;
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tbase, ncols);
}

// W_k = L_k^-1 in FP64: L_k is staged in shared memory, one thread solves
// one column by forward substitution; written as FP32 DP x DP, zero padded.
template <typename T>
__global__ void invert_factors_kernel(const T *__restrict__ L, int d, int DP, int first, float *__restrict__ w) {
    const int k = first + blockIdx.x;
    extern __shared__ double sm_inv[];
    double *Ls = sm_inv;            // d x d column-major
    double *Ws = sm_inv + d * d;    // d x d column-major
    const T *Lk = L + (size_t)k * d * d;
    for (int e = threadIdx.x; e < d * d; e += blockDim.x) Ls[e] = (double)Lk[e];
    __syncthreads();
    for (int c = threadIdx.x; c < d; c += blockDim.x) {
        for (int r = 0; r < c; ++r) Ws[r + c * d] = 0.0;
        for (int r = c; r < d; ++r) {
            double v = (r == c) ? 1.0 : 0.0;
            for (int q = c; q < r; ++q) v -= Ls[r + q * d] * Ws[q + c * d];
            Ws[r + c * d] = v / Ls[r + r * d];
        }
    }
    __syncthreads();
    float *wk = w + (size_t)k * DP * DP;
    for (int e = threadIdx.x; e < DP * DP; e += blockDim.x) {
        const int j = e / DP, c = e % DP;
        wk[e] = (j < d && c < d) ? (float)Ws[j + c * d] : 0.f;
    }
}

int invert_factors(const issm_bank *bk, int first, int count, float *out, cudaStream_t stream) {
    const int d = bk->dim;
    if (d > 64) return ISSM_E_UNSUPPORTED;
    const int DP = d <= 16 ? 16 : d <= 32 ? 32 : 64;
    const size_t smem = 2 * sizeof(double) * d * d;
    if (count <= 0) return 0;
    cudaError_t e = cudaFuncSetAttribute(bk->dtype == ISSM_F32 ? (const void *)invert_factors_kernel<float>
                                                               : (const void *)invert_factors_kernel<double>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return (int)e;
    if (bk->dtype == ISSM_F32) {
        { invert_factors_kernel<float><<<count, 64, smem, stream>>>((const float *)bk->scales, d, DP, first, out);
          note_launch(); }
    } else {
        { invert_factors_kernel<double><<<count, 64, smem, stream>>>((const double *)bk->scales, d, DP, first, out);
          note_launch(); }
    }
    return (int)cudaGetLastError();
}

size_t tc_workspace_bytes(int k, int d) {
    const int DP = d <= 16 ? 16 : d <= 32 ? 32 : 64;
    return sizeof(float) * ((size_t)k * DP * DP + (size_t)k * DP + DP) + 64;
}

template <int KIND, int SPLIT, int DP>
static int launch_tc(TcParams p, cudaStream_t stream) {
    constexpr int EB = KIND == tc::kBF16 ? 2 : 4;
    constexpr int NPART = SPLIT == 3 ? 2 : 1;
    const int nslots = p.last_slot - p.first_slot + 1;
    const int maxcols = 256;  // two CTAs per SM share the 512 TMEM columns
    int chunk = maxcols / DP;
    if (chunk > nslots) chunk = nslots;
    p.chunk = chunk;
    size_t smem = (size_t)NPART * kTcTile * DP * EB + (size_t)NPART * chunk * DP * DP * EB +
                  sizeof(float) * chunk * DP;
    // never more resident CTAs per SM than TMEM holds, so allocations never wait
    const int ncols = chunk * DP <= 32 ? 32 : chunk * DP <= 64 ? 64 : chunk * DP <= 128 ? 128 : 256;
    const int tmem_ctas = 512 / ncols;
    const size_t floor_smem = 233472 / (tmem_ctas + 1) + 1024;
    if (smem < floor_smem) smem = floor_smem;
    auto kern = mixture_tc_kernel<KIND, SPLIT, DP>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return (int)e;
    int occ = 1;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kTcThreads, smem);
    if (e != cudaSuccess) return (int)e;
    occ = max(1, min(occ, tmem_ctas));
    p.ntile_total = (int)((p.n + kTcTile - 1) / kTcTile);
    const int blocks = min(p.ntile_total, kSMs * occ);
    if (blocks < 1) return 0;
    { kern<<<blocks, kTcThreads, smem, stream>>>(p); note_launch(); }
    return (int)cudaGetLastError();
}

// precision: ISSM_PREC_TF32 or ISSM_PREC_BF16 (split x3)
int tc_mixture(const issm_bank *bk, const issm_denominator *den, int mode, int first, int last,
               const void *x, int64_t n, const int32_t *slots, int fixed_slot, const void *coef,
               void *out_logden, void *out_generating, void *lognum, uint64_t *failures, int64_t index_base,
               int precision, void *ws, size_t ws_bytes, int *error, cudaStream_t stream) {
    const int d = bk->dim;
    if (bk->dtype != ISSM_F32 || bk->scale_kind != ISSM_SCALE_FACTOR || d > 64) return ISSM_E_UNSUPPORTED;
    const int DP = d <= 16 ? 16 : d <= 32 ? 32 : 64;
    if (ws_bytes < tc_workspace_bytes(bk->count, d)) return ISSM_E_WORKSPACE;
    float *w = (float *)ws;
    float *center = w + (size_t)bk->count * DP * DP + (size_t)bk->count * DP;
    // shift: the generating (or appended) slot's mean
    const int cslot = (mode == 1) ? first : fixed_slot;
    cudaError_t e = cudaMemsetAsync(center, 0, sizeof(float) * DP, stream);
    if (e != cudaSuccess) return (int)e;
    e = cudaMemcpyAsync(center, (const float *)bk->locations + (size_t)cslot * d, sizeof(float) * d,
                        cudaMemcpyDeviceToDevice, stream);
    if (e != cudaSuccess) return (int)e;
    if (bk->inverse_factors) {
        w = const_cast<float *>(bk->inverse_factors);
    } else {
        const int st = invert_factors(bk, first, last - first + 1, w, stream);
        if (st) return st;
    }
    TcParams p{};
    p.d = d; p.k = bk->count; p.family = bk->family; p.mode = mode;
    p.first_slot = first; p.last_slot = last;
    p.den_kind = den ? den->kind : ISSM_DENOM_FULL;
    p.n = n; p.x = (const float *)x; p.w = w; p.loc = (const float *)bk->locations;
    p.lognorm = (const float *)bk->lognormalizers; p.coef = (const float *)coef; p.dofs = (const float *)bk->dofs;
    p.slots = slots; p.group = den ? den->group_of_slot : nullptr; p.fixed_slot = fixed_slot;
    p.center = center; p.out_logden = (float *)out_logden; p.out_generating = (float *)out_generating;
    p.lognum = (float *)lognum; p.failures = failures; p.index_base = index_base; p.error = error;
    const bool tf32 = precision == ISSM_PREC_TF32;
    if (DP == 16) return tf32 ? launch_tc<tc::kTF32, 1, 16>(p, stream) : launch_tc<tc::kBF16, 3, 16>(p, stream);
    if (DP == 32) return tf32 ? launch_tc<tc::kTF32, 1, 32>(p, stream) : launch_tc<tc::kBF16, 3, 32>(p, stream);
    return tf32 ? launch_tc<tc::kTF32, 1, 64>(p, stream) : launch_tc<tc::kBF16, 3, 64>(p, stream);
}

}  // namespace issm
