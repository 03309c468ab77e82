// moments_tc.cu — tensor-core form of the weighted moments that drive AMIS /
// N-PMC adaptation (_weighted_moments!, src/adaptive_gaussian_execution.jl:268-273).
//
// One streaming pass over the retained samples. For a tile of samples the
// operand is the 128 x K matrix A whose rows 0..d-1 hold sqrt(w) (x - c)
// (c = previous proposal mean), row 64 holds sqrt(w), other rows zero; then
//   D[128 x 80] += A A[0:80]^T
// accumulates S2 = sum w z z^T (rows/cols 0..63), S1 = sum w z (row 64 or
// col 64) and S0 = sum w (D[64][64]) in FP32 tensor memory over all tiles of
// the CTA. A and B are the same shared-memory tile (B = its first 80 rows).
// Two tile buffers alternate so staging overlaps the previous tile's MMAs.
// Per-CTA partials are summed in FP64 and mean = c + S1/S0,
// cov = S2/S0 - (S1/S0)(S1/S0)^T.
#include "issm_device.cuh"
#include "issm_internal.h"
#include "tcgen05.cuh"

namespace issm {

constexpr int kMtThreads = 128;
constexpr int kMtRows = 128;  // MMA M
constexpr int kMtCols = 80;   // MMA N (64 dims + sqrt(w) + padding)

template <int KIND>
__global__ void __launch_bounds__(kMtThreads) moments_tc_kernel(const float *__restrict__ x, int d, int64_t n,
                                                                 const float *__restrict__ lw,
                                                                 const double *__restrict__ summary,
                                                                 const double *__restrict__ center,
                                                                 float *__restrict__ partial, int *error) {
    constexpr int EB = KIND == tc::kBF16 ? 2 : 4;
    constexpr int TS = KIND == tc::kBF16 ? 128 : 64;  // samples per tile = MMA K extent per tile
    constexpr int PER = 16 / EB;
    constexpr int KG = TS / PER;                       // 16 core groups per row (256 bytes)
    constexpr int BUF = kMtRows * TS * EB;             // 32 KB
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ uint32_t tmem_base;
    __shared__ int abort_flag;
    __shared__ float cshift[64];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (warp == 0) tc::tmem_alloc(&tmem_base, 128);
    if (tid == 0) {
        tc::mbar_init(&bar[0], 1);
        tc::mbar_init(&bar[1], 1);
        tc::fence_mbar_init();
        abort_flag = 0;
    }
    for (int c = tid; c < 64; c += kMtThreads) cshift[c] = c < d ? (float)center[c] : 0.f;
    for (int e = tid; e < 2 * BUF / 16; e += kMtThreads) reinterpret_cast<uint4 *>(smem)[e] = make_uint4(0, 0, 0, 0);
    const float m = (float)summary[0];
    const float inv = (float)(1.0 / summary[1]);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = tmem_base;
    const int64_t ntiles = (n + TS - 1) / TS;
    uint32_t uses[2] = {0u, 0u};
    int it = 0, last_buf = -1;
    const uint32_t idesc = tc::instr_desc(KIND, kMtRows, kMtCols);
    // thread -> (sample column, dimension half): TF32 tiles have 64 samples, so
    // two threads share a sample, each staging 32 dimensions
    constexpr int HALVES = kMtThreads / TS;   // 1 (bf16) or 2 (tf32)
    constexpr int DH = 64 / HALVES;           // dimensions per thread
    const int col = tid % TS, half = tid / TS, j0 = half * DH;
    const bool vec = (d % 4 == 0) && ((reinterpret_cast<uintptr_t>(x) & 15) == 0);
    float xr[DH];
    float lr = -INFINITY;
    auto load_col = [&](int64_t tile) {
        const int64_t i = tile * TS + col;
#pragma unroll
        for (int c = 0; c < DH; ++c) xr[c] = 0.f;
        lr = -INFINITY;
        if (tile < ntiles && i < n) {
            lr = __ldg(lw + i);
            const float *xi = x + i * d + j0;
            if (vec) {
#pragma unroll
                for (int c = 0; c < DH; c += 4)
                    if (j0 + c < d) {
                        const float4 q = __ldg(reinterpret_cast<const float4 *>(xi + c));
                        xr[c] = q.x; xr[c + 1] = q.y; xr[c + 2] = q.z; xr[c + 3] = q.w;
                    }
            } else {
#pragma unroll
                for (int c = 0; c < DH; ++c)
                    if (j0 + c < d) xr[c] = __ldg(xi + c);
            }
        }
    };
    load_col(blockIdx.x);
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
        const int buf = it & 1;
        if (it >= 2) {
            if (tid == 0 && !tc::mbar_wait(&bar[buf], (uses[buf] - 1) & 1)) {
                atomicExch(error, 1);
                abort_flag = 1;
            }
            tc::fence_before_sync();
            __syncthreads();
            tc::fence_after_sync();
            if (abort_flag) break;
        }
        unsigned char *sa = smem + buf * BUF;
        // ---- stage this thread's (sample, dimension-half) of the tile ----
        {
            const float sw = lr == -INFINITY ? 0.f : sqrtf(expf(lr - m) * inv);
            float z[DH];
#pragma unroll
            for (int c = 0; c < DH; ++c) z[c] = (j0 + c < d) ? sw * (xr[c] - cshift[j0 + c]) : 0.f;
            load_col(tile + gridDim.x);  // next tile's column is in flight during the stores and MMAs
            const int kq = col / PER, kr = col % PER;
#pragma unroll
            for (int jj = 0; jj <= DH; ++jj) {
                if (jj == DH && half != HALVES - 1) break;
                const int j = jj < DH ? j0 + jj : 64;
                const float v = jj < DH ? z[jj] : sw;
                const uint32_t off = (uint32_t)((((j >> 3) * KG + kq) << 7) + ((j & 7) << 4) + kr * EB);
                if (EB == 2) *reinterpret_cast<uint16_t *>(sa + off) = tc::bf16_bits(v);
                else *reinterpret_cast<float *>(sa + off) = v;
            }
        }
        tc::fence_proxy_async();
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        if (tid == 0) {
            const uint32_t a0 = tc::smem_u32(sa);
            for (int s = 0; s < TS * EB / 32; ++s) {
                const uint64_t da = tc::smem_desc(a0 + s * 256, 128, KG * 128);
                if (KIND == tc::kTF32) tc::mma_tf32(tbase, da, da, idesc, it > 0 || s > 0);
                else tc::mma(tbase, da, da, idesc, it > 0 || s > 0);
            }
            tc::commit(&bar[buf]);
        }
        uses[buf] += 1;
        last_buf = buf;
    }
    // ---- wait for the last MMA group (commits track every earlier MMA) ----
    if (last_buf >= 0 && !abort_flag) {
        if (tid == 0 && !tc::mbar_wait(&bar[last_buf], (uses[last_buf] - 1) & 1)) {
            atomicExch(error, 1);
            abort_flag = 1;
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    float *out = partial + (size_t)blockIdx.x * 65 * kMtCols;
    if (!abort_flag && warp < 3) {
        const int row = 32 * warp + lane;
#pragma unroll
        for (int c0 = 0; c0 < kMtCols; c0 += 16) {
            float v[16];
            if (last_buf >= 0) {
                tc::tmem_ld16(tbase + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, v);
            } else {
                for (int j = 0; j < 16; ++j) v[j] = 0.f;
            }
            if (row <= 64) {
                for (int j = 0; j < 16; ++j) out[row * kMtCols + c0 + j] = v[j];
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tbase, 128);
}

// Partials are [block][65][80] FP32; stage 1 sums them over blocks in FP64
// (32 entries x 8 block-strided lanes per CTA, coalesced), stage 2 forms the
// mean and covariance from the 65 x 80 sums.
__global__ void moments_tc_reduce_kernel(const float *__restrict__ partial, int blocks, double *__restrict__ sums) {
    __shared__ double acc_s[8][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int e = blockIdx.x * 32 + tx;
    double acc = 0.0;
    if (e < 65 * kMtCols)
        for (int b = ty; b < blocks; b += 8) acc += (double)partial[(size_t)b * 65 * kMtCols + e];
    acc_s[ty][tx] = acc;
    __syncthreads();
    if (ty == 0 && e < 65 * kMtCols) {
        double t = 0.0;
        for (int r = 0; r < 8; ++r) t += acc_s[r][tx];
        sums[e] = t;
    }
}

__global__ void moments_tc_finish_kernel(const double *__restrict__ sums, int d, const double *__restrict__ center,
                                         double *__restrict__ mean, double *__restrict__ cov) {
    const double s0 = sums[64 * kMtCols + 64];
    for (int j = threadIdx.x; j < d; j += blockDim.x) mean[j] = center[j] + sums[64 * kMtCols + j] / s0;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < d * d; e += gridDim.x * blockDim.x) {
        const int r = e % d, c = e / d;
        const double mr = sums[64 * kMtCols + r] / s0, mc = sums[64 * kMtCols + c] / s0;
        cov[e] = sums[r * kMtCols + c] / s0 - mr * mc;
    }
}

static int moments_tc_blocks(int64_t n, int ts) {
    int64_t t = (n + ts - 1) / ts;
    int64_t b = kSMs * 2;
    return (int)(t < b ? (t < 1 ? 1 : t) : b);
}

size_t moments_tc_workspace_bytes(int64_t n) {
    return sizeof(float) * (size_t)moments_tc_blocks(n, 64) * 65 * kMtCols + sizeof(double) * 65 * kMtCols + 128;
}

int moments_tc(const void *x, int d, int64_t n, const void *lw, const double *summary, const double *shift,
               double *mean, double *cov, int precision, void *ws, size_t ws_bytes, int *error, cudaStream_t stream) {
    if (d > 64) return ISSM_E_UNSUPPORTED;
    if (ws_bytes < moments_tc_workspace_bytes(n)) return ISSM_E_WORKSPACE;
    const bool bf16 = precision == ISSM_PREC_BF16;
    const int ts = bf16 ? 128 : 64;
    const int blocks = moments_tc_blocks(n, ts);
    const size_t smem = 2 * (size_t)kMtRows * ts * (bf16 ? 2 : 4);
    float *partial = (float *)ws;
    if (bf16) {
        auto kern = moments_tc_kernel<tc::kBF16>;
        const int e = allow_dynamic_smem((const void *)kern);
        if (e) return e;
        { kern<<<blocks, kMtThreads, smem, stream>>>((const float *)x, d, n, (const float *)lw, summary, shift,
                                                     partial, error); note_launch(); }
    } else {
        auto kern = moments_tc_kernel<tc::kTF32>;
        const int e = allow_dynamic_smem((const void *)kern);
        if (e) return e;
        { kern<<<blocks, kMtThreads, smem, stream>>>((const float *)x, d, n, (const float *)lw, summary, shift,
                                                     partial, error); note_launch(); }
    }
    double *sums = reinterpret_cast<double *>(partial + (size_t)moments_tc_blocks(n, 64) * 65 * kMtCols);
    { moments_tc_reduce_kernel<<<(65 * kMtCols + 31) / 32, 256, 0, stream>>>(partial, blocks, sums); note_launch(); }
    { moments_tc_finish_kernel<<<(d * d + 255) / 256, 256, 0, stream>>>(sums, d, shift, mean, cov); note_launch(); }
    return (int)cudaGetLastError();
}

}  // namespace issm
