// moments.cu — weighted mean / covariance of the retained samples and the
// FP64 candidate fit (ridge, Cholesky, Student-t scaling, lognormalizer).
//
// weighted_moments is a literal two-pass restatement of _weighted_moments!
// (src/adaptive_gaussian_execution.jl:268-273): pass 1 the weighted mean about
// `shift`, pass 2 the weighted covariance about that mean. Weights are
// w_i = exp(l_i - max) / S from the device summary words. Each block stages a
// tile of samples in shared memory (centred, in the sample dtype) and
// accumulates its share of the d or d x d sums; per-block partials are summed
// in FP64 by a second kernel. fit_factor runs in one CTA with the covariance
// in shared memory (d <= 64).
#include "issm_device.cuh"
#include "issm_internal.h"
#include "trinv.cuh"

namespace issm {

constexpr int kMomThreads = 256;
constexpr int kMomTile = 64;

static int moment_blocks(int64_t n) {
    int64_t b = (n + 2047) / 2048;
    if (b > kSMs * 2) b = kSMs * 2;
    return b < 1 ? 1 : (int)b;
}

size_t moments_workspace_bytes(int64_t n, int d) {
    return sizeof(double) * ((size_t)moment_blocks(n) * (size_t)d * (size_t)d + (size_t)d * (size_t)d + 2 * (size_t)d + 16);
}

// pass: 0 -> partial[b][c] = sum w (x_c - shift_c); 1 -> partial[b][r + c d] = sum w z_r z_c
template <typename T>
__global__ void __launch_bounds__(kMomThreads) moments_partial_kernel(const T *__restrict__ x, int d, int64_t n,
                                                                      const T *__restrict__ lw,
                                                                      const double *__restrict__ summary,
                                                                      const double *__restrict__ center, int pass,
                                                                      double *__restrict__ partial) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *tile = reinterpret_cast<T *>(smem_raw);               // kMomTile x d (centred)
    T *wt = tile + (size_t)kMomTile * d;                      // kMomTile weights
    const T m = (T)summary[0];
    const T inv = (T)(1.0 / summary[1]);
    const int entries = pass == 0 ? d : d * d;
    // each thread owns up to 16 entries of the output
    T acc[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) acc[j] = T(0);
    const int64_t per_block = (n + gridDim.x - 1) / gridDim.x;
    const int64_t lo = (int64_t)blockIdx.x * per_block;
    const int64_t hi = min(n, lo + per_block);
    for (int64_t t0 = lo; t0 < hi; t0 += kMomTile) {
        const int cnt = (int)min((int64_t)kMomTile, hi - t0);
        __syncthreads();
        for (int e = threadIdx.x; e < cnt * d; e += blockDim.x) {
            const int s = e / d, c = e - s * d;
            tile[e] = (T)((double)x[(t0 + s) * d + c] - center[c]);
        }
        for (int s = threadIdx.x; s < cnt; s += blockDim.x) {
            const T w = dexp(lw[t0 + s] - m) * inv;
            wt[s] = (pass == 1) ? w : w;
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            const int e = threadIdx.x + j * kMomThreads;
            if (e < entries) {
                T a = acc[j];
                if (pass == 0) {
                    for (int s = 0; s < cnt; ++s) a += wt[s] * tile[s * d + e];
                } else {
                    const int r = e % d, c = e / d;
                    for (int s = 0; s < cnt; ++s) a += wt[s] * tile[s * d + r] * tile[s * d + c];
                }
                acc[j] = a;
            }
        }
    }
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        const int e = threadIdx.x + j * kMomThreads;
        if (e < entries) partial[(size_t)blockIdx.x * entries + e] = (double)acc[j];
    }
}

// Sum block partials in FP64. pass 0: mean = center + S1 (weights sum to one);
// pass 1: cov = S2 - s1 s1^T where s1 = sum w (x - mean) (nearly zero).
__global__ void moments_finish_kernel(const double *__restrict__ partial, int blocks, int d, int pass,
                                      const double *__restrict__ center, double *__restrict__ out,
                                      const double *__restrict__ s1) {
    const int entries = pass == 0 ? d : d * d;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < entries; e += gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int b = 0; b < blocks; ++b) acc += partial[(size_t)b * entries + e];
        if (pass == 0) {
            out[e] = center[e] + acc;
        } else {
            const int r = e % d, c = e / d;
            out[e] = acc - (s1 ? s1[r] * s1[c] : 0.0);
        }
    }
}

// residual mean about the pass-1 mean, to correct pass 2
__global__ void moments_residual_kernel(const double *__restrict__ partial, int blocks, int d,
                                        double *__restrict__ s1) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < d; e += gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int b = 0; b < blocks; ++b) acc += partial[(size_t)b * d + e];
        s1[e] = acc;
    }
}

template <typename T>
static int moments_t(const T *x, int d, int64_t n, const T *lw, const double *summary, const double *shift,
                     double *mean, double *cov, double *ws, cudaStream_t stream) {
    const int blocks = moment_blocks(n);
    double *partial = ws;
    double *s1 = ws + (size_t)blocks * d * d;
    const size_t smem = sizeof(T) * ((size_t)kMomTile * d + kMomTile);
    if (d * d > 16 * kMomThreads) return ISSM_E_UNSUPPORTED;
    auto kern = moments_partial_kernel<T>;
    if (smem > 48 * 1024) {
        const int e = allow_dynamic_smem((const void *)kern);
        if (e) return e;
    }
    { kern<<<blocks, kMomThreads, smem, stream>>>(x, d, n, lw, summary, shift, 0, partial); note_launch(); }
    { moments_finish_kernel<<<1, 256, 0, stream>>>(partial, blocks, d, 0, shift, mean, nullptr); note_launch(); }
    { kern<<<blocks, kMomThreads, smem, stream>>>(x, d, n, lw, summary, mean, 1, partial); note_launch(); }
    { moments_finish_kernel<<<(d * d + 255) / 256, 256, 0, stream>>>(partial, blocks, d, 1, mean, cov, nullptr); note_launch(); }
    (void)s1;
    return (int)cudaGetLastError();
}

int weighted_moments(const void *x, int d, int64_t n, const void *lw, int dtype, const double *summary,
                     const double *shift, double *mean, double *cov, void *ws, size_t ws_bytes,
                     cudaStream_t stream) {
    if (ws_bytes < moments_workspace_bytes(n, d)) return ISSM_E_WORKSPACE;
    if (dtype == ISSM_F32)
        return moments_t<float>((const float *)x, d, n, (const float *)lw, summary, shift, mean, cov, (double *)ws,
                                stream);
    return moments_t<double>((const double *)x, d, n, (const double *)lw, summary, shift, mean, cov, (double *)ws,
                             stream);
}

// ---- candidate fit ---------------------------------------------------------------
// ridge = reg * tr(L_prev L_prev^T) * c_nu / d with the overflow fallback of
// _factor_scale_aware_ridge (src/adaptive_gaussian_execution.jl:283-301);
// right-looking Cholesky in FP64; factor *= sqrt(1/c_nu) for Student-t
// (src/proposals.jl:73-80); zero upper triangle; lognormalizer and validity
// (:493-528).
// 1 / a in FP64 with few FP64 instructions: an FP32 reciprocal seed refined
// by two Newton-Raphson steps r <- r + r (1 - a r) (about 23 -> 46 -> full
// double bits; the seed is the hardware's approximate FP32 reciprocal). Each
// FP64 instruction occupies a warp's FP64 pipe for about 64 cycles on this
// GPU (and takes as long to complete), so the factorisation's
// sequential chain is built from as few of them as possible. Values outside
// the FP32 seed's range, zero, negative or non-finite values take the exact
// division (and give its NaN / Inf).
__device__ __forceinline__ double rcp_nr(double a) {
    const float af = (float)a;
    if (!(af > 1e-30f && af < 1e30f)) return 1.0 / a;
    float rf;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rf) : "f"(af));  // one MUFU op; Newton makes up the bits
    double r = (double)rf;
    double e = fma(-a, r, 1.0);
    r = fma(r, e, r);
    e = fma(-a, r, 1.0);
    return fma(r, e, r);
}

template <typename V> __device__ __forceinline__ V warp_sum_all(V v) {
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

// Candidate fit of one moment round (src/adaptive_gaussian_execution.jl:283-528):
// cov + ridge I with ridge = reg tr(L_prev L_prev^T) c_nu / d (reg = sqrt(eps(T)),
// c_nu = nu/(nu-2) for Student-t, 1 for Gaussian; when that product is not
// finite the ridge is summed from the scaled factor, as the reference does),
// an FP64 factorisation, Student-t scaling of the factor by sqrt((nu-2)/nu),
// rounding to T, the validity rule and the lognormalizer, plus (optionally)
// the FP32 inverse of the stored factor for the tensor-core forms.
//
// The factorisation is a blocked right-looking LDL^T, A = L D L^T with unit
// lower L, in 8-column panels; the Cholesky factor is L diag(sqrt(d)). Each
// FP64 instruction holds a warp's FP64 pipe for about 64 cycles on this GPU
// (and takes as long to complete), so:
//  * the sequential chain per column is only 1/d_j (an FP32 seed and two
//    Newton steps), run by warp 0 on the 8 x 8 diagonal block, which it
//    holds in registers (one element per lane, shuffles between steps);
//  * one thread per row solves its panel row, l_ic = (a_ic - sum_q l_iq d_q
//    l_cq) / d_c;
//  * while warp 0 updates and factors the next diagonal block (lookahead),
//    warps 1-3 and 5-7 apply the rank-8 update to the rest of the trailing
//    lower triangle, each thread holding up to nine independent elements
//    (column pairs (k, m-1-k) balance the work), so the pipe, not latency,
//    bounds it; warp 4 stays out, since it would queue FP64 instructions on
//    warp 0's sub-partition ahead of the pivot chain.
// The pivots fail exactly when Cholesky's would (d_j <= 0 or not finite).
template <typename T>
__global__ void __launch_bounds__(256) fit_factor_kernel(const double *__restrict__ mean,
                                                         const double *__restrict__ cov, int d,
                                                         const T *__restrict__ prev, double ridge_scale,
                                                         double ridge_fallback_scale, double lognorm_const,
                                                         double tscale, T *out_loc, T *out_factor, T *out_lognorm,
                                                         uint64_t *failures, int64_t failure_index,
                                                         float *out_inverse) {
    extern __shared__ __align__(16) double A[];  // d x d column-major
    __shared__ double s_red[8];
    __shared__ double s_ridge;
    __shared__ double s_dg[64];
    __shared__ double s_rinv[8];
    __shared__ double s_w[2][8][64];  // w_c[i] = l_ic d_c of a panel (double-buffered by panel)
    __shared__ double s_scale[64];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int dd = d * d;
    // ---- stage the covariance with all loads in flight; trace of the previous factor ----
    T tr = T(0);
    for (int e0 = tid; e0 < dd; e0 += 256 * 8) {
        double v[8];
        T pv[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int e = e0 + 256 * u;
            v[u] = e < dd ? cov[e] : 0.0;
            pv[u] = e < dd ? prev[e] : T(0);
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int e = e0 + 256 * u;
            if (e < dd) {
                A[e] = v[u];
                if (e % d >= e / d) tr += pv[u] * pv[u];  // lower triangle, in T as the reference sums it
            }
        }
    }
    tr = warp_sum_all(tr);
    if (lane == 0) s_red[warp] = (double)tr;
    __syncthreads();
    if (tid == 0) {
        double t = 0.0;
        for (int w = 0; w < 8; ++w) t += s_red[w];
        s_ridge = t * ridge_scale;
    }
    __syncthreads();
    double ridge = s_ridge;
    if (!isfinite(ridge)) {
        // the scaled-factor route of _factor_scale_aware_ridge (rare)
        double acc = 0.0;
        if (ridge_fallback_scale != 0.0)
            for (int e = tid; e < dd; e += 256)
                if (e % d >= e / d) {
                    const double v = (double)prev[e] * ridge_fallback_scale;
                    acc += v * v;
                }
        acc = warp_sum_all(acc);
        __syncthreads();
        if (lane == 0) s_red[warp] = acc;
        __syncthreads();
        if (tid == 0) {
            double t = 0.0;
            for (int w = 0; w < 8; ++w) t += s_red[w];
            s_ridge = t;
        }
        __syncthreads();
        ridge = s_ridge;
    }
    for (int c = tid; c < d; c += 256) A[c + c * d] += ridge;
    __syncthreads();

    // ---- blocked LDL^T ----
    // warp 0: LDL^T of the nb x nb diagonal block at (kb, kb), in registers.
    // Lane e < 28 holds the strictly-lower element (ei, ec) of the block
    // (row-major lower order, e = ei (ei - 1) / 2 + ec) and lanes 0..nb-1 the
    // diagonal; a column step is a pivot broadcast, the reciprocal chain, one
    // scaling and one update per held element, with the operands exchanged by
    // warp shuffles, so the chain holds no shared-memory round trip
    auto factor_diag = [&](int kb, int nb, double (*w)[64]) {  // warp 0
        int ei = 1, ec = 0;
        {
            int t = lane;
            while (ei < 8 && t >= ei) {
                t -= ei;
                ++ei;
            }
            ec = t;
        }
        const bool hasl = lane < 28 && ei < nb;
        const bool hasd = lane < nb;
        double vl = hasl ? A[(kb + ei) + (kb + ec) * d] : 0.0;
        double vd = hasd ? A[(kb + lane) + (kb + lane) * d] : 0.0;
        double ul = 0.0;  // u = l d of this lane's lower element, once its column is done
        const int lane_d = lane * (lane - 1) / 2;  // lanes of row `lane`'s lower elements start here
        for (int j = 0; j < nb; ++j) {
            const double dj = __shfl_sync(0xffffffffu, vd, j);
            const double rj = rcp_nr(dj);
            if (lane == 0) {
                s_dg[kb + j] = dj;
                s_rinv[j] = rj;
            }
            // column j: element (ei, j) becomes l = u / d_j
            if (hasl && ec == j) {
                ul = vl;
                vl = vl * rj;
                w[j][kb + ei] = ul;
            }
            // (ei, ec), ec > j: -= l(ei, j) u(ec, j); diagonal (c, c), c > j: -= l(c, j) u(c, j)
            const double l_i = __shfl_sync(0xffffffffu, vl, (ei * (ei - 1) / 2 + j) & 31);
            const double u_c = __shfl_sync(0xffffffffu, ul, (ec * (ec - 1) / 2 + j) & 31);
            const double l_d = __shfl_sync(0xffffffffu, vl, (lane_d + j) & 31);
            const double u_d = __shfl_sync(0xffffffffu, ul, (lane_d + j) & 31);
            if (hasl && ec > j) vl = fma(-l_i, u_c, vl);
            if (hasd && lane > j) vd = fma(-l_d, u_d, vd);
        }
        if (hasl) A[(kb + ei) + (kb + ec) * d] = vl;
        if (hasd) A[(kb + lane) + (kb + lane) * d] = vd;  // the pivot d_lane
        __syncwarp();
    };
    if (warp == 0) factor_diag(0, min(8, d), s_w[0]);
    __syncthreads();
    for (int kb = 0; kb < d; kb += 8) {
        const int nb = min(8, d - kb), base = kb + nb, m = d - base;
        if (m <= 0) break;
        double (*wc)[64] = s_w[(kb >> 3) & 1];
        double (*wn)[64] = s_w[((kb >> 3) + 1) & 1];
        // panel: one thread per row i below the diagonal block
        for (int r = tid; r < m; r += 256) {
            const int i = base + r;
            double w[8];
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                if (c < nb) {
                    double v = A[i + (kb + c) * d];
#pragma unroll
                    for (int q = 0; q < 8; ++q)
                        if (q < c) v = fma(-w[q], A[(kb + c) + (kb + q) * d], v);
                    w[c] = v;                            // l_ic d_c
                    A[i + (kb + c) * d] = v * s_rinv[c];  // l_ic
                    wc[c][i] = v;
                } else {
                    w[c] = 0.0;
                }
            }
        }
        __syncthreads();
        const int nbn = min(8, m);
        if (warp == 0) {
            // lookahead: the next diagonal block gets its rank-nb update first, then is factored
            for (int e = lane; e < nbn * (nbn + 1) / 2; e += 32) {
                int c = 0, t = e;
                while (t >= nbn - c) {
                    t -= nbn - c;
                    ++c;
                }
                const int i = c + t;
                double acc = A[(base + i) + (base + c) * d];
                for (int q = 0; q < nb; ++q) acc = fma(-A[(base + i) + (kb + q) * d], wc[q][base + c], acc);
                A[(base + i) + (base + c) * d] = acc;
            }
            __syncwarp();
            factor_diag(base, nbn, wn);
        } else if (warp != 4) {
            // rank-nb update of the trailing lower triangle outside the next
            // diagonal block, by warps 1-3 and 5-7: warp 4 shares warp 0's
            // sub-partition (warp id mod 4) and so its FP64 pipe, which the
            // pivot chain needs free
            const int wt = (warp < 4 ? warp - 1 : warp - 2) * 32 + lane, half = (m + 1) >> 1,
                      total = half * (m + 1);
            constexpr int kT = 9;  // elements per thread: 192 x 9 >= 28 x 57, the largest trailing triangle
            int ei[kT], ek[kT];
#pragma unroll
            for (int t = 0; t < kT; ++t) {
                ei[t] = -1;
                ek[t] = 0;
                const int e = wt + t * 192;
                if (e < total) {
                    const int c = e / (m + 1), r = e - c * (m + 1);
                    int i = -1, k = 0;
                    if (r < m - c) {
                        k = c;
                        i = c + r;
                    } else {
                        const int k2 = m - 1 - c;
                        if (k2 != c) {
                            k = k2;
                            i = k2 + (r - (m - c));
                        }
                    }
                    if (i >= 0 && !(i < nbn && k < nbn)) {
                        ei[t] = i;
                        ek[t] = k;
                    }
                }
            }
            double acc[kT];
#pragma unroll
            for (int t = 0; t < kT; ++t) acc[t] = ei[t] >= 0 ? A[(base + ei[t]) + (base + ek[t]) * d] : 0.0;
            for (int c = 0; c < nb; ++c) {
#pragma unroll
                for (int t = 0; t < kT; ++t)
                    if (ei[t] >= 0) acc[t] = fma(-A[(base + ei[t]) + (kb + c) * d], wc[c][base + ek[t]], acc[t]);
            }
#pragma unroll
            for (int t = 0; t < kT; ++t)
                if (ei[t] >= 0) A[(base + ei[t]) + (base + ek[t]) * d] = acc[t];
        }
        __syncthreads();
    }

    // ---- factor = L diag(sqrt(d)) * Student-t scale, rounded to T ----
    int invalid = 0;
    for (int c = tid; c < d; c += 256) {
        const double dg = s_dg[c];
        invalid |= !(dg > 0.0) || !isfinite(dg);
        s_scale[c] = sqrt(dg) * tscale;
    }
    __syncthreads();
    constexpr int LDI = 65;
    float *Lf = reinterpret_cast<float *>(A + dd);  // FP32 copy of the stored factor for the inverse
    for (int e = tid; e < dd; e += 256) {
        const int r = e % d, c = e / d;
        const T v = r > c ? (T)(A[e] * s_scale[c]) : r == c ? (T)s_scale[c] : T(0);
        out_factor[e] = v;
        if (out_inverse != nullptr) Lf[r * LDI + c] = (float)v;
        if (r > c) invalid |= !isfinite(v);
    }
    // log|L_jj| in the factor's own precision, summed across lanes then in FP64
    T lg = T(0);
    for (int c = tid; c < d; c += 256) {
        const T v = (T)s_scale[c];
        invalid |= !isfinite(v) || !(v > T(0));
        lg += dlog(fabs(v));
    }
    for (int c = tid; c < d; c += 256) {
        const T v = (T)mean[c];
        out_loc[c] = v;
        invalid |= !isfinite(v);
    }
    lg = warp_sum_all(lg);
    if (lane == 0) s_red[warp] = (double)lg;
    invalid = __syncthreads_or(invalid);
    if (tid == 0) {
        double logabsdet = 0.0;
        for (int w = 0; w < 8; ++w) logabsdet += s_red[w];
        const double ln = lognorm_const - logabsdet;
        *out_lognorm = (T)ln;
        const bool valid = !invalid && isfinite((T)ln);
        if (!valid) record_failure(failures, failure_index, 0, ISSM_REASON_MOMENT_FIT_INVALID);
    }
    // inverse factor for the tensor-core forms: W = (stored factor)^-1 in
    // FP32, DP x DP row-major zero padded
    if (out_inverse != nullptr) {
        float *Wf = Lf + 64 * LDI;
        __syncthreads();
        invert_lower_f32(Lf, Wf, d, LDI);
        const int DP = d <= 16 ? 16 : d <= 32 ? 32 : 64;
        for (int e = tid; e < DP * DP; e += 256) {
            const int j = e / DP, c = e % DP;
            out_inverse[e] = (j < d && c < d) ? Wf[j * LDI + c] : 0.f;
        }
    }
}

int fit_factor(const double *mean, const double *cov, int d, const void *prev, double dof, double logconst,
               int dtype, void *out_loc, void *out_factor, void *out_lognorm, uint64_t *failures,
               int64_t failure_index, float *out_inverse, double regularization, cudaStream_t stream) {
    if (d > 64) return ISSM_E_UNSUPPORTED;
    size_t smem = sizeof(double) * (size_t)d * d;
    if (out_inverse != nullptr) {
        smem += sizeof(float) * 2 * 64 * 65;
        const int e = allow_dynamic_smem(dtype == ISSM_F32 ? (const void *)fit_factor_kernel<float>
                                                           : (const void *)fit_factor_kernel<double>);
        if (e) return e;
    }
    // scalar constants formed once on the host
    const double mult = dof > 0.0 ? dof / (dof - 2.0) : 1.0;
    // sqrt(eps(T)) of the factor type unless the caller gives the coefficient
    const double reg = regularization >= 0.0 ? regularization
                       : dtype == ISSM_F32 ? sqrt((double)FLT_EPSILON) : sqrt(DBL_EPSILON);
    const double ridge_scale = reg * mult / (double)d;
    const double ridge_fallback = reg != 0.0 ? sqrt(reg) * sqrt(mult / (double)d) : 0.0;
    const double lognorm_const = dof > 0.0 ? logconst : -0.5 * (double)d * log(2.0 * 3.14159265358979323846);
    const double tscale = dof > 0.0 ? sqrt(1.0 / mult) : 1.0;
    if (dtype == ISSM_F32) {
        { fit_factor_kernel<float><<<1, 256, smem, stream>>>(mean, cov, d, (const float *)prev, ridge_scale,
                                                           ridge_fallback, lognorm_const, tscale, (float *)out_loc,
                                                           (float *)out_factor, (float *)out_lognorm, failures,
                                                           failure_index, out_inverse); note_launch(); }
    } else {
        { fit_factor_kernel<double><<<1, 256, smem, stream>>>(mean, cov, d, (const double *)prev, ridge_scale,
                                                            ridge_fallback, lognorm_const, tscale,
                                                            (double *)out_loc, (double *)out_factor,
                                                            (double *)out_lognorm, failures, failure_index,
                                                            out_inverse); note_launch(); }
    }
    return (int)cudaGetLastError();
}

}  // namespace issm
