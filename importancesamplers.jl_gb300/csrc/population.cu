// population.cu — per-proposal ("local") weights, covariances and factors of
// a population of proposals, the adaptation step of the population methods
// (src/population_covariance.jl):
//
//   population_local_weights  _population_local_weights! (:115-480): for each
//       proposal slot, its own samples' log weights normalised to weights, the
//       raw local ESS, the weighted raw mean, and -- when the ESS is below the
//       slot's threshold -- a bisection on a tempering power p in (0, 1) for
//       the largest p whose tempered weights w^p keep the ESS at or above the
//       threshold;
//   population_covariances    _fit_population_covariances! (:482-805): the
//       weighted covariance of each ready slot about its centre (the weighted
//       mean when tempered, else the slot's location); slots that are not
//       ready keep their current covariance (L L^T times the family's
//       covariance multiplier);
//   population_factors        _factor_population_covariances! (:807-957) and
//       _scale_population_factors! (:959-973): a lower Cholesky factor per
//       ready slot with LAPACK potrf's info convention (-1 for a non-finite
//       covariance, the failing column otherwise), then the Student-t scaling
//       sqrt((nu - 2) / nu).
//
// One CTA per proposal slot. Samples are d x N column-major (sample i
// contiguous); a slot's samples are the contiguous range starts[k] ..
// starts[k] + counts[k] - 1 (0-based), as the deterministic allocation lays
// them out. Sums run in FP64 whatever the storage type (the reference sums in
// the storage type), the Cholesky too; outputs are written in the storage type.
#include "issm_device.cuh"
#include "issm_internal.h"

namespace issm {

constexpr int kPopThreads = 256;
constexpr uint8_t kPopReady = 0, kPopAllZero = 1, kPopTemperingFailed = 2;

__device__ __forceinline__ double block_sum(double v, double *red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();  // red is reused across calls
    if (l == 0) red[w] = v;
    __syncthreads();
    double t = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += red[i];
    return t;
}

__device__ __forceinline__ double block_max(double v, double *red) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    double t = -INFINITY;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t = fmax(t, red[i]);
    return t;
}

// (sum e^{p (l - m)}, sum e^{2 p (l - m)}) over the slot's samples
template <typename T>
__device__ void tempered_sums(const T *lw, int64_t s0, int64_t cnt, double m, double p, double *red, double &s,
                              double &s2) {
    double a = 0.0, b = 0.0;
    for (int64_t i = threadIdx.x; i < cnt; i += blockDim.x) {
        const double w = exp(p * ((double)lw[s0 + i] - m));
        a += w;
        b += w * w;
    }
    s = block_sum(a, red);
    s2 = block_sum(b, red);
}

template <typename T>
__global__ void __launch_bounds__(kPopThreads) population_local_weights_kernel(
    const T *__restrict__ lw, const T *__restrict__ x, int d, const int64_t *__restrict__ starts,
    const int64_t *__restrict__ counts, const double *__restrict__ thresholds, double tolerance, int max_iterations,
    T *__restrict__ weights, T *__restrict__ local_ess, T *__restrict__ powers, uint8_t *__restrict__ status,
    T *__restrict__ raw_means) {
    __shared__ double red[32];
    const int k = blockIdx.x;
    const int64_t s0 = starts[k], cnt = counts[k];
    double mx = -INFINITY;
    for (int64_t i = threadIdx.x; i < cnt; i += blockDim.x) mx = fmax(mx, (double)lw[s0 + i]);
    mx = block_max(mx, red);
    if (mx == -INFINITY || cnt == 0) {
        if (threadIdx.x == 0) {
            local_ess[k] = T(0);
            powers[k] = T(0);
            status[k] = kPopAllZero;
        }
        return;
    }
    double s, s2;
    tempered_sums(lw, s0, cnt, mx, 1.0, red, s, s2);
    const double inv = 1.0 / s;
    for (int64_t i = threadIdx.x; i < cnt; i += blockDim.x)
        weights[s0 + i] = (T)(exp((double)lw[s0 + i] - mx) * inv);
    __syncthreads();
    if (raw_means != nullptr) {
        // the weighted raw mean, one coordinate per pass (coalesced over samples of a row)
        for (int c = 0; c < d; ++c) {
            double a = 0.0;
            for (int64_t i = threadIdx.x; i < cnt; i += blockDim.x)
                a += (double)weights[s0 + i] * (double)x[(s0 + i) * d + c];
            a = block_sum(a, red);
            if (threadIdx.x == 0) raw_means[(size_t)k * d + c] = (T)a;
        }
    }
    const double ess = s * s / s2;
    const double thr = thresholds[k];
    if (ess >= thr) {
        if (threadIdx.x == 0) {
            local_ess[k] = (T)ess;
            powers[k] = T(1);
            status[k] = kPopReady;
        }
        return;
    }
    // bisection: the largest power whose tempered ESS reaches the threshold
    double lo = 0.0, hi = 1.0, lo_ess = 0.0, lo_total = 0.0;
    for (int iter = 0; iter < max_iterations; ++iter) {
        const double p = 0.5 * (lo + hi);
        double ts, ts2;
        tempered_sums(lw, s0, cnt, mx, p, red, ts, ts2);
        const double e = ts * ts / ts2;
        if (e >= thr) {
            lo = p;
            lo_ess = e;
            lo_total = ts;
        } else {
            hi = p;
        }
        if (hi - lo <= tolerance) break;
    }
    if (lo > 0.0) {
        const double tinv = 1.0 / lo_total;
        for (int64_t i = threadIdx.x; i < cnt; i += blockDim.x)
            weights[s0 + i] = (T)(exp(lo * ((double)lw[s0 + i] - mx)) * tinv);
        if (threadIdx.x == 0) {
            local_ess[k] = (T)lo_ess;
            powers[k] = (T)lo;
            status[k] = kPopReady;
        }
    } else if (threadIdx.x == 0) {
        local_ess[k] = (T)ess;
        powers[k] = T(0);
        status[k] = kPopTemperingFailed;
    }
}

// Current covariance entry (r, c) of slot k of a bank: (L L^T)(r, c), or the
// squared diagonal/spherical scale, times the family's covariance multiplier
// nu / (nu - 2) (1 for Gaussian).
template <typename T> __device__ double bank_covariance(const issm_bank &b, int k, int r, int c) {
    const int d = b.dim;
    const T *sc = (const T *)b.scales;
    double v = 0.0;
    if (b.scale_kind == ISSM_SCALE_FACTOR) {
        const T *L = sc + (size_t)k * d * d;  // column-major: (r, j) at r + j d
        const int m = r < c ? r : c;
        for (int j = 0; j <= m; ++j) v += (double)L[r + (size_t)j * d] * (double)L[c + (size_t)j * d];
    } else if (r == c) {
        const double s = b.scale_kind == ISSM_SCALE_DIAGONAL ? (double)sc[(size_t)k * d + r] : (double)sc[k];
        v = s * s;
    }
    if (b.family == ISSM_STUDENT_T) {
        const double nu = (double)((const T *)b.dofs)[k];
        v *= nu / (nu - 2.0);
    }
    return v;
}

constexpr int kPopTile = 32;  // samples staged per pass of the covariance kernel

template <typename T>
__global__ void __launch_bounds__(kPopThreads) population_covariances_kernel(
    const T *__restrict__ x, int d, const T *__restrict__ weights, const T *__restrict__ powers,
    const uint8_t *__restrict__ status, const T *__restrict__ locations, issm_bank bank,
    const int64_t *__restrict__ starts, const int64_t *__restrict__ counts, T *__restrict__ centres,
    T *__restrict__ covs) {
    __shared__ double red[32];
    __shared__ double cen[64];
    __shared__ double zt[kPopTile][65];  // sqrt-free centred rows of the staged samples
    __shared__ double wt[kPopTile];
    const int k = blockIdx.x;
    const int64_t s0 = starts[k], cnt = counts[k];
    const bool ready = status[k] == kPopReady;
    const bool tempered = ready && (double)powers[k] < 1.0;
    // centre: the weighted mean when tempered, else the slot's location
    for (int c = 0; c < d; ++c) {
        double a = 0.0;
        if (tempered)
            for (int64_t i = threadIdx.x; i < cnt; i += blockDim.x)
                a += (double)weights[s0 + i] * (double)x[(s0 + i) * d + c];
        a = tempered ? block_sum(a, red) : (double)locations[(size_t)k * d + c];
        if (threadIdx.x == 0) {
            cen[c] = tempered ? (double)(T)a : a;  // the centre as stored
            centres[(size_t)k * d + c] = (T)a;
        }
    }
    __syncthreads();
    T *ck = covs + (size_t)k * d * d;
    const int tri = d * (d + 1) / 2;
    if (!ready) {
        for (int q = threadIdx.x; q < tri; q += blockDim.x) {
            int r = (int)((sqrtf(8.f * (float)q + 1.f) - 1.f) * 0.5f);
            if ((r + 1) * (r + 2) / 2 <= q) ++r;
            if (r * (r + 1) / 2 > q) --r;
            const int c = q - r * (r + 1) / 2;
            const T v = (T)bank_covariance<T>(bank, k, r, c);
            ck[r + (size_t)c * d] = v;
            ck[c + (size_t)r * d] = v;
        }
        return;
    }
    // lower triangle q -> (r, c); each thread keeps up to 9 entries (d <= 64: 2080 / 256 < 9)
    constexpr int kMaxPer = 9;
    double acc[kMaxPer];
    int er[kMaxPer], ec[kMaxPer];
#pragma unroll
    for (int u = 0; u < kMaxPer; ++u) {
        acc[u] = 0.0;
        const int q = threadIdx.x + u * kPopThreads;
        int r = 0, c = 0;
        if (q < tri) {
            r = (int)((sqrtf(8.f * (float)q + 1.f) - 1.f) * 0.5f);
            if ((r + 1) * (r + 2) / 2 <= q) ++r;
            if (r * (r + 1) / 2 > q) --r;
            c = q - r * (r + 1) / 2;
        }
        er[u] = r;
        ec[u] = c;
    }
    for (int64_t t0 = 0; t0 < cnt; t0 += kPopTile) {
        const int rows = (int)min((int64_t)kPopTile, cnt - t0);
        __syncthreads();
        for (int e = threadIdx.x; e < rows * d; e += blockDim.x) {
            const int r = e / d, c = e - r * d;
            zt[r][c] = (double)x[(s0 + t0 + r) * d + c] - cen[c];
        }
        for (int r = threadIdx.x; r < rows; r += blockDim.x) wt[r] = (double)weights[s0 + t0 + r];
        __syncthreads();
        for (int s = 0; s < rows; ++s) {
            const double w = wt[s];
#pragma unroll
            for (int u = 0; u < kMaxPer; ++u)
                if (threadIdx.x + u * kPopThreads < tri) acc[u] += w * zt[s][er[u]] * zt[s][ec[u]];
        }
    }
#pragma unroll
    for (int u = 0; u < kMaxPer; ++u) {
        if (threadIdx.x + u * kPopThreads < tri) {
            const T v = (T)acc[u];
            ck[er[u] + (size_t)ec[u] * d] = v;
            ck[ec[u] + (size_t)er[u] * d] = v;
        }
    }
}

// Unblocked Cholesky of each ready slot's covariance in FP64 in shared
// memory (d <= 64), potrf's info convention; zeros above the diagonal.
template <typename T>
__global__ void __launch_bounds__(kPopThreads) population_factors_kernel(const T *__restrict__ covs, int d,
                                                                       const uint8_t *__restrict__ status,
                                                                       const T *__restrict__ dofs,
                                                                       T *__restrict__ factors,
                                                                       int32_t *__restrict__ info) {
    __shared__ double A[64][65];
    __shared__ int s_info;
    const int k = blockIdx.x;
    if (status[k] != kPopReady) {
        if (threadIdx.x == 0) info[k] = 0;
        return;
    }
    const T *ck = covs + (size_t)k * d * d;
    int bad = 0;
    for (int e = threadIdx.x; e < d * d; e += blockDim.x) {
        const int r = e % d, c = e / d;
        const double v = (double)ck[e];
        bad |= !isfinite(v);
        A[r][c] = v;
    }
    bad = __syncthreads_or(bad);
    if (threadIdx.x == 0) s_info = bad ? -1 : 0;
    __syncthreads();
    if (!bad) {
        for (int j = 0; j < d; ++j) {
            if (threadIdx.x == 0) {
                double piv = A[j][j];
                for (int q = 0; q < j; ++q) piv -= A[j][q] * A[j][q];
                if (isfinite(piv) && piv > 0.0) A[j][j] = sqrt(piv);
                else s_info = j + 1;
            }
            __syncthreads();
            if (s_info != 0) break;
            const double dj = A[j][j];
            for (int r = j + 1 + threadIdx.x; r < d; r += blockDim.x) {
                double v = A[r][j];
                for (int q = 0; q < j; ++q) v -= A[r][q] * A[j][q];
                A[r][j] = v / dj;
            }
            __syncthreads();
        }
    }
    __syncthreads();
    const int inf = s_info;
    // the Student-t scaling sqrt((nu - 2) / nu) of _scale_population_factors!
    const double scale = dofs != nullptr ? sqrt(((double)dofs[k] - 2.0) / (double)dofs[k]) : 1.0;
    T *fk = factors + (size_t)k * d * d;
    for (int e = threadIdx.x; e < d * d; e += blockDim.x) {
        const int r = e % d, c = e / d;
        double v;
        if (inf == -1) v = (double)ck[e] * (r >= c ? 1.0 : 0.0);
        else v = r >= c ? A[r][c] : 0.0;
        fk[e] = (T)(v * scale);
    }
    if (threadIdx.x == 0) info[k] = inf;
}

int population_local_weights(const void *lw, const void *x, int d, int dtype, const int64_t *starts,
                             const int64_t *counts, const double *thresholds, int k, double tolerance,
                             int max_iterations, void *weights, void *local_ess, void *powers, uint8_t *status,
                             void *raw_means, cudaStream_t stream) {
    if (dtype == ISSM_F32) {
        population_local_weights_kernel<float><<<k, kPopThreads, 0, stream>>>(
            (const float *)lw, (const float *)x, d, starts, counts, thresholds, tolerance, max_iterations,
            (float *)weights, (float *)local_ess, (float *)powers, status, (float *)raw_means);
    } else {
        population_local_weights_kernel<double><<<k, kPopThreads, 0, stream>>>(
            (const double *)lw, (const double *)x, d, starts, counts, thresholds, tolerance, max_iterations,
            (double *)weights, (double *)local_ess, (double *)powers, status, (double *)raw_means);
    }
    note_launch();
    return (int)cudaGetLastError();
}

int population_covariances(const void *x, int d, int dtype, const void *weights, const void *powers,
                           const uint8_t *status, const void *locations, const issm_bank *bank,
                           const int64_t *starts, const int64_t *counts, int k, void *centres, void *covs,
                           cudaStream_t stream) {
    if (dtype == ISSM_F32) {
        population_covariances_kernel<float><<<k, kPopThreads, 0, stream>>>(
            (const float *)x, d, (const float *)weights, (const float *)powers, status, (const float *)locations,
            *bank, starts, counts, (float *)centres, (float *)covs);
    } else {
        population_covariances_kernel<double><<<k, kPopThreads, 0, stream>>>(
            (const double *)x, d, (const double *)weights, (const double *)powers, status,
            (const double *)locations, *bank, starts, counts, (double *)centres, (double *)covs);
    }
    note_launch();
    return (int)cudaGetLastError();
}

int population_factors(const void *covs, int d, int k, int dtype, const uint8_t *status, const void *dofs,
                       void *factors, int32_t *info, cudaStream_t stream) {
    if (dtype == ISSM_F32) {
        population_factors_kernel<float><<<k, kPopThreads, 0, stream>>>((const float *)covs, d, status,
                                                                        (const float *)dofs, (float *)factors,
                                                                        info);
    } else {
        population_factors_kernel<double><<<k, kPopThreads, 0, stream>>>((const double *)covs, d, status,
                                                                         (const double *)dofs, (double *)factors,
                                                                         info);
    }
    note_launch();
    return (int)cudaGetLastError();
}

}  // namespace issm
