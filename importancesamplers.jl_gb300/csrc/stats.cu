// stats.cu — result statistics on the device (src/statistics.jl):
//
//   weighted_sum      sum_i w_i x_i per coordinate with the self-normalised
//                     weights w_i = e^{l_i - m} / S of the result's summary
//                     (Statistics.mean(result) and, on f's values,
//                     Statistics.mean(f, result), :11-33): FP64 sums for FP64
//                     data, compensated FP32 sums merged in FP64 for FP32 data,
//                     per-block partials reduced in a fixed order (bitwise
//                     reproducible);
//   weighted_quantile component-wise weighted quantiles with the StatsBase
//                     generic-weight interpolation rule of _weighted_quantile
//                     (:114-154), which the reference evaluates on the host
//                     after sorting. Here no sort: for every (coordinate,
//                     probability) the element at which the cumulative weight
//                     of the value-sorted positive-weight samples first exceeds
//                     the threshold p (W - w_first) + w_first is found by a
//                     weighted most-significant-digit radix select (per-bin
//                     weight sums, FP64, fixed-order reduction), followed by
//                     the neighbours the interpolation needs.
//
// Samples are n x d row-major (sample i contiguous). Keys order like the
// values (see select.cu); a coordinate holding a NaN returns NaN, as the
// reference does.
#include "issm_device.cuh"
#include "issm_internal.h"

namespace issm {

constexpr int kSumThreads = 256;
constexpr int kSumTile = 64;  // samples per block-iteration staged in shared memory

// per-block partial sums of w_i x_i (d <= 64 per pass over coordinate blocks)
template <typename T>
__global__ void weighted_sum_partial_kernel(const T *__restrict__ x, int d, int64_t n, const T *__restrict__ lw,
                                            const double *__restrict__ summary, double *__restrict__ partial) {
    __shared__ double tile[kSumTile][65];
    __shared__ double ws[kSumTile];
    const double m = summary[0], inv = 1.0 / summary[1];
    const int c0 = blockIdx.y * 64, dc = min(64, d - c0);
    double acc = 0.0;  // thread t < dc owns coordinate c0 + t
    const int64_t tiles = (n + kSumTile - 1) / kSumTile;
    for (int64_t tt = blockIdx.x; tt < tiles; tt += gridDim.x) {
        const int64_t r0 = tt * kSumTile;
        const int rows = (int)min((int64_t)kSumTile, n - r0);
        __syncthreads();
        for (int e = threadIdx.x; e < rows * dc; e += blockDim.x) {
            const int r = e / dc, c = e - r * dc;
            tile[r][c] = (double)x[(r0 + r) * d + c0 + c];
        }
        for (int r = threadIdx.x; r < rows; r += blockDim.x) {
            const double l = (double)lw[r0 + r];
            ws[r] = l == -INFINITY ? 0.0 : exp(l - m) * inv;
        }
        __syncthreads();
        if (threadIdx.x < dc)
            for (int r = 0; r < rows; ++r)
                if (ws[r] != 0.0) acc += ws[r] * tile[r][threadIdx.x];
    }
    if (threadIdx.x < dc) partial[((size_t)blockIdx.x * gridDim.y + blockIdx.y) * 64 + threadIdx.x] = acc;
}

// FP32 samples: per-thread compensated FP32 (Kahan) sums of w x with w in
// FP32 (expf of the FP32 log weight less the summary's max, times 1/S), four
// row groups per coordinate merged in FP64 in a fixed order. In FP64 the pass
// ran on this GPU's narrow FP64 pipe (a conversion and an FMA per element)
// at several times its memory time. Thread t owns coordinate t % 64 of every
// fourth row, so a warp reads consecutive coordinates of one row.
__global__ void __launch_bounds__(kSumThreads) weighted_sum_partial_f32_kernel(const float *__restrict__ x, int d,
                                                                              int64_t n,
                                                                              const float *__restrict__ lw,
                                                                              const double *__restrict__ summary,
                                                                              double *__restrict__ partial) {
    __shared__ float ws[kSumTile];
    __shared__ double s4[4][64];
    const float m = (float)summary[0], inv = (float)(1.0 / summary[1]);
    const int c0 = blockIdx.y * 64, dc = min(64, d - c0);
    const int c = threadIdx.x & 63, rg = threadIdx.x >> 6;
    float s = 0.f, k = 0.f;
    const int64_t tiles = (n + kSumTile - 1) / kSumTile;
    for (int64_t tt = blockIdx.x; tt < tiles; tt += gridDim.x) {
        const int64_t r0 = tt * kSumTile;
        const int rows = (int)min((int64_t)kSumTile, n - r0);
        __syncthreads();
        if (threadIdx.x < rows) {
            const float l = lw[r0 + threadIdx.x];
            ws[threadIdx.x] = l == -INFINITY ? 0.f : expf(l - m) * inv;
        }
        __syncthreads();
        if (c < dc) {
#pragma unroll 4
            for (int r = rg; r < rows; r += 4) {
                const float w = ws[r];
                if (w == 0.f) continue;  // a zero weight contributes nothing (not even a NaN)
                const float y = fmaf(w, x[(r0 + r) * d + c0 + c], -k);
                const float t = s + y;
                k = (t - s) - y;
                s = t;
            }
        }
    }
    s4[rg][c] = (double)s - (double)k;
    __syncthreads();
    if (threadIdx.x < dc)
        partial[((size_t)blockIdx.x * gridDim.y + blockIdx.y) * 64 + threadIdx.x] =
            ((s4[0][threadIdx.x] + s4[1][threadIdx.x]) + s4[2][threadIdx.x]) + s4[3][threadIdx.x];
}

__global__ void weighted_sum_finish_kernel(const double *__restrict__ partial, int blocks, int d, double *out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d) return;
    const int cb = c / 64, cc = c % 64, ncb = (d + 63) / 64;
    double s = 0.0;
    for (int b = 0; b < blocks; ++b) s += partial[((size_t)b * ncb + cb) * 64 + cc];
    out[c] = s;
}

constexpr int kSumBlocksPerSm = 8;  // enough loads in flight to stream the samples

static int sum_blocks(int64_t n) {
    const int64_t t = (n + kSumTile - 1) / kSumTile;
    const int64_t cap = (int64_t)device_sms() * kSumBlocksPerSm;
    return (int)(t < cap ? (t < 1 ? 1 : t) : cap);
}

size_t weighted_sum_workspace_bytes(int64_t n, int d) {
    return sizeof(double) * (size_t)kSMs * kSumBlocksPerSm * (size_t)((d + 63) / 64) * 64;
}

int weighted_sum(const void *x, int d, int64_t n, const void *lw, int dtype, const double *summary, double *out,
                 void *ws, cudaStream_t stream) {
    const int blocks = sum_blocks(n);
    const dim3 grid(blocks, (d + 63) / 64);
    double *partial = (double *)ws;
    if (dtype == ISSM_F32)
        weighted_sum_partial_f32_kernel<<<grid, kSumThreads, 0, stream>>>((const float *)x, d, n,
                                                                         (const float *)lw, summary, partial);
    else
        weighted_sum_partial_kernel<double><<<grid, kSumThreads, 0, stream>>>((const double *)x, d, n,
                                                                             (const double *)lw, summary, partial);
    note_launch();
    weighted_sum_finish_kernel<<<(d + 127) / 128, 128, 0, stream>>>(partial, blocks, d, out);
    note_launch();
    return (int)cudaGetLastError();
}

// ---- weighted quantile ---------------------------------------------------------
template <typename T> struct QKey;
template <> struct QKey<float> {
    using K = unsigned long long;
    static constexpr int kBits = 32;
    __device__ static K key(float v) {
        const uint32_t u = __float_as_uint(v);
        return (K)((u & 0x80000000u) ? ~u : (u | 0x80000000u));
    }
    __device__ static double value(K k) {
        const uint32_t u = (uint32_t)k;
        return (double)__uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
    }
};
template <> struct QKey<double> {
    using K = unsigned long long;
    static constexpr int kBits = 64;
    __device__ static K key(double v) {
        const unsigned long long u = (unsigned long long)__double_as_longlong(v);
        return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
    }
    __device__ static double value(K k) {
        return __longlong_as_double((long long)((k & 0x8000000000000000ull) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k));
    }
};

constexpr int kQBlocks = 32;    // blocks per (coordinate, probability) problem
constexpr int kQThreads = 256;

// Per problem: [0] prefix key, [1] state flags, then doubles: threshold,
// remaining threshold, cumulative weight below the prefix, total W, w_first,
// nan flag; plus the partial bins kQBlocks x 256 and scratch for the final
// reductions.
struct QState {
    unsigned long long prefix;
    int beyond;     // the threshold is not exceeded: the result is the largest value
    int nan;
    double thr, below, total, w_first;
    unsigned long long min_key;     // smallest positive-weight key
    long long min_key_index;        // its first index
};
struct QScratch {
    double bins[kQBlocks][256];
    unsigned long long kmin[kQBlocks];
    long long imin[kQBlocks];
    double tot[kQBlocks];
    int nan[kQBlocks];
    unsigned long long klow[kQBlocks];   // largest key below the selected key
    long long iup[kQBlocks];             // first index holding the selected key
};

__device__ __forceinline__ double qweight(double l, double m, double inv) {
    return l == -INFINITY ? 0.0 : exp(l - m) * inv;
}

// pass 0: total weight, NaN flag, smallest key and its first index (per block)
template <typename T>
__global__ void quantile_setup_kernel(const T *__restrict__ x, int d, int64_t n, const T *__restrict__ lw,
                                      const double *__restrict__ summary, QScratch *__restrict__ scr) {
    using QK = QKey<T>;
    const int prob = blockIdx.y, c = prob % d;
    const double m = summary[0], inv = 1.0 / summary[1];
    double tot = 0.0;
    int nan = 0;
    unsigned long long kmin = ~0ull;
    long long imin = LLONG_MAX;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const T v = x[i * d + c];
        if (isnan(v)) nan = 1;
        const double w = qweight((double)lw[i], m, inv);
        if (w > 0.0 && !isnan(v)) {
            tot += w;
            const unsigned long long k = QK::key(v);
            if (k < kmin || (k == kmin && i < imin)) { kmin = k; imin = i; }
        }
    }
    __shared__ double s_tot[kQThreads];
    __shared__ unsigned long long s_k[kQThreads];
    __shared__ long long s_i[kQThreads];
    __shared__ int s_nan[kQThreads];
    s_tot[threadIdx.x] = tot;
    s_k[threadIdx.x] = kmin;
    s_i[threadIdx.x] = imin;
    s_nan[threadIdx.x] = nan;
    __syncthreads();
    for (int o = kQThreads / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            s_tot[threadIdx.x] += s_tot[threadIdx.x + o];
            s_nan[threadIdx.x] |= s_nan[threadIdx.x + o];
            const unsigned long long k2 = s_k[threadIdx.x + o];
            const long long i2 = s_i[threadIdx.x + o];
            if (k2 < s_k[threadIdx.x] || (k2 == s_k[threadIdx.x] && i2 < s_i[threadIdx.x])) {
                s_k[threadIdx.x] = k2;
                s_i[threadIdx.x] = i2;
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        QScratch &s = scr[prob];
        s.tot[blockIdx.x] = s_tot[0];
        s.nan[blockIdx.x] = s_nan[0];
        s.kmin[blockIdx.x] = s_k[0];
        s.imin[blockIdx.x] = s_i[0];
    }
}

// one thread per problem: W, w_first, the threshold, the state
template <typename T>
__global__ void quantile_init_kernel(int nprob_total, int d, const T *__restrict__ x, const T *__restrict__ lw,
                                     const double *__restrict__ summary, const double *__restrict__ probs,
                                     QScratch *__restrict__ scr, QState *__restrict__ st) {
    const int prob = blockIdx.x * blockDim.x + threadIdx.x;
    if (prob >= nprob_total) return;
    const QScratch &s = scr[prob];
    double tot = 0.0;
    int nan = 0;
    unsigned long long kmin = ~0ull;
    long long imin = LLONG_MAX;
    for (int b = 0; b < kQBlocks; ++b) {
        tot += s.tot[b];
        nan |= s.nan[b];
        if (s.kmin[b] < kmin || (s.kmin[b] == kmin && s.imin[b] < imin)) { kmin = s.kmin[b]; imin = s.imin[b]; }
    }
    const double m = summary[0], inv = 1.0 / summary[1];
    QState &q = st[prob];
    q.prefix = 0ull;
    q.nan = nan;
    q.total = tot;
    q.min_key = kmin;
    q.min_key_index = imin;
    q.w_first = imin == LLONG_MAX ? 0.0 : qweight((double)lw[imin], m, inv);
    const double p = probs[prob / d];
    q.thr = p * (tot - q.w_first) + q.w_first;
    q.below = 0.0;
    q.beyond = 0;
}

// weighted histogram of one 8-bit digit over the keys matching the prefix
template <typename T>
__global__ void quantile_hist_kernel(const T *__restrict__ x, int d, int64_t n, const T *__restrict__ lw,
                                     const double *__restrict__ summary, int digit, const QState *__restrict__ st,
                                     QScratch *__restrict__ scr) {
    using QK = QKey<T>;
    const int prob = blockIdx.y, c = prob % d;
    __shared__ double bins[256];
    for (int b = threadIdx.x; b < 256; b += blockDim.x) bins[b] = 0.0;
    __syncthreads();
    const QState &q = st[prob];
    if (!q.nan && !q.beyond) {
        const double m = summary[0], inv = 1.0 / summary[1];
        const int shift = QK::kBits - 8 * (digit + 1);
        const unsigned long long hi_mask =
            digit == 0 ? 0ull : ((~0ull << (shift + 8)) & (QK::kBits == 32 ? 0xFFFFFFFFull : ~0ull));
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
            const double w = qweight((double)lw[i], m, inv);
            if (!(w > 0.0)) continue;
            const unsigned long long k = QK::key(x[i * d + c]);
            if ((k & hi_mask) == (q.prefix & hi_mask)) atomicAdd(&bins[(k >> shift) & 0xFFu], w);
        }
    }
    __syncthreads();
    for (int b = threadIdx.x; b < 256; b += blockDim.x) scr[prob].bins[blockIdx.x][b] = bins[b];
}

// one thread per problem: fixed-order bin sums; the first bin whose
// cumulative weight exceeds the threshold extends the prefix
template <typename T>
__global__ void quantile_step_kernel(int nprob_total, int digit, QScratch *__restrict__ scr,
                                     QState *__restrict__ st) {
    using QK = QKey<T>;
    const int prob = blockIdx.x * blockDim.x + threadIdx.x;
    if (prob >= nprob_total) return;
    QState &q = st[prob];
    if (q.nan || q.beyond) return;
    const QScratch &s = scr[prob];
    const int shift = QK::kBits - 8 * (digit + 1);
    double cum = q.below;
    for (int b = 0; b < 256; ++b) {
        double w = 0.0;
        for (int k = 0; k < kQBlocks; ++k) w += s.bins[k][b];
        if (cum + w > q.thr) {
            q.prefix |= (unsigned long long)b << shift;
            q.below = cum;
            return;
        }
        cum += w;
    }
    q.beyond = 1;  // rounding left the threshold at or above W: the largest value
}

// after the digits: the largest key below the selected one and the first
// index holding the selected key (per block)
template <typename T>
__global__ void quantile_neighbours_kernel(const T *__restrict__ x, int d, int64_t n, const T *__restrict__ lw,
                                           const double *__restrict__ summary, const QState *__restrict__ st,
                                           QScratch *__restrict__ scr) {
    using QK = QKey<T>;
    const int prob = blockIdx.y, c = prob % d;
    const QState &q = st[prob];
    const double m = summary[0], inv = 1.0 / summary[1];
    unsigned long long klow = 0ull;  // 0 = none (no finite or NaN-free value maps to key 0)
    long long iup = LLONG_MAX;
    const bool want_max = q.beyond != 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (!(qweight((double)lw[i], m, inv) > 0.0)) continue;
        const unsigned long long k = QK::key(x[i * d + c]);
        if (want_max) {
            if (k > klow) klow = k;  // the largest key
        } else {
            if (k < q.prefix && k > klow) klow = k;
            if (k == q.prefix && i < iup) iup = i;
        }
    }
    __shared__ unsigned long long s_k[kQThreads];
    __shared__ long long s_i[kQThreads];
    s_k[threadIdx.x] = klow;
    s_i[threadIdx.x] = iup;
    __syncthreads();
    for (int o = kQThreads / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            if (s_k[threadIdx.x + o] > s_k[threadIdx.x]) s_k[threadIdx.x] = s_k[threadIdx.x + o];
            if (s_i[threadIdx.x + o] < s_i[threadIdx.x]) s_i[threadIdx.x] = s_i[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        scr[prob].klow[blockIdx.x] = s_k[0];
        scr[prob].iup[blockIdx.x] = s_i[0];
    }
}

// the interpolation of _weighted_quantile (src/statistics.jl:140-153)
template <typename T>
__global__ void quantile_finish_kernel(int nprob_total, int d, const T *__restrict__ lw,
                                       const double *__restrict__ summary, const QScratch *__restrict__ scr,
                                       const QState *__restrict__ st, double *__restrict__ out) {
    using QK = QKey<T>;
    const int prob = blockIdx.x * blockDim.x + threadIdx.x;
    if (prob >= nprob_total) return;
    const QState &q = st[prob];
    const QScratch &s = scr[prob];
    unsigned long long klow = 0ull;
    long long iup = LLONG_MAX;
    for (int b = 0; b < kQBlocks; ++b) {
        if (s.klow[b] > klow) klow = s.klow[b];
        if (s.iup[b] < iup) iup = s.iup[b];
    }
    double v;
    if (q.nan) {
        v = nan("");
    } else if (q.beyond) {
        v = QK::value(klow);  // the largest value
    } else {
        const double m = summary[0], inv = 1.0 / summary[1];
        const double v_up = QK::value(q.prefix), w_up = qweight((double)lw[iup], m, inv);
        if (q.below + w_up > q.thr) {
            // lower = the last sample below the selected value
            const double v_lo = QK::value(klow);
            const double f = (q.thr - q.below) / w_up;
            if (f == 0.0) {
                v = v_lo;
            } else {
                const double diff = v_up - v_lo;
                v = isfinite(diff) ? v_lo + f * diff : (1.0 - f) * v_lo + f * v_up;
            }
        } else {
            v = v_up;  // lower and upper both hold the selected value
        }
    }
    out[prob] = (double)(T)v;
}

size_t weighted_quantile_workspace_bytes(int d, int nprob) {
    const size_t p = (size_t)d * (size_t)nprob;
    return p * (sizeof(QScratch) + sizeof(QState)) + 256;
}

template <typename T>
static int weighted_quantile_t(const T *x, int d, int64_t n, const T *lw, const double *summary, const double *probs,
                               int nprob, double *out, void *ws, cudaStream_t stream) {
    const int P = d * nprob;
    QScratch *scr = (QScratch *)ws;
    QState *st = (QState *)((char *)ws + (size_t)P * sizeof(QScratch));
    const dim3 grid(kQBlocks, P);
    const int pb = (P + 127) / 128;
    quantile_setup_kernel<T><<<grid, kQThreads, 0, stream>>>(x, d, n, lw, summary, scr);
    note_launch();
    quantile_init_kernel<T><<<pb, 128, 0, stream>>>(P, d, x, lw, summary, probs, scr, st);
    note_launch();
    for (int digit = 0; digit < QKey<T>::kBits / 8; ++digit) {
        quantile_hist_kernel<T><<<grid, kQThreads, 0, stream>>>(x, d, n, lw, summary, digit, st, scr);
        note_launch();
        quantile_step_kernel<T><<<pb, 128, 0, stream>>>(P, digit, scr, st);
        note_launch();
    }
    quantile_neighbours_kernel<T><<<grid, kQThreads, 0, stream>>>(x, d, n, lw, summary, st, scr);
    note_launch();
    quantile_finish_kernel<T><<<pb, 128, 0, stream>>>(P, d, lw, summary, scr, st, out);
    note_launch();
    return (int)cudaGetLastError();
}

int weighted_quantile(const void *x, int d, int64_t n, const void *lw, int dtype, const double *summary,
                      const double *probs, int nprob, double *out, void *ws, cudaStream_t stream) {
    if (dtype == ISSM_F32)
        return weighted_quantile_t<float>((const float *)x, d, n, (const float *)lw, summary, probs, nprob, out, ws,
                                          stream);
    return weighted_quantile_t<double>((const double *)x, d, n, (const double *)lw, summary, probs, nprob, out, ws,
                                       stream);
}

}  // namespace issm
