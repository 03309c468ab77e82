// reduce.cu — log-weight reductions (HBM-bound, one read of the log weights).
//
// logweight_summary: single pass; each thread keeps an online (max, S, S2)
// with S = sum exp(l - max) computed in the weight dtype (FP32 data: Kahan
// FP32 per thread, then compensated FP32 pairs; FP64 data: FP64); warps and
// blocks merge with the reference's rescaling rule
// (_merge_logweight_moments, src/execution.jl:166-173); the last block to
// finish merges the per-block partials, so one launch yields the final three
// FP64 words with no host round trip.
// resampling_cdf: exp(l - max) in the weight dtype, an FP64 three-phase scan,
// and cdf = prefix / total rounded to the weight dtype
// (_resampling_cdf!, src/resampling.jl:199-225).
#include "issm_device.cuh"
#include "issm_internal.h"
#include "scan.cuh"

namespace issm {

struct Moments3 {
    double m, s, s2;
};

// exp of a difference of two maxima; the maxima are log weights of dtype T,
// so the factor is formed in T (FP64 exponentials are slow on this GPU and
// add nothing for FP32 data).
template <typename T> __device__ __forceinline__ double scale_factor(double a, double b) {
    return (double)dexp((T)(a - b));
}

__device__ __forceinline__ double warp_max(double v) {
    for (int off = 16; off > 0; off >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, off));
    return v;
}
__device__ __forceinline__ double warp_sum(double v) {
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

// Block-wide merge: take the block maximum first, then rescale every
// thread's sums once and add them (one exponential per thread).
template <typename T> __device__ Moments3 block_merge3(Moments3 v) {
    __shared__ double red[3][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    double m = warp_max(v.s == 0.0 ? -INFINITY : v.m);
    if (lane == 0) red[0][warp] = m;
    __syncthreads();
    double M = -INFINITY;
    for (int w = 0; w < nw; ++w) M = fmax(M, red[0][w]);
    double s = 0.0, s2 = 0.0;
    if (v.s != 0.0) {
        const double f = scale_factor<T>(v.m, M);
        s = v.s * f;
        s2 = v.s2 * (f * f);
    }
    s = warp_sum(s);
    s2 = warp_sum(s2);
    __syncthreads();
    if (lane == 0) {
        red[1][warp] = s;
        red[2][warp] = s2;
    }
    __syncthreads();
    double ts = 0.0, ts2 = 0.0;
    for (int w = 0; w < nw; ++w) {
        ts += red[1][w];
        ts2 += red[2][w];
    }
    __syncthreads();
    return Moments3{M, ts, ts2};
}

// Per-thread running (max, S, S2). FP64 data accumulates in FP64; FP32 data
// accumulates in FP32 with Kahan compensation (error about 2 ulp of the
// thread's sum however many terms it takes, and none of the slow FP64
// additions per element); its merges above the thread carry hi + lo FP32
// pairs (summary_finish below).
template <typename T> struct ThreadSums {
    T m = -num<T>::inf();
    double s = 0.0, s2 = 0.0;
    __device__ __forceinline__ void add(T l) {
        if (l == -num<T>::inf()) return;
        if (l > m) {
            if (m != -num<T>::inf()) {
                const double r = (double)dexp(m - l);
                s *= r;
                s2 *= r * r;
            }
            m = l;
        }
        const double e = (double)dexp(l - m);
        s += e;
        s2 += e * e;
    }
    __device__ __forceinline__ Moments3 result() const { return Moments3{(double)m, s, s2}; }
};
template <> struct ThreadSums<float> {
    float m = -INFINITY;
    float s = 0.f, cs = 0.f, s2 = 0.f, cs2 = 0.f;
    __device__ __forceinline__ static void kahan(float &sum, float &c, float x) {
        const float y = x - c;
        const float t = sum + y;
        c = (t - sum) - y;
        sum = t;
    }
    __device__ __forceinline__ void add(float l) {
        if (l == -INFINITY) return;
        if (l > m) {
            if (m != -INFINITY) {
                const float r = expf(m - l);
                s *= r;
                cs *= r;
                s2 *= r * r;
                cs2 *= r * r;
            }
            m = l;
        }
        const float e = expf(l - m);
        kahan(s, cs, e);
        kahan(s2, cs2, e * e);
    }
    __device__ __forceinline__ Moments3 result() const {
        return Moments3{(double)m, (double)s - (double)cs, (double)s2 - (double)cs2};
    }
};

// Block merge of the threads' (max, S, S2), then the last block to finish
// merges the per-block partials in the same launch and writes the FP64 words.
// FP64 data: FP64 throughout.
__device__ void summary_finish(const ThreadSums<double> &ts, double *out, Moments3 *partials,
                               unsigned int *counter) {
    Moments3 v = block_merge3<double>(ts.result());
    __shared__ bool last;
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = v;
        __threadfence();
        unsigned int done = atomicAdd(counter, 1u);
        last = (done == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    // the last block merges the per-block partials the same way
    const volatile double *pv = reinterpret_cast<const volatile double *>(partials);
    double pm = -INFINITY, ps = 0.0, ps2 = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
        const double bm = pv[3 * b], bs = pv[3 * b + 1], bs2 = pv[3 * b + 2];
        if (bs == 0.0) continue;
        if (ps == 0.0 || bm > pm) {
            if (ps != 0.0) {
                const double f = scale_factor<double>(pm, bm);
                ps *= f;
                ps2 *= f * f;
            }
            pm = bm;
        }
        const double f = scale_factor<double>(bm, pm);
        ps += bs * f;
        ps2 += bs2 * (f * f);
    }
    const Moments3 acc = block_merge3<double>(Moments3{pm, ps, ps2});
    if (threadIdx.x == 0) {
        out[0] = acc.s == 0.0 ? -INFINITY : acc.m;
        out[1] = acc.s;
        out[2] = acc.s2;
        *counter = 0u;
    }
}

// FP32 data: every merge in FP32 with the sums carried as unevaluated pairs
// hi + lo (error-free two-sum; about 44 significant bits), because FP64
// instructions hold a warp's FP64 pipe for about 64 cycles on this GPU and a
// few dozen of them per thread would cost more than the pass's HBM traffic.
// Only the last block's three output words are formed in FP64.
struct Pair {
    float h, l;
};
__device__ __forceinline__ Pair pair_add(Pair a, Pair b) {
    const float s = a.h + b.h, bb = s - a.h;
    const float e = ((a.h - (s - bb)) + (b.h - bb)) + (a.l + b.l);
    const float h = s + e;
    return Pair{h, e - (h - s)};
}
__device__ __forceinline__ Pair pair_scale(Pair a, float f) {
    const float p = a.h * f;
    const float l = fmaf(a.l, f, fmaf(a.h, f, -p));
    const float h = p + l;
    return Pair{h, l - (h - p)};
}
__device__ __forceinline__ Pair shfl_pair(Pair a, int off) {
    return Pair{__shfl_xor_sync(0xffffffffu, a.h, off), __shfl_xor_sync(0xffffffffu, a.l, off)};
}
struct Partial3f {
    float m;
    Pair s, s2;
};
static_assert(sizeof(Partial3f) <= sizeof(Moments3), "FP32 partials reuse the FP64 partial slots");

// block max of m over entries with s != 0, then sum s f, s2 f^2 with f = exp(m - M)
__device__ Partial3f block_merge3f(float m, Pair s, Pair s2) {
    __shared__ float red_m[32];
    __shared__ Pair red_s[32], red_s2[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    const bool live = s.h != 0.f;
    float wm = live ? m : -INFINITY;
    for (int off = 16; off > 0; off >>= 1) wm = fmaxf(wm, __shfl_xor_sync(0xffffffffu, wm, off));
    if (lane == 0) red_m[warp] = wm;
    __syncthreads();
    float M = -INFINITY;
    for (int w = 0; w < nw; ++w) M = fmaxf(M, red_m[w]);
    Pair a{0.f, 0.f}, b{0.f, 0.f};
    if (live) {
        const float f = expf(m - M);
        a = pair_scale(s, f);
        b = pair_scale(s2, f * f);
    }
    for (int off = 16; off > 0; off >>= 1) {
        a = pair_add(a, shfl_pair(a, off));
        b = pair_add(b, shfl_pair(b, off));
    }
    if (lane == 0) {
        red_s[warp] = a;
        red_s2[warp] = b;
    }
    __syncthreads();
    Pair ta{0.f, 0.f}, tb{0.f, 0.f};
    for (int w = 0; w < nw; ++w) {
        ta = pair_add(ta, red_s[w]);
        tb = pair_add(tb, red_s2[w]);
    }
    __syncthreads();
    return Partial3f{M, ta, tb};
}

__device__ void summary_finish(const ThreadSums<float> &ts, double *out, Moments3 *partials_d,
                               unsigned int *counter) {
    Partial3f *partials = reinterpret_cast<Partial3f *>(partials_d);
    const Partial3f v = block_merge3f(ts.m, Pair{ts.s, -ts.cs}, Pair{ts.s2, -ts.cs2});
    __shared__ bool last;
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = v;
        __threadfence();
        unsigned int done = atomicAdd(counter, 1u);
        last = (done == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    // the last block: this thread's partials about their own maximum, then the block merge
    const volatile float *pv = reinterpret_cast<const volatile float *>(partials);
    constexpr int kW = sizeof(Partial3f) / sizeof(float);
    float pm = -INFINITY;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
        if (pv[kW * b + 1] != 0.f) pm = fmaxf(pm, pv[kW * b]);
    Pair ps{0.f, 0.f}, ps2{0.f, 0.f};
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
        const Pair bs{pv[kW * b + 1], pv[kW * b + 2]}, bs2{pv[kW * b + 3], pv[kW * b + 4]};
        if (bs.h == 0.f) continue;
        const float f = expf(pv[kW * b] - pm);
        ps = pair_add(ps, pair_scale(bs, f));
        ps2 = pair_add(ps2, pair_scale(bs2, f * f));
    }
    const Partial3f acc = block_merge3f(pm, ps, ps2);
    if (threadIdx.x == 0) {
        const double S = (double)acc.s.h + (double)acc.s.l;
        out[0] = S == 0.0 ? -INFINITY : (double)acc.m;
        out[1] = S;
        out[2] = (double)acc.s2.h + (double)acc.s2.l;
        *counter = 0u;
    }
}

template <typename T>
__global__ void __launch_bounds__(256) summary_kernel(const T *__restrict__ lw, int64_t n, double *out,
                                                      Moments3 *partials, unsigned int *counter) {
    ThreadSums<T> ts;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (sizeof(T) == 4 && (reinterpret_cast<uintptr_t>(lw) & 15) == 0) {
        // four weights per load; the tail (< 4 weights) goes to the first threads
        const int64_t n4 = n >> 2;
        const float4 *lw4 = reinterpret_cast<const float4 *>(lw);
        for (int64_t i = t0; i < n4; i += stride) {
            const float4 q = lw4[i];
            ts.add((T)q.x);
            ts.add((T)q.y);
            ts.add((T)q.z);
            ts.add((T)q.w);
        }
        if (t0 < (n & 3)) ts.add(lw[(n4 << 2) + t0]);
    } else {
        for (int64_t i = t0; i < n; i += stride) ts.add(lw[i]);
    }
    summary_finish(ts, out, partials, counter);
}

// AMIS log weights of rounds 1..t and their summary in one pass
// (_form_amis_logweights_kernel!, src/amis_execution.jl:107-134, then
// _logweight_summary): logw_i = logtarget_i - (lognum_i - logtotal) for
// round_ids[i] != 0, recording invalid weights; only the weights written
// enter the summary.
template <typename T>
__global__ void __launch_bounds__(256) form_summary_kernel(const T *__restrict__ lt, const T *__restrict__ lnum,
                                                           const int64_t *__restrict__ round_ids, T logtotal,
                                                           int64_t n, T *__restrict__ lw, uint64_t *failures,
                                                           double *out, Moments3 *partials, unsigned int *counter) {
    ThreadSums<T> ts;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    auto one = [&](int64_t i, T target, T num) {
        T v;
        const uint16_t r = subtract_logweight(target, num - logtotal, &v);
        if (r) {
            record_failure(failures, i + 1, 0, r);
        } else {
            lw[i] = v;
            ts.add(v);
        }
    };
    const bool vec = sizeof(T) == 4 && ((reinterpret_cast<uintptr_t>(lt) | reinterpret_cast<uintptr_t>(lnum) |
                                         reinterpret_cast<uintptr_t>(lw) | reinterpret_cast<uintptr_t>(round_ids)) & 15) == 0;
    int64_t done = 0;
    if (vec) {
        // four samples per iteration: 16-byte loads of both inputs and the round ids
        const int64_t n4 = n >> 2;
        for (int64_t q = t0; q < n4; q += stride) {
            const float4 a = reinterpret_cast<const float4 *>(lt)[q];
            const float4 b = reinterpret_cast<const float4 *>(lnum)[q];
            bool keep[4] = {true, true, true, true};
            if (round_ids) {
                const longlong2 r0 = reinterpret_cast<const longlong2 *>(round_ids)[2 * q];
                const longlong2 r1 = reinterpret_cast<const longlong2 *>(round_ids)[2 * q + 1];
                keep[0] = r0.x != 0; keep[1] = r0.y != 0; keep[2] = r1.x != 0; keep[3] = r1.y != 0;
            }
            const int64_t i = q << 2;
            if (keep[0]) one(i, (T)a.x, (T)b.x);
            if (keep[1]) one(i + 1, (T)a.y, (T)b.y);
            if (keep[2]) one(i + 2, (T)a.z, (T)b.z);
            if (keep[3]) one(i + 3, (T)a.w, (T)b.w);
        }
        done = n4 << 2;
    }
    for (int64_t i = done + t0; i < n; i += stride) {
        if (round_ids && round_ids[i] == 0) continue;
        one(i, lt[i], lnum[i]);
    }
    summary_finish(ts, out, partials, counter);
}

static int summary_blocks(int64_t n) {
    int64_t b = (n + 256 * 16 - 1) / (256 * 16);
    if (b > kSMs * 8) b = kSMs * 8;
    return b < 1 ? 1 : (int)b;
}

// Workspace layout shared by the summary and the CDF:
//   [0, 4)      completion counter of the summary kernel
//   [128, 152)  summary words written by resampling_cdf
//   [256, ...)  per-block summary partials, later reused as scan tile sums
size_t reduce_workspace_bytes(int64_t n) {
    size_t a = sizeof(Moments3) * (size_t)(kSMs * 8);
    size_t tiles = (size_t)((n + kScanTile - 1) / kScanTile) + 1;
    size_t b = sizeof(double) * tiles;
    return 256 + (a > b ? a : b);
}

static int summary_launch(const void *lw, int64_t n, int dtype, double *out, void *ws, cudaStream_t stream) {
    unsigned int *counter = (unsigned int *)ws;
    Moments3 *partials = (Moments3 *)((char *)ws + 256);
    cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(unsigned int), stream);
    if (e != cudaSuccess) return (int)e;
    const int blocks = summary_blocks(n);
    if (dtype == ISSM_F32)
        { summary_kernel<float><<<blocks, 256, 0, stream>>>((const float *)lw, n, out, partials, counter); note_launch(); }
    else
        { summary_kernel<double><<<blocks, 256, 0, stream>>>((const double *)lw, n, out, partials, counter); note_launch(); }
    return (int)cudaGetLastError();
}

int logweight_summary(const void *lw, int64_t n, int dtype, double *out, void *ws, size_t ws_bytes,
                      cudaStream_t stream) {
    if (ws_bytes < reduce_workspace_bytes(n)) return ISSM_E_WORKSPACE;
    return summary_launch(lw, n, dtype, out, ws, stream);
}

int amis_form_summary(const void *lt, const void *lnum, const int64_t *round_ids, double logtotal, int64_t n,
                      int dtype, void *lw, uint64_t *failures, double *out, void *ws, size_t ws_bytes,
                      cudaStream_t stream) {
    if (ws_bytes < reduce_workspace_bytes(n)) return ISSM_E_WORKSPACE;
    unsigned int *counter = (unsigned int *)ws;
    Moments3 *partials = (Moments3 *)((char *)ws + 256);
    cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(unsigned int), stream);
    if (e != cudaSuccess) return (int)e;
    const int blocks = summary_blocks(n);
    if (dtype == ISSM_F32)
        { form_summary_kernel<float><<<blocks, 256, 0, stream>>>((const float *)lt, (const float *)lnum, round_ids,
                                                               (float)logtotal, n, (float *)lw, failures, out,
                                                               partials, counter); note_launch(); }
    else
        { form_summary_kernel<double><<<blocks, 256, 0, stream>>>((const double *)lt, (const double *)lnum,
                                                                round_ids, logtotal, n, (double *)lw, failures,
                                                                out, partials, counter); note_launch(); }
    return (int)cudaGetLastError();
}

template <typename T>
__global__ void normalize_kernel(const T *__restrict__ lw, int64_t n, const double *__restrict__ summary,
                                 T *__restrict__ w) {
    const T m = (T)summary[0];
    const T inv = (T)(1.0 / summary[1]);
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        w[i] = dexp(lw[i] - m) * inv;
}

int normalize(const void *lw, int64_t n, int dtype, const double *summary, void *w, cudaStream_t stream) {
    const int blocks = grid_for(n, 256, 4);
    if (dtype == ISSM_F32)
        { normalize_kernel<float><<<blocks, 256, 0, stream>>>((const float *)lw, n, summary, (float *)w); note_launch(); }
    else
        { normalize_kernel<double><<<blocks, 256, 0, stream>>>((const double *)lw, n, summary, (double *)w); note_launch(); }
    return (int)cudaGetLastError();
}

// ---- reference-compatible CDF ------------------------------------------------
template <typename T> struct ExpWeight {
    const T *lw;
    const double *summary;
    __device__ double operator()(int64_t i) const { return (double)dexp(lw[i] - (T)summary[0]); }
};

template <typename T> struct CdfWrite {
    T *cdf;
    __device__ void operator()(int64_t i, double prefix, double total) const { cdf[i] = (T)(prefix / total); }
};

int resampling_cdf(const void *lw, int64_t n, int dtype, void *cdf, void *ws, size_t ws_bytes,
                   cudaStream_t stream) {
    if (ws_bytes < reduce_workspace_bytes(n)) return ISSM_E_WORKSPACE;
    double *summary = (double *)((char *)ws + 128);
    int st = summary_launch(lw, n, dtype, summary, ws, stream);
    if (st) return st;
    double *scan_ws = (double *)((char *)ws + 256);
    if (dtype == ISSM_F32)
        return scan_apply<double>(n, ExpWeight<float>{(const float *)lw, summary}, CdfWrite<float>{(float *)cdf},
                                  scan_ws, stream);
    return scan_apply<double>(n, ExpWeight<double>{(const double *)lw, summary}, CdfWrite<double>{(double *)cdf},
                              scan_ws, stream);
}

}  // namespace issm
