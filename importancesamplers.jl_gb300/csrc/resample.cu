// resample.cu — multinomial and systematic resampling, gather and the DM-PMC
// per-proposal (local) selection.
//
// Two CDF conventions:
//  * resample_select: the reference's float CDF (src/resampling.jl:199-225)
//    searched with strict < and the -Inf plateau repair (:92-118); bit-exact
//    with the reference for a given CDF and uniforms.
//  * resample_fixed: an exact 64-bit fixed-point CDF. w_j = e^(l_j - max) is
//    evaluated by det_exp (Cody-Waite reduction, degree-13 Taylor polynomial,
//    IEEE-exact operations only), quantised to q_j = floor(w_j 2^s + 1/2) with
//    s = min(52, 62 - ceil(log2 n)), and summed in uint64, which is
//    associative: ancestors are bit-identical on any scan order, on the GPU and
//    in the FP64 oracle. A uniform u selects the first j with
//    umulhi(floor(u 2^64), total) < prefix_j; zero-weight samples have empty
//    intervals, so no plateau repair is needed. Systematic resampling uses
//    tau_i = floor((i * total + umulhi(U, total)) / count).
#include "issm_device.cuh"
#include "issm_internal.h"
#include "scan.cuh"

namespace issm {

// ---- reference CDF select ----------------------------------------------------
template <typename T>
__global__ void select_kernel(const T *__restrict__ cdf, const T *__restrict__ lw, int64_t n,
                              const T *__restrict__ u, int64_t count, int64_t *__restrict__ anc) {
    const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= count) return;
    const T uniform = u[o];
    int64_t first = 1, last = n;
    while (first < last) {
        const int64_t mid = first + ((last - first) >> 1);
        if (uniform < cdf[mid - 1]) last = mid; else first = mid + 1;
    }
    if (lw[first - 1] == -num<T>::inf()) {
        while (first > 1 && lw[first - 1] == -num<T>::inf()) first -= 1;
        while (first < n && lw[first - 1] == -num<T>::inf()) first += 1;
    }
    anc[o] = first;
}

int resample_select(const void *cdf, const void *lw, int64_t n, const void *u, int64_t count, int dtype,
                    int64_t *anc, cudaStream_t stream) {
    if (count <= 0) return 0;
    const unsigned blocks = (unsigned)((count + 255) / 256);
    if (dtype == ISSM_F32)
        { select_kernel<float><<<blocks, 256, 0, stream>>>((const float *)cdf, (const float *)lw, n,
                                                         (const float *)u, count, anc); note_launch(); }
    else
        { select_kernel<double><<<blocks, 256, 0, stream>>>((const double *)cdf, (const double *)lw, n,
                                                          (const double *)u, count, anc); note_launch(); }
    return (int)cudaGetLastError();
}

// ---- deterministic fixed-point CDF ----------------------------------------------
__device__ __forceinline__ double det_exp(double x) {
    const double kInvLn2 = 0x1.71547652b82fep+0;
    const double kLn2Hi = 0x1.62e42ff000000p-1;   // ln 2 rounded to 32 bits
    const double kLn2Lo = -0x1.718432a1b0e26p-35; // ln 2 - kLn2Hi
    if (isnan(x)) return x;
    if (x < -708.0) return 0.0;
    if (x > 0.0) x = 0.0;
    const double k = floor(__dadd_rn(__dmul_rn(x, kInvLn2), 0.5));
    double r = __fma_rn(-k, kLn2Hi, x);
    r = __fma_rn(-k, kLn2Lo, r);
    double p = 1.0 / 6227020800.0;  // 1/13!
    const double inv_fact[13] = {1.0, 1.0, 1.0 / 2.0, 1.0 / 6.0, 1.0 / 24.0, 1.0 / 120.0, 1.0 / 720.0,
                                 1.0 / 5040.0, 1.0 / 40320.0, 1.0 / 362880.0, 1.0 / 3628800.0,
                                 1.0 / 39916800.0, 1.0 / 479001600.0};
#pragma unroll
    for (int i = 12; i >= 0; --i) p = __fma_rn(p, r, inv_fact[i]);
    return ldexp(p, (int)k);
}

static int fixed_scale_bits(int64_t n) {
    int b = 0;
    while (((int64_t)1 << b) < n) ++b;
    int s = 62 - b;
    return s > 52 ? 52 : s;
}

template <typename T> struct FixedWeight {
    const T *lw;
    const double *summary;
    double scale;
    __device__ unsigned long long operator()(int64_t i) const {
        const double w = det_exp(__dadd_rn((double)lw[i], -summary[0]));
        return (unsigned long long)floor(__dadd_rn(__dmul_rn(w, scale), 0.5));
    }
};

struct PrefixWrite {
    unsigned long long *prefix;
    __device__ void operator()(int64_t i, unsigned long long p, unsigned long long) const { prefix[i] = p; }
};

__device__ __forceinline__ unsigned long long u64_from_unit(double u) {
    if (!(u > 0.0)) return 0ull;
    if (u >= 1.0) return ~0ull;
    return (unsigned long long)ldexp(u, 64);
}

__device__ __forceinline__ int64_t first_greater(const unsigned long long *__restrict__ prefix, int64_t n,
                                                 unsigned long long tau) {
    int64_t lo = 0, hi = n - 1;
    while (lo < hi) {
        const int64_t mid = lo + ((hi - lo) >> 1);
        if (tau < prefix[mid]) hi = mid; else lo = mid + 1;
    }
    return lo + 1;
}

__global__ void fixed_select_kernel(const unsigned long long *__restrict__ prefix, int64_t n,
                                    const double *__restrict__ uniforms, double u, int systematic, int64_t count,
                                    int64_t *__restrict__ anc) {
    const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= count) return;
    const unsigned long long total = prefix[n - 1];
    unsigned long long tau;
    if (systematic) {
        const unsigned long long base = __umul64hi(u64_from_unit(u), total);
        const unsigned __int128 num = (unsigned __int128)total * (unsigned long long)o + base;
        tau = (unsigned long long)(num / (unsigned long long)count);
    } else {
        tau = __umul64hi(u64_from_unit(uniforms[o]), total);
    }
    anc[o] = first_greater(prefix, n, tau);
}

size_t resample_workspace_bytes(int64_t n) {
    return reduce_workspace_bytes(n) + 256 + sizeof(unsigned long long) * (size_t)(n + 1) +
           sizeof(unsigned long long) * (size_t)((n + kScanTile - 1) / kScanTile + 2);
}

int resample_fixed(const void *lw, int64_t n, int dtype, const double *uniforms, double u, int systematic,
                   int64_t count, int64_t *anc, void *ws, size_t ws_bytes, cudaStream_t stream) {
    if (ws_bytes < resample_workspace_bytes(n)) return ISSM_E_WORKSPACE;
    char *base = (char *)ws;
    const size_t red = reduce_workspace_bytes(n);
    double *summary = (double *)(base + red);
    unsigned long long *prefix = (unsigned long long *)(base + red + 256);
    unsigned long long *tiles = prefix + (n + 1);
    int st = logweight_summary(lw, n, dtype, summary, base, red, stream);
    if (st) return st;
    const double scale = ldexp(1.0, fixed_scale_bits(n));
    if (dtype == ISSM_F32)
        st = scan_apply<unsigned long long>(n, FixedWeight<float>{(const float *)lw, summary, scale},
                                            PrefixWrite{prefix}, tiles, stream);
    else
        st = scan_apply<unsigned long long>(n, FixedWeight<double>{(const double *)lw, summary, scale},
                                            PrefixWrite{prefix}, tiles, stream);
    if (st) return st;
    if (count <= 0) return 0;
    { fixed_select_kernel<<<(unsigned)((count + 255) / 256), 256, 0, stream>>>(prefix, n, uniforms, u, systematic,
                                                                             count, anc); note_launch(); }
    return (int)cudaGetLastError();
}

// ---- gather ------------------------------------------------------------------------
template <typename T>
__global__ void gather_kernel(const T *__restrict__ src, int d, const int64_t *__restrict__ anc, int64_t count,
                              T *__restrict__ dst) {
    const int64_t total = count * d;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += stride) {
        const int64_t o = e / d;
        const int c = (int)(e - o * d);
        dst[e] = src[(anc[o] - 1) * d + c];
    }
}

int gather(const void *src, int d, int64_t n_src, const int64_t *anc, int64_t count, int dtype, void *dst,
           cudaStream_t stream) {
    (void)n_src;
    if (count <= 0) return 0;
    const int blocks = grid_for(count * d, 256, 8);
    if (dtype == ISSM_F32)
        { gather_kernel<float><<<blocks, 256, 0, stream>>>((const float *)src, d, anc, count, (float *)dst); note_launch(); }
    else
        { gather_kernel<double><<<blocks, 256, 0, stream>>>((const double *)src, d, anc, count, (double *)dst); note_launch(); }
    return (int)cudaGetLastError();
}

// ---- DM-PMC local resampling -------------------------------------------------------
// One block per proposal slot over its contiguous run of samples; lane chunks
// as in _cooperative_local_resample_locations_kernel!
// (src/dm_pmc_execution.jl:184-265), chunk totals accumulated in FP64.
template <typename T>
__global__ void __launch_bounds__(256) local_resample_kernel(const T *__restrict__ lw, const int64_t *__restrict__ counts,
                                                             int k, const T *__restrict__ u,
                                                             const T *__restrict__ samples, int d,
                                                             int64_t *__restrict__ anc, T *__restrict__ dst) {
    const int slot = blockIdx.x;
    __shared__ int64_t first_s;
    __shared__ double chunk_totals[256];
    __shared__ T maxima[256];
    __shared__ int chosen;
    __shared__ double remainder_s;
    if (threadIdx.x == 0) {
        int64_t f = 0;
        for (int s = 0; s < slot; ++s) f += counts[s];
        first_s = f;
        chosen = -1;
    }
    __syncthreads();
    const int64_t first = first_s, cnt = counts[slot], last = first + cnt - 1;
    T lm = -num<T>::inf();
    for (int64_t i = first + threadIdx.x; i <= last; i += blockDim.x) lm = fmax(lm, lw[i]);
    maxima[threadIdx.x] = lm;
    __syncthreads();
    for (int off = 128; off > 0; off >>= 1) {
        if (threadIdx.x < off) maxima[threadIdx.x] = fmax(maxima[threadIdx.x], maxima[threadIdx.x + off]);
        __syncthreads();
    }
    const T m = maxima[0];
    const int64_t chunk = (cnt + blockDim.x - 1) / blockDim.x;
    const int64_t c0 = first + (int64_t)threadIdx.x * chunk;
    const int64_t c1 = min(c0 + chunk - 1, last);
    double acc = 0.0;
    if (m != -num<T>::inf())
        for (int64_t i = c0; i <= c1; ++i) acc += (double)dexp(lw[i] - m);
    chunk_totals[threadIdx.x] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double total = 0.0;
        for (int l = 0; l < (int)blockDim.x; ++l) total += chunk_totals[l];
        if (m != -num<T>::inf() && isfinite(total) && total > 0.0) {
            const double draw = (double)u[slot] * total;
            double prefix = 0.0;
            int pick = (int)min((int64_t)blockDim.x, cnt) - 1;
            double rem = chunk_totals[pick];
            for (int l = 0; l < (int)blockDim.x; ++l) {
                const double next = prefix + chunk_totals[l];
                if (draw < next) { pick = l; rem = draw - prefix; break; }
                prefix = next;
            }
            chosen = pick;
            remainder_s = rem;
        }
    }
    __syncthreads();
    if ((int)threadIdx.x == chosen) {
        double cum = 0.0;
        int64_t a = c1;
        for (int64_t i = c0; i <= c1; ++i) {
            cum += (double)dexp(lw[i] - m);
            if (remainder_s < cum) { a = i; break; }
        }
        anc[slot] = a + 1;
        if (dst)
            for (int c = 0; c < d; ++c) dst[(int64_t)slot * d + c] = samples[a * d + c];
    }
    if (threadIdx.x == 0 && chosen < 0) anc[slot] = 0;
}

int local_resample(const void *lw, const int64_t *counts, int k, const void *u, const void *samples, int d,
                   int dtype, int64_t *anc, void *dst, cudaStream_t stream) {
    if (k <= 0) return 0;
    if (dtype == ISSM_F32)
        { local_resample_kernel<float><<<k, 256, 0, stream>>>((const float *)lw, counts, k, (const float *)u,
                                                            (const float *)samples, d, anc, (float *)dst); note_launch(); }
    else
        { local_resample_kernel<double><<<k, 256, 0, stream>>>((const double *)lw, counts, k, (const double *)u,
                                                             (const double *)samples, d, anc, (double *)dst); note_launch(); }
    return (int)cudaGetLastError();
}

}  // namespace issm
