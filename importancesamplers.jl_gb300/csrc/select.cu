// select.cu — the N-PMC weight clipping of src/npmc_execution.jl:22-33: the
// k-th smallest of a round's n log weights (k = n - isqrt(n) + 1, the
// reference's partialsort! / sort! order statistic) and the clipped weights
// min(raw, threshold), on the device with no host round trip.
//
// The order statistic is a most-significant-digit radix select over keys that
// order like the values: an IEEE value maps to its bits with the sign bit
// set (non-negative) or all bits flipped (negative), and every NaN maps to
// the largest key, so NaNs sort last as in Julia's isless. Each 8-bit digit
// takes two launches: a histogram of the digit over the keys whose higher
// digits match the prefix found so far, then one block that scans the 256
// bins, picks the bin holding rank k, extends the prefix and clears the
// histogram. Four digits for FP32 keys, eight for FP64. The state (prefix,
// remaining rank, histogram) lives in the caller's workspace, so the sequence
// is fixed and graph-capturable.
#include "issm_device.cuh"
#include "issm_internal.h"

namespace issm {

template <typename T> struct KeyOf;
template <> struct KeyOf<float> {
    using K = uint32_t;
    static constexpr int kDigits = 4;
    __device__ static K key(float v) {
        if (isnan(v)) return 0xFFFFFFFFu;
        const uint32_t u = __float_as_uint(v);
        return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
    }
    __device__ static float value(K k) {
        if (k == 0xFFFFFFFFu) return __uint_as_float(0x7FC00000u);
        return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
    }
};
template <> struct KeyOf<double> {
    using K = unsigned long long;
    static constexpr int kDigits = 8;
    __device__ static K key(double v) {
        if (isnan(v)) return 0xFFFFFFFFFFFFFFFFull;
        const unsigned long long u = (unsigned long long)__double_as_longlong(v);
        return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
    }
    __device__ static double value(K k) {
        if (k == 0xFFFFFFFFFFFFFFFFull) return __longlong_as_double(0x7FF8000000000000ll);
        return __longlong_as_double((long long)((k & 0x8000000000000000ull) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k));
    }
};

// workspace: [0, 2048) 256 histogram bins (uint64); then the state
struct SelectState {
    unsigned long long prefix;  // key bits fixed so far
    long long rank;             // 1-based rank within the keys matching the prefix
};

template <typename T>
__global__ void select_histogram_kernel(const T *__restrict__ v, int64_t n, int digit,
                                        unsigned long long *__restrict__ hist, const SelectState *__restrict__ st) {
    using KO = KeyOf<T>;
    __shared__ unsigned int bins[256];
    for (int b = threadIdx.x; b < 256; b += blockDim.x) bins[b] = 0u;
    __syncthreads();
    constexpr int kBits = 8 * (int)sizeof(typename KO::K);
    const int shift = kBits - 8 * (digit + 1);
    const unsigned long long prefix = st->prefix;
    // keys match when their bits above this digit equal the prefix's
    const unsigned long long hi_mask = digit == 0 ? 0ull : (~0ull << (shift + 8)) & (kBits == 32 ? 0xFFFFFFFFull : ~0ull);
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const unsigned long long k = (unsigned long long)KO::key(v[i]);
        if ((k & hi_mask) == (prefix & hi_mask)) atomicAdd(&bins[(k >> shift) & 0xFFu], 1u);
    }
    __syncthreads();
    for (int b = threadIdx.x; b < 256; b += blockDim.x)
        if (bins[b]) atomicAdd(&hist[b], (unsigned long long)bins[b]);
}

template <typename T>
__global__ void select_step_kernel(int digit, unsigned long long *__restrict__ hist, SelectState *__restrict__ st,
                                   T *__restrict__ out) {
    using KO = KeyOf<T>;
    constexpr int kBits = 8 * (int)sizeof(typename KO::K);
    const int shift = kBits - 8 * (digit + 1);
    if (threadIdx.x == 0) {
        long long rank = st->rank;
        int b = 0;
        for (; b < 255; ++b) {
            const long long c = (long long)hist[b];
            if (rank <= c) break;
            rank -= c;
        }
        st->rank = rank;
        st->prefix |= (unsigned long long)b << shift;
        if (digit == KO::kDigits - 1) *out = KO::value((typename KO::K)st->prefix);
    }
    __syncthreads();
    for (int b = threadIdx.x; b < 256; b += blockDim.x) hist[b] = 0ull;
}

template <typename T> __global__ void select_init_kernel(SelectState *st, long long rank, unsigned long long *hist) {
    if (threadIdx.x == 0) {
        st->prefix = 0ull;
        st->rank = rank;
    }
    for (int b = threadIdx.x; b < 256; b += blockDim.x) hist[b] = 0ull;
}

// Julia's min: NaN when either argument is NaN
template <typename T>
__global__ void clip_kernel(const T *__restrict__ raw, int64_t n, const T *__restrict__ threshold, T *__restrict__ out) {
    const T t = *threshold;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const T x = raw[i];
        out[i] = (isnan(x) || isnan(t)) ? (isnan(x) ? x : t) : (x < t ? x : t);
    }
}

size_t select_workspace_bytes() { return 256 * sizeof(unsigned long long) + sizeof(SelectState) + 64; }

template <typename T>
static int select_kth_t(const T *v, int64_t n, int64_t k, T *out, void *ws, cudaStream_t stream) {
    unsigned long long *hist = (unsigned long long *)ws;
    SelectState *st = (SelectState *)(hist + 256);
    select_init_kernel<T><<<1, 256, 0, stream>>>(st, (long long)k, hist);
    note_launch();
    const int blocks = grid_for(n, 256, 4);
    for (int digit = 0; digit < KeyOf<T>::kDigits; ++digit) {
        select_histogram_kernel<T><<<blocks, 256, 0, stream>>>(v, n, digit, hist, st);
        note_launch();
        select_step_kernel<T><<<1, 256, 0, stream>>>(digit, hist, st, out);
        note_launch();
    }
    return (int)cudaGetLastError();
}

int select_kth(const void *v, int64_t n, int64_t k, int dtype, void *out, void *ws, cudaStream_t stream) {
    if (dtype == ISSM_F32) return select_kth_t<float>((const float *)v, n, k, (float *)out, ws, stream);
    return select_kth_t<double>((const double *)v, n, k, (double *)out, ws, stream);
}

int clip_logweights(const void *raw, int64_t n, int dtype, const void *threshold, void *out, cudaStream_t stream) {
    const int blocks = grid_for(n, 256, 4);
    if (dtype == ISSM_F32)
        clip_kernel<float><<<blocks, 256, 0, stream>>>((const float *)raw, n, (const float *)threshold, (float *)out);
    else
        clip_kernel<double><<<blocks, 256, 0, stream>>>((const double *)raw, n, (const double *)threshold,
                                                        (double *)out);
    note_launch();
    return (int)cudaGetLastError();
}

}  // namespace issm
