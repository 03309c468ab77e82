// issm_device.cuh — device helpers shared by the sm_103a kernels of
// libissm103.so: numeric traits, the LogExpFunctions-compatible logaddexp,
// an online log-sum-exp state, the packed 3-word failure record, and launch
// utilities.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cfloat>
#include <cmath>

#include "../../include/issm.h"

namespace issm {

// GB300: 2 dies x 76 SMs. The largest SM count that per-CTA scratch
// (summary partials, moment partials) is sized for; grids of persistent
// kernels take the current device's own count from device_sms().
constexpr int kSMs = 152;

// SM count of the current device (cudaDevAttrMultiProcessorCount, cached per
// device), at most kSMs.
int device_sms();

template <typename T> struct num;
template <> struct num<float> {
    __device__ __host__ static constexpr float inf() { return __builtin_huge_valf(); }
    __device__ __host__ static constexpr float fmin() { return FLT_MIN; }
    __device__ __host__ static constexpr float eps() { return FLT_EPSILON; }
    static constexpr int emin_half = 126 / 2;
};
template <> struct num<double> {
    __device__ __host__ static constexpr double inf() { return __builtin_huge_val(); }
    __device__ __host__ static constexpr double fmin() { return DBL_MIN; }
    __device__ __host__ static constexpr double eps() { return DBL_EPSILON; }
    static constexpr int emin_half = 1022 / 2;
};

__device__ __forceinline__ float dlog(float x) { return logf(x); }
__device__ __forceinline__ double dlog(double x) { return log(x); }
__device__ __forceinline__ float dexp(float x) { return expf(x); }
__device__ __forceinline__ double dexp(double x) { return exp(x); }
__device__ __forceinline__ float dlog1p(float x) { return log1pf(x); }
__device__ __forceinline__ double dlog1p(double x) { return log1p(x); }
__device__ __forceinline__ float dsqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double dsqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float dfrexp(float x, int *e) { return frexpf(x, e); }
__device__ __forceinline__ double dfrexp(double x, int *e) { return frexp(x, e); }
__device__ __forceinline__ float dldexp(float x, int e) { return ldexpf(x, e); }
__device__ __forceinline__ double dldexp(double x, int e) { return ldexp(x, e); }
__device__ __forceinline__ float dpow(float x, float y) { return powf(x, y); }
__device__ __forceinline__ double dpow(double x, double y) { return pow(x, y); }

// LogExpFunctions.log1pexp / logaddexp (x == y guard keeps logaddexp(Inf, Inf) = Inf).
template <typename T> __device__ __forceinline__ T log1pexp(T x) {
    if (x > T(33.3)) return x;
    if (x > T(18)) return x + dexp(-x);
    if (x < T(-37)) return dexp(x);
    return dlog1p(dexp(x));
}
template <typename T> __device__ __forceinline__ T logaddexp(T x, T y) {
    if (isnan(x) || isnan(y)) return x + y;
    T delta = (x == y) ? T(0) : fabs(x - y);
    T m = x > y ? x : y;
    return m + log1pexp(-delta);
}

template <typename T> __device__ __forceinline__ T qnan();
template <> __device__ __forceinline__ float qnan<float>() { return __int_as_float(0x7fffffff); }
template <> __device__ __forceinline__ double qnan<double>() { return __longlong_as_double(0x7ff8000000000000ll); }

// Online log-sum-exp over terms: one exp per term, exact special values
// (NaN propagates, -Inf terms vanish, equal infinities collapse as logaddexp).
template <typename T> struct LseState {
    T m = -num<T>::inf();
    T s = T(0);
    bool nan = false;
    __device__ __forceinline__ void add(T t) {
        if (isnan(t)) {
            nan = true;
        } else if (t > m) {
            s = (m == -num<T>::inf()) ? T(1) : s * dexp(m - t) + T(1);
            m = t;
        } else if (t > -num<T>::inf()) {
            s += (t == m) ? T(1) : dexp(t - m);
        }
    }
    __device__ __forceinline__ T value() const {
        if (nan) return qnan<T>();
        if (m == -num<T>::inf()) return m;
        return m + dlog(s);
    }
};

// Packed failure record (src/execution.jl:677-699): word0 = count, word1 =
// max(inverse 1-based index << 32 | inverse block << 16 | reason bits),
// word2 = the same max restricted to draw reasons.
constexpr uint16_t kDrawReasons = 0x000f | 0x0800 | 0x0010;
__device__ __forceinline__ void record_failure(uint64_t *rec, int64_t logical_index,
                                               uint32_t block, uint16_t reason) {
    if (rec == nullptr) return;
    uint32_t inv_index = (uint32_t)(0xFFFFFFFFu - (uint32_t)logical_index + 1u);
    uint16_t inv_block = (uint16_t)(0xFFFFu - (uint16_t)block + 1u);
    unsigned long long packed = ((unsigned long long)inv_index << 32) |
                                ((unsigned long long)inv_block << 16) | reason;
    atomicAdd((unsigned long long *)&rec[0], 1ull);
    atomicMax((unsigned long long *)&rec[1], packed);
    if (reason & kDrawReasons) atomicMax((unsigned long long *)&rec[2], packed);
}

// _subtract_logweight (src/methods/importance_sampling.jl:1261-1266)
template <typename T> __device__ __forceinline__ uint16_t subtract_logweight(T target, T proposal, T *out) {
    T w = target - proposal;
    *out = w;
    return (isnan(w) || w == num<T>::inf()) ? 0x1000 : 0;
}
// _native_target_reason (src/execution.jl:769-773)
template <typename T> __device__ __forceinline__ uint16_t target_reason(T v) {
    if (isnan(v)) return 0x0100;
    if (v == num<T>::inf()) return 0x0200;
    return 0;
}

// Host-side count of kernels this library has launched (issm_kernel_launches).
void note_launch();

// Raise a kernel's dynamic shared-memory limit to the per-block maximum, once
// per kernel and device. The limit is never lowered afterwards: a recorded
// CUDA graph replays launches of several sizes and each must stay allowed.
int allow_dynamic_smem(const void *kernel);

inline int grid_for(int64_t n, int threads, int per_sm = 8) {
    int64_t blocks = (n + threads - 1) / threads;
    int64_t cap = (int64_t)device_sms() * per_sm * 64;
    if (blocks > cap) blocks = cap;
    return blocks < 1 ? 1 : (int)blocks;
}

}  // namespace issm
