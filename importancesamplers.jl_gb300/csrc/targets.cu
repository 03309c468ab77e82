// targets.cu — built-in batch targets used by the benchmark configurations.
// In the reference the target is user code compiled into the sampling kernel
// or a batch callback (src/batched_targets.jl:54-114); these kernels are the
// native equivalents of the callbacks the benchmark workloads need.
#include "issm_device.cuh"
#include "issm_internal.h"

namespace issm {

constexpr double kLog2Pi = 1.8378770664093454835606594728112;

template <typename T>
__global__ void target_simple_kernel(issm_target t, const T *__restrict__ x, int64_t n, T *__restrict__ out) {
    const int d = t.dim;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const T *a = (const T *)t.a;
    const T *b = (const T *)t.b;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const T *xi = x + i * d;
        T v = T(0);
        if (t.kind == ISSM_TARGET_STD_NORMAL) {
            T r2 = T(0);
            for (int c = 0; c < d; ++c) r2 += xi[c] * xi[c];
            v = T(-0.5 * kLog2Pi) * T(d) - T(0.5) * r2;
        } else if (t.kind == ISSM_TARGET_QUADRATIC) {
            T r2 = T(0);
            for (int c = 0; c < d; ++c) { T z = xi[c] - a[c]; r2 += z * z; }
            v = -r2 / T(t.p0);
        } else if (t.kind == ISSM_TARGET_GAUSS_MIX) {
            LseState<T> lse;
            for (int j = 0; j < t.count; ++j) {
                T r2 = T(0);
                for (int c = 0; c < d; ++c) { T z = xi[c] - a[(size_t)j * d + c]; r2 += z * z; }
                lse.add(T(-0.5) * r2);
            }
            v = lse.value() - dlog(T(t.count)) - T(0.5 * kLog2Pi) * T(d);
        } else if (t.kind == ISSM_TARGET_STUDENT_T) {
            // normalised multivariate t with location a, scale factor b (column-major), nu = p0,
            // log constant p1 (already minus log|L|)
            T z[64];
            T r2 = T(0);
            for (int r = 0; r < d; ++r) {
                T s = xi[r] - a[r];
                for (int c = 0; c < r; ++c) s -= b[r + (size_t)c * d] * z[c];
                s /= b[r + (size_t)r * d];
                z[r] = s;
                r2 += s * s;
            }
            const T nu = T(t.p0);
            v = T(t.p1) - (nu + T(d)) * T(0.5) * dlog1p(r2 / nu);
        }
        out[i] = v;
    }
}

// Regression likelihoods: one warp per sample, lanes stride the observations;
// X is n_obs x d column-major, beta = the sample.
template <typename T>
__global__ void target_regression_kernel(issm_target t, const T *__restrict__ x, int64_t n, T *__restrict__ out) {
    const int d = t.dim;
    const int nobs = t.count;
    const T *X = (const T *)t.a;
    const T *y = (const T *)t.b;
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = warp; i < n; i += nwarps) {
        const T *beta = x + i * d;
        T acc = T(0);
        for (int o = lane; o < nobs; o += 32) {
            T eta = T(0);
            for (int c = 0; c < d; ++c) eta += X[o + (size_t)c * nobs] * beta[c];
            if (t.kind == ISSM_TARGET_LINREG) {
                const T r = y[o] - eta;
                acc += r * r;
            } else {
                acc += y[o] * eta - log1pexp(eta);
            }
        }
        for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
        if (lane == 0) {
            T bb = T(0);
            for (int c = 0; c < d; ++c) bb += beta[c] * beta[c];
            const T pv = T(t.p1);
            const T prior = T(-0.5) * T(d) * (T(kLog2Pi) + dlog(pv)) - bb / (T(2) * pv);
            if (t.kind == ISSM_TARGET_LINREG) {
                const T sigma = T(t.p0);
                out[i] = T(-0.5) * T(nobs) * (T(kLog2Pi) + T(2) * dlog(sigma)) - acc / (T(2) * sigma * sigma) + prior;
            } else {
                out[i] = acc + prior;
            }
        }
    }
}

int target_logdensity(const issm_target *t, const void *x, int64_t n, void *out, cudaStream_t stream) {
    if (n <= 0) return 0;
    if (t->kind == ISSM_TARGET_LINREG || t->kind == ISSM_TARGET_LOGISTIC) {
        const int blocks = grid_for(n * 32, 256, 8);
        if (t->dtype == ISSM_F32)
            { target_regression_kernel<float><<<blocks, 256, 0, stream>>>(*t, (const float *)x, n, (float *)out); note_launch(); }
        else
            { target_regression_kernel<double><<<blocks, 256, 0, stream>>>(*t, (const double *)x, n, (double *)out); note_launch(); }
    } else {
        if (t->kind == ISSM_TARGET_STUDENT_T && t->dim > 64) return ISSM_E_UNSUPPORTED;
        const int blocks = grid_for(n, 128, 8);
        if (t->dtype == ISSM_F32)
            { target_simple_kernel<float><<<blocks, 128, 0, stream>>>(*t, (const float *)x, n, (float *)out); note_launch(); }
        else
            { target_simple_kernel<double><<<blocks, 128, 0, stream>>>(*t, (const double *)x, n, (double *)out); note_launch(); }
    }
    return (int)cudaGetLastError();
}

}  // namespace issm
