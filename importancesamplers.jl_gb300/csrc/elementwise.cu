// elementwise.cu — one-pass per-sample kernels: static assignment, log-weight
// formation and the batch-target finish, each with the reference's failure
// records.
#include "issm_device.cuh"
#include "issm_internal.h"

namespace issm {

// src/methods/static_mis.jl:171-211 — first slot with u' <= cdf[slot].
template <typename T>
__global__ void assign_kernel(const T *__restrict__ cdf, int k, const T *__restrict__ u, int64_t n, int stratified,
                              int32_t *__restrict__ slots) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const T mapped = stratified ? (T(i) + u[i]) / T(n) : u[i];
        int lo = 0, hi = k - 1;
        while (lo < hi) {
            const int mid = lo + (hi - lo) / 2;
            if (mapped <= cdf[mid]) hi = mid; else lo = mid + 1;
        }
        slots[i] = lo;
    }
}

int static_assign(const void *cdf, int k, const void *u, int64_t n, int stratified, int32_t *slots, int dtype,
                  cudaStream_t stream) {
    if (n <= 0) return 0;
    const int blocks = grid_for(n, 256, 4);
    if (dtype == ISSM_F32)
        { assign_kernel<float><<<blocks, 256, 0, stream>>>((const float *)cdf, k, (const float *)u, n, stratified, slots); note_launch(); }
    else
        { assign_kernel<double><<<blocks, 256, 0, stream>>>((const double *)cdf, k, (const double *)u, n, stratified, slots); note_launch(); }
    return (int)cudaGetLastError();
}

// _finish_batch_weights! (src/batched_targets.jl:204-214): samples whose
// weight is already -Inf (failed earlier) stay untouched.
template <typename T>
__global__ void add_values_kernel(T *__restrict__ lw, const T *__restrict__ v, int64_t n, uint64_t *failures,
                                  int64_t index_base) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const T cur = lw[i];
        if (cur == -num<T>::inf()) continue;
        const T val = v[i];
        uint16_t r = target_reason(val);
        if (r) {
            record_failure(failures, index_base + i + 1, 0, r);
            lw[i] = -num<T>::inf();
            continue;
        }
        T w = cur + val;
        if (isnan(w) || w == num<T>::inf()) {
            record_failure(failures, index_base + i + 1, 0, ISSM_REASON_LOGWEIGHT_INVALID);
            w = -num<T>::inf();
        }
        lw[i] = w;
    }
}

int add_target_values(void *lw, const void *values, int64_t n, int dtype, uint64_t *failures, int64_t index_base,
                      cudaStream_t stream) {
    if (n <= 0) return 0;
    const int blocks = grid_for(n, 256, 4);
    if (dtype == ISSM_F32)
        { add_values_kernel<float><<<blocks, 256, 0, stream>>>((float *)lw, (const float *)values, n, failures, index_base); note_launch(); }
    else
        { add_values_kernel<double><<<blocks, 256, 0, stream>>>((double *)lw, (const double *)values, n, failures,
                                                              index_base); note_launch(); }
    return (int)cudaGetLastError();
}

template <typename T>
__global__ void subtract_kernel(const T *__restrict__ lt, const T *__restrict__ ld, int64_t n, T *__restrict__ lw,
                                uint64_t *failures, int64_t index_base) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const T t = lt[i];
        uint16_t r = target_reason(t);
        T w = -num<T>::inf();
        if (!r) {
            T v;
            r = subtract_logweight(t, ld[i], &v);
            if (!r) w = v;
        }
        if (r) record_failure(failures, index_base + i + 1, 0, r);
        lw[i] = w;
    }
}

int subtract_logweights(const void *lt, const void *ld, int64_t n, int dtype, void *lw, uint64_t *failures,
                        int64_t index_base, cudaStream_t stream) {
    if (n <= 0) return 0;
    const int blocks = grid_for(n, 256, 4);
    if (dtype == ISSM_F32)
        { subtract_kernel<float><<<blocks, 256, 0, stream>>>((const float *)lt, (const float *)ld, n, (float *)lw,
                                                           failures, index_base); note_launch(); }
    else
        { subtract_kernel<double><<<blocks, 256, 0, stream>>>((const double *)lt, (const double *)ld, n, (double *)lw,
                                                            failures, index_base); note_launch(); }
    return (int)cudaGetLastError();
}

// _form_amis_logweights_kernel! (src/amis_execution.jl:107-134)
template <typename T>
__global__ void amis_form_kernel(const T *__restrict__ lt, const T *__restrict__ lnum,
                                 const int64_t *__restrict__ round_ids, T logtotal, int64_t n, T *__restrict__ lw,
                                 uint64_t *failures) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        if (round_ids && round_ids[i] == 0) continue;
        T v;
        const uint16_t r = subtract_logweight(lt[i], lnum[i] - logtotal, &v);
        if (r) record_failure(failures, i + 1, 0, r);
        else lw[i] = v;
    }
}

int amis_form(const void *lt, const void *lnum, const int64_t *round_ids, double logtotal, int64_t n, int dtype,
              void *lw, uint64_t *failures, cudaStream_t stream) {
    if (n <= 0) return 0;
    const int blocks = grid_for(n, 256, 4);
    if (dtype == ISSM_F32)
        { amis_form_kernel<float><<<blocks, 256, 0, stream>>>((const float *)lt, (const float *)lnum, round_ids,
                                                            (float)logtotal, n, (float *)lw, failures); note_launch(); }
    else
        { amis_form_kernel<double><<<blocks, 256, 0, stream>>>((const double *)lt, (const double *)lnum, round_ids,
                                                             logtotal, n, (double *)lw, failures); note_launch(); }
    return (int)cudaGetLastError();
}

// Target validity for targets evaluated outside the sampling kernel: a NaN or
// +Inf value is recorded (_native_target_reason, src/execution.jl:769-773) and
// the sample leaves the round (its round id becomes 0, as the reference's
// _gaussian_round_launch_kernel! leaves it, src/mis_execution.jl:722-771).
template <typename T>
__global__ void check_targets_kernel(const T *__restrict__ v, int64_t n, int64_t *round_ids, uint64_t *failures,
                                     int64_t index_base) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint16_t r = target_reason(v[i]);
        if (r) {
            record_failure(failures, index_base + i + 1, 0, r);
            if (round_ids) round_ids[i] = 0;
        }
    }
}

int check_target_values(const void *values, int64_t n, int dtype, int64_t *round_ids, uint64_t *failures,
                        int64_t index_base, cudaStream_t stream) {
    if (n <= 0) return 0;
    const int blocks = grid_for(n, 256, 4);
    if (dtype == ISSM_F32)
        { check_targets_kernel<float><<<blocks, 256, 0, stream>>>((const float *)values, n, round_ids, failures,
                                                                  index_base); note_launch(); }
    else
        { check_targets_kernel<double><<<blocks, 256, 0, stream>>>((const double *)values, n, round_ids, failures,
                                                                   index_base); note_launch(); }
    return (int)cudaGetLastError();
}

int failure_reset(uint64_t *f, cudaStream_t stream) {
    return (int)cudaMemsetAsync(f, 0, 3 * sizeof(uint64_t), stream);
}

}  // namespace issm
