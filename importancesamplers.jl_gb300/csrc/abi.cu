// abi.cu — the extern "C" boundary of libissm103.so (declared in
// include/issm.h). Validates arguments, maps them to the kernel entry points
// and returns 0 / cudaError_t / ISSM_E_*; no exception crosses the ABI.
#include <stdio.h>

#include "issm_device.cuh"
#include "issm_internal.h"

#include <atomic>
#include <mutex>
#include <utility>
#include <vector>

using namespace issm;

namespace issm {
static std::atomic<unsigned long long> g_launches{0};
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

int device_sms() {
    constexpr int kMaxDevices = 64;
    static std::atomic<int> cached[kMaxDevices];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return kSMs;
    if (dev < kMaxDevices) {
        const int c = cached[dev].load(std::memory_order_relaxed);
        if (c > 0) return c;
    }
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) return kSMs;
    if (sms > kSMs) sms = kSMs;  // scratch is sized for at most kSMs
    if (dev < kMaxDevices) cached[dev].store(sms, std::memory_order_relaxed);
    return sms;
}

int allow_dynamic_smem(const void *kernel) {
    static std::mutex mu;
    static std::vector<std::pair<int, const void *>> done;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return (int)e;
    std::lock_guard<std::mutex> lock(mu);
    for (const auto &k : done)
        if (k.first == dev && k.second == kernel) return 0;
    int optin = 0;
    e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e != cudaSuccess) return (int)e;
    cudaFuncAttributes fa;
    e = cudaFuncGetAttributes(&fa, kernel);
    if (e != cudaSuccess) return (int)e;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
    if (e != cudaSuccess) return (int)e;
    done.emplace_back(dev, kernel);
    return 0;
}
}  // namespace issm

namespace {

int check_bank(const issm_bank *b) {
    if (!b || !b->locations || !b->scales || !b->lognormalizers) return ISSM_E_NULL;
    if (b->dim < 1 || b->count < 1) return ISSM_E_SIZE;
    if (b->dtype != ISSM_F32 && b->dtype != ISSM_F64) return ISSM_E_DTYPE;
    if (b->family != ISSM_GAUSSIAN && b->family != ISSM_STUDENT_T) return ISSM_E_KIND;
    if (b->scale_kind < ISSM_SCALE_FACTOR || b->scale_kind > ISSM_SCALE_SPHERICAL) return ISSM_E_KIND;
    if (b->family == ISSM_STUDENT_T && !b->dofs) return ISSM_E_NULL;
    return ISSM_OK;
}

int check_den(const issm_bank *b, const issm_denominator *den) {
    if (!den) return ISSM_E_NULL;
    switch (den->kind) {
    case ISSM_DENOM_FULL:
        return den->logcoefficients ? ISSM_OK : ISSM_E_NULL;
    case ISSM_DENOM_GENERATING:
        return ISSM_OK;
    case ISSM_DENOM_PARTIAL:
        return (den->logcoefficients && den->group_of_slot) ? ISSM_OK : ISSM_E_NULL;
    case ISSM_DENOM_PREFIX:
        if (!den->logcoefficients) return ISSM_E_NULL;
        return (den->terms >= 1 && den->terms <= b->count) ? ISSM_OK : ISSM_E_SIZE;
    }
    return ISSM_E_KIND;
}

int check_dtype(int dtype) { return (dtype == ISSM_F32 || dtype == ISSM_F64) ? ISSM_OK : ISSM_E_DTYPE; }

}  // namespace

#define ISSM_TRY(expr)            \
    do {                          \
        int _st = (expr);         \
        if (_st != 0) return _st; \
    } while (0)

extern "C" {

const char *issm_version(void) { return "issm103 1.0.0 sm_103a"; }

uint64_t issm_kernel_launches(void) { return g_launches.load(std::memory_order_relaxed); }

const char *issm_status_string(int status) {
    switch (status) {
    case ISSM_OK: return "success";
    case ISSM_E_NULL: return "a required pointer is NULL";
    case ISSM_E_SIZE: return "a size is negative or out of range";
    case ISSM_E_DTYPE: return "unsupported or mismatched dtype";
    case ISSM_E_KIND: return "unknown family, scale or denominator kind";
    case ISSM_E_ALL_ZERO: return "normalized weights are undefined because all raw weights are zero";
    case ISSM_E_UNSUPPORTED: return "request not supported by this library";
    case ISSM_E_WORKSPACE: return "workspace too small";
    case ISSM_E_NOT_POSDEF: return "covariance is not positive definite";
    case ISSM_E_SCRATCH_LIMIT: return "input larger than the fixed scratch of a no-allocation entry point allows";
    }
    if (status > 0) return cudaGetErrorString((cudaError_t)status);
    return "unknown status";
}

int issm_failure_reset(uint64_t *failures, issm_stream_t stream) {
    if (!failures) return ISSM_E_NULL;
    return failure_reset(failures, (cudaStream_t)stream);
}

int issm_fill_normals(uint64_t seed, uint64_t offset, int64_t n, void *out, int32_t dtype, issm_stream_t stream) {
    if (n < 0) return ISSM_E_SIZE;
    if (n > 0 && !out) return ISSM_E_NULL;
    ISSM_TRY(check_dtype(dtype));
    return fill_normals(seed, nullptr, offset, n, out, dtype, (cudaStream_t)stream);
}

int issm_fill_uniforms(uint64_t seed, uint64_t offset, int64_t n, void *out, int32_t dtype, issm_stream_t stream) {
    if (n < 0) return ISSM_E_SIZE;
    if (n > 0 && !out) return ISSM_E_NULL;
    ISSM_TRY(check_dtype(dtype));
    return fill_uniforms(seed, nullptr, offset, n, out, dtype, (cudaStream_t)stream);
}

int issm_fill_normals_at(uint64_t seed, const uint64_t *offset_base, uint64_t offset, int64_t n, void *out,
                         int32_t dtype, issm_stream_t stream) {
    if (n < 0) return ISSM_E_SIZE;
    if (n > 0 && (!out || !offset_base)) return ISSM_E_NULL;
    ISSM_TRY(check_dtype(dtype));
    return fill_normals(seed, offset_base, offset, n, out, dtype, (cudaStream_t)stream);
}

int issm_fill_uniforms_at(uint64_t seed, const uint64_t *offset_base, uint64_t offset, int64_t n, void *out,
                          int32_t dtype, issm_stream_t stream) {
    if (n < 0) return ISSM_E_SIZE;
    if (n > 0 && (!out || !offset_base)) return ISSM_E_NULL;
    ISSM_TRY(check_dtype(dtype));
    return fill_uniforms(seed, offset_base, offset, n, out, dtype, (cudaStream_t)stream);
}

int issm_counter_advance(uint64_t *counter, uint64_t increment, issm_stream_t stream) {
    if (!counter) return ISSM_E_NULL;
    return counter_advance(counter, increment, (cudaStream_t)stream);
}

int issm_static_assign(const void *cdf, int32_t k, const void *uniforms, int64_t n, int32_t stratified,
                       int32_t *slots, int32_t dtype, issm_stream_t stream) {
    if (n < 0 || k < 1) return ISSM_E_SIZE;
    if (n == 0) return ISSM_OK;
    if (!cdf || !uniforms || !slots) return ISSM_E_NULL;
    ISSM_TRY(check_dtype(dtype));
    return static_assign(cdf, k, uniforms, n, stratified, slots, dtype, (cudaStream_t)stream);
}

int issm_draw(const issm_bank *bank, const int32_t *slots, int32_t fixed_slot, const void *normals,
              const void *radial_normals, int32_t radial_normal_stride, const void *radial_uniforms,
              int32_t radial_uniform_stride, int64_t n, void *samples, uint64_t *failures, int64_t index_base,
              issm_stream_t stream) {
    ISSM_TRY(check_bank(bank));
    if (n < 0) return ISSM_E_SIZE;
    if (n == 0) return ISSM_OK;
    if (!normals || !samples) return ISSM_E_NULL;
    if (!slots && (fixed_slot < 0 || fixed_slot >= bank->count)) return ISSM_E_SIZE;
    if (bank->family == ISSM_STUDENT_T && !radial_normals) return ISSM_E_NULL;
    return simt_draw(bank, slots, fixed_slot, normals, radial_normals, radial_normal_stride, radial_uniforms,
                     radial_uniform_stride, n, samples, failures, index_base, (cudaStream_t)stream);
}

int issm_draw_philox(const issm_bank *bank, int32_t fixed_slot, uint64_t seed, const uint64_t *counter,
                     uint64_t offset, const void *radial_normals, int32_t radial_normal_stride,
                     const void *radial_uniforms, int32_t radial_uniform_stride, int64_t n, void *samples,
                     uint64_t *failures, int64_t index_base, issm_stream_t stream) {
    ISSM_TRY(check_bank(bank));
    if (n < 0) return ISSM_E_SIZE;
    if (n == 0) return ISSM_OK;
    if (!samples) return ISSM_E_NULL;
    if (fixed_slot < 0 || fixed_slot >= bank->count) return ISSM_E_SIZE;
    if (bank->family == ISSM_STUDENT_T && !radial_normals) return ISSM_E_NULL;
    return simt_draw_fused(bank, fixed_slot, seed, counter, offset, radial_normals, radial_normal_stride,
                           radial_uniforms, radial_uniform_stride, n, samples, failures, index_base,
                           (cudaStream_t)stream);
}

int issm_mixture_logdensity(const issm_bank *bank, const issm_denominator *den, const void *x, int64_t n,
                            const int32_t *slots, int32_t fixed_slot, void *out_logden, void *out_generating,
                            uint64_t *failures, int64_t index_base, int32_t precision, issm_stream_t stream) {
    ISSM_TRY(check_bank(bank));
    ISSM_TRY(check_den(bank, den));
    if (n < 0) return ISSM_E_SIZE;
    if (n == 0) return ISSM_OK;
    if (!x || !out_logden) return ISSM_E_NULL;
    if (!slots && (fixed_slot < 0 || fixed_slot >= bank->count)) return ISSM_E_SIZE;
    if (precision == ISSM_PREC_NATIVE)
        return simt_mixture(bank, den, x, n, slots, fixed_slot, out_logden, out_generating, failures, index_base,
                            (cudaStream_t)stream);
    return ISSM_E_UNSUPPORTED;
}

size_t issm_tc_workspace_bytes(int32_t k, int32_t d) {
    return tc_workspace_bytes(k < 1 ? 1 : k, d < 1 ? 1 : d) + 64;
}

int issm_invert_factors(const issm_bank *bank, int32_t first, int32_t count, float *out, issm_stream_t stream) {
    ISSM_TRY(check_bank(bank));
    if (!out) return ISSM_E_NULL;
    if (bank->scale_kind != ISSM_SCALE_FACTOR) return ISSM_E_KIND;
    if (bank->dim > 64) return ISSM_E_UNSUPPORTED;
    if (first < 0 || count < 0 || first + count > bank->count) return ISSM_E_SIZE;
    return invert_factors(bank, first, count, out, (cudaStream_t)stream);
}

static int tc_args_ok(const issm_bank *bank, int precision) {
    if (precision != ISSM_PREC_TF32 && precision != ISSM_PREC_BF16) return ISSM_E_KIND;
    if (bank->dtype != ISSM_F32 || bank->scale_kind != ISSM_SCALE_FACTOR || bank->dim > 64) return ISSM_E_UNSUPPORTED;
    return ISSM_OK;
}

int issm_mixture_logdensity_ws(const issm_bank *bank, const issm_denominator *den, const void *x, int64_t n,
                               const int32_t *slots, int32_t fixed_slot, void *out_logden, void *out_generating,
                               uint64_t *failures, int64_t index_base, int32_t precision, void *workspace,
                               size_t workspace_bytes, issm_stream_t stream) {
    if (precision == ISSM_PREC_NATIVE)
        return issm_mixture_logdensity(bank, den, x, n, slots, fixed_slot, out_logden, out_generating, failures,
                                       index_base, precision, stream);
    ISSM_TRY(check_bank(bank));
    ISSM_TRY(check_den(bank, den));
    ISSM_TRY(tc_args_ok(bank, precision));
    if (n < 0) return ISSM_E_SIZE;
    if (n == 0) return ISSM_OK;
    if (!x || !out_logden || !workspace) return ISSM_E_NULL;
    if (slots == nullptr && (fixed_slot < 0 || fixed_slot >= bank->count)) return ISSM_E_SIZE;
    if (slots != nullptr) return ISSM_E_UNSUPPORTED;  // tensor form centres on one fixed slot
    if (workspace_bytes < issm_tc_workspace_bytes(bank->count, bank->dim)) return ISSM_E_WORKSPACE;
    const int last = den->kind == ISSM_DENOM_PREFIX ? den->terms - 1 : bank->count - 1;
    int *err = (int *)((char *)workspace + workspace_bytes - 64);
    return tc_mixture(bank, den, 0, 0, last, x, n, slots, fixed_slot,
                      den->kind == ISSM_DENOM_GENERATING ? nullptr : den->logcoefficients, out_logden,
                      out_generating, nullptr, failures, index_base, precision, workspace, workspace_bytes - 64,
                      err, (cudaStream_t)stream);
}

int issm_amis_append_ws(const issm_bank *history, int32_t slot, const void *logcounts, const void *x, int64_t n,
                        void *lognumerators, uint64_t *failures, int32_t precision, void *workspace,
                        size_t workspace_bytes, issm_stream_t stream) {
    if (precision == ISSM_PREC_NATIVE)
        return issm_amis_append(history, slot, logcounts, x, n, lognumerators, failures, precision, stream);
    ISSM_TRY(check_bank(history));
    ISSM_TRY(tc_args_ok(history, precision));
    if (n < 0 || slot < 0 || slot >= history->count) return ISSM_E_SIZE;
    if (n == 0) return ISSM_OK;
    if (!logcounts || !x || !lognumerators || !workspace) return ISSM_E_NULL;
    if (workspace_bytes < issm_tc_workspace_bytes(history->count, history->dim)) return ISSM_E_WORKSPACE;
    int *err = (int *)((char *)workspace + workspace_bytes - 64);
    return tc_mixture(history, nullptr, 1, slot, slot, x, n, nullptr, slot, logcounts, nullptr, nullptr,
                      lognumerators, failures, 0, precision, workspace, workspace_bytes - 64, err,
                      (cudaStream_t)stream);
}

int issm_mis_round(const issm_bank *bank, const issm_denominator *den, const int32_t *slots, const void *normals,
                   const void *radial_normals, int32_t radial_normal_stride, const void *radial_uniforms,
                   int32_t radial_uniform_stride, const void *logtargets, int64_t n, void *samples,
                   void *logweights, const int64_t *proposal_ids, int64_t *proposal_ids_out, uint64_t *failures,
                   int32_t precision, issm_stream_t stream) {
    ISSM_TRY(check_bank(bank));
    ISSM_TRY(check_den(bank, den));
    if (n < 0) return ISSM_E_SIZE;
    if (n == 0) return ISSM_OK;
    if (!slots || !normals || !samples || !logweights) return ISSM_E_NULL;
    if (bank->family == ISSM_STUDENT_T && !radial_normals) return ISSM_E_NULL;
    if (precision != ISSM_PREC_NATIVE) return ISSM_E_UNSUPPORTED;
    return simt_round(bank, den, slots, normals, radial_normals, radial_normal_stride, radial_uniforms,
                      radial_uniform_stride, logtargets, n, samples, logweights, proposal_ids, proposal_ids_out,
                      failures, (cudaStream_t)stream);
}

int issm_add_target_values(void *logweights, const void *values, int64_t n, int32_t dtype, uint64_t *failures,
                           int64_t index_base, issm_stream_t stream) {
    if (n < 0) return ISSM_E_SIZE;
    if (n == 0) return ISSM_OK;
    if (!logweights || !values) return ISSM_E_NULL;
    ISSM_TRY(check_dtype(dtype));
    return add_target_values(logweights, values, n, dtype, failures, index_base, (cudaStream_t)stream);
}

int issm_check_target_values(const void *values, int64_t n, int32_t dtype, int64_t *round_ids,
                             uint64_t *failures, int64_t index_base, issm_stream_t stream) {
    if (n < 0) return ISSM_E_SIZE;
    if (n == 0) return ISSM_OK;
    if (!values) return ISSM_E_NULL;
    ISSM_TRY(check_dtype(dtype));
    return check_target_values(values, n, dtype, round_ids, failures, index_base, (cudaStream_t)stream);
}

int issm_subtract_logweights(const void *logtargets, const void *logden, int64_t n, int32_t dtype,
                             void *logweights, uint64_t *failures, int64_t index_base, issm_stream_t stream) {
    if (n < 0) return ISSM_E_SIZE;
    if (n == 0) return ISSM_OK;
    if (!logtargets || !logden || !logweights) return ISSM_E_NULL;
    ISSM_TRY(check_dtype(dtype));
    return subtract_logweights(logtargets, logden, n, dtype, logweights, failures, index_base,
                               (cudaStream_t)stream);
}

int issm_amis_append(const issm_bank *history, int32_t slot, const void *logcounts, const void *x, int64_t n,
                     void *lognumerators, uint64_t *failures, int32_t precision, issm_stream_t stream) {
    ISSM_TRY(check_bank(history));
    if (n < 0 || slot < 0 || slot >= history->count) return ISSM_E_SIZE;
    if (n == 0) return ISSM_OK;
    if (!logcounts || !x || !lognumerators) return ISSM_E_NULL;
    if (precision != ISSM_PREC_NATIVE) return ISSM_E_UNSUPPORTED;
    return simt_append(history, slot, logcounts, x, n, lognumerators, failures, (cudaStream_t)stream);
}

int issm_amis_form(const void *logtargets, const void *lognumerators, const int64_t *round_ids, double logtotal,
                   int64_t n, int32_t dtype, void *logweights, uint64_t *failures, issm_stream_t stream) {
    if (n < 0) return ISSM_E_SIZE;
    if (n == 0) return ISSM_OK;
    if (!logtargets || !lognumerators || !logweights) return ISSM_E_NULL;
    ISSM_TRY(check_dtype(dtype));
    return amis_form(logtargets, lognumerators, round_ids, logtotal, n, dtype, logweights, failures,
                     (cudaStream_t)stream);
}

int issm_amis_form_summary(const void *logtargets, const void *lognumerators, const int64_t *round_ids,
                           double logtotal, int64_t n, int32_t dtype, void *logweights, uint64_t *failures,
                           double *summary, void *workspace, size_t workspace_bytes, issm_stream_t stream) {
    if (n < 1) return ISSM_E_SIZE;
    if (!logtargets || !lognumerators || !logweights || !summary || !workspace) return ISSM_E_NULL;
    ISSM_TRY(check_dtype(dtype));
    return amis_form_summary(logtargets, lognumerators, round_ids, logtotal, n, dtype, logweights, failures, summary,
                             workspace, workspace_bytes, (cudaStream_t)stream);
}

size_t issm_reduce_workspace_bytes(int64_t n) { return reduce_workspace_bytes(n < 1 ? 1 : n); }

int issm_logweight_summary(const void *logweights, int64_t n, int32_t dtype, double *out, void *workspace,
                           size_t workspace_bytes, issm_stream_t stream) {
    if (n < 1) return ISSM_E_SIZE;
    if (!logweights || !out || !workspace) return ISSM_E_NULL;
    ISSM_TRY(check_dtype(dtype));
    return logweight_summary(logweights, n, dtype, out, workspace, workspace_bytes, (cudaStream_t)stream);
}

int issm_normalize(const void *logweights, int64_t n, int32_t dtype, const double *summary, void *weights,
                   issm_stream_t stream) {
    if (n < 1) return ISSM_E_SIZE;
    if (!logweights || !summary || !weights) return ISSM_E_NULL;
    ISSM_TRY(check_dtype(dtype));
    return normalize(logweights, n, dtype, summary, weights, (cudaStream_t)stream);
}

int issm_resampling_cdf(const void *logweights, int64_t n, int32_t dtype, void *cdf, void *workspace,
                        size_t workspace_bytes, issm_stream_t stream) {
    if (n < 1) return ISSM_E_SIZE;
    if (!logweights || !cdf || !workspace) return ISSM_E_NULL;
    ISSM_TRY(check_dtype(dtype));
    return resampling_cdf(logweights, n, dtype, cdf, workspace, workspace_bytes, (cudaStream_t)stream);
}

int issm_resample_select(const void *cdf, const void *logweights, int64_t n, const void *uniforms, int64_t count,
                         int32_t dtype, int64_t *ancestors, issm_stream_t stream) {
    if (n < 1 || count < 0) return ISSM_E_SIZE;
    if (count == 0) return ISSM_OK;
    if (!cdf || !logweights || !uniforms || !ancestors) return ISSM_E_NULL;
    ISSM_TRY(check_dtype(dtype));
    return resample_select(cdf, logweights, n, uniforms, count, dtype, ancestors, (cudaStream_t)stream);
}

size_t issm_resample_workspace_bytes(int64_t n) { return resample_workspace_bytes(n < 1 ? 1 : n); }

int issm_resample_multinomial(const void *logweights, int64_t n, int32_t dtype, const double *uniforms,
                              int64_t count, int64_t *ancestors, void *workspace, size_t workspace_bytes,
                              issm_stream_t stream) {
    if (n < 1 || count < 0 || n > ((int64_t)1 << 40)) return ISSM_E_SIZE;
    if (!logweights || !workspace || (count > 0 && (!uniforms || !ancestors))) return ISSM_E_NULL;
    ISSM_TRY(check_dtype(dtype));
    return resample_fixed(logweights, n, dtype, uniforms, 0.0, 0, count, ancestors, workspace, workspace_bytes,
                          (cudaStream_t)stream);
}

int issm_resample_systematic(const void *logweights, int64_t n, int32_t dtype, double u, int64_t count,
                             int64_t *ancestors, void *workspace, size_t workspace_bytes, issm_stream_t stream) {
    if (n < 1 || count < 0 || n > ((int64_t)1 << 40)) return ISSM_E_SIZE;
    if (!(u >= 0.0 && u < 1.0)) return ISSM_E_SIZE;
    if (!logweights || !workspace || (count > 0 && !ancestors)) return ISSM_E_NULL;
    ISSM_TRY(check_dtype(dtype));
    return resample_fixed(logweights, n, dtype, nullptr, u, 1, count, ancestors, workspace, workspace_bytes,
                          (cudaStream_t)stream);
}

int issm_gather(const void *src, int32_t d, int64_t n_src, const int64_t *ancestors, int64_t count, int32_t dtype,
                void *dst, issm_stream_t stream) {
    if (d < 1 || n_src < 1 || count < 0) return ISSM_E_SIZE;
    if (count == 0) return ISSM_OK;
    if (!src || !ancestors || !dst) return ISSM_E_NULL;
    ISSM_TRY(check_dtype(dtype));
    return gather(src, d, n_src, ancestors, count, dtype, dst, (cudaStream_t)stream);
}

int issm_local_resample(const void *logweights, const int64_t *counts, int32_t k, const void *uniforms,
                        const void *samples, int32_t d, int32_t dtype, int64_t *ancestors, void *destination,
                        issm_stream_t stream) {
    if (k < 0 || d < 1) return ISSM_E_SIZE;
    if (k == 0) return ISSM_OK;
    if (!logweights || !counts || !uniforms || !ancestors) return ISSM_E_NULL;
    if (destination && !samples) return ISSM_E_NULL;
    ISSM_TRY(check_dtype(dtype));
    return local_resample(logweights, counts, k, uniforms, samples, d, dtype, ancestors, destination,
                          (cudaStream_t)stream);
}

size_t issm_moments_workspace_bytes(int64_t n, int32_t d) {
    const size_t a = moments_workspace_bytes(n < 1 ? 1 : n, d < 1 ? 1 : d);
    const size_t b = moments_tc_workspace_bytes(n < 1 ? 1 : n);
    return (a > b ? a : b) + 64;
}

int issm_weighted_moments_ws(const void *x, int32_t d, int64_t n, const void *logweights, int32_t dtype,
                             const double *summary, const double *shift, const void *prev_factor, double *mean,
                             double *cov, int32_t precision, void *workspace, size_t workspace_bytes,
                             issm_stream_t stream) {
    if (d < 1 || n < 1) return ISSM_E_SIZE;
    if (d > 64) return ISSM_E_UNSUPPORTED;
    if (!x || !logweights || !summary || !shift || !mean || !cov || !workspace) return ISSM_E_NULL;
    ISSM_TRY(check_dtype(dtype));
    if (workspace_bytes < issm_moments_workspace_bytes(n, d)) return ISSM_E_WORKSPACE;
    if (precision == ISSM_PREC_NATIVE)
        return weighted_moments(x, d, n, logweights, dtype, summary, shift, mean, cov, workspace,
                                workspace_bytes - 64, (cudaStream_t)stream);
    if (precision != ISSM_PREC_TF32 && precision != ISSM_PREC_BF16) return ISSM_E_KIND;
    if (dtype != ISSM_F32) return ISSM_E_UNSUPPORTED;
    int *err = (int *)((char *)workspace + workspace_bytes - 64);
    return moments_tc(x, d, n, logweights, summary, shift, (const float *)prev_factor, mean, cov, precision, workspace,
                      workspace_bytes - 64, err, (cudaStream_t)stream);
}

int issm_weighted_moments(const void *x, int32_t d, int64_t n, const void *logweights, int32_t dtype,
                          const double *summary, const double *shift, double *mean, double *cov, void *workspace,
                          size_t workspace_bytes, issm_stream_t stream) {
    if (d < 1 || n < 1) return ISSM_E_SIZE;
    if (d > 64) return ISSM_E_UNSUPPORTED;
    if (!x || !logweights || !summary || !shift || !mean || !cov || !workspace) return ISSM_E_NULL;
    ISSM_TRY(check_dtype(dtype));
    return weighted_moments(x, d, n, logweights, dtype, summary, shift, mean, cov, workspace, workspace_bytes,
                            (cudaStream_t)stream);
}

int issm_fit_factor_reg(const double *mean, const double *cov, int32_t d, const void *previous_factor, double dof,
                        double logconstant, int32_t dtype, double regularization, void *out_location,
                        void *out_factor, void *out_lognormalizer, float *out_inverse, uint64_t *failures,
                        int64_t failure_index, issm_stream_t stream) {
    if (d < 1) return ISSM_E_SIZE;
    if (d > 64) return ISSM_E_UNSUPPORTED;
    if (!mean || !cov || !previous_factor || !out_location || !out_factor || !out_lognormalizer)
        return ISSM_E_NULL;
    if (dof > 0.0 && !(dof > 2.0)) return ISSM_E_KIND;
    if (regularization != regularization) return ISSM_E_KIND;  // NaN
    ISSM_TRY(check_dtype(dtype));
    return fit_factor(mean, cov, d, previous_factor, dof, logconstant, dtype, out_location, out_factor,
                      out_lognormalizer, failures, failure_index, out_inverse, regularization, (cudaStream_t)stream);
}

int issm_fit_factor_ex(const double *mean, const double *cov, int32_t d, const void *previous_factor, double dof,
                       double logconstant, int32_t dtype, void *out_location, void *out_factor,
                       void *out_lognormalizer, float *out_inverse, uint64_t *failures, int64_t failure_index,
                       issm_stream_t stream) {
    return issm_fit_factor_reg(mean, cov, d, previous_factor, dof, logconstant, dtype, -1.0, out_location, out_factor,
                               out_lognormalizer, out_inverse, failures, failure_index, stream);
}

int issm_fit_factor(const double *mean, const double *cov, int32_t d, const void *previous_factor, double dof,
                    double logconstant, int32_t dtype, void *out_location, void *out_factor,
                    void *out_lognormalizer, uint64_t *failures, int64_t failure_index, issm_stream_t stream) {
    return issm_fit_factor_ex(mean, cov, d, previous_factor, dof, logconstant, dtype, out_location, out_factor,
                              out_lognormalizer, nullptr, failures, failure_index, stream);
}

size_t issm_weighted_sum_workspace_bytes(int64_t n, int32_t d) {
    if (n < 1 || d < 1) return 0;
    return weighted_sum_workspace_bytes(n, d);
}

int issm_weighted_sum(const void *x, int32_t d, int64_t n, const void *logweights, int32_t dtype,
                      const double *summary, double *out, void *workspace, size_t workspace_bytes,
                      issm_stream_t stream) {
    if (n < 1 || d < 1) return ISSM_E_SIZE;
    if (!x || !logweights || !summary || !out || !workspace) return ISSM_E_NULL;
    ISSM_TRY(check_dtype(dtype));
    if (workspace_bytes < weighted_sum_workspace_bytes(n, d)) return ISSM_E_WORKSPACE;
    return weighted_sum(x, d, n, logweights, dtype, summary, out, workspace, (cudaStream_t)stream);
}

size_t issm_weighted_quantile_workspace_bytes(int32_t d, int32_t nprob) {
    if (d < 1 || nprob < 1) return 0;
    return weighted_quantile_workspace_bytes(d, nprob);
}

int issm_weighted_quantile(const void *x, int32_t d, int64_t n, const void *logweights, int32_t dtype,
                           const double *summary, const double *probabilities, int32_t nprob, double *out,
                           void *workspace, size_t workspace_bytes, issm_stream_t stream) {
    if (n < 1 || d < 1 || nprob < 1) return ISSM_E_SIZE;
    if (!x || !logweights || !summary || !probabilities || !out || !workspace) return ISSM_E_NULL;
    ISSM_TRY(check_dtype(dtype));
    if (workspace_bytes < weighted_quantile_workspace_bytes(d, nprob)) return ISSM_E_WORKSPACE;
    if (((uintptr_t)workspace & 15) != 0) return ISSM_E_UNSUPPORTED;
    return weighted_quantile(x, d, n, logweights, dtype, summary, probabilities, nprob, out, workspace,
                             (cudaStream_t)stream);
}

static int glm_check(const issm_target *t, int32_t precision) {
    if (!t) return ISSM_E_NULL;
    if (t->kind != ISSM_TARGET_LINREG && t->kind != ISSM_TARGET_LOGISTIC) return ISSM_E_KIND;
    if (t->dtype != ISSM_F32) return ISSM_E_DTYPE;
    if (t->dim < 1 || t->count < 1) return ISSM_E_SIZE;
    if (t->dim > 64) return ISSM_E_UNSUPPORTED;
    if (precision != ISSM_PREC_BF16 && precision != ISSM_PREC_TF32 && precision != ISSM_PREC_BF16X1)
        return ISSM_E_KIND;
    if (!t->a || !t->b) return ISSM_E_NULL;
    return ISSM_OK;
}

size_t issm_glm_operand_bytes(int32_t nobs, int32_t d, int32_t precision) {
    if (nobs < 1 || d < 1 || d > 64) return 0;
    return glm_operand_bytes(nobs, d, precision);
}

int issm_glm_prepare(const issm_target *target, int32_t precision, void *operand, size_t operand_bytes,
                     issm_stream_t stream) {
    ISSM_TRY(glm_check(target, precision));
    if (!operand) return ISSM_E_NULL;
    if (operand_bytes < glm_operand_bytes(target->count, target->dim, precision)) return ISSM_E_WORKSPACE;
    if (((uintptr_t)operand & 15) != 0) return ISSM_E_UNSUPPORTED;
    return glm_prepare(target, precision, operand, (cudaStream_t)stream);
}

int issm_glm_logdensity(const issm_target *target, int32_t precision, const void *operand, const float *x,
                        int64_t n, float *out, int32_t *error, issm_stream_t stream) {
    ISSM_TRY(glm_check(target, precision));
    if (n < 0) return ISSM_E_SIZE;
    if (n == 0) return ISSM_OK;
    if (!operand || !x || !out || !error) return ISSM_E_NULL;
    if (((uintptr_t)operand & 15) != 0) return ISSM_E_UNSUPPORTED;
    return glm_logdensity(target, precision, operand, x, n, out, error, (cudaStream_t)stream);
}

size_t issm_select_workspace_bytes(void) { return select_workspace_bytes(); }

int issm_select_kth(const void *values, int64_t n, int64_t k, int32_t dtype, void *out, void *workspace,
                    size_t workspace_bytes, issm_stream_t stream) {
    if (n < 1 || k < 1 || k > n) return ISSM_E_SIZE;
    if (!values || !out || !workspace) return ISSM_E_NULL;
    ISSM_TRY(check_dtype(dtype));
    if (workspace_bytes < select_workspace_bytes()) return ISSM_E_WORKSPACE;
    return select_kth(values, n, k, dtype, out, workspace, (cudaStream_t)stream);
}

int issm_npmc_clip(const void *raw_logweights, int64_t n, int32_t dtype, void *clipped, void *threshold,
                   void *workspace, size_t workspace_bytes, issm_stream_t stream) {
    if (n < 1) return ISSM_E_SIZE;
    if (!raw_logweights || !clipped || !threshold || !workspace) return ISSM_E_NULL;
    ISSM_TRY(check_dtype(dtype));
    if (workspace_bytes < select_workspace_bytes()) return ISSM_E_WORKSPACE;
    int64_t r = (int64_t)std::sqrt((double)n);  // isqrt(n)
    while (r * r > n) --r;
    while ((r + 1) * (r + 1) <= n) ++r;
    ISSM_TRY(select_kth(raw_logweights, n, n - r + 1, dtype, threshold, workspace, (cudaStream_t)stream));
    return clip_logweights(raw_logweights, n, dtype, threshold, clipped, (cudaStream_t)stream);
}

int issm_population_local_weights(const void *local_logweights, const void *samples, int32_t d, int32_t dtype,
                                  const int64_t *starts, const int64_t *counts, const double *thresholds,
                                  int32_t k, double tolerance, int32_t max_iterations, void *normalized_weights,
                                  void *local_ess, void *tempering_powers, uint8_t *status, void *raw_means,
                                  issm_stream_t stream) {
    if (k < 0 || d < 1 || max_iterations < 0) return ISSM_E_SIZE;
    if (k == 0) return ISSM_OK;
    if (!local_logweights || !starts || !counts || !thresholds || !normalized_weights || !local_ess ||
        !tempering_powers || !status)
        return ISSM_E_NULL;
    if (raw_means && !samples) return ISSM_E_NULL;
    if (!(tolerance >= 0.0)) return ISSM_E_KIND;
    ISSM_TRY(check_dtype(dtype));
    return population_local_weights(local_logweights, samples, d, dtype, starts, counts, thresholds, k, tolerance,
                                    max_iterations, normalized_weights, local_ess, tempering_powers, status,
                                    raw_means, (cudaStream_t)stream);
}

int issm_population_covariances(const void *samples, int32_t d, int32_t dtype, const void *normalized_weights,
                                const void *tempering_powers, const uint8_t *status, const void *locations,
                                const issm_bank *current, const int64_t *starts, const int64_t *counts, int32_t k,
                                void *centres, void *covariances, issm_stream_t stream) {
    if (k < 0 || d < 1) return ISSM_E_SIZE;
    if (d > 64) return ISSM_E_UNSUPPORTED;
    if (k == 0) return ISSM_OK;
    if (!samples || !normalized_weights || !tempering_powers || !status || !locations || !current || !starts ||
        !counts || !centres || !covariances || !current->scales)
        return ISSM_E_NULL;
    ISSM_TRY(check_dtype(dtype));
    if (current->dtype != dtype || current->dim != d || current->count < k) return ISSM_E_DTYPE;
    if (current->scale_kind < ISSM_SCALE_FACTOR || current->scale_kind > ISSM_SCALE_SPHERICAL) return ISSM_E_KIND;
    if (current->family == ISSM_STUDENT_T && !current->dofs) return ISSM_E_NULL;
    return population_covariances(samples, d, dtype, normalized_weights, tempering_powers, status, locations, current,
                                  starts, counts, k, centres, covariances, (cudaStream_t)stream);
}

int issm_population_factors(const void *covariances, int32_t d, int32_t k, int32_t dtype, const uint8_t *status,
                            const void *dofs, void *factors, int32_t *info, issm_stream_t stream) {
    if (k < 0 || d < 1) return ISSM_E_SIZE;
    if (d > 64) return ISSM_E_UNSUPPORTED;
    if (k == 0) return ISSM_OK;
    if (!covariances || !status || !factors || !info) return ISSM_E_NULL;
    ISSM_TRY(check_dtype(dtype));
    return population_factors(covariances, d, k, dtype, status, dofs, factors, info, (cudaStream_t)stream);
}

int issm_target_logdensity(const issm_target *target, const void *x, int64_t n, void *out, issm_stream_t stream) {
    if (!target) return ISSM_E_NULL;
    if (n < 0 || target->dim < 1) return ISSM_E_SIZE;
    if (n == 0) return ISSM_OK;
    if (!x || !out) return ISSM_E_NULL;
    ISSM_TRY(check_dtype(target->dtype));
    if (target->kind < ISSM_TARGET_GAUSS_MIX || target->kind > ISSM_TARGET_QUADRATIC) return ISSM_E_KIND;
    return target_logdensity(target, x, n, out, (cudaStream_t)stream);
}

int issm_tc_selftest(const float *a, const float *b, float *c, int32_t n, int32_t k, int32_t kind,
                     int32_t *status, issm_stream_t stream) {
    if (!a || !b || !c || !status) return ISSM_E_NULL;
    const int layout = (kind >> 8) & 3;
    kind &= ~0x300;
    if (kind != ISSM_PREC_BF16 && kind != ISSM_PREC_TF32) return ISSM_E_KIND;
    if (layout == 3) return ISSM_E_KIND;
    if (layout == 2 && kind != ISSM_PREC_BF16) return ISSM_E_UNSUPPORTED;  // MN-major: 16-bit types only
    if (n < 16 || n > 256 || n % 16 != 0) return ISSM_E_SIZE;
    const int kstep = kind == ISSM_PREC_BF16 ? 16 : 8;
    if (k < kstep || k > (layout >= 2 ? 128 : 64) || k % kstep != 0) return ISSM_E_SIZE;
    return tc_gemm_selftest(a, b, c, n, k, (kind == ISSM_PREC_BF16 ? 1 : 2) | (layout << 8), status,
                            (cudaStream_t)stream);
}

}  // extern "C"
