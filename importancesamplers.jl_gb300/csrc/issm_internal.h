// issm_internal.h — host-side entry points between the C ABI layer (abi.cu)
// and the kernel translation units.
#pragma once

#include <cuda.h>  // CUtensorMap (types only; driver calls are resolved through the runtime)
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "../../include/issm.h"

namespace issm {

int simt_mixture(const issm_bank *b, const issm_denominator *den, const void *x, int64_t n,
                 const int32_t *slots, int32_t fixed_slot, void *out_logden, void *out_generating,
                 uint64_t *failures, int64_t index_base, cudaStream_t stream);
int simt_round(const issm_bank *b, const issm_denominator *den, const int32_t *slots, const void *normals,
               const void *rn, int rn_stride, const void *ru, int ru_stride, const void *logtargets,
               int64_t n, void *samples, void *logweights, const int64_t *proposal_ids,
               int64_t *proposal_ids_out, uint64_t *failures, cudaStream_t stream);
int simt_draw(const issm_bank *b, const int32_t *slots, int32_t fixed_slot, const void *normals,
              const void *rn, int rn_stride, const void *ru, int ru_stride, int64_t n, void *samples,
              uint64_t *failures, int64_t index_base, cudaStream_t stream);
int simt_draw_fused(const issm_bank *b, int32_t fixed_slot, uint64_t seed, const uint64_t *counter,
                    uint64_t offset, const void *rn, int rn_stride, const void *ru, int ru_stride, int64_t n,
                    void *samples, uint64_t *failures, int64_t index_base, cudaStream_t stream);
int simt_append(const issm_bank *b, int slot, const void *logcounts, const void *x, int64_t n, void *lognum,
                uint64_t *failures, cudaStream_t stream);

// reductions (reduce.cu)
size_t reduce_workspace_bytes(int64_t n);
int logweight_summary(const void *lw, int64_t n, int dtype, double *out, void *ws, size_t ws_bytes,
                      cudaStream_t stream);
int normalize(const void *lw, int64_t n, int dtype, const double *summary, void *w, cudaStream_t stream);
int amis_form_summary(const void *lt, const void *lnum, const int64_t *round_ids, double logtotal, int64_t n,
                      int dtype, void *lw, uint64_t *failures, double *out, void *ws, size_t ws_bytes,
                      cudaStream_t stream);
int resampling_cdf(const void *lw, int64_t n, int dtype, void *cdf, void *ws, size_t ws_bytes,
                   cudaStream_t stream);

// resampling (resample.cu)
size_t resample_workspace_bytes(int64_t n);
int resample_select(const void *cdf, const void *lw, int64_t n, const void *u, int64_t count, int dtype,
                    int64_t *anc, cudaStream_t stream);
int resample_fixed(const void *lw, int64_t n, int dtype, const double *uniforms, double u, int systematic,
                   int64_t count, int64_t *anc, void *ws, size_t ws_bytes, cudaStream_t stream);
int gather(const void *src, int d, int64_t n_src, const int64_t *anc, int64_t count, int dtype, void *dst,
           cudaStream_t stream);
int local_resample(const void *lw, const int64_t *counts, int k, const void *u, const void *samples, int d,
                   int dtype, int64_t *anc, void *dst, cudaStream_t stream);

// moments and fit (moments.cu)
size_t moments_workspace_bytes(int64_t n, int d);
int weighted_moments(const void *x, int d, int64_t n, const void *lw, int dtype, const double *summary,
                     const double *shift, double *mean, double *cov, void *ws, size_t ws_bytes,
                     cudaStream_t stream);
int fit_factor(const double *mean, const double *cov, int d, const void *prev, double dof, double logconst,
               int dtype, void *out_loc, void *out_factor, void *out_lognorm, uint64_t *failures,
               int64_t failure_index, float *out_inverse, double regularization, cudaStream_t stream);

// population local weights, covariances, factors (population.cu)
int population_local_weights(const void *lw, const void *x, int d, int dtype, const int64_t *starts,
                             const int64_t *counts, const double *thresholds, int k, double tolerance,
                             int max_iterations, void *weights, void *local_ess, void *powers, uint8_t *status,
                             void *raw_means, cudaStream_t stream);
int population_covariances(const void *x, int d, int dtype, const void *weights, const void *powers,
                           const uint8_t *status, const void *locations, const issm_bank *bank,
                           const int64_t *starts, const int64_t *counts, int k, void *centres, void *covs,
                           cudaStream_t stream);
int population_factors(const void *covs, int d, int k, int dtype, const uint8_t *status, const void *dofs,
                       void *factors, int32_t *info, cudaStream_t stream);

// tensor maps of n x d FP32 sample arrays, 32-float x 128-row boxes (tma.cu)
bool row_tiles_supported(const void *x, int d, int64_t n);
int encode_row_tiles(CUtensorMap *map, const void *x, int d, int64_t n);

// one launch per phase across the in-flight runs of a serving loop (group.cu)
int group_step(const void *runs, int nruns, int64_t blocks_new, int64_t blocks_all, int64_t blocks_mom,
               cudaStream_t stream);

// result statistics (stats.cu)
size_t weighted_sum_workspace_bytes(int64_t n, int d);
int weighted_sum(const void *x, int d, int64_t n, const void *lw, int dtype, const double *summary, double *out,
                 void *ws, cudaStream_t stream);
size_t weighted_quantile_workspace_bytes(int d, int nprob);
int weighted_quantile(const void *x, int d, int64_t n, const void *lw, int dtype, const double *summary,
                      const double *probs, int nprob, double *out, void *ws, cudaStream_t stream);

// regression likelihood on tensor cores (glm_tc.cu)
size_t glm_operand_bytes(int nobs, int d, int precision);
int glm_prepare(const issm_target *t, int precision, void *ops, cudaStream_t stream);
int glm_logdensity(const issm_target *t, int precision, const void *ops, const float *x, int64_t n, float *out,
                   int *error, cudaStream_t stream);

// order statistic and N-PMC clipping (select.cu)
size_t select_workspace_bytes();
int select_kth(const void *v, int64_t n, int64_t k, int dtype, void *out, void *ws, cudaStream_t stream);
int clip_logweights(const void *raw, int64_t n, int dtype, const void *threshold, void *out, cudaStream_t stream);

// elementwise (elementwise.cu)
int static_assign(const void *cdf, int k, const void *u, int64_t n, int stratified, int32_t *slots, int dtype,
                  cudaStream_t stream);
int add_target_values(void *lw, const void *values, int64_t n, int dtype, uint64_t *failures,
                      int64_t index_base, cudaStream_t stream);
int subtract_logweights(const void *lt, const void *ld, int64_t n, int dtype, void *lw, uint64_t *failures,
                        int64_t index_base, cudaStream_t stream);
int amis_form(const void *lt, const void *lnum, const int64_t *round_ids, double logtotal, int64_t n,
              int dtype, void *lw, uint64_t *failures, cudaStream_t stream);
int failure_reset(uint64_t *f, cudaStream_t stream);
int check_target_values(const void *values, int64_t n, int dtype, int64_t *round_ids, uint64_t *failures,
                        int64_t index_base, cudaStream_t stream);

// built-in targets (targets.cu)
int target_logdensity(const issm_target *t, const void *x, int64_t n, void *out, cudaStream_t stream);

// tensor-core mixture density (mixture_tc.cu)
size_t tc_workspace_bytes(int k, int d);
int invert_factors(const issm_bank *bk, int first, int count, float *out, cudaStream_t stream);
int tc_mixture(const issm_bank *bk, const issm_denominator *den, int mode, int first, int last, const void *x,
               int64_t n, const int32_t *slots, int fixed_slot, const void *coef, void *out_logden,
               void *out_generating, void *lognum, uint64_t *failures, int64_t index_base, int precision, void *ws,
               size_t ws_bytes, int *error, cudaStream_t stream);

// tensor-core weighted moments (moments_tc.cu)
size_t moments_tc_workspace_bytes(int64_t n);
int moments_tc(const void *x, int d, int64_t n, const void *lw, const double *summary, const double *shift,
               const float *prev_factor,
               double *mean, double *cov, int precision, void *ws, size_t ws_bytes, int *error, cudaStream_t stream);

// tensor-core self-test (tc_selftest.cu)
int tc_gemm_selftest(const float *a, const float *b, float *c, int n, int k, int kind, int *status,
                     cudaStream_t stream);

// random streams (rng.cu)
int fill_normals(uint64_t seed, const uint64_t *base, uint64_t offset, int64_t n, void *out, int dtype,
                 cudaStream_t stream);
int fill_uniforms(uint64_t seed, const uint64_t *base, uint64_t offset, int64_t n, void *out, int dtype,
                  cudaStream_t stream);
int counter_advance(uint64_t *counter, uint64_t inc, cudaStream_t stream);

}  // namespace issm
