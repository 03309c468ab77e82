/*
 * issm.h — C ABI of libissm103.so, the sm_103a importance-sampling hot path.
 *
 * Every entry point is `extern "C"`, takes plain device pointers, element
 * counts and a CUDA stream, never allocates caller-visible memory, never calls
 * cudaDeviceSynchronize, and returns an int status:
 *   0                       success
 *   > 0                     a cudaError_t raised by a launch on the stream
 *   < 0                     an argument error (ISSM_E_*)
 * Sample-level numeric failures are NOT return errors: they are recorded in
 * the caller's 3-word failure record exactly as the reference packs them
 * (src/execution.jl:669-699, reason bits :758-767), so the reference's
 * `_device_failure_snapshot` -> `SamplerExecutionError` path reads them as-is.
 *
 * Layouts follow the reference's column-major Julia arrays:
 *   samples      d x N   sample i at x[i*d .. i*d+d-1]
 *   locations    d x K   component k at loc[k*d ..]
 *   factors      d x d x K, column-major lower-triangular L_k (zeros above)
 *   counts/coefs K x R   column r is one round
 * All float arrays of one call share the dtype given in the call (or in the
 * bank); reductions that the reference accumulates in >= Float32 are kept in
 * FP64 here and written to caller-provided FP64 device words.
 *
 * Threading: entry points are reentrant for distinct output/workspace
 * buffers; a prepared sampler that owns them is non-reentrant
 * (src/methods/importance_sampling.jl:105-116).
 */
#ifndef ISSM_H
#define ISSM_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same object as cudaStream_t (struct CUstream_st*); NULL = legacy stream. */
typedef struct CUstream_st *issm_stream_t;

/* ---- status codes ------------------------------------------------------ */
#define ISSM_OK                 0
#define ISSM_E_NULL           (-1)   /* a required pointer is NULL            */
#define ISSM_E_SIZE           (-2)   /* a size is negative or out of range    */
#define ISSM_E_DTYPE          (-3)   /* unsupported dtype / dtype mismatch    */
#define ISSM_E_KIND           (-4)   /* unknown family/scale/denominator kind */
#define ISSM_E_ALL_ZERO       (-5)   /* every log weight is -Inf (AllZeroWeightsError, src/results.jl:133-144) */
#define ISSM_E_UNSUPPORTED    (-6)   /* valid request this library does not run */
#define ISSM_E_WORKSPACE      (-7)   /* workspace too small                   */
#define ISSM_E_NOT_POSDEF     (-8)   /* Cholesky met a non-positive pivot     */
#define ISSM_E_SCRATCH_LIMIT  (-9)   /* input larger than a fixed scratch allows */

/* ---- enums ------------------------------------------------------------- */
#define ISSM_F32 0
#define ISSM_F64 1

#define ISSM_GAUSSIAN  0   /* GaussianFamily  src/proposals.jl:15            */
#define ISSM_STUDENT_T 1   /* StudentTFamily  src/proposals.jl:17-20         */

#define ISSM_SCALE_FACTOR    0  /* _FactorGaussianScale: L lower d x d      */
#define ISSM_SCALE_DIAGONAL  1  /* _DiagonalGaussianScale: d scales         */
#define ISSM_SCALE_SPHERICAL 2  /* _SphericalGaussianScale: 1 scale         */

/* Denominator kinds (src/mis_execution.jl:30-65 and the term policies):     */
#define ISSM_DENOM_FULL       0 /* all K slots, coef[k]   (_FullMixtureDenominator, src/methods/static_mis.jl:389-417;
                                   _RealizedMixtureDenominator, src/mis_execution.jl:67-89) */
#define ISSM_DENOM_GENERATING 1 /* generating slot only, coef 0 (_GeneratingDenominator, static_mis.jl:402-443) */
#define ISSM_DENOM_PARTIAL    2 /* slots in the generating slot's group, coef[k] (_PartialMixtureDenominator) */
#define ISSM_DENOM_PREFIX     3 /* slots 0..terms-1, coef[k] (_AMISMixtureDenominator, src/amis_execution.jl:12-35) */

/* Contraction precision of the Mahalanobis term. */
#define ISSM_PREC_NATIVE 0  /* SIMT in the bank dtype: the drop-in FP32/FP64 path */
#define ISSM_PREC_TF32   1  /* tcgen05 kind::tf32, FP32 accumulate, centred inputs */
#define ISSM_PREC_BF16   2  /* tcgen05 kind::f16 (bf16), FP32 accumulate, centred inputs */
#define ISSM_PREC_BF16X1 3  /* regression likelihood only: one bf16 product per K slice (no split) */

/* Failure reason bits (src/execution.jl:758-767, adaptive_gaussian_execution.jl:9) */
#define ISSM_REASON_TARGET_NAN          0x0100u
#define ISSM_REASON_TARGET_POS_INF      0x0200u
#define ISSM_REASON_PROPOSAL_INVALID    0x0400u
#define ISSM_REASON_GENERATED_NONFINITE 0x0800u
#define ISSM_REASON_LOGWEIGHT_INVALID   0x1000u
#define ISSM_REASON_DRAW_EXHAUSTED      0x0010u
#define ISSM_REASON_MOMENT_FIT_INVALID  0x2000u

/* A proposal bank packed as the reference's _PackedFactorBank /
 * _PackedDiagonalBank (src/proposal_banks.jl:139-163). All float arrays have
 * `dtype`. `dofs` is NULL for Gaussian banks; Student-t lognormalizers already
 * include the per-slot Student-t log constant (src/proposals.jl:413-437).
 * `range_risk` (optional, K bytes) marks slots whose factor exponent bound
 * makes the Student-t density take the full-range radius
 * (src/student_t_range.jl:35-36). */
typedef struct issm_bank {
    int32_t dim;           /* d >= 1                                     */
    int32_t count;         /* K >= 1 active slots                        */
    int32_t family;        /* ISSM_GAUSSIAN / ISSM_STUDENT_T             */
    int32_t scale_kind;    /* ISSM_SCALE_*                               */
    int32_t dtype;         /* ISSM_F32 / ISSM_F64                        */
    int32_t reserved;
    const void *locations;       /* d x K                                 */
    const void *scales;          /* factor d x d x K | diag d x K | sph K */
    const void *lognormalizers;  /* K                                     */
    const void *dofs;            /* K or NULL                             */
    const uint8_t *range_risk;   /* K or NULL                             */
    /* Optional FP32 inverse factors W_k = L_k^-1 for the tensor-core forms,
     * K x DP x DP row-major (row j holds W_k[j, :]), DP = 16 / 32 / 64 for
     * d <= 16 / 32 / 64, zero padded (issm_invert_factors writes them).
     * NULL: the tensor-core entry points form them per call. */
    const float *inverse_factors;
} issm_bank;

typedef struct issm_denominator {
    int32_t kind;                /* ISSM_DENOM_*                          */
    int32_t terms;               /* PREFIX: number of leading slots       */
    const void *logcoefficients; /* K, bank dtype (unused for GENERATING)  */
    const int32_t *group_of_slot;/* PARTIAL: group id per slot            */
} issm_denominator;

/* ---- introspection ----------------------------------------------------- */
/* Library version string, e.g. "issm103 1.0.0 sm_103a". */
const char *issm_version(void);
/* Human-readable message for a status code. */
const char *issm_status_string(int status);
/* Number of kernels this library has launched in this process (all threads). */
uint64_t issm_kernel_launches(void);

/* ---- failure record (src/execution.jl:669-756) ------------------------- */
/* Zero the 3-word record on the stream (replaces _reset_native_failure_scratch!,
 * src/execution.jl:652-657). */
int issm_failure_reset(uint64_t *failures, issm_stream_t stream);

/* ---- device random streams (replace CUDA.RNG draws,
 *      ext/ImportanceSamplersCUDAExt.jl:253-256) --------------------------- */
/* Standard normals / U[0,1) uniforms from counter-based Philox-4x32-10 with
 * Box-Muller; element i depends only on (seed, offset + i). */
int issm_fill_normals(uint64_t seed, uint64_t offset, int64_t n, void *out,
                      int32_t dtype, issm_stream_t stream);
int issm_fill_uniforms(uint64_t seed, uint64_t offset, int64_t n, void *out,
                       int32_t dtype, issm_stream_t stream);
/* Same streams at offset (*offset_base + offset) with the base read on the
 * device, so a captured CUDA graph draws fresh numbers on every replay once
 * issm_counter_advance moves the base. */
int issm_fill_normals_at(uint64_t seed, const uint64_t *offset_base,
                         uint64_t offset, int64_t n, void *out, int32_t dtype,
                         issm_stream_t stream);
int issm_fill_uniforms_at(uint64_t seed, const uint64_t *offset_base,
                          uint64_t offset, int64_t n, void *out, int32_t dtype,
                          issm_stream_t stream);
/* *counter += increment, stream-ordered (one-thread kernel). */
int issm_counter_advance(uint64_t *counter, uint64_t increment,
                         issm_stream_t stream);

/* ---- assignment and draw ---------------------------------------------- */
/* Static-MIS assignment: u' = (i + u_i)/N (stratified) or u_i (random), then
 * the first slot with u' <= cdf[slot]. Replaces _static_mis_assignment_kernel!
 * (src/static_mis_execution.jl:125-139; rule src/methods/static_mis.jl:171-211).
 * Writes 0-based slots. */
int issm_static_assign(const void *cdf, int32_t k, const void *uniforms,
                       int64_t n, int32_t stratified, int32_t *slots,
                       int32_t dtype, issm_stream_t stream);

/* Draw x_i = mu_s + L_s * (m_i * n_i) for slot s = slots[i] (or `fixed_slot`
 * when slots == NULL). Student-t banks compute the radial multiplier m_i from
 * the buffered Marsaglia-Tsang gamma draw (8 attempts) on `radial_normals`
 * and `radial_uniforms` with the given per-sample strides. Replaces
 * _native_store_sample! (src/native_execution.jl:488-528),
 * _scale_mis_normals_kernel! (:184-199) and _student_t_radial_multiplier
 * (:153-180). Non-finite draws record ISSM_REASON_GENERATED_NONFINITE.
 * `index_base` is added to the 0-based sample index before it is packed
 * (1-based logical index = index_base + i + 1). */
int issm_draw(const issm_bank *bank, const int32_t *slots, int32_t fixed_slot,
              const void *normals, const void *radial_normals,
              int32_t radial_normal_stride, const void *radial_uniforms,
              int32_t radial_uniform_stride, int64_t n, void *samples,
              uint64_t *failures, int64_t index_base, issm_stream_t stream);

/* issm_draw from component `fixed_slot` of a factor bank with the standard
 * normals generated in the kernel: row i, coordinate e takes element
 * offset + (*counter if counter) + i d + e of the (seed) stream that
 * issm_fill_normals_at writes, so the samples are bitwise those of
 * issm_fill_normals_at followed by issm_draw, and no normal is stored.
 * ISSM_E_UNSUPPORTED for scalar or spherical scales. No reference
 * counterpart: the reference fills a normal buffer and then draws from it
 * (_launch_prefilled_amis_factor_batch!, src/amis_execution.jl:162-194). */
int issm_draw_philox(const issm_bank *bank, int32_t fixed_slot, uint64_t seed,
                     const uint64_t *counter, uint64_t offset,
                     const void *radial_normals, int32_t radial_normal_stride,
                     const void *radial_uniforms, int32_t radial_uniform_stride,
                     int64_t n, void *samples, uint64_t *failures,
                     int64_t index_base, issm_stream_t stream);

/* ---- balance-heuristic denominators ------------------------------------ */
/* out_logden[i] = log sum_{k in terms(i)} exp(coef_k + log q_k(x_i)),
 * out_generating[i] = log q_{slots[i]}(x_i) (optional). Records
 * ISSM_REASON_PROPOSAL_INVALID when the generating density or the
 * denominator is NaN or -Inf, and then writes -Inf.
 * Replaces _mis_logdenominator_core (src/mis_execution.jl:30-65) over
 * _packed_gaussian_logdensity! (src/native_execution.jl:346-384) and
 * _radial_logdensity (src/proposals.jl:24-55). `precision` selects the SIMT
 * path (NATIVE) or the tcgen05 contraction (TF32/BF16; factor-Gaussian and
 * factor-Student-t banks, FP32 samples, d <= 64). */
int issm_mixture_logdensity(const issm_bank *bank, const issm_denominator *den,
                            const void *x, int64_t n, const int32_t *slots,
                            int32_t fixed_slot, void *out_logden,
                            void *out_generating, uint64_t *failures,
                            int64_t index_base, int32_t precision,
                            issm_stream_t stream);

/* Workspace variants that also run the tensor-core precision forms
 * (ISSM_PREC_TF32, ISSM_PREC_BF16 = bf16 split in three products) for
 * factor-Gaussian / factor-Student-t FP32 banks with d <= 64; NATIVE
 * precision runs the SIMT path and ignores the workspace. The workspace
 * holds the per-call MMA operand forms [W_k | -W_k (mu_k - c)] of the slots
 * (c = the centre slot's mean), the centre, and — when the bank carries no
 * inverse_factors — the inverse factors formed for the call; its last 64
 * bytes hold a sticky error word that a timed-out tensor-core completion
 * wait sets to 1 (zero the workspace once when it is created).
 * workspace_bytes >= issm_tc_workspace_bytes(K, d). */
size_t issm_tc_workspace_bytes(int32_t k, int32_t d);
/* W_k = L_k^-1 for factor slots [first, first + count) of an FP32 or FP64
 * factor bank, formed in FP32 by blocked triangular inversion and written
 * into out (K x DP x DP, layout of issm_bank.inverse_factors). */
int issm_invert_factors(const issm_bank *bank, int32_t first, int32_t count,
                        float *out, issm_stream_t stream);
int issm_mixture_logdensity_ws(const issm_bank *bank, const issm_denominator *den,
                               const void *x, int64_t n, const int32_t *slots,
                               int32_t fixed_slot, void *out_logden,
                               void *out_generating, uint64_t *failures,
                               int64_t index_base, int32_t precision,
                               void *workspace, size_t workspace_bytes,
                               issm_stream_t stream);
int issm_amis_append_ws(const issm_bank *history, int32_t slot,
                        const void *logcounts, const void *x, int64_t n,
                        void *lognumerators, uint64_t *failures,
                        int32_t precision, void *workspace,
                        size_t workspace_bytes, issm_stream_t stream);

/* Fused static-MIS / DM-PMC round: draw + denominator + log weight.
 * logw_i = logtarget_i - logden_i when `logtargets` is non-NULL; with
 * logtargets == NULL the target is deferred (the reference's batch-target
 * path, src/batched_targets.jl:70-77) and logw_i = -logden_i, finished later
 * by issm_add_target_values. proposal_ids_out[i] = proposal_ids[slot] (or 0
 * on failure). Replaces _mis_round_launch_kernel! (src/mis_execution.jl:674-720). */
int issm_mis_round(const issm_bank *bank, const issm_denominator *den,
                   const int32_t *slots, const void *normals,
                   const void *radial_normals, int32_t radial_normal_stride,
                   const void *radial_uniforms, int32_t radial_uniform_stride,
                   const void *logtargets, int64_t n, void *samples,
                   void *logweights, const int64_t *proposal_ids,
                   int64_t *proposal_ids_out, uint64_t *failures,
                   int32_t precision, issm_stream_t stream);

/* Batch-target finish: logw_i += values_i, recording target NaN/+Inf and
 * invalid log weights. Replaces _finish_batch_weights! (src/batched_targets.jl:204-214). */
int issm_add_target_values(void *logweights, const void *values, int64_t n,
                           int32_t dtype, uint64_t *failures,
                           int64_t index_base, issm_stream_t stream);

/* Record NaN / +Inf target values of a batch target (_native_target_reason,
 * src/execution.jl:769-773) and, when round_ids is given, set the failed
 * samples' round id to 0 so later stages skip them, as the reference's round
 * kernel leaves them (src/mis_execution.jl:722-771). */
int issm_check_target_values(const void *values, int64_t n, int32_t dtype,
                             int64_t *round_ids, uint64_t *failures,
                             int64_t index_base, issm_stream_t stream);

/* logw_i = logtarget_i - logden_i with the reference's invalid-weight check
 * (_subtract_logweight, src/methods/importance_sampling.jl:1261-1266). */
int issm_subtract_logweights(const void *logtargets, const void *logden,
                             int64_t n, int32_t dtype, void *logweights,
                             uint64_t *failures, int64_t index_base,
                             issm_stream_t stream);

/* ---- AMIS retrospective recurrence (src/amis_execution.jl) -------------- */
/* Old samples: lognum_i <- logaddexp(lognum_i, logcounts[slot] + log q_slot(x_i)).
 * Replaces _append_logmixture_kernel! (src/amis_execution.jl:37-71). */
int issm_amis_append(const issm_bank *history, int32_t slot,
                     const void *logcounts, const void *x, int64_t n,
                     void *lognumerators, uint64_t *failures,
                     int32_t precision, issm_stream_t stream);

/* All samples of rounds 1..t: logw_i = logtarget_i - (lognum_i - logtotal)
 * for round_ids[i] != 0. Replaces _form_amis_logweights_kernel!
 * (src/amis_execution.jl:107-134). */
int issm_amis_form(const void *logtargets, const void *lognumerators,
                   const int64_t *round_ids, double logtotal, int64_t n,
                   int32_t dtype, void *logweights, uint64_t *failures,
                   issm_stream_t stream);

/* issm_amis_form and issm_logweight_summary in one pass: the summary covers
 * the log weights this call writes (samples with round_ids[i] != 0 and a
 * valid weight). workspace: issm_reduce_workspace_bytes(n) bytes. */
int issm_amis_form_summary(const void *logtargets, const void *lognumerators,
                           const int64_t *round_ids, double logtotal, int64_t n,
                           int32_t dtype, void *logweights, uint64_t *failures,
                           double *summary, void *workspace,
                           size_t workspace_bytes, issm_stream_t stream);

/* ---- log-weight reductions (src/execution.jl:103-186, src/results.jl:6-36,560-626) */
/* out[0..2] = (max, sum exp(l-max), sum exp(2(l-max))) in FP64 over n log
 * weights, merged as _merge_logweight_moments. out is 3 FP64 device words.
 * workspace: issm_reduce_workspace_bytes(n) bytes of device memory. */
size_t issm_reduce_workspace_bytes(int64_t n);
int issm_logweight_summary(const void *logweights, int64_t n, int32_t dtype,
                           double *out, void *workspace, size_t workspace_bytes,
                           issm_stream_t stream);

/* w_i = exp(l_i - max) / S using a summary produced by
 * issm_logweight_summary (device FP64 words). Replaces normalized_weights
 * (src/results.jl:589-598) and _normalize_moment_weights! (adaptive_gaussian_execution.jl:207-247). */
int issm_normalize(const void *logweights, int64_t n, int32_t dtype,
                   const double *summary, void *weights, issm_stream_t stream);

/* ---- resampling (src/resampling.jl) ------------------------------------ */
/* Reference-compatible CDF: cdf = cumsum(exp(l - max)) / total in the
 * logweight dtype (>= F32). Replaces _resampling_cdf! (src/resampling.jl:199-225). */
int issm_resampling_cdf(const void *logweights, int64_t n, int32_t dtype,
                        void *cdf, void *workspace, size_t workspace_bytes,
                        issm_stream_t stream);
/* No-allocation variant of issm_resampling_cdf, with no counterpart in the
 * reference. For callers that cannot allocate device memory around the call
 * (a binding holding only the log-weight and CDF pointers, a host with a
 * fixed device-memory budget): the workspace is one fixed 264 KiB __device__
 * array inside the library, so the call allocates nothing. At most
 * issm_resampling_cdf_static_max() = 2^27 log weights; larger n returns
 * ISSM_E_SCRATCH_LIMIT. The first call in each CUDA context (each device's
 * primary context, again after a device reset, and any context the host
 * creates itself) looks up the array's address there (cudaGetSymbolAddress),
 * which may load the module: make that call before any stream capture. The
 * array is shared by all calls on a device, so calls
 * that overlap in time there (other streams or threads) race and corrupt each
 * other's results: serialise them. Same results as issm_resampling_cdf. */
int64_t issm_resampling_cdf_static_max(void);
int issm_resampling_cdf_static(const void *logweights, int64_t n, int32_t dtype,
                               void *cdf, issm_stream_t stream);
/* Ancestors (1-based, as the reference) for given uniforms: first j with
 * u < cdf[j] (strict), then the -Inf plateau repair. Replaces
 * _select_resampling_ancestors_kernel! (src/resampling.jl:92-118). */
int issm_resample_select(const void *cdf, const void *logweights, int64_t n,
                         const void *uniforms, int64_t count, int32_t dtype,
                         int64_t *ancestors, issm_stream_t stream);
/* Deterministic multinomial / systematic resampling on an exact 64-bit
 * fixed-point CDF of w_j = exp(l_j - max) (see docs); ancestors 1-based.
 * Systematic uses one uniform u: u_i = (i + u)/count. */
size_t issm_resample_workspace_bytes(int64_t n);
int issm_resample_multinomial(const void *logweights, int64_t n, int32_t dtype,
                              const double *uniforms, int64_t count,
                              int64_t *ancestors, void *workspace,
                              size_t workspace_bytes, issm_stream_t stream);
int issm_resample_systematic(const void *logweights, int64_t n, int32_t dtype,
                             double u, int64_t count, int64_t *ancestors,
                             void *workspace, size_t workspace_bytes,
                             issm_stream_t stream);
/* dst[:, i] = src[:, ancestors[i]] (1-based ancestors). Replaces
 * _gather_resampled_samples_kernel! (src/resampling.jl:160-164). */
int issm_gather(const void *src, int32_t d, int64_t n_src,
                const int64_t *ancestors, int64_t count, int32_t dtype,
                void *dst, issm_stream_t stream);
/* DM-PMC local resampling: one ancestor per proposal slot from that slot's
 * contiguous run of `counts[slot]` samples, threshold u_slot * total with a
 * strict < scan; ancestor 0 when the slot has no positive weight. Replaces
 * _local_resample_locations_kernel! and the cooperative GPU variant
 * (src/dm_pmc_execution.jl:80-265). */
int issm_local_resample(const void *logweights, const int64_t *counts,
                        int32_t k, const void *uniforms, const void *samples,
                        int32_t d, int32_t dtype, int64_t *ancestors,
                        void *destination, issm_stream_t stream);

/* ---- adaptation moments (src/adaptive_gaussian_execution.jl:186-528) ---- */
/* Weighted mean and covariance with normalised weights exp(l - max)/S taken
 * from a device summary: mean = sum w x, cov = sum w (x-mean)(x-mean)^T, in
 * FP64, accumulated about `shift` (d FP64 device words, e.g. the previous
 * mean). Replaces _weighted_moments! (:268-273). workspace:
 * issm_moments_workspace_bytes(n, d). */
size_t issm_moments_workspace_bytes(int64_t n, int32_t d);
int issm_weighted_moments(const void *x, int32_t d, int64_t n,
                          const void *logweights, int32_t dtype,
                          const double *summary, const double *shift,
                          double *mean, double *cov, void *workspace,
                          size_t workspace_bytes, issm_stream_t stream);
/* As issm_weighted_moments with a precision: ISSM_PREC_TF32 / ISSM_PREC_BF16
 * run a tensor-core pass over FP32 samples about `shift`, accumulating
 * sum w z z^T, sum w z and sum w in FP32 tensor memory and finishing in FP64
 * (d <= 64; the split products form the Gram matrix of the bf16 hi/lo
 * operand, so the covariance is semidefinite), and a second pass centred at
 * the first pass's mean when the first pass's cancellation error
 * (2^-16 of a diagonal second moment about `shift`) exceeds 2^-8 of that
 * variance plus 2^-4 of R = sqrt(eps(Float32)) tr(L L^T) / d, L =
 * `prev_factor` (the previous proposal's d x d factor in `dtype`, column-major;
 * NULL takes R = 0). NATIVE runs the two-pass SIMT kernels and ignores
 * `prev_factor`. workspace_bytes >=
 * issm_moments_workspace_bytes(n, d); its last 64 bytes hold the sticky
 * tensor-core timeout word and a completion counter (zero the workspace once
 * when it is created; every call leaves the counter at zero). */
int issm_weighted_moments_ws(const void *x, int32_t d, int64_t n,
                             const void *logweights, int32_t dtype,
                             const double *summary, const double *shift,
                             const void *prev_factor,
                             double *mean, double *cov, int32_t precision,
                             void *workspace, size_t workspace_bytes,
                             issm_stream_t stream);

/* Candidate fit: cov + ridge I with ridge = sqrt(eps(T)) tr(L_prev L_prev^T)
 * * c_nu / d (src/adaptive_gaussian_execution.jl:283-301, src/execution.jl:188-194),
 * FP64 Cholesky, Student-t scaling by sqrt((nu-2)/nu), lognormalizer and the
 * validity rule (:475-528). Writes mean/factor/lognormalizer in `dtype` into
 * the history slot pointers; records ISSM_REASON_MOMENT_FIT_INVALID at
 * logical index `failure_index` on failure. `dof` <= 0 means Gaussian. */
int issm_fit_factor(const double *mean, const double *cov, int32_t d,
                    const void *previous_factor, double dof,
                    double logconstant, int32_t dtype, void *out_location,
                    void *out_factor, void *out_lognormalizer,
                    uint64_t *failures, int64_t failure_index,
                    issm_stream_t stream);
/* As issm_fit_factor, also writing the FP32 inverse of the new factor
 * (issm_bank.inverse_factors layout, one slot) when out_inverse != NULL, so a
 * proposal history keeps its tensor-core operands current. */
int issm_fit_factor_ex(const double *mean, const double *cov, int32_t d,
                       const void *previous_factor, double dof,
                       double logconstant, int32_t dtype, void *out_location,
                       void *out_factor, void *out_lognormalizer,
                       float *out_inverse, uint64_t *failures,
                       int64_t failure_index, issm_stream_t stream);
/* As issm_fit_factor_ex with the ridge coefficient given: `regularization`
 * >= 0 replaces sqrt(eps(T)) of _factor_scale_aware_ridge
 * (src/adaptive_gaussian_execution.jl:385-389, which fixes it to the
 * element type); a negative value keeps sqrt(eps(T)). An FP64 run that
 * passes sqrt(eps(Float32)) fits with the same ridge as an FP32 run, so the
 * two differ by their arithmetic alone. NaN is ISSM_E_KIND. */
int issm_fit_factor_reg(const double *mean, const double *cov, int32_t d,
                        const void *previous_factor, double dof,
                        double logconstant, int32_t dtype,
                        double regularization, void *out_location,
                        void *out_factor, void *out_lognormalizer,
                        float *out_inverse, uint64_t *failures,
                        int64_t failure_index, issm_stream_t stream);

/* ---- result statistics ------------------------------------------------------
 * Statistics.mean(result) / mean(f, result) (src/statistics.jl:11-33): the
 * self-normalised weighted sum out[c] = sum_i w_i x[i, c] (FP64, d >= 1),
 * with w_i = e^{l_i - m} / S from the 3-word summary of the log weights;
 * bitwise reproducible (per-block partials reduced in a fixed order). For
 * the functional mean pass f's values as x with d = 1. */
size_t issm_weighted_sum_workspace_bytes(int64_t n, int32_t d);
int issm_weighted_sum(const void *x, int32_t d, int64_t n, const void *logweights,
                      int32_t dtype, const double *summary, double *out,
                      void *workspace, size_t workspace_bytes, issm_stream_t stream);
/* Statistics.quantile(result, probabilities) (src/statistics.jl:106-154):
 * component-wise weighted quantiles with the StatsBase generic-weight rule
 * (threshold p (W - w_first) + w_first over the value-sorted positive-weight
 * samples, linear interpolation between the neighbours), on the device with
 * no sort (a weighted radix select); out[q * d + c] for probability q and
 * coordinate c, in FP64 holding the sample type's value; NaN for a
 * coordinate with a NaN sample. probabilities: device FP64, each in [0, 1]
 * (the caller checks). The reference evaluates it on the host only. */
size_t issm_weighted_quantile_workspace_bytes(int32_t d, int32_t nprob);
int issm_weighted_quantile(const void *x, int32_t d, int64_t n, const void *logweights,
                           int32_t dtype, const double *summary,
                           const double *probabilities, int32_t nprob, double *out,
                           void *workspace, size_t workspace_bytes,
                           issm_stream_t stream);

/* ---- N-PMC weight clipping ---------------------------------------------------
 * _moment_adaptation_workspace!(::NPMC, ...) (src/npmc_execution.jl:22-33):
 * the isqrt(n) largest of a round's n log weights are clipped to the
 * (n - isqrt(n) + 1)-th smallest, clipped = min(raw, threshold) (NaN when
 * either is NaN, as Julia's min), with the order statistic of the
 * reference's sort (NaN last) found on the device by a radix select: no host
 * read. `threshold` is a device scalar of `dtype` that receives the order
 * statistic. issm_select_kth is the order statistic alone: the k-th smallest
 * (1-based) of n values into the device scalar `out`. The workspace is
 * issm_select_workspace_bytes() bytes; calls sharing one must be ordered. */
size_t issm_select_workspace_bytes(void);
int issm_select_kth(const void *values, int64_t n, int64_t k, int32_t dtype,
                    void *out, void *workspace, size_t workspace_bytes,
                    issm_stream_t stream);
int issm_npmc_clip(const void *raw_logweights, int64_t n, int32_t dtype,
                   void *clipped, void *threshold, void *workspace,
                   size_t workspace_bytes, issm_stream_t stream);

/* ---- population adaptation --------------------------------------------------
 * The per-proposal ("local") weights, covariances and factors of a
 * population of K proposals (src/population_covariance.jl). Slot k's samples
 * are the contiguous range starts[k] .. starts[k] + counts[k] - 1 (0-based;
 * the reference's starts[k, round] - 1) of `samples` (d x N column-major) and
 * of the per-sample arrays; starts/counts/thresholds are the round's columns,
 * device arrays of K entries. status: 0 ready, 1 every local log weight is
 * -Inf, 2 the tempering search found no feasible power. Sums and the
 * Cholesky run in FP64; outputs are written in `dtype`. */

/* _population_local_weights! (src/population_covariance.jl:115-480): per slot
 * the normalised weights exp(l - max) / sum (into normalized_weights at the
 * slot's samples), the local ESS, the tempering power (1 when the raw ESS
 * reaches thresholds[k], else the largest power in (0, 1) found by bisection
 * to `tolerance` in at most `max_iterations` steps whose tempered ESS does,
 * with the weights re-normalised at that power) and the status. raw_means
 * (d x K, or NULL) receives the untempered weighted mean. */
int issm_population_local_weights(const void *local_logweights, const void *samples,
                                  int32_t d, int32_t dtype, const int64_t *starts,
                                  const int64_t *counts, const double *thresholds,
                                  int32_t k, double tolerance, int32_t max_iterations,
                                  void *normalized_weights, void *local_ess,
                                  void *tempering_powers, uint8_t *status,
                                  void *raw_means, issm_stream_t stream);
/* _fit_population_covariances! (src/population_covariance.jl:482-805): for a
 * ready slot the weighted covariance sum w (x - c)(x - c)^T about its centre
 * c (the weighted mean when the slot was tempered, its location otherwise);
 * a slot that is not ready keeps the current covariance of slot k of
 * `current` (L L^T, or the squared diagonal/spherical scale, times
 * nu / (nu - 2) for Student-t). centres (d x K) and covariances (d x d x K,
 * symmetric) are written; d <= 64. */
int issm_population_covariances(const void *samples, int32_t d, int32_t dtype,
                                const void *normalized_weights,
                                const void *tempering_powers, const uint8_t *status,
                                const void *locations, const issm_bank *current,
                                const int64_t *starts, const int64_t *counts,
                                int32_t k, void *centres, void *covariances,
                                issm_stream_t stream);
/* _factor_population_covariances! and _scale_population_factors!
 * (src/population_covariance.jl:807-973): the lower Cholesky factor of each
 * ready slot's covariance (zeros above the diagonal) with potrf's info
 * (0, the failing column, or -1 for a non-finite covariance; 0 and no write
 * for slots that are not ready), then, when `dofs` (K entries) is given, the
 * Student-t scaling sqrt((nu - 2) / nu) of every ready slot. d <= 64. */
int issm_population_factors(const void *covariances, int32_t d, int32_t k,
                            int32_t dtype, const uint8_t *status, const void *dofs,
                            void *factors, int32_t *info, issm_stream_t stream);

/* ---- built-in batch targets ------------------------------------------------
 * Native equivalents of the batch callbacks the benchmark workloads pass to
 * LogTarget(...; batch=...) (src/targets.jl:65-76, src/batched_targets.jl:54-114):
 *   STD_NORMAL  N(0, I)                              (normalised)
 *   QUADRATIC   -|x - a|^2 / p0                      (a: d)
 *   GAUSS_MIX   equal-weight N(a_j, I), j < count    (a: d x count; normalised)
 *   STUDENT_T   t_nu(a, b b^T), nu = p0, p1 = log constant - log|b|  (b: d x d)
 *   LINREG      N(y | X beta, p0^2 I) N(beta | 0, p1 I)  (X: count x d, y: count)
 *   LOGISTIC    Bernoulli-logit(y | X beta) N(beta | 0, p1 I)                    */
#define ISSM_TARGET_GAUSS_MIX  0
#define ISSM_TARGET_STUDENT_T  1
#define ISSM_TARGET_LINREG     2
#define ISSM_TARGET_LOGISTIC   3
#define ISSM_TARGET_STD_NORMAL 4
#define ISSM_TARGET_QUADRATIC  5
typedef struct issm_target {
    int32_t kind, dim, count, dtype;
    const void *a, *b, *c;
    double p0, p1;
} issm_target;
/* out[i] = log target(x_i) for n samples (d x n, target dtype). */
int issm_target_logdensity(const issm_target *target, const void *x, int64_t n,
                           void *out, issm_stream_t stream);

/* The LINREG / LOGISTIC targets' likelihood as a tensor-core GEMM: X beta
 * for every (sample, observation) pair on tcgen05 with the Gaussian or
 * Bernoulli-logit log-likelihood reduced in the epilogue, plus the prior
 * (the batch callbacks of src/batched_targets.jl:54-214 and
 * examples/batched_linear_regression.jl:18-37, whose X beta is a GEMM).
 * FP32 target, d <= 64. precision: ISSM_PREC_BF16 (bf16 x3 split),
 * ISSM_PREC_TF32, or ISSM_PREC_BF16X1 (one bf16 product: the plain BF16
 * GEMM form, about 8 bits per product). issm_glm_prepare writes the
 * observations' operand form (issm_glm_operand_bytes) once per target and
 * precision; issm_glm_logdensity then evaluates n samples (d x n). `error`
 * is a device int the caller zeroes; it becomes 1 if a completion wait
 * timed out. Results stay within the form's log-density tolerance of
 * issm_target_logdensity. */
size_t issm_glm_operand_bytes(int32_t nobs, int32_t d, int32_t precision);
int issm_glm_prepare(const issm_target *target, int32_t precision, void *operand,
                     size_t operand_bytes, issm_stream_t stream);
int issm_glm_logdensity(const issm_target *target, int32_t precision,
                        const void *operand, const float *x, int64_t n,
                        float *out, int32_t *error, issm_stream_t stream);

/* ---- one AMIS run in one call --------------------------------------------
 * Every launch of an AMIS run with a Gaussian factor proposal (draws with
 * in-kernel normals, target, retrospective append, prefix mixture, weights
 * and per-round summary, moments, FP64 fit), stream-ordered with no host
 * synchronisation: the same library calls, in the same order, as the host
 * round loop, so the results are bitwise those of issuing them one by one.
 * Replaces the round loop over _launch_prefilled_amis_round!
 * (src/amis_execution.jl:261-357) and _fit_moment_proposal!
 * (src/adaptive_gaussian_execution.jl:348-425).
 * history: `rounds` (or more) slots; slot 0 is overwritten with the initial
 * proposal, slot t + 1 receives round t's fit; inverse_factors is required
 * for the tensor-core precisions. Sample t of round r takes normal stream
 * elements from normal_offset (+ *counter); *counter advances by the run's
 * total at the end. The workspace (issm_amis_run_workspace_bytes) is zeroed
 * by the run itself at its start; it holds, in order, the tensor-core scratch
 * (issm_tc_workspace_bytes(rounds, d), rounded up to 256 bytes), the moments
 * scratch (issm_moments_workspace_bytes(total, d), rounded up) and the
 * reduction scratch; the first two end in their sticky timeout words.
 * target_operand, when not NULL, is the regression target's operand form
 * (issm_glm_prepare for target_precision) and the target runs through
 * issm_glm_logdensity, its timeout word shared with the tensor-core
 * scratch's; NULL runs issm_target_logdensity (SIMT, the target's type).
 * target_bank, when not NULL, is a target that is itself a radial mixture
 * (a normalised Student-t or Gaussian, one slot or several): it runs through
 * issm_mixture_logdensity[_ws] with target_den at target_bank_precision, the
 * tensor-core scratch shared, and `target` may then be NULL.
 * ISSM_E_UNSUPPORTED for Student-t or non-factor histories. */
typedef struct issm_amis_run_desc {
    issm_bank history;
    const issm_target *target;
    int32_t rounds, precision;
    const int64_t *round_sizes;      /* host, rounds entries */
    double logconstant;              /* radial log constant of the family (0 for Gaussian) */
    uint64_t seed, normal_offset;
    uint64_t *counter;               /* device normal-stream base, or NULL */
    const void *logcounts;           /* device, log(round_sizes) in the history dtype */
    const int64_t *round_ids_init;   /* device, round id (1-based) of each sample */
    const void *initial_location, *initial_factor, *initial_lognormalizer;
    void *samples, *logtargets, *lognum, *logweights;  /* total (x d) entries */
    int64_t *round_ids;
    double *summaries;               /* rounds x 3: (max, S, S2) of each round's weights */
    int64_t *round_failures;         /* rounds x 3 failure records */
    double *mean, *cov, *shift;      /* FP64 scratch: d, d x d, d */
    void *cand_location, *cand_factor, *cand_lognormalizer;  /* the last round's fit */
    void *workspace;
    size_t workspace_bytes;
    const void *target_operand;      /* issm_glm_prepare output, or NULL */
    int32_t target_precision, reserved;
    const issm_bank *target_bank;            /* a normalised radial target, or NULL */
    const issm_denominator *target_den;      /* its denominator (slot 0 generating, or full) */
    int32_t target_bank_precision, reserved2;
} issm_amis_run_desc;
size_t issm_amis_run_workspace_bytes(int32_t d, int64_t total, int32_t rounds);
int issm_amis_run(const issm_amis_run_desc *run, issm_stream_t stream);
/* sizeof(issm_amis_run_desc) and the offset of its workspace_bytes field,
 * for bindings that mirror the struct (checked by the CPU tests). */
size_t issm_amis_run_desc_bytes(void);
size_t issm_amis_run_desc_workspace_offset(void);

/* ---- many runs per launch (serving) -----------------------------------------
 * No one-call counterpart in the reference, which runs each sampler's rounds
 * on its own (the per-run sequence is _launch_prefilled_amis_round!,
 * src/amis_execution.jl:261-357, then _fit_moment_proposal!,
 * src/adaptive_gaussian_execution.jl:348-425). issm_group_step advances every
 * run of a device table of issm_group_run rows by one AMIS round with seven
 * launches in all, however many runs: draws from the counter-based normal
 * stream, the linear-regression target in its mode-centred quadratic form,
 * the retrospective mixture, weights and their summary, moment sums about the
 * previous location (compensated FP32 per block, merged in FP64), and the FP64
 * fit of the next proposal. Gaussian
 * factor proposals, FP32 samples, d <= 64, one sample count per round per
 * run. Rows are ordered by their block offsets: blk_new0 (ceil(n_round /
 * ISSM_GROUP_TILE) blocks per run), blk_all0 (ceil((n_old + n_round) /
 * ISSM_GROUP_TILE)) and blk_mom0 (ceil((n_old + n_round) /
 * ISSM_GROUP_MOMENT_SAMPLES), = nmom) are each run's cumulative starts and
 * blocks_new / blocks_all / blocks_mom the totals. `partial` holds 3 doubles
 * per blk_all block and `mpartial` ISSM_GROUP_MOMENT_WORDS per moment block.
 * A run only touches its own arrays and every per-run reduction has a fixed
 * order, so its results do not depend on the other runs in the table. */
#define ISSM_GROUP_TILE 128
#define ISSM_GROUP_MOMENT_SAMPLES 2048
#define ISSM_GROUP_MOMENT_WORDS 2145
typedef struct issm_group_run {
    int64_t d, rounds, round, n_round, n_old;   /* round: 0-based round of this step */
    uint64_t seed, normal_offset;               /* normal stream position of this round */
    int64_t blk_new0, blk_all0, blk_mom0, nmom;
    float *samples, *logtargets, *lognum, *logweights;   /* rounds * n_round (x d) */
    float *loc, *fac, *lognorm;                 /* history: rounds slots, factors column-major */
    float *cand_loc, *cand_fac, *cand_lognorm;  /* the last round's fit */
    const float *t_mode, *t_chol;               /* target: mode (d), U (d x d column-major, upper) */
    double *summaries;                          /* rounds x 3: (max, S, S2) of each round's weights */
    double *mean, *cov;                         /* FP64 d, d x d: the last fit's moments */
    uint64_t *failures;                         /* rounds x 3 failure records */
    double *partial, *mpartial;                 /* scratch of this step */
    double t_const;                             /* target: log p(y, mode) */
    double logcount;                            /* log n_round */
} issm_group_run;
size_t issm_group_run_bytes(void);
int issm_group_step(const issm_group_run *runs, int32_t nruns, int64_t blocks_new,
                    int64_t blocks_all, int64_t blocks_mom, issm_stream_t stream);

/* ---- tensor-core self-test ------------------------------------------------
 * No counterpart in the reference: a one-CTA tcgen05 GEMM
 * C[128 x n] = A[128 x k] B[n x k]^T (row-major FP32 in and out; inputs rounded
 * to bf16 when kind = ISSM_PREC_BF16 or read as tf32 when kind = ISSM_PREC_TF32)
 * that pins the shared-memory and instruction descriptor encodings used by
 * the tensor-core kernels. n in {16, 32, ..., 256}; k a multiple of 16 (bf16)
 * or 8 (tf32), k <= 64 (k <= 128 MN-major). kind | 0x100 stages both operands in the
 * row-contiguous layout (each 16-byte K group holds the rows consecutively)
 * instead of 8-row core-matrix blocks; kind | 0x200 (bf16 only) stages them
 * MN-major (8 rows of one K index per 16 bytes). *status (device int,
 * zeroed by the caller) becomes 1 if the MMA completion wait timed out. */
int issm_tc_selftest(const float *a, const float *b, float *c, int32_t n,
                     int32_t k, int32_t kind, int32_t *status,
                     issm_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif /* ISSM_H */
