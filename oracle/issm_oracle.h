/*
 * issm_oracle.h — CPU restatement (FP64, plain C99 + OpenMP) of the
 * reference's importance-sampling hot path. TEST INFRASTRUCTURE ONLY: the
 * parity checker for the CUDA library and the timed CPU baseline. Nothing in
 * the product links it.
 *
 * Pinned against the literal vectors of the reference's own tests (see
 * tests/golden/); systematic resampling has no reference implementation and
 * its parity is unpinned (the rule here is the textbook one on the same
 * deterministic fixed-point CDF the GPU uses).
 *
 * Conventions: samples d x N column-major (sample i at x + i*d); slots are
 * 0-based; resampling ancestors are 1-based like the reference.
 */
#ifndef ISSM_ORACLE_H
#define ISSM_ORACLE_H
#include <stdint.h>

#define ORC_GAUSSIAN 0
#define ORC_STUDENT_T 1
#define ORC_SCALE_FACTOR 0
#define ORC_SCALE_DIAGONAL 1
#define ORC_SCALE_SPHERICAL 2
#define ORC_DENOM_FULL 0
#define ORC_DENOM_GENERATING 1
#define ORC_DENOM_PARTIAL 2
#define ORC_DENOM_PREFIX 3

#define ORC_REASON_TARGET_NAN 0x0100u
#define ORC_REASON_TARGET_POS_INF 0x0200u
#define ORC_REASON_PROPOSAL_INVALID 0x0400u
#define ORC_REASON_GENERATED_NONFINITE 0x0800u
#define ORC_REASON_LOGWEIGHT_INVALID 0x1000u
#define ORC_REASON_DRAW_EXHAUSTED 0x0010u
#define ORC_REASON_MOMENT_FIT_INVALID 0x2000u

typedef struct orc_bank {
    int d, k, family, scale_kind;
    const double *loc;      /* d x K */
    const double *scales;   /* d x d x K | d x K | K */
    const double *lognorm;  /* K */
    const double *dofs;     /* K or NULL */
    const unsigned char *range_risk; /* K or NULL */
} orc_bank;

typedef struct orc_target {
    int kind;          /* ORC_TARGET_* */
    int d, j;          /* dimension, components / observations */
    const double *a;   /* kind-specific arrays, see issm_oracle.c */
    const double *b;
    const double *c;
    double p0, p1;
} orc_target;
#define ORC_TARGET_GAUSS_MIX 0   /* j equal-weight N(a[:,c], I) components        */
#define ORC_TARGET_STUDENT_T 1   /* loc a (d), scale factor b (d x d), nu = p0     */
#define ORC_TARGET_LINREG 2      /* X a (j x d col-major), y b (j), sigma p0, prior N(0, p1 I) */
#define ORC_TARGET_LOGISTIC 3    /* X a (j x d), y b (j), prior N(0, p1 I)         */
#define ORC_TARGET_STD_NORMAL 4  /* N(0, I), normalised                          */
#define ORC_TARGET_QUADRATIC 5   /* -|x - a|^2 / p0 (unnormalised test target)    */

int orc_num_threads(void);
void orc_set_threads(int threads);

double orc_log1pexp(double x);
double orc_logaddexp(double x, double y);
double orc_student_t_logconstant(double dof, int d);
double orc_gaussian_lognormalizer(int d, double logabsdet);
int orc_factor_exponent_bound(const double *factor, int d);
double orc_component_logdensity(const orc_bank *bank, int slot, const double *x,
                                double *scratch_values, int *scratch_exponents);
void orc_mixture_logdensity(const orc_bank *bank, int denom_kind, int terms,
                            const double *coef, const int *group_of_slot,
                            const double *x, int64_t n, const int *slots,
                            int fixed_slot, double *out_logden,
                            double *out_generating, uint32_t *reasons);
double orc_radial_multiplier(double dof, const double *radial_normals,
                             const double *radial_uniforms, int has_uniforms,
                             uint32_t *reason);
void orc_draw(const orc_bank *bank, const int *slots, int fixed_slot,
              const double *normals, const double *radial_normals,
              int rn_stride, const double *radial_uniforms, int ru_stride,
              int64_t n, double *samples, uint32_t *reasons);
void orc_static_assign(const double *cdf, int k, const double *uniforms,
                       int64_t n, int stratified, int *slots);
double orc_target_logdensity(const orc_target *t, const double *x);
void orc_logweight_summary(const double *lw, int64_t n, double out[3]);
void orc_normalize(const double *lw, int64_t n, double *w);
void orc_resampling_cdf_f32(const float *lw, int64_t n, float *cdf);
void orc_resampling_cdf_f64(const double *lw, int64_t n, double *cdf);
void orc_resample_select(const double *cdf, const double *lw, int64_t n,
                         const double *uniforms, int64_t count, int64_t *anc);
double orc_det_exp(double x);
int orc_fixed_scale_bits(int64_t n);
int orc_fixed_prefix(const double *lw, int64_t n, uint64_t *prefix);
void orc_resample_multinomial_fixed(const double *lw, int64_t n,
                                    const double *uniforms, int64_t count,
                                    int64_t *anc);
void orc_resample_systematic_fixed(const double *lw, int64_t n, double u,
                                   int64_t count, int64_t *anc);
void orc_local_resample(const double *lw, const int64_t *counts, int k,
                        const double *uniforms, int64_t *anc);
void orc_weighted_moments(const double *x, int d, int64_t n, const double *lw,
                          double *mean, double *cov, double *weights);
int orc_fit_factor(const double *mean, const double *cov, int d,
                   const double *prev_factor, double dof, double logconstant,
                   double regularization, double *out_factor,
                   double *out_lognorm);
void orc_weighted_quantile(const double *x, int d, int64_t n, const double *w, const double *probs, int nprob,
                           double *out);
int orc_npmc_run(const orc_target *target, int d, int family, double dof, const double *loc0,
                 const double *factor0, int rounds, const int64_t *schedule, const double *normals,
                 const double *rn, int rn_stride, const double *ru, int ru_stride, double regularization,
                 double *samples, double *logweights, double *round_ess, double *round_logz,
                 double *adaptation_ess, double *hist_loc, double *hist_factor, double *hist_lognorm);
void orc_population_local_weights(const double *lw, const double *x, int d, const int64_t *starts,
                                  const int64_t *counts, const double *thresholds, int k, double tolerance,
                                  int max_iterations, double *weights, double *local_ess, double *powers,
                                  uint8_t *status, double *raw_means);
void orc_population_covariances(const double *x, int d, const double *weights, const double *powers,
                                const uint8_t *status, const double *locations, const double *factors,
                                const double *dofs, const int64_t *starts, const int64_t *counts, int k,
                                double *centres, double *covs);
void orc_population_factors(const double *covs, int d, int k, const uint8_t *status, const double *dofs,
                            double *factors, int32_t *info);
void orc_philox_normals(uint64_t seed, uint64_t offset, int64_t n, double *out);
void orc_philox_uniforms(uint64_t seed, uint64_t offset, int64_t n, double *out);
int orc_amis_run(const orc_target *target, int d, int family, double dof,
                 const double *loc0, const double *factor0, int rounds,
                 const int64_t *schedule, const double *normals,
                 const double *radial_normals, int rn_stride,
                 const double *radial_uniforms, int ru_stride,
                 double regularization, double *samples, double *logtargets,
                 double *lognum, double *logweights, double *round_ess,
                 double *round_logz, double *hist_loc, double *hist_factor,
                 double *hist_lognorm, uint32_t *reasons);
#endif
