/*
 * issm_oracle.c — FP64 CPU restatement of ImportanceSamplers.jl's hot path.
 *
 * TEST INFRASTRUCTURE ONLY (parity checker and timed CPU baseline). Each
 * function names the reference lines it follows. Compile with
 * -ffp-contract=off so that orc_det_exp and the fixed-point CDF round exactly
 * as the CUDA kernels do.
 */
#include "issm_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static const double LOG2PI = 1.8378770664093454835606594728112;

static int g_threads = 0;
void orc_set_threads(int threads) { g_threads = threads; }
int orc_num_threads(void) {
#ifdef _OPENMP
    return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
    return 1;
#endif
}

/* LogExpFunctions.log1pexp for the x <= 0 arguments used here, and
 * logaddexp with the x == y guard (LogExpFunctions 1.0 `logaddexp`). */
double orc_log1pexp(double x) {
    if (x > 33.3) return x;
    if (x > 18.0) return x + exp(-x);
    if (x < -37.0) return exp(x);
    return log1p(exp(x));
}
double orc_logaddexp(double x, double y) {
    if (isnan(x) || isnan(y)) return NAN;
    double delta = (x == y) ? 0.0 : fabs(x - y);
    double m = x > y ? x : y;
    return m + orc_log1pexp(-delta);
}

/* src/proposals.jl:237-240 */
double orc_gaussian_lognormalizer(int d, double logabsdet) {
    return -0.5 * (double)d * log(2.0 * M_PI) - logabsdet;
}

/* src/proposals.jl:413-437: shifted gamma-ratio recurrence + six Stirling
 * terms for odd d, log1p sums over the even offsets. */
double orc_student_t_logconstant(double dof, int d) {
    double value = -(double)d * log(2.0 * M_PI) / 2.0;
    if (d % 2 == 1) {
        double shifted = dof, correction = 0.0;
        while (shifted < 32.0) {
            if (shifted < 1.0)
                correction += (log(shifted) + log(shifted + 2.0)) / 2.0 - log1p(shifted);
            else {
                double r = 1.0 / (shifted + 1.0);
                correction += log1p(-(r * r)) / 2.0;
            }
            shifted += 2.0;
        }
        double r = 1.0 / shifted, r2 = r * r;
        const double c[6] = {-1.0 / 4.0, 1.0 / 24.0, -1.0 / 20.0,
                             17.0 / 112.0, -31.0 / 36.0, 691.0 / 88.0};
        double poly = c[5];
        for (int i = 4; i >= 0; --i) poly = poly * r2 + c[i];
        correction += r * poly;
        value += correction;
    }
    for (int offset = (d % 2 == 1) ? 1 : 0; offset <= d - 2; offset += 2) {
        double x = (double)offset;
        value += (x <= dof) ? log1p(x / dof) : log(x) + log1p(dof / x) - log(dof);
    }
    return value;
}

/* src/student_t_range.jl:21-31 */
int orc_factor_exponent_bound(const double *factor, int d) {
    int bound = 0;
    for (int c = 0; c < d; ++c)
        for (int r = c; r < d; ++r) {
            double v = factor[r + (size_t)c * d];
            if (v == 0.0) continue;
            if (!isfinite(v)) return 0x7fffffff;
            int e;
            frexp(v, &e);
            int a = abs(e), b = abs(e - 1);
            if (a > bound) bound = a;
            if (b > bound) bound = b;
        }
    return bound;
}

/* ---- range arithmetic, src/student_t_range.jl:59-80 ------------------- */
typedef struct { double m; int e; } rng_t;
static rng_t rfrexp(double v) { rng_t r; r.m = frexp(v, &r.e); return r; }
static rng_t range_subtract(rng_t l, rng_t r) {
    if (l.m == 0.0) { rng_t o = {-r.m, r.e}; return o; }
    if (r.m == 0.0) return l;
    int e = l.e > r.e ? l.e : r.e;
    int shift;
    double m = frexp(ldexp(l.m, l.e - e) - ldexp(r.m, r.e - e), &shift);
    rng_t o = {m, m == 0.0 ? 0 : e + shift};
    return o;
}
static rng_t range_multiply(rng_t v, double factor) {
    int fe, s;
    double fm = frexp(factor, &fe);
    double p = frexp(v.m * fm, &s);
    rng_t o = {p, p == 0.0 ? 0 : v.e + fe + s};
    return o;
}
static rng_t range_divide(rng_t v, double divisor) {
    int de, s;
    double dm = frexp(divisor, &de);
    double q = frexp(v.m / dm, &s);
    rng_t o = {q, q == 0.0 ? 0 : v.e - de + s};
    return o;
}

/* src/student_t_range.jl:82-87 */
static double standardized_difference(double sample, double location, double scale) {
    double diff = sample - location;
    if (isfinite(diff) || !isfinite(sample) || !isfinite(location)) return diff / scale;
    return sample / scale - location / scale;
}

/* src/student_t_range.jl:89-109; L column-major, prev = already solved rows */
static double factor_standardized_coordinate(double sample, double location, int row,
                                             const double *L, int d, const double *prev) {
    double z = sample - location;
    for (int c = 0; c < row; ++c) z -= L[row + (size_t)c * d] * prev[c];
    double diag = L[row + (size_t)row * d];
    z /= diag;
    if (isfinite(z) || !isfinite(sample) || !isfinite(location)) return z;
    rng_t value = range_subtract(rfrexp(sample), rfrexp(location));
    for (int c = 0; c < row; ++c) {
        double p = prev[c];
        if (!isfinite(p)) return p;
        value = range_subtract(value, range_multiply(rfrexp(p), L[row + (size_t)c * d]));
    }
    rng_t q = range_divide(value, diag);
    return ldexp(q.m, q.e);
}

/* src/student_t_range.jl:123-131 */
static double logabsdiff(double l, double r) {
    double diff = l - r;
    if (isfinite(diff) || !isfinite(l) || !isfinite(r)) return log(fabs(diff));
    double al = fabs(l), ar = fabs(r);
    double largest = al > ar ? al : ar, smallest = al > ar ? ar : al;
    return log(largest) + log1p(smallest / largest);
}

/* src/student_t_range.jl:133-153: exponent-extended radii */
static double diagonal_range_logradius(int d, const double *x, const double *mu,
                                       const double *scales, int spherical) {
    double total = -INFINITY;
    for (int c = 0; c < d; ++c) {
        double s = spherical ? scales[0] : scales[c];
        double v = logabsdiff(x[c], mu[c]) - log(s);
        total = orc_logaddexp(total, 2.0 * v);
    }
    return total;
}
static double factor_range_logradius(int d, const double *x, const double *mu,
                                     const double *L, double *vals, int *exps) {
    double total = -INFINITY;
    for (int row = 0; row < d; ++row) {
        rng_t value = range_subtract(rfrexp(x[row]), rfrexp(mu[row]));
        for (int c = 0; c < row; ++c) {
            rng_t p = {vals[c], exps[c]};
            value = range_subtract(value, range_multiply(p, L[row + (size_t)c * d]));
        }
        rng_t q = range_divide(value, L[row + (size_t)row * d]);
        vals[row] = q.m;
        exps[row] = q.e;
        double logabs = log(fabs(q.m)) + (double)q.e * log(2.0);
        total = orc_logaddexp(total, 2.0 * logabs);
    }
    return total;
}

/* One component's normalised log density: _packed_gaussian_logdensity!
 * (src/native_execution.jl:346-384), _packed_gaussian_logdensity
 * (:447-469) and _radial_logdensity (src/proposals.jl:24-70). */
double orc_component_logdensity(const orc_bank *b, int slot, const double *x,
                                double *vals, int *exps) {
    const int d = b->d;
    const double *mu = b->loc + (size_t)slot * d;
    const double lognorm = b->lognorm[slot];
    double r2 = 0.0;
    int range_risk = 0;
    const double *L = NULL, *sc = NULL;
    if (b->scale_kind == ORC_SCALE_FACTOR) {
        L = b->scales + (size_t)slot * d * d;
        for (int row = 0; row < d; ++row) {
            double z = x[row] - mu[row];
            for (int c = 0; c < row; ++c) z -= L[row + (size_t)c * d] * vals[c];
            z /= L[row + (size_t)row * d];
            vals[row] = z;
            r2 += z * z;
        }
        if (!isfinite(r2)) {
            int all_finite = 1;
            for (int c = 0; c < d; ++c) all_finite &= isfinite(vals[c]) ? 1 : 0;
            if (!all_finite) {
                r2 = 0.0;
                for (int row = 0; row < d; ++row) {
                    double z = factor_standardized_coordinate(x[row], mu[row], row, L, d, vals);
                    vals[row] = z;
                    r2 += z * z;
                }
            }
        }
        if (b->family == ORC_STUDENT_T && b->range_risk) range_risk = b->range_risk[slot];
    } else {
        int sph = b->scale_kind == ORC_SCALE_SPHERICAL;
        sc = sph ? b->scales + slot : b->scales + (size_t)slot * d;
        for (int c = 0; c < d; ++c) {
            double z = (x[c] - mu[c]) / (sph ? sc[0] : sc[c]);
            r2 += z * z;
        }
        for (int c = 0; c < d; ++c) vals[c] = standardized_difference(x[c], mu[c], sph ? sc[0] : sc[c]);
    }
    if (b->family == ORC_GAUSSIAN) {
        double half = 0.5 * r2;
        if (!isfinite(r2)) {
            half = 0.0;
            for (int c = 0; c < d; ++c) half += (0.5 * vals[c]) * vals[c];
        }
        return lognorm - half;
    }
    const double dof = b->dofs[slot];
    const double ratio = r2 / dof;
    double radial;
    if (range_risk) {
        double lr = (b->scale_kind == ORC_SCALE_FACTOR)
                        ? factor_range_logradius(d, x, mu, L, vals, exps)
                        : diagonal_range_logradius(d, x, mu, sc, b->scale_kind == ORC_SCALE_SPHERICAL);
        radial = orc_log1pexp(lr - log(dof));
    } else if (r2 < DBL_MIN) {
        double s = sqrt(dof), acc = 0.0;
        for (int c = 0; c < d; ++c) { double v = vals[c] / s; acc += v * v; }
        radial = log1p(acc);
    } else if (isfinite(ratio)) {
        radial = log1p(ratio);
    } else if (isfinite(r2)) {
        radial = log(r2) - log(dof);
    } else {
        double scale = 0.0;
        for (int c = 0; c < d; ++c) { double a = fabs(vals[c]); if (a > scale) scale = a; }
        if (!isfinite(scale)) {
            double lr = (b->scale_kind == ORC_SCALE_FACTOR)
                            ? factor_range_logradius(d, x, mu, L, vals, exps)
                            : diagonal_range_logradius(d, x, mu, sc, b->scale_kind == ORC_SCALE_SPHERICAL);
            radial = orc_log1pexp(lr - log(dof));
        } else {
            double acc = 0.0;
            for (int c = 0; c < d; ++c) { double v = vals[c] / scale; acc += v * v; }
            radial = orc_log1pexp(2.0 * log(scale) + log(acc) - log(dof));
        }
    }
    return lognorm - (dof + (double)d) / 2.0 * radial;
}

/* Balance-heuristic denominator: _mis_logdenominator_core
 * (src/mis_execution.jl:30-65) with the term policies of
 * src/methods/static_mis.jl:389-443, src/mis_execution.jl:67-89 and
 * src/amis_execution.jl:12-35. */
void orc_mixture_logdensity(const orc_bank *b, int kind, int terms,
                            const double *coef, const int *group_of_slot,
                            const double *x, int64_t n, const int *slots,
                            int fixed_slot, double *out_logden,
                            double *out_generating, uint32_t *reasons) {
    const int d = b->d;
#pragma omp parallel num_threads(orc_num_threads())
    {
        double *vals = (double *)malloc(sizeof(double) * (size_t)d);
        int *exps = (int *)malloc(sizeof(int) * (size_t)d);
#pragma omp for schedule(static)
        for (int64_t i = 0; i < n; ++i) {
            const double *xi = x + (size_t)i * d;
            int gen = slots ? slots[i] : fixed_slot;
            int first = 0, last = b->k - 1;
            if (kind == ORC_DENOM_GENERATING) first = last = gen;
            else if (kind == ORC_DENOM_PREFIX) last = terms - 1;
            double value = -INFINITY, gen_log = 0.0;
            for (int s = first; s <= last; ++s) {
                if (kind == ORC_DENOM_PARTIAL && group_of_slot[s] != group_of_slot[gen]) continue;
                double c = (kind == ORC_DENOM_GENERATING) ? 0.0 : coef[s];
                double lq = orc_component_logdensity(b, s, xi, vals, exps);
                if (s == gen) gen_log = lq;
                value = orc_logaddexp(value, c + lq);
            }
            uint32_t reason = (isnan(gen_log) || gen_log == -INFINITY || isnan(value) || value == -INFINITY)
                                  ? ORC_REASON_PROPOSAL_INVALID : 0u;
            out_logden[i] = value;
            if (out_generating) out_generating[i] = gen_log;
            if (reasons) reasons[i] = reason;
        }
        free(vals);
        free(exps);
    }
}

/* Marsaglia-Tsang candidate and the 8-attempt buffered gamma,
 * src/proposals.jl:738-751, src/native_execution.jl:153-180. */
static int gamma_candidate(double offset, double coef, double normal, double uniform, double *gamma) {
    double root = 1.0 + coef * normal;
    if (!(root > 0.0)) { *gamma = 0.0; return 0; }
    double cube = root * root * root;
    double n2 = normal * normal;
    int accepted = uniform < 1.0 - 0.0331 * (n2 * n2) ||
                   log(uniform) < 0.5 * n2 + offset * (1.0 - cube + log(cube));
    *gamma = offset * cube;
    return accepted;
}
double orc_radial_multiplier(double dof, const double *rn, const double *ru,
                             int has_uniforms, uint32_t *reason) {
    *reason = 0;
    if (!has_uniforms || dof == 1.0) {
        double den = fabs(rn[0]);
        if (!(isfinite(den) && den > 0.0)) { *reason = ORC_REASON_DRAW_EXHAUSTED; return 0.0; }
        return 1.0 / den;
    }
    double shape = dof / 2.0;
    double adjusted = shape < 1.0 ? shape + 1.0 : shape;
    double offset = adjusted - 1.0 / 3.0;
    double coef = 1.0 / sqrt(offset) / 3.0;
    for (int a = 0; a < 8; ++a) {
        double g;
        if (!gamma_candidate(offset, coef, rn[a], ru[a], &g)) continue;
        if (shape < 1.0) g *= pow(ru[8], 1.0 / shape);
        if (!(isfinite(g) && g > 0.0)) break;
        return sqrt(dof / (2.0 * g));
    }
    *reason = ORC_REASON_DRAW_EXHAUSTED;
    return 0.0;
}

/* Packed draw x = mu + L (m n): _native_proposal_coordinate
 * (src/native_execution.jl:238-264) and _scale_mis_normals_kernel! (:184-199). */
void orc_draw(const orc_bank *b, const int *slots, int fixed_slot,
              const double *normals, const double *rn, int rn_stride,
              const double *ru, int ru_stride, int64_t n, double *samples,
              uint32_t *reasons) {
    const int d = b->d;
#pragma omp parallel for schedule(static) num_threads(orc_num_threads())
    for (int64_t i = 0; i < n; ++i) {
        int s = slots ? slots[i] : fixed_slot;
        uint32_t reason = 0;
        double m = 1.0;
        if (b->family == ORC_STUDENT_T) {
            uint32_t r;
            m = orc_radial_multiplier(b->dofs[s], rn + (size_t)i * rn_stride,
                                      ru ? ru + (size_t)i * ru_stride : NULL,
                                      ru != NULL && ru_stride > 0, &r);
            if (r) { reason |= r; m = NAN; }
        }
        const double *mu = b->loc + (size_t)s * d;
        const double *nz = normals + (size_t)i * d;
        double *xi = samples + (size_t)i * d;
        int valid = 1;
        for (int row = 0; row < d; ++row) {
            double v = mu[row];
            if (b->scale_kind == ORC_SCALE_FACTOR) {
                const double *L = b->scales + (size_t)s * d * d;
                for (int c = 0; c <= row; ++c) v += L[row + (size_t)c * d] * (nz[c] * m);
            } else {
                double sc = b->scale_kind == ORC_SCALE_SPHERICAL ? b->scales[s] : b->scales[(size_t)s * d + row];
                v = mu[row] + sc * (nz[row] * m);
            }
            xi[row] = v;
            valid &= isfinite(v) ? 1 : 0;
        }
        if (!valid) reason |= ORC_REASON_GENERATED_NONFINITE;
        if (reasons) reasons[i] = reason;
    }
}

/* src/methods/static_mis.jl:171-211: first slot with u' <= cdf[slot]. */
void orc_static_assign(const double *cdf, int k, const double *u, int64_t n,
                       int stratified, int *slots) {
    for (int64_t i = 0; i < n; ++i) {
        double mapped = stratified ? ((double)i + u[i]) / (double)n : u[i];
        int lo = 0, hi = k - 1;
        while (lo < hi) {
            int mid = lo + (hi - lo) / 2;
            if (mapped <= cdf[mid]) hi = mid; else lo = mid + 1;
        }
        slots[i] = lo;
    }
}

/* Targets used by the benchmark configurations (user code in the reference). */
double orc_target_logdensity(const orc_target *t, const double *x) {
    const int d = t->d;
    switch (t->kind) {
    case ORC_TARGET_STD_NORMAL: {
        double r2 = 0.0;
        for (int c = 0; c < d; ++c) r2 += x[c] * x[c];
        return -0.5 * d * LOG2PI - 0.5 * r2;
    }
    case ORC_TARGET_QUADRATIC: {
        double r2 = 0.0;
        for (int c = 0; c < d; ++c) { double z = x[c] - t->a[c]; r2 += z * z; }
        return -r2 / t->p0;
    }
    case ORC_TARGET_GAUSS_MIX: {
        double acc = -INFINITY;
        for (int j = 0; j < t->j; ++j) {
            double r2 = 0.0;
            for (int c = 0; c < d; ++c) { double z = x[c] - t->a[(size_t)j * d + c]; r2 += z * z; }
            acc = orc_logaddexp(acc, -0.5 * r2);
        }
        return acc - log((double)t->j) - 0.5 * d * LOG2PI;
    }
    case ORC_TARGET_STUDENT_T: {
        const double *L = t->b;
        double z[512];
        double r2 = 0.0, logdet = 0.0;
        for (int row = 0; row < d; ++row) {
            double v = x[row] - t->a[row];
            for (int c = 0; c < row; ++c) v -= L[row + (size_t)c * d] * z[c];
            v /= L[row + (size_t)row * d];
            z[row] = v;
            r2 += v * v;
            logdet += log(L[row + (size_t)row * d]);
        }
        double nu = t->p0;
        return orc_student_t_logconstant(nu, d) - logdet - (nu + d) / 2.0 * log1p(r2 / nu);
    }
    case ORC_TARGET_LINREG: {
        const int nobs = t->j;
        double sigma = t->p0, pv = t->p1, ss = 0.0, bb = 0.0;
        for (int i = 0; i < nobs; ++i) {
            double eta = 0.0;
            for (int c = 0; c < d; ++c) eta += t->a[i + (size_t)c * nobs] * x[c];
            double r = t->b[i] - eta;
            ss += r * r;
        }
        for (int c = 0; c < d; ++c) bb += x[c] * x[c];
        return -0.5 * nobs * (LOG2PI + 2.0 * log(sigma)) - ss / (2.0 * sigma * sigma) -
               0.5 * d * (LOG2PI + log(pv)) - bb / (2.0 * pv);
    }
    case ORC_TARGET_LOGISTIC: {
        const int nobs = t->j;
        double pv = t->p1, ll = 0.0, bb = 0.0;
        for (int i = 0; i < nobs; ++i) {
            double eta = 0.0;
            for (int c = 0; c < d; ++c) eta += t->a[i + (size_t)c * nobs] * x[c];
            ll += t->b[i] * eta - orc_log1pexp(eta);
        }
        for (int c = 0; c < d; ++c) bb += x[c] * x[c];
        return ll - 0.5 * d * (LOG2PI + log(pv)) - bb / (2.0 * pv);
    }
    }
    return NAN;
}

/* src/execution.jl:103-186: (max, S, S2) and the summary. */
/* Sums are compensated (Neumaier) so that the oracle stays accurate to a few
 * ulps at any n: a plain sequential sum drops the many terms far below one
 * ulp of the running total. */
void orc_logweight_summary(const double *lw, int64_t n, double out[3]) {
    double m = -INFINITY;
    for (int64_t i = 0; i < n; ++i) if (lw[i] > m) m = lw[i];
    double s = 0.0, s2 = 0.0, cs = 0.0, cs2 = 0.0;
    if (m != -INFINITY)
        for (int64_t i = 0; i < n; ++i) {
            double w = exp(lw[i] - m), w2 = w * w;
            double t = s + w;
            cs += fabs(s) >= fabs(w) ? (s - t) + w : (w - t) + s;
            s = t;
            t = s2 + w2;
            cs2 += fabs(s2) >= fabs(w2) ? (s2 - t) + w2 : (w2 - t) + s2;
            s2 = t;
        }
    out[0] = m; out[1] = s + cs; out[2] = s2 + cs2;
}

/* src/results.jl:589-598 */
void orc_normalize(const double *lw, int64_t n, double *w) {
    double sm[3];
    orc_logweight_summary(lw, n, sm);
    for (int64_t i = 0; i < n; ++i) w[i] = exp(lw[i] - sm[0]) / sm[1];
}

/* src/resampling.jl:199-225, serial cumsum as the CPU reference does. */
void orc_resampling_cdf_f32(const float *lw, int64_t n, float *cdf) {
    float m = -INFINITY;
    for (int64_t i = 0; i < n; ++i) if (lw[i] > m) m = lw[i];
    for (int64_t i = 0; i < n; ++i) cdf[i] = expf(lw[i] - m);
    for (int64_t i = 1; i < n; ++i) cdf[i] = cdf[i - 1] + cdf[i];
    float total = cdf[n - 1];
    for (int64_t i = 0; i < n; ++i) cdf[i] = cdf[i] / total;
}
void orc_resampling_cdf_f64(const double *lw, int64_t n, double *cdf) {
    double m = -INFINITY;
    for (int64_t i = 0; i < n; ++i) if (lw[i] > m) m = lw[i];
    for (int64_t i = 0; i < n; ++i) cdf[i] = exp(lw[i] - m);
    for (int64_t i = 1; i < n; ++i) cdf[i] = cdf[i - 1] + cdf[i];
    double total = cdf[n - 1];
    for (int64_t i = 0; i < n; ++i) cdf[i] = cdf[i] / total;
}

/* src/resampling.jl:92-118: strict-< search and the -Inf plateau repair. */
void orc_resample_select(const double *cdf, const double *lw, int64_t n,
                         const double *u, int64_t count, int64_t *anc) {
    for (int64_t o = 0; o < count; ++o) {
        int64_t first = 1, last = n;
        while (first < last) {
            int64_t mid = first + ((last - first) >> 1);
            if (u[o] < cdf[mid - 1]) last = mid; else first = mid + 1;
        }
        if (lw[first - 1] == -INFINITY) {
            while (first > 1 && lw[first - 1] == -INFINITY) first -= 1;
            while (first < n && lw[first - 1] == -INFINITY) first += 1;
        }
        anc[o] = first;
    }
}

/* Deterministic exp for x <= 0 (used only to define resampling weights
 * identically on CPU and GPU): Cody-Waite reduction x = k ln2 + r with ln2
 * split into a 32-bit head and a tail (Cody & Waite 1980), then a degree-13
 * Taylor polynomial of e^r by Horner with fused multiply-adds, scaled by 2^k.
 * Only IEEE-exact operations are used, so every platform rounds alike. */
static const double DET_INV_LN2 = 0x1.71547652b82fep+0;
static const double DET_LN2_HI = 0x1.62e42ff000000p-1;   /* ln2 rounded to 32 bits */
static const double DET_LN2_LO = -0x1.718432a1b0e26p-35;  /* ln2 - DET_LN2_HI */
double orc_det_exp(double x) {
    if (isnan(x)) return NAN;
    if (x == -INFINITY || x < -708.0) return 0.0;
    if (x > 0.0) x = 0.0;
    double k = floor(x * DET_INV_LN2 + 0.5);
    double r = fma(-k, DET_LN2_HI, x);
    r = fma(-k, DET_LN2_LO, r);
    double p = 1.0 / 6227020800.0;                 /* 1/13! */
    static const double inv_fact[13] = {1.0, 1.0, 1.0 / 2.0, 1.0 / 6.0, 1.0 / 24.0, 1.0 / 120.0,
                                        1.0 / 720.0, 1.0 / 5040.0, 1.0 / 40320.0, 1.0 / 362880.0,
                                        1.0 / 3628800.0, 1.0 / 39916800.0, 1.0 / 479001600.0};
    for (int i = 12; i >= 0; --i) p = fma(p, r, inv_fact[i]);
    return ldexp(p, (int)k);
}

/* Fixed-point weights q_j = floor(det_exp(l_j - max) * 2^s + 1/2) with
 * s = 62 - ceil(log2 n), summed exactly in uint64. */
int orc_fixed_scale_bits(int64_t n) {
    int b = 0;
    while (((int64_t)1 << b) < n) ++b;
    int s = 62 - b;
    return s > 52 ? 52 : s;
}
int orc_fixed_prefix(const double *lw, int64_t n, uint64_t *prefix) {
    double m = -INFINITY;
    for (int64_t i = 0; i < n; ++i) if (lw[i] > m) m = lw[i];
    if (m == -INFINITY || isnan(m)) return -1;
    double scale = ldexp(1.0, orc_fixed_scale_bits(n));
    uint64_t acc = 0;
    for (int64_t i = 0; i < n; ++i) {
        double w = orc_det_exp(lw[i] - m);
        uint64_t q = (uint64_t)floor(w * scale + 0.5);
        acc += q;
        prefix[i] = acc;
    }
    return 0;
}
static uint64_t umulhi64(uint64_t a, uint64_t b) {
    return (uint64_t)(((unsigned __int128)a * (unsigned __int128)b) >> 64);
}
static uint64_t u64_from_unit(double u) {
    if (!(u > 0.0)) return 0;
    if (u >= 1.0) return UINT64_MAX;
    return (uint64_t)ldexp(u, 64);
}
static int64_t first_greater(const uint64_t *prefix, int64_t n, uint64_t tau) {
    int64_t lo = 0, hi = n - 1;
    while (lo < hi) {
        int64_t mid = lo + ((hi - lo) >> 1);
        if (tau < prefix[mid]) hi = mid; else lo = mid + 1;
    }
    return lo + 1;
}
void orc_resample_multinomial_fixed(const double *lw, int64_t n, const double *u,
                                    int64_t count, int64_t *anc) {
    uint64_t *prefix = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)n);
    if (orc_fixed_prefix(lw, n, prefix) != 0) { free(prefix); return; }
    uint64_t total = prefix[n - 1];
    for (int64_t o = 0; o < count; ++o) anc[o] = first_greater(prefix, n, umulhi64(u64_from_unit(u[o]), total));
    free(prefix);
}
void orc_resample_systematic_fixed(const double *lw, int64_t n, double u,
                                   int64_t count, int64_t *anc) {
    uint64_t *prefix = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)n);
    if (orc_fixed_prefix(lw, n, prefix) != 0) { free(prefix); return; }
    uint64_t total = prefix[n - 1];
    uint64_t base = umulhi64(u64_from_unit(u), total);
    for (int64_t o = 0; o < count; ++o) {
        unsigned __int128 num = (unsigned __int128)total * (uint64_t)o + base;
        uint64_t tau = (uint64_t)(num / (uint64_t)count);
        anc[o] = first_greater(prefix, n, tau);
    }
    free(prefix);
}

/* src/dm_pmc_execution.jl:80-125 (CPU local resampling). */
void orc_local_resample(const double *lw, const int64_t *counts, int k,
                        const double *u, int64_t *anc) {
    int64_t first = 0;
    for (int s = 0; s < k; ++s) {
        int64_t last = first + counts[s] - 1;
        double m = -INFINITY;
        for (int64_t i = first; i <= last; ++i) if (lw[i] > m) m = lw[i];
        int64_t a = 0;
        if (m != -INFINITY) {
            double total = 0.0;
            for (int64_t i = first; i <= last; ++i) total += exp(lw[i] - m);
            if (isfinite(total) && total > 0.0) {
                double threshold = u[s] * total, cum = 0.0;
                a = last + 1;
                for (int64_t i = first; i <= last; ++i) {
                    cum += exp(lw[i] - m);
                    if (threshold < cum) { a = i + 1; break; }
                }
            }
        }
        anc[s] = a;
        first = last + 1;
    }
}

/* Literal two-pass moments: _normalize_moment_weights! and
 * _fit_moment_proposal! (src/adaptive_gaussian_execution.jl:186-205,341-372). */
void orc_weighted_moments(const double *x, int d, int64_t n, const double *lw,
                          double *mean, double *cov, double *weights) {
    double *w = weights ? weights : (double *)malloc(sizeof(double) * (size_t)n);
    double m = -INFINITY;
    for (int64_t i = 0; i < n; ++i) if (lw[i] > m) m = lw[i];
    double total = 0.0;
    for (int64_t i = 0; i < n; ++i) { w[i] = exp(lw[i] - m); total += w[i]; }
    for (int64_t i = 0; i < n; ++i) w[i] *= 1.0 / total;
    for (int c = 0; c < d; ++c) mean[c] = 0.0;
    for (int64_t i = 0; i < n; ++i)
        for (int c = 0; c < d; ++c) mean[c] += w[i] * x[(size_t)i * d + c];
    for (int a = 0; a < d * d; ++a) cov[a] = 0.0;
    int nt = orc_num_threads();
#pragma omp parallel num_threads(nt)
    {
        double *loc = (double *)calloc((size_t)d * d, sizeof(double));
        double *z = (double *)malloc(sizeof(double) * (size_t)d);
#pragma omp for schedule(static)
        for (int64_t i = 0; i < n; ++i) {
            double s = sqrt(w[i]);
            for (int c = 0; c < d; ++c) z[c] = (x[(size_t)i * d + c] - mean[c]) * s;
            for (int c = 0; c < d; ++c)
                for (int r = c; r < d; ++r) loc[r + (size_t)c * d] += z[r] * z[c];
        }
#pragma omp critical
        for (int a = 0; a < d * d; ++a) cov[a] += loc[a];
        free(loc);
        free(z);
    }
    for (int c = 0; c < d; ++c)
        for (int r = c + 1; r < d; ++r) cov[c + (size_t)r * d] = cov[r + (size_t)c * d];
    if (!weights) free(w);
}

/* Candidate fit: ridge (src/adaptive_gaussian_execution.jl:283-301,
 * src/execution.jl:188-194), potrf, Student-t scaling (src/proposals.jl:73-80),
 * zero upper triangle, logabsdet, lognormalizer and validity (:475-528). */
int orc_fit_factor(const double *mean, const double *cov, int d,
                   const double *prev, double dof, double logconstant,
                   double regularization, double *L, double *lognorm) {
    double mult = dof > 0.0 ? dof / (dof - 2.0) : 1.0;
    double trace = 0.0;
    for (int c = 0; c < d; ++c)
        for (int r = c; r < d; ++r) trace += prev[r + (size_t)c * d] * prev[r + (size_t)c * d];
    double ridge = regularization * (trace * mult) / (double)d;
    if (!isfinite(ridge)) {
        ridge = 0.0;
        if (regularization != 0.0) {
            double scale = sqrt(regularization) * sqrt(mult / (double)d);
            for (int c = 0; c < d; ++c)
                for (int r = c; r < d; ++r) { double v = prev[r + (size_t)c * d] * scale; ridge += v * v; }
        }
    }
    for (int a = 0; a < d * d; ++a) L[a] = cov[a];
    for (int c = 0; c < d; ++c) L[c + (size_t)c * d] += ridge;
    for (int j = 0; j < d; ++j) {
        double djj = L[j + (size_t)j * d];
        for (int k = 0; k < j; ++k) djj -= L[j + (size_t)k * d] * L[j + (size_t)k * d];
        if (!(djj > 0.0) || !isfinite(djj)) return -1;
        double ljj = sqrt(djj);
        L[j + (size_t)j * d] = ljj;
        for (int i = j + 1; i < d; ++i) {
            double v = L[i + (size_t)j * d];
            for (int k = 0; k < j; ++k) v -= L[i + (size_t)k * d] * L[j + (size_t)k * d];
            L[i + (size_t)j * d] = v / ljj;
        }
    }
    if (dof > 0.0) {
        double f = sqrt(1.0 / mult);
        for (int a = 0; a < d * d; ++a) L[a] *= f;
    }
    for (int c = 0; c < d; ++c)
        for (int r = 0; r < c; ++r) L[r + (size_t)c * d] = 0.0;
    double logabsdet = 0.0;
    for (int c = 0; c < d; ++c) logabsdet += log(fabs(L[c + (size_t)c * d]));
    *lognorm = dof > 0.0 ? logconstant - logabsdet : orc_gaussian_lognormalizer(d, logabsdet);
    int valid = isfinite(*lognorm);
    for (int c = 0; c < d; ++c) valid &= isfinite(mean[c]) ? 1 : 0;
    for (int c = 0; c < d; ++c)
        for (int r = c; r < d; ++r) {
            double v = L[r + (size_t)c * d];
            valid &= isfinite(v) ? 1 : 0;
            if (r == c) valid &= v > 0.0 ? 1 : 0;
        }
    return valid ? 0 : -2;
}

/* Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) counter-based stream,
 * FP64 form: block b -> two doubles from 53-bit uniforms; Box-Muller. */
static void philox(uint32_t ctr[4], uint32_t key[2]) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)M0 * ctr[0], p1 = (uint64_t)M1 * ctr[2];
        uint32_t h0 = (uint32_t)(p0 >> 32), l0 = (uint32_t)p0;
        uint32_t h1 = (uint32_t)(p1 >> 32), l1 = (uint32_t)p1;
        uint32_t n0 = h1 ^ ctr[1] ^ key[0], n2 = h0 ^ ctr[3] ^ key[1];
        ctr[0] = n0; ctr[1] = l1; ctr[2] = n2; ctr[3] = l0;
        key[0] += W0; key[1] += W1;
    }
}
static void philox_block(uint64_t seed, uint64_t block, uint32_t out[4]) {
    uint32_t ctr[4] = {(uint32_t)block, (uint32_t)(block >> 32), 0u, 0u};
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    philox(ctr, key);
    memcpy(out, ctr, sizeof(ctr));
}
void orc_philox_uniforms(uint64_t seed, uint64_t offset, int64_t n, double *out) {
    for (int64_t i = 0; i < n; ++i) {
        uint64_t e = offset + (uint64_t)i;
        uint32_t o[4];
        philox_block(seed, e >> 1, o);
        uint64_t bits = (e & 1) ? (((uint64_t)o[3] << 32) | o[2]) : (((uint64_t)o[1] << 32) | o[0]);
        out[i] = (double)(bits >> 11) * 0x1.0p-53;
    }
}
void orc_philox_normals(uint64_t seed, uint64_t offset, int64_t n, double *out) {
#pragma omp parallel for schedule(static) num_threads(orc_num_threads()) if (n > 65536)
    for (int64_t i = 0; i < n; ++i) {
        uint64_t e = offset + (uint64_t)i;
        uint32_t o[4];
        philox_block(seed, e >> 1, o);
        uint64_t b1 = ((uint64_t)o[1] << 32) | o[0], b2 = ((uint64_t)o[3] << 32) | o[2];
        double u1 = ((double)(b1 >> 11) + 1.0) * 0x1.0p-53; /* (0, 1] */
        double u2 = (double)(b2 >> 11) * 0x1.0p-53;
        double r = sqrt(-2.0 * log(u1));
        out[i] = (e & 1) ? r * sin(2.0 * M_PI * u2) : r * cos(2.0 * M_PI * u2);
    }
}

/* Complete AMIS run on fed draws: _importance_sample_cpu! for
 * _PreparedMomentSampler (src/adaptive_gaussian_execution.jl:897-1112) with
 * the retrospective recurrence of src/amis_execution.jl:261-357. Returns 0 or
 * the 1-based failing round (negative for a failed fit). */
int orc_amis_run(const orc_target *target, int d, int family, double dof,
                 const double *loc0, const double *factor0, int rounds,
                 const int64_t *schedule, const double *normals,
                 const double *rn, int rn_stride, const double *ru, int ru_stride,
                 double regularization, double *samples, double *logtargets,
                 double *lognum, double *logw, double *round_ess,
                 double *round_logz, double *hist_loc, double *hist_factor,
                 double *hist_lognorm, uint32_t *reasons) {
    double logconst = family == ORC_STUDENT_T ? orc_student_t_logconstant(dof, d) : 0.0;
    double *dofs = (double *)malloc(sizeof(double) * (size_t)rounds);
    double *logcounts = (double *)malloc(sizeof(double) * (size_t)rounds);
    for (int r = 0; r < rounds; ++r) { dofs[r] = dof; logcounts[r] = log((double)schedule[r]); }
    memcpy(hist_loc, loc0, sizeof(double) * (size_t)d);
    memcpy(hist_factor, factor0, sizeof(double) * (size_t)d * d);
    double logabsdet = 0.0;
    for (int c = 0; c < d; ++c) logabsdet += log(factor0[c + (size_t)c * d]);
    hist_lognorm[0] = family == ORC_STUDENT_T ? logconst - logabsdet : orc_gaussian_lognormalizer(d, logabsdet);
    double *mean = (double *)malloc(sizeof(double) * (size_t)d);
    double *cov = (double *)malloc(sizeof(double) * (size_t)d * d);
    int64_t total = 0;
    int status = 0;
    for (int t = 0; t < rounds; ++t) {
        orc_bank hist = {d, t + 1, family, ORC_SCALE_FACTOR, hist_loc, hist_factor, hist_lognorm, dofs, NULL};
        int64_t n_old = total, n_new = schedule[t];
        double *x_new = samples + (size_t)n_old * d;
        orc_draw(&hist, NULL, t, normals + (size_t)n_old * d,
                 rn ? rn + (size_t)n_old * rn_stride : NULL, rn_stride,
                 ru ? ru + (size_t)n_old * ru_stride : NULL, ru_stride, n_new, x_new,
                 reasons ? reasons + n_old : NULL);
        if (n_old > 0) {
            /* old samples gain the newest component */
#pragma omp parallel num_threads(orc_num_threads())
            {
                double *vals = (double *)malloc(sizeof(double) * (size_t)d);
                int *exps = (int *)malloc(sizeof(int) * (size_t)d);
#pragma omp for schedule(static)
                for (int64_t i = 0; i < n_old; ++i) {
                    double lq = orc_component_logdensity(&hist, t, samples + (size_t)i * d, vals, exps);
                    lognum[i] = orc_logaddexp(lognum[i], logcounts[t] + lq);
                }
                free(vals);
                free(exps);
            }
        }
#pragma omp parallel for schedule(static) num_threads(orc_num_threads())
        for (int64_t i = 0; i < n_new; ++i) logtargets[n_old + i] = orc_target_logdensity(target, x_new + (size_t)i * d);
        orc_mixture_logdensity(&hist, ORC_DENOM_PREFIX, t + 1, logcounts, NULL, x_new, n_new, NULL, t,
                               lognum + n_old, NULL, NULL);
        total += n_new;
        double logtotal = log((double)total);
        for (int64_t i = 0; i < total; ++i) logw[i] = logtargets[i] - (lognum[i] - logtotal);
        double sm[3];
        orc_logweight_summary(logw, total, sm);
        round_ess[t] = sm[1] * sm[1] / sm[2];
        round_logz[t] = sm[0] + log(sm[1]) - log((double)total);
        orc_weighted_moments(samples, d, total, logw, mean, cov, NULL);
        if (t + 1 < rounds) {
            double *L = hist_factor + (size_t)(t + 1) * d * d;
            if (orc_fit_factor(mean, cov, d, hist_factor + (size_t)t * d * d,
                               family == ORC_STUDENT_T ? dof : 0.0, logconst, regularization, L,
                               hist_lognorm + t + 1) != 0) { status = -(t + 1); break; }
            memcpy(hist_loc + (size_t)(t + 1) * d, mean, sizeof(double) * (size_t)d);
        }
    }
    free(dofs); free(logcounts); free(mean); free(cov);
    return status;
}

/* ---- weighted quantile (src/statistics.jl:114-154) ---------------------------- */
typedef struct { double v; int64_t i; } orc_vi;
static int cmp_vi(const void *a, const void *b) {  /* value, then index: a stable sort */
    const orc_vi *x = (const orc_vi *)a, *y = (const orc_vi *)b;
    if (x->v < y->v) return -1;
    if (x->v > y->v) return 1;
    /* -0.0 sorts before 0.0 (Julia's isless) */
    if (signbit(x->v) != signbit(y->v)) return signbit(x->v) ? -1 : 1;
    return (x->i > y->i) - (x->i < y->i);
}

/* Component-wise weighted quantiles of x (n x d row-major) under normalised
 * weights w: positive-weight samples sorted by value (stable), cumulative
 * weights, threshold p (W - w_first) + w_first, upper = first index whose
 * cumulative weight exceeds it (searchsortedlast + 1), linear interpolation
 * with lower = upper - 1; NaN for a coordinate holding a NaN.
 * out[q * d + c]. */
void orc_weighted_quantile(const double *x, int d, int64_t n, const double *w, const double *probs, int nprob,
                           double *out) {
    orc_vi *buf = (orc_vi *)malloc(sizeof(orc_vi) * (size_t)n);
    double *cum = (double *)malloc(sizeof(double) * (size_t)n);
    for (int c = 0; c < d; ++c) {
        int nan = 0;
        int64_t m = 0;
        for (int64_t i = 0; i < n; ++i) {
            const double v = x[(size_t)i * d + c];
            if (isnan(v)) nan = 1;
            if (w[i] != 0.0) { buf[m].v = v; buf[m].i = i; ++m; }
        }
        if (nan || m == 0) {
            for (int q = 0; q < nprob; ++q) out[(size_t)q * d + c] = NAN;
            continue;
        }
        qsort(buf, (size_t)m, sizeof(orc_vi), cmp_vi);
        double s = 0.0;
        for (int64_t j = 0; j < m; ++j) { s += w[buf[j].i]; cum[j] = s; }
        const double total = cum[m - 1], first = w[buf[0].i];
        for (int q = 0; q < nprob; ++q) {
            const double thr = probs[q] * (total - first) + first;
            int64_t upper = 0;  /* 0-based: first j with cum[j] > thr */
            while (upper < m && !(cum[upper] > thr)) ++upper;
            double v;
            if (upper >= m) {
                v = buf[m - 1].v;
            } else {
                const int64_t lower = upper - 1;
                const double f = (thr - cum[lower]) / (cum[upper] - cum[lower]);
                if (f == 0.0) v = buf[lower].v;
                else {
                    const double diff = buf[upper].v - buf[lower].v;
                    v = isfinite(diff) ? buf[lower].v + f * diff : (1.0 - f) * buf[lower].v + f * buf[upper].v;
                }
            }
            out[(size_t)q * d + c] = v;
        }
    }
    free(buf);
    free(cum);
}

static int cmp_double_nan_last(const void *a, const void *b) {
    const double x = *(const double *)a, y = *(const double *)b;
    if (isnan(x)) return isnan(y) ? 0 : 1;
    if (isnan(y)) return -1;
    return (x > y) - (x < y);
}

/* Complete N-PMC on fed draws (src/npmc_execution.jl with the moment loop of
 * src/adaptive_gaussian_execution.jl:897-1112): each round draws from the
 * current proposal, weighs by the generating density alone, clips the
 * isqrt(n) largest log weights to the (n - isqrt(n) + 1)-th smallest
 * (:22-33, Julia's min) and fits the next proposal to the round's samples
 * with the clipped weights. Per-round ESS / log Z of the raw weights and the
 * ESS of the clipped ones. Returns 0 or -(round) for a failed fit. */
int orc_npmc_run(const orc_target *target, int d, int family, double dof, const double *loc0,
                 const double *factor0, int rounds, const int64_t *schedule, const double *normals,
                 const double *rn, int rn_stride, const double *ru, int ru_stride, double regularization,
                 double *samples, double *logweights, double *round_ess, double *round_logz,
                 double *adaptation_ess, double *hist_loc, double *hist_factor, double *hist_lognorm) {
    double logconst = family == ORC_STUDENT_T ? orc_student_t_logconstant(dof, d) : 0.0;
    double *dofs = (double *)malloc(sizeof(double) * (size_t)rounds);
    for (int r = 0; r < rounds; ++r) dofs[r] = dof;
    memcpy(hist_loc, loc0, sizeof(double) * (size_t)d);
    memcpy(hist_factor, factor0, sizeof(double) * (size_t)d * d);
    double logabsdet = 0.0;
    for (int c = 0; c < d; ++c) logabsdet += log(factor0[c + (size_t)c * d]);
    hist_lognorm[0] = family == ORC_STUDENT_T ? logconst - logabsdet : orc_gaussian_lognormalizer(d, logabsdet);
    int64_t maxn = 0;
    for (int r = 0; r < rounds; ++r) maxn = schedule[r] > maxn ? schedule[r] : maxn;
    double *mean = (double *)malloc(sizeof(double) * (size_t)d);
    double *cov = (double *)malloc(sizeof(double) * (size_t)d * d);
    double *sorted = (double *)malloc(sizeof(double) * (size_t)maxn);
    double *clipped = (double *)malloc(sizeof(double) * (size_t)maxn);
    double *wbuf = (double *)malloc(sizeof(double) * (size_t)maxn);
    double *vals = (double *)malloc(sizeof(double) * (size_t)d);
    int *exps = (int *)malloc(sizeof(int) * (size_t)d);
    int64_t off = 0;
    int status = 0;
    for (int t = 0; t < rounds; ++t) {
        orc_bank hist = {d, t + 1, family, ORC_SCALE_FACTOR, hist_loc, hist_factor, hist_lognorm, dofs, NULL};
        const int64_t n = schedule[t];
        double *x = samples + (size_t)off * d;
        double *lw = logweights + off;
        orc_draw(&hist, NULL, t, normals + (size_t)off * d, rn ? rn + (size_t)off * rn_stride : NULL, rn_stride,
                 ru ? ru + (size_t)off * ru_stride : NULL, ru_stride, n, x, NULL);
        for (int64_t i = 0; i < n; ++i)
            lw[i] = orc_target_logdensity(target, x + (size_t)i * d) -
                    orc_component_logdensity(&hist, t, x + (size_t)i * d, vals, exps);
        double sm[3];
        orc_logweight_summary(lw, n, sm);
        round_ess[t] = sm[1] * sm[1] / sm[2];
        round_logz[t] = sm[0] + log(sm[1]) - log((double)n);
        int64_t r = (int64_t)sqrt((double)n);
        while (r * r > n) --r;
        while ((r + 1) * (r + 1) <= n) ++r;
        memcpy(sorted, lw, sizeof(double) * (size_t)n);
        qsort(sorted, (size_t)n, sizeof(double), cmp_double_nan_last);
        const double thr = sorted[n - r];  /* the (n - r + 1)-th smallest */
        for (int64_t i = 0; i < n; ++i)
            clipped[i] = (isnan(lw[i]) || isnan(thr)) ? (isnan(lw[i]) ? lw[i] : thr) : (lw[i] < thr ? lw[i] : thr);
        double cs[3];
        orc_logweight_summary(clipped, n, cs);
        adaptation_ess[t] = cs[1] * cs[1] / cs[2];
        off += n;
        if (t + 1 < rounds) {
            orc_weighted_moments(x, d, n, clipped, mean, cov, wbuf);
            double *L = hist_factor + (size_t)(t + 1) * d * d;
            if (orc_fit_factor(mean, cov, d, hist_factor + (size_t)t * d * d, family == ORC_STUDENT_T ? dof : 0.0,
                               logconst, regularization, L, hist_lognorm + t + 1) != 0) { status = -(t + 1); break; }
            memcpy(hist_loc + (size_t)(t + 1) * d, mean, sizeof(double) * (size_t)d);
        }
    }
    free(dofs); free(mean); free(cov); free(sorted); free(clipped); free(wbuf); free(vals); free(exps);
    return status;
}

/* ---- population adaptation (src/population_covariance.jl) ------------------ */

static double orc_power_ess(const double *lw, int64_t s0, int64_t cnt, double m, double p, double *total) {
    double s = 0.0, s2 = 0.0;
    for (int64_t i = 0; i < cnt; ++i) {
        const double w = exp(p * (lw[s0 + i] - m));
        s += w;
        s2 += w * w;
    }
    if (total) *total = s;
    return s * s / s2;
}

/* _population_local_weights_slot! (src/population_covariance.jl:136-233) for
 * every slot: normalised local weights, raw ESS and weighted raw mean, then
 * the bisection on the tempering power when the ESS is below the threshold.
 * status: 0 ready, 1 all -Inf, 2 tempering failed. */
void orc_population_local_weights(const double *lw, const double *x, int d, const int64_t *starts,
                                  const int64_t *counts, const double *thresholds, int k, double tolerance,
                                  int max_iterations, double *weights, double *local_ess, double *powers,
                                  uint8_t *status, double *raw_means) {
    for (int s = 0; s < k; ++s) {
        const int64_t s0 = starts[s], cnt = counts[s];
        double m = -INFINITY;
        for (int64_t i = 0; i < cnt; ++i) m = lw[s0 + i] > m ? lw[s0 + i] : m;
        if (m == -INFINITY || cnt == 0) {
            local_ess[s] = 0.0;
            powers[s] = 0.0;
            status[s] = 1;
            continue;
        }
        double total = 0.0, sq = 0.0;
        for (int64_t i = 0; i < cnt; ++i) {
            const double w = exp(lw[s0 + i] - m);
            weights[s0 + i] = w;
            total += w;
            sq += w * w;
        }
        const double inv = 1.0 / total;
        for (int64_t i = 0; i < cnt; ++i) weights[s0 + i] *= inv;
        if (raw_means)
            for (int c = 0; c < d; ++c) {
                double a = 0.0;
                for (int64_t i = 0; i < cnt; ++i) a += weights[s0 + i] * x[(s0 + i) * d + c];
                raw_means[(size_t)s * d + c] = a;
            }
        const double ess = total * total / sq;
        local_ess[s] = ess;
        powers[s] = 1.0;
        status[s] = 0;
        if (ess >= thresholds[s]) continue;
        double lo = 0.0, hi = 1.0, lo_ess = 0.0;
        for (int it = 0; it < max_iterations; ++it) {
            const double p = 0.5 * (lo + hi);
            const double e = orc_power_ess(lw, s0, cnt, m, p, NULL);
            if (e >= thresholds[s]) { lo = p; lo_ess = e; } else { hi = p; }
            if (hi - lo <= tolerance) break;
        }
        if (lo == 0.0) {
            powers[s] = 0.0;
            status[s] = 2;
            continue;
        }
        double t;
        orc_power_ess(lw, s0, cnt, m, lo, &t);
        for (int64_t i = 0; i < cnt; ++i) weights[s0 + i] = exp(lo * (lw[s0 + i] - m)) / t;
        local_ess[s] = lo_ess;
        powers[s] = lo;
    }
}

/* _fit_population_covariance_slot! (src/population_covariance.jl:482-545):
 * ready slots: centre (weighted mean when tempered, else the location) and
 * the weighted covariance about it; other slots: the current covariance
 * L L^T * multiplier from `factors` (d x d x K column-major) and `dofs`
 * (NULL for Gaussian). */
void orc_population_covariances(const double *x, int d, const double *weights, const double *powers,
                                const uint8_t *status, const double *locations, const double *factors,
                                const double *dofs, const int64_t *starts, const int64_t *counts, int k,
                                double *centres, double *covs) {
    for (int s = 0; s < k; ++s) {
        const int64_t s0 = starts[s], cnt = counts[s];
        double *cs = centres + (size_t)s * d;
        double *ck = covs + (size_t)s * d * d;
        const int tempered = status[s] == 0 && powers[s] < 1.0;
        for (int c = 0; c < d; ++c) {
            double a = locations[(size_t)s * d + c];
            if (tempered) {
                a = 0.0;
                for (int64_t i = 0; i < cnt; ++i) a += weights[s0 + i] * x[(s0 + i) * d + c];
            }
            cs[c] = a;
        }
        for (int c = 0; c < d; ++c)
            for (int r = c; r < d; ++r) {
                double v = 0.0;
                if (status[s] != 0) {
                    const double *L = factors + (size_t)s * d * d;
                    for (int j = 0; j <= c; ++j) v += L[r + (size_t)j * d] * L[c + (size_t)j * d];
                    if (dofs) v *= dofs[s] / (dofs[s] - 2.0);
                } else {
                    for (int64_t i = 0; i < cnt; ++i)
                        v += weights[s0 + i] * (x[(s0 + i) * d + r] - cs[r]) * (x[(s0 + i) * d + c] - cs[c]);
                }
                ck[r + (size_t)c * d] = v;
                ck[c + (size_t)r * d] = v;
            }
    }
}

/* _factor_population_slot! and _scale_population_factors!
 * (src/population_covariance.jl:807-828,959-973): potrf of each ready slot
 * (info -1 for a non-finite covariance, else the failing column), zeros above
 * the diagonal, then the Student-t scaling sqrt((nu-2)/nu) when dofs != NULL. */
void orc_population_factors(const double *covs, int d, int k, const uint8_t *status, const double *dofs,
                            double *factors, int32_t *info) {
    for (int s = 0; s < k; ++s) {
        info[s] = 0;
        if (status[s] != 0) continue;
        const double *ck = covs + (size_t)s * d * d;
        double *f = factors + (size_t)s * d * d;
        int bad = 0;
        for (int e = 0; e < d * d; ++e) {
            const int r = e % d, c = e / d;
            if (!isfinite(ck[e])) bad = 1;
            f[e] = r >= c ? ck[e] : 0.0;
        }
        if (bad) info[s] = -1;
        for (int j = 0; j < d && !bad; ++j) {
            double piv = f[j + (size_t)j * d];
            for (int q = 0; q < j; ++q) piv -= f[j + (size_t)q * d] * f[j + (size_t)q * d];
            if (!(isfinite(piv) && piv > 0.0)) { info[s] = j + 1; break; }
            f[j + (size_t)j * d] = sqrt(piv);
            for (int r = j + 1; r < d; ++r) {
                double v = f[r + (size_t)j * d];
                for (int q = 0; q < j; ++q) v -= f[r + (size_t)q * d] * f[j + (size_t)q * d];
                f[r + (size_t)j * d] = v / f[j + (size_t)j * d];
            }
        }
        if (dofs) {
            const double sc = sqrt((dofs[s] - 2.0) / dofs[s]);
            for (int e = 0; e < d * d; ++e) f[e] *= sc;
        }
    }
}
