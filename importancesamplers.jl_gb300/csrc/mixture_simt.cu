// mixture_simt.cu — SIMT (CUDA-core) kernels for the balance-heuristic
// mixture density in the bank's own precision. This is the drop-in path for
// FP32 and FP64 banks: one thread owns one sample (held in registers), the
// bank is staged in shared memory in chunks, and each (sample, component)
// pair runs the reference's forward substitution
// (_packed_gaussian_logdensity!, src/native_execution.jl:346-384) followed by
// the radial density (src/proposals.jl:24-70). The balance-heuristic sum is an
// online log-sum-exp (one exp per pair) instead of the reference's chained
// logaddexp (src/mis_execution.jl:30-65): same value, two fewer
// transcendentals per term, same NaN / -Inf semantics.
//
// Non-finite radii, subnormal Student-t radii and range-risk Student-t slots
// leave the fast path for `slow_component_logdensity`, a restatement of the
// reference's exponent-extended solves (src/student_t_range.jl:82-153).
#include "issm_device.cuh"
#include "issm_internal.h"
#include "rng.cuh"
#include "tcgen05.cuh"

namespace issm {

// Shared-memory layout of one staged component (units of T):
//   [0] lognormalizer  [1] coefficient  [2] dof  [3] range-risk flag
//   mu[D]  invdiag[D] (factor) | scale[D] (diagonal)
//   factor: packed lower triangle, row r at r(r+1)/2 .. + r   (compile-time offsets)
//   diagonal: inverse scale[D]
template <int D, bool FACTOR> struct Layout {
    static constexpr int kHdr = 4;
    static constexpr int kMu = kHdr;
    static constexpr int kAux = kMu + D;              // invdiag or scale
    static constexpr int kTri = kAux + D;             // packed L, or inverse scale
    static constexpr int kBody = FACTOR ? D * (D + 1) / 2 : D;
    static constexpr int kStride = ((kTri + kBody) + 3) / 4 * 4;
    __device__ static constexpr int tri(int r, int c) { return kTri + r * (r + 1) / 2 + c; }
};

template <typename T> struct MixParams {
    // bank
    int d, k, family, scale_kind;
    const T *loc, *scales, *lognorm, *dofs;
    const uint8_t *range_risk;
    // denominator
    int den_kind, terms;
    const T *coef;
    const int32_t *group;
    // samples / slots
    int64_t n;
    const T *x;            // input samples (DENOM / APPEND)
    const int32_t *slots;  // generating slots or NULL
    int fixed_slot;
    // draw inputs (ROUND)
    const T *normals, *rnormals, *runiforms;
    // fused normals (fixed-slot factor draws): element e of row i is element
    // noffset (+ *nbase) + i d + e of the (nseed) normal stream
    int fused;
    uint64_t nseed, noffset;
    const uint64_t *nbase;
    int rn_stride, ru_stride;
    T *samples_out;
    // outputs
    T *out_logden, *out_generating;
    const T *logtargets;
    T *logweights;
    const int64_t *proposal_ids;
    int64_t *proposal_ids_out;
    T *lognum;             // APPEND in/out
    uint64_t *failures;
    int64_t index_base;
    int mode;
    int first_slot, last_slot, chunk;
};

// ---- slow path ----------------------------------------------------------
template <typename T> struct Rng { T m; int e; };
template <typename T> __device__ Rng<T> rfrexp(T v) { Rng<T> r; r.m = dfrexp(v, &r.e); return r; }
template <typename T> __device__ Rng<T> range_subtract(Rng<T> l, Rng<T> r) {
    if (l.m == T(0)) return Rng<T>{-r.m, r.e};
    if (r.m == T(0)) return l;
    int e = l.e > r.e ? l.e : r.e;
    int s;
    T m = dfrexp(dldexp(l.m, l.e - e) - dldexp(r.m, r.e - e), &s);
    return Rng<T>{m, m == T(0) ? 0 : e + s};
}
template <typename T> __device__ Rng<T> range_multiply(Rng<T> v, T f) {
    int fe, s;
    T fm = dfrexp(f, &fe);
    T p = dfrexp(v.m * fm, &s);
    return Rng<T>{p, p == T(0) ? 0 : v.e + fe + s};
}
template <typename T> __device__ Rng<T> range_divide(Rng<T> v, T dv) {
    int de, s;
    T dm = dfrexp(dv, &de);
    T q = dfrexp(v.m / dm, &s);
    return Rng<T>{q, q == T(0) ? 0 : v.e - de + s};
}
template <typename T> __device__ T logabsdiff(T l, T r) {
    T diff = l - r;
    if (isfinite(diff) || !isfinite(l) || !isfinite(r)) return dlog(fabs(diff));
    T al = fabs(l), ar = fabs(r);
    T big = al > ar ? al : ar, small = al > ar ? ar : al;
    return dlog(big) + dlog1p(small / big);
}

// Full reference semantics for one pair, reading the component from its
// global (reference-layout) arrays. Only taken for exceptional radii.
template <typename T>
__device__ __noinline__ T slow_component_logdensity(const MixParams<T> &p, int slot, const T *x) {
    const int d = p.d;
    T z[64];
    int ex[64];
    const T *mu = p.loc + (size_t)slot * d;
    T lognorm = p.lognorm[slot];
    T r2 = T(0);
    const bool factor = p.scale_kind == ISSM_SCALE_FACTOR;
    const T *L = factor ? p.scales + (size_t)slot * d * d : nullptr;
    const T *sc = p.scale_kind == ISSM_SCALE_SPHERICAL ? p.scales + slot : p.scales + (size_t)slot * d;
    auto scale_at = [&](int c) { return p.scale_kind == ISSM_SCALE_SPHERICAL ? sc[0] : sc[c]; };
    if (factor) {
        for (int r = 0; r < d; ++r) {
            T v = x[r] - mu[r];
            for (int c = 0; c < r; ++c) v -= L[r + (size_t)c * d] * z[c];
            v /= L[r + (size_t)r * d];
            z[r] = v;
            r2 += v * v;
        }
        if (!isfinite(r2)) {
            bool all_finite = true;
            for (int c = 0; c < d; ++c) all_finite &= (bool)isfinite(z[c]);
            if (!all_finite) {
                r2 = T(0);
                for (int r = 0; r < d; ++r) {
                    // _factor_standardized_coordinate (src/student_t_range.jl:89-109)
                    T v = x[r] - mu[r];
                    for (int c = 0; c < r; ++c) v -= L[r + (size_t)c * d] * z[c];
                    T dg = L[r + (size_t)r * d];
                    v /= dg;
                    if (!(isfinite(v) || !isfinite(x[r]) || !isfinite(mu[r]))) {
                        Rng<T> val = range_subtract(rfrexp(x[r]), rfrexp(mu[r]));
                        bool done = false;
                        for (int c = 0; c < r && !done; ++c) {
                            if (!isfinite(z[c])) { v = z[c]; done = true; break; }
                            val = range_subtract(val, range_multiply(rfrexp(z[c]), L[r + (size_t)c * d]));
                        }
                        if (!done) {
                            Rng<T> q = range_divide(val, dg);
                            v = dldexp(q.m, q.e);
                        }
                    }
                    z[r] = v;
                    r2 += v * v;
                }
            }
        }
    } else {
        for (int c = 0; c < d; ++c) {
            T v = (x[c] - mu[c]) / scale_at(c);
            r2 += v * v;
        }
        for (int c = 0; c < d; ++c) {
            T diff = x[c] - mu[c];
            z[c] = (isfinite(diff) || !isfinite(x[c]) || !isfinite(mu[c])) ? diff / scale_at(c)
                                                                           : x[c] / scale_at(c) - mu[c] / scale_at(c);
        }
    }
    auto logradius = [&]() -> T {
        T total = -num<T>::inf();
        if (factor) {
            for (int r = 0; r < d; ++r) {
                Rng<T> val = range_subtract(rfrexp(x[r]), rfrexp(mu[r]));
                for (int c = 0; c < r; ++c)
                    val = range_subtract(val, range_multiply(Rng<T>{z[c], ex[c]}, L[r + (size_t)c * d]));
                Rng<T> q = range_divide(val, L[r + (size_t)r * d]);
                z[r] = q.m;
                ex[r] = q.e;
                T la = dlog(fabs(q.m)) + T(q.e) * dlog(T(2));
                total = logaddexp(total, T(2) * la);
            }
        } else {
            for (int c = 0; c < d; ++c) {
                T v = logabsdiff(x[c], mu[c]) - dlog(scale_at(c));
                total = logaddexp(total, T(2) * v);
            }
        }
        return total;
    };
    if (p.family == ISSM_GAUSSIAN) {
        T half = T(0.5) * r2;
        if (!isfinite(r2)) {
            half = T(0);
            for (int c = 0; c < d; ++c) half += (T(0.5) * z[c]) * z[c];
        }
        return lognorm - half;
    }
    const T dof = p.dofs[slot];
    const bool risk = factor && p.range_risk != nullptr && p.range_risk[slot];
    const T ratio = r2 / dof;
    T radial;
    if (risk) {
        radial = log1pexp(logradius() - dlog(dof));
    } else if (r2 < num<T>::fmin()) {
        T s = dsqrt(dof), acc = T(0);
        for (int c = 0; c < d; ++c) { T v = z[c] / s; acc += v * v; }
        radial = dlog1p(acc);
    } else if (isfinite(ratio)) {
        radial = dlog1p(ratio);
    } else if (isfinite(r2)) {
        radial = dlog(r2) - dlog(dof);
    } else {
        T scale = T(0);
        for (int c = 0; c < d; ++c) scale = fmax(scale, fabs(z[c]));
        if (!isfinite(scale)) {
            radial = log1pexp(logradius() - dlog(dof));
        } else {
            T acc = T(0);
            for (int c = 0; c < d; ++c) { T v = z[c] / scale; acc += v * v; }
            radial = log1pexp(T(2) * dlog(scale) + dlog(acc) - dlog(dof));
        }
    }
    return lognorm - (dof + T(d)) / T(2) * radial;
}

// ---- fast path ------------------------------------------------------------
template <typename T> __device__ __forceinline__ T mul_or_div(T v, T inv, T dg);
template <> __device__ __forceinline__ float mul_or_div<float>(float v, float inv, float) { return v * inv; }
template <> __device__ __forceinline__ double mul_or_div<double>(double v, double, double dg) { return v / dg; }

template <typename T, int D, bool FACTOR>
__device__ __forceinline__ T fast_component_logdensity(const T *__restrict__ c, const T (&x)[D], int d,
                                                       int family, bool *slow) {
    using Ly = Layout<D, FACTOR>;
    T r2 = T(0);
    if constexpr (FACTOR) {
        T z[D];
#pragma unroll
        for (int r = 0; r < D; ++r) {
            if (r < d) {
                T v = x[r] - c[Ly::kMu + r];
#pragma unroll
                for (int q = 0; q < r; ++q) v -= c[Ly::tri(r, q)] * z[q];
                v = mul_or_div(v, c[Ly::kAux + r], c[Ly::tri(r, r)]);
                z[r] = v;
                r2 += v * v;
            }
        }
    } else {
#pragma unroll
        for (int r = 0; r < D; ++r) {
            if (r < d) {
                T v = mul_or_div(x[r] - c[Ly::kMu + r], c[Ly::kTri + r], c[Ly::kAux + r]);
                r2 += v * v;
            }
        }
    }
    const T lognorm = c[0];
    if (family == ISSM_GAUSSIAN) {
        if (!isfinite(r2)) { *slow = true; return T(0); }
        return lognorm - T(0.5) * r2;
    }
    const T dof = c[2];
    const T ratio = r2 / dof;
    if (c[3] != T(0) || r2 < num<T>::fmin() || !isfinite(ratio)) { *slow = true; return T(0); }
    return lognorm - (dof + T(d)) * T(0.5) * dlog1p(ratio);
}

// Stage components [k0, k0 + count) of the bank into shared memory.
template <typename T, int D, bool FACTOR>
__device__ void stage_components(T *sm, const MixParams<T> &p, int k0, int count) {
    using Ly = Layout<D, FACTOR>;
    const int d = p.d;
    const int total = count * Ly::kStride;
    for (int e = threadIdx.x; e < total; e += blockDim.x) {
        const int kk = e / Ly::kStride, off = e - kk * Ly::kStride;
        const int k = k0 + kk;
        T v = T(0);
        if (off == 0) v = p.lognorm[k];
        else if (off == 1) v = (p.den_kind == ISSM_DENOM_GENERATING || p.coef == nullptr) ? T(0) : p.coef[k];
        else if (off == 2) v = p.dofs ? p.dofs[k] : T(0);
        else if (off == 3) v = (p.range_risk && p.scale_kind == ISSM_SCALE_FACTOR && p.family == ISSM_STUDENT_T) ? T(p.range_risk[k]) : T(0);
        else if (off < Ly::kAux) { int r = off - Ly::kMu; if (r < d) v = p.loc[(size_t)k * d + r]; }
        else if (off < Ly::kTri) {
            int r = off - Ly::kAux;
            if (r < d) {
                if (FACTOR) v = T(1) / p.scales[(size_t)k * d * d + (size_t)r * d + r];
                else v = p.scale_kind == ISSM_SCALE_SPHERICAL ? p.scales[k] : p.scales[(size_t)k * d + r];
            }
        } else if (off < Ly::kTri + Ly::kBody) {
            int t = off - Ly::kTri;
            if (FACTOR) {
                int r = 0;
                while ((r + 1) * (r + 2) / 2 <= t) ++r;
                int q = t - r * (r + 1) / 2;
                if (r < d && q < d) v = p.scales[(size_t)k * d * d + (size_t)q * d + r];
            } else {
                int r = t;
                if (r < d) v = T(1) / (p.scale_kind == ISSM_SCALE_SPHERICAL ? p.scales[k] : p.scales[(size_t)k * d + r]);
            }
        }
        sm[e] = v;
    }
}

// Student-t radial multiplier from buffered draws (src/native_execution.jl:153-180).
template <typename T>
__device__ T radial_multiplier(T dof, const T *rn, const T *ru, bool has_u, uint16_t *reason) {
    *reason = 0;
    if (!has_u || dof == T(1)) {
        T den = fabs(rn[0]);
        if (!(isfinite(den) && den > T(0))) { *reason = ISSM_REASON_DRAW_EXHAUSTED; return T(0); }
        return T(1) / den;
    }
    const T shape = dof / T(2);
    const T adjusted = shape < T(1) ? shape + T(1) : shape;
    const T offset = adjusted - T(1) / T(3);
    const T coefm = T(1) / dsqrt(offset) / T(3);
    for (int a = 0; a < 8; ++a) {
        const T normal = rn[a], uniform = ru[a];
        const T root = T(1) + coefm * normal;
        if (!(root > T(0))) continue;
        const T cube = root * root * root;
        const T n2 = normal * normal;
        const bool acc = uniform < T(1) - T(0.0331) * (n2 * n2) ||
                         dlog(uniform) < T(0.5) * n2 + offset * (T(1) - cube + dlog(cube));
        if (!acc) continue;
        T g = offset * cube;
        if (shape < T(1)) g *= dpow(ru[8], T(1) / shape);
        if (!(isfinite(g) && g > T(0))) break;
        return dsqrt(dof / (T(2) * g));
    }
    *reason = ISSM_REASON_DRAW_EXHAUSTED;
    return T(0);
}

// x = mu_s + L_s (m n) with the packed-bank summation order
// (_native_proposal_coordinate, src/native_execution.jl:238-264).
template <typename T, int D>
__device__ bool draw_sample(const MixParams<T> &p, int64_t i, int s, T (&x)[D], uint16_t *reason) {
    const int d = p.d;
    T m = T(1);
    *reason = 0;
    if (p.family == ISSM_STUDENT_T) {
        uint16_t r;
        m = radial_multiplier(p.dofs[s], p.rnormals + (size_t)i * p.rn_stride,
                              p.runiforms ? p.runiforms + (size_t)i * p.ru_stride : nullptr,
                              p.runiforms != nullptr && p.ru_stride > 0, &r);
        if (r) {
            record_failure(p.failures, p.index_base + i + 1, 0, r);
            m = qnan<T>();
        }
    }
    const T *mu = p.loc + (size_t)s * d;
    const T *nz = p.normals + (size_t)i * d;
    bool valid = true;
    T nm[D];
#pragma unroll
    for (int c = 0; c < D; ++c) if (c < d) nm[c] = nz[c] * m;
    if (p.scale_kind == ISSM_SCALE_FACTOR) {
        const T *L = p.scales + (size_t)s * d * d;
#pragma unroll
        for (int r = 0; r < D; ++r) {
            if (r < d) {
                T v = mu[r];
#pragma unroll
                for (int c = 0; c <= r; ++c) v += L[r + (size_t)c * d] * nm[c];
                x[r] = v;
                valid &= (bool)isfinite(v);
            }
        }
    } else {
#pragma unroll
        for (int r = 0; r < D; ++r) {
            if (r < d) {
                T sc = p.scale_kind == ISSM_SCALE_SPHERICAL ? p.scales[s] : p.scales[(size_t)s * d + r];
                T v = mu[r] + sc * nm[r];
                x[r] = v;
                valid &= (bool)isfinite(v);
            }
        }
    }
    if (p.samples_out) {
        T *out = p.samples_out + (size_t)i * d;
#pragma unroll
        for (int r = 0; r < D; ++r) if (r < d) out[r] = x[r];
    }
    if (!valid) *reason = ISSM_REASON_GENERATED_NONFINITE;
    return valid;
}

// Same draw with the component already staged in shared memory (fixed-slot
// draws: every sample of the launch comes from one proposal).
template <typename T, int D, bool FACTOR>
__device__ bool draw_sample_staged(const MixParams<T> &p, int64_t i, const T *__restrict__ c, T (&x)[D],
                                   uint16_t *reason) {
    using Ly = Layout<D, FACTOR>;
    const int d = p.d;
    T m = T(1);
    *reason = 0;
    if (p.family == ISSM_STUDENT_T) {
        uint16_t r;
        m = radial_multiplier(c[2], p.rnormals + (size_t)i * p.rn_stride,
                              p.runiforms ? p.runiforms + (size_t)i * p.ru_stride : nullptr,
                              p.runiforms != nullptr && p.ru_stride > 0, &r);
        if (r) {
            record_failure(p.failures, p.index_base + i + 1, 0, r);
            m = qnan<T>();
        }
    }
    const T *nz = p.normals + (size_t)i * d;
    T nm[D];
#pragma unroll
    for (int q = 0; q < D; ++q) nm[q] = q < d ? nz[q] * m : T(0);
    bool valid = true;
#pragma unroll
    for (int r = 0; r < D; ++r) {
        if (r < d) {
            T v = c[Ly::kMu + r];
            if constexpr (FACTOR) {
#pragma unroll
                for (int q = 0; q <= r; ++q) v += c[Ly::tri(r, q)] * nm[q];
            } else {
                v += c[Ly::kAux + r] * nm[r];
            }
            x[r] = v;
            valid &= (bool)isfinite(v);
        }
    }
    if (p.samples_out) {
        T *out = p.samples_out + (size_t)i * d;
#pragma unroll
        for (int r = 0; r < D; ++r) if (r < d) out[r] = x[r];
    }
    if (!valid) *reason = ISSM_REASON_GENERATED_NONFINITE;
    return valid;
}

enum Mode { kModeDenominator = 0, kModeRound = 1, kModeAppend = 2, kModeDraw = 3 };

template <typename T, int D, bool FACTOR>
__global__ void __launch_bounds__(128) mixture_simt_kernel(MixParams<T> p) {
    using Ly = Layout<D, FACTOR>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *sm = reinterpret_cast<T *>(smem_raw);
    const int d = p.d;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = i < p.n;
    T x[D];
#pragma unroll
    for (int r = 0; r < D; ++r) x[r] = T(0);
    const int gen = active ? (p.slots ? p.slots[i] : p.fixed_slot) : 0;
    bool ok = active;
    if (p.mode == kModeDraw && p.slots == nullptr) {
        stage_components<T, D, FACTOR>(sm, p, p.fixed_slot, 1);
        __syncthreads();
        if (active) {
            uint16_t reason;
            if (!draw_sample_staged<T, D, FACTOR>(p, i, sm, x, &reason))
                record_failure(p.failures, p.index_base + i + 1, 0, reason);
        }
        return;
    }
    if (active) {
        if (p.mode == kModeRound || p.mode == kModeDraw) {
            uint16_t reason;
            if (!draw_sample<T, D>(p, i, gen, x, &reason)) {
                record_failure(p.failures, p.index_base + i + 1, 0, reason);
                ok = false;
            }
        } else {
            const T *xi = p.x + (size_t)i * d;
#pragma unroll
            for (int r = 0; r < D; ++r) if (r < d) x[r] = xi[r];
        }
    }
    if (p.mode == kModeDraw) return;

    LseState<T> lse;
    T gen_lq = T(0);
    T append_lq = T(0);
    bool any_slow = false;
    const int g_gen = (p.den_kind == ISSM_DENOM_PARTIAL && active) ? p.group[gen] : 0;
    for (int k0 = p.first_slot; k0 <= p.last_slot; k0 += p.chunk) {
        const int count = min(p.chunk, p.last_slot - k0 + 1);
        __syncthreads();
        stage_components<T, D, FACTOR>(sm, p, k0, count);
        __syncthreads();
        if (!ok) continue;
        for (int kk = 0; kk < count; ++kk) {
            const int k = k0 + kk;
            if (p.den_kind == ISSM_DENOM_GENERATING && k != gen) continue;
            if (p.den_kind == ISSM_DENOM_PARTIAL && p.group[k] != g_gen) continue;
            const T *c = sm + (size_t)kk * Ly::kStride;
            bool slow = false;
            T lq = fast_component_logdensity<T, D, FACTOR>(c, x, d, p.family, &slow);
            if (slow) {
                any_slow = true;
                const T *xg = (p.mode == kModeRound) ? p.samples_out + (size_t)i * d : p.x + (size_t)i * d;
                lq = slow_component_logdensity<T>(p, k, xg);
            }
            if (k == gen) gen_lq = lq;
            append_lq = lq;
            lse.add(c[1] + lq);
        }
    }
    (void)any_slow;
    if (!active) return;
    if (p.mode == kModeAppend) {
        if (!ok) return;
        uint16_t reason = isnan(append_lq) ? ISSM_REASON_PROPOSAL_INVALID : 0;
        if (!reason) {
            T v = logaddexp(p.lognum[i], p.coef[p.first_slot] + append_lq);
            if (isnan(v) || v == -num<T>::inf()) reason = ISSM_REASON_PROPOSAL_INVALID;
            else p.lognum[i] = v;
        }
        if (reason) record_failure(p.failures, p.index_base + i + 1, 0, reason);
        return;
    }
    T den = -num<T>::inf();
    if (ok) {
        den = lse.value();
        if (isnan(gen_lq) || gen_lq == -num<T>::inf() || isnan(den) || den == -num<T>::inf()) {
            record_failure(p.failures, p.index_base + i + 1, 0, ISSM_REASON_PROPOSAL_INVALID);
            ok = false;
            den = -num<T>::inf();
        }
    }
    if (p.mode == kModeDenominator) {
        p.out_logden[i] = den;
        if (p.out_generating) p.out_generating[i] = ok ? gen_lq : -num<T>::inf();
        return;
    }
    // kModeRound: _mis_round_launch_kernel! (src/mis_execution.jl:674-720)
    T lw = -num<T>::inf();
    int64_t pid = 0;
    if (ok) {
        T target = p.logtargets ? p.logtargets[i] : T(0);
        uint16_t tr = p.logtargets ? target_reason(target) : 0;
        if (tr) {
            record_failure(p.failures, p.index_base + i + 1, 0, tr);
        } else {
            T w;
            uint16_t r = subtract_logweight(target, den, &w);
            if (r) record_failure(p.failures, p.index_base + i + 1, 0, r);
            else { lw = w; pid = p.proposal_ids ? p.proposal_ids[gen] : (int64_t)gen + 1; }
        }
    }
    p.logweights[i] = lw;
    if (p.proposal_ids_out) p.proposal_ids_out[i] = pid;
    if (p.out_logden) p.out_logden[i] = den;
    if (p.out_generating) p.out_generating[i] = gen_lq;
}

// Fixed-slot draws from one factor component, x = mu + L (m z) with the
// reference's summation order (mu first, then q = 0..r). A CTA of 256 threads
// takes a tile of 64 rows:
//  * the factor is staged once per CTA, column-major (column q holds L[., q],
//    so 4 consecutive rows of a column are one 16-byte broadcast load), with
//    its upper triangle zeroed;
//  * the tile's normals are staged transposed, zT[q][row], from coalesced
//    loads or, with fused normals, generated there from the counter-based
//    stream (the tile's elements are contiguous in the stream, so the threads
//    take its Philox blocks in turn and no normal touches HBM);
//  * four threads share a row and split its output coordinates where the
//    triangular work quarters; each forms 4 coordinates at a time as
//    independent FMA chains over q = 0..r0+3 (the zero upper triangle makes
//    the extra terms exact no-ops), reading z[q] of 32 consecutive rows from
//    32 banks, so the loops stay compact (a fully unrolled triangle overflows
//    the instruction cache);
//  * x goes to a row-major staging tile and is stored coalesced.
constexpr int kDrawRows = 64;     // rows per tile
constexpr int kDrawParts = 4;     // threads per row
template <int D> struct DrawSplit {
    // first output coordinate of part i: 4 * ceil(D sqrt(i / 4) / 4), the triangle's quarters
    static constexpr int at(int i) {
        return i == 0 ? 0 : i >= 4 ? D : D == 64 ? (i == 1 ? 32 : i == 2 ? 44 : 56)
                                       : D == 32 ? (i == 1 ? 16 : i == 2 ? 24 : 28)
                                       : D == 16 ? (i == 1 ? 8 : i == 2 ? 12 : 16)
                                                 : D;
    }
};

template <typename T, int D>
__global__ void __launch_bounds__(kDrawRows * kDrawParts) draw_fixed_kernel(MixParams<T> p) {
    constexpr int LC = D + 4;          // column stride of the staged factor (16-byte aligned columns)
    constexpr int LR = kDrawRows + 4;  // row stride of zT (per coordinate)
    constexpr int LX = D + 4;          // row stride of the x tile
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *Lc = reinterpret_cast<T *>(smem_raw);  // D columns of LC
    T *mus = Lc + D * LC;                      // D
    T *zT = mus + D;                           // D x LR
    T *xs = zT + D * LR;                       // kDrawRows x LX
    __shared__ T s_mult[kDrawRows];
    __shared__ int s_bad[kDrawRows];
    const int d = p.d, k = p.fixed_slot, tid = threadIdx.x;
    const int row = tid % kDrawRows, part = tid / kDrawRows;  // warp-uniform parts
    const T *Lk = p.scales + (size_t)k * d * d;
    // rows of whole 16-byte vectors, both buffers 16-byte aligned
    const bool vec = (d * sizeof(T)) % 16 == 0 && (p.fused || (reinterpret_cast<uintptr_t>(p.normals) & 15) == 0) &&
                     (reinterpret_cast<uintptr_t>(p.samples_out) & 15) == 0;
    if (d == D && (reinterpret_cast<uintptr_t>(Lk) & 15) == 0) {
        // every column in flight at once (16-byte asynchronous copies; the padding is never read)
        constexpr int V = 16 / sizeof(T), CV = D / V;
        for (int e = tid; e < D * CV; e += blockDim.x) {
            const int q = e / CV, c = e - q * CV;
            tc::cp_async16(Lc + q * LC + c * V, Lk + (size_t)q * D + c * V);
        }
        tc::cp_async_commit();
        tc::cp_async_wait_all();
        __syncthreads();
        for (int e = tid; e < D * D; e += blockDim.x) {
            const int q = e / D, r = e - q * D;
            if (r < q) Lc[q * LC + r] = T(0);
        }
    } else {
        for (int e = tid; e < D * LC; e += blockDim.x) {
            const int q = e / LC, r = e - q * LC;
            Lc[e] = (q < d && r < d && r >= q) ? Lk[(size_t)q * d + r] : T(0);
        }
    }
    for (int r = tid; r < D; r += blockDim.x) mus[r] = r < d ? p.loc[(size_t)k * d + r] : T(0);
    const T dof = p.family == ISSM_STUDENT_T ? p.dofs[k] : T(0);
    const uint64_t noff = p.fused ? p.noffset + (p.nbase ? *p.nbase : 0ull) : 0ull;
    // coordinates d..D-1 of z stay zero
    for (int e = tid; e < (D - d) * LR; e += blockDim.x) zT[d * LR + e] = T(0);
    __syncthreads();
    const int lo = DrawSplit<D>::at(part), hi = DrawSplit<D>::at(part + 1);
    const int64_t ntiles = (p.n + kDrawRows - 1) / kDrawRows;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t row0 = tile * kDrawRows;
        const int rows = (int)min((int64_t)kDrawRows, p.n - row0);
        if (p.fused) {
            using NB = NormalBlock<T>;
            const uint64_t first = noff + (uint64_t)row0 * d;
            const int count = rows * d;
            const uint64_t b0 = first >> NB::kShift;
            if (d == D && (first & (NB::kPer - 1)) == 0) {
                // every Philox block is kPer consecutive coordinates of one row;
                // consecutive lanes take consecutive rows (conflict-free stores into zT)
                constexpr int BPR = D / NB::kPer;
                for (int j = tid; j < kDrawRows * BPR; j += blockDim.x) {
                    const int r = j % kDrawRows, cb = j / kDrawRows;
                    if (r >= rows) continue;
                    T v[NB::kPer];
                    NB::eval(b0 + (uint64_t)(r * BPR + cb), p.nseed, v);
#pragma unroll
                    for (int l = 0; l < NB::kPer; ++l) zT[(cb * NB::kPer + l) * LR + r] = v[l];
                }
            } else {
                const int nb = (int)(((first + (uint64_t)count - 1) >> NB::kShift) - b0 + 1);
                for (int j = tid; j < nb; j += blockDim.x) {
                    const uint64_t blk = b0 + (uint64_t)j;
                    T v[NB::kPer];
                    NB::eval(blk, p.nseed, v);
                    const int q0 = (int)(int64_t)((blk << NB::kShift) - first);  // negative in a split first block
                    int r = q0 >= 0 ? q0 / d : -1;
                    int c = q0 - r * d;
#pragma unroll
                    for (int l = 0; l < NB::kPer; ++l) {
                        if (c >= d) { c -= d; ++r; }
                        if (q0 + l >= 0 && q0 + l < count) zT[c * LR + r] = v[l];
                        ++c;
                    }
                }
            }
        } else {
            const T *nz = p.normals + row0 * d;
            for (int e = tid; e < rows * d; e += blockDim.x) {
                const int r = e / d, c = e - r * d;
                zT[c * LR + r] = nz[e];
            }
        }
        // the radial multiplier of each row (Student-t), once per row
        if (part == 0 && row < rows) {
            T m = T(1);
            if (p.family == ISSM_STUDENT_T) {
                const int64_t i = row0 + row;
                uint16_t rr;
                m = radial_multiplier(dof, p.rnormals + (size_t)i * p.rn_stride,
                                      p.runiforms ? p.runiforms + (size_t)i * p.ru_stride : nullptr,
                                      p.runiforms != nullptr && p.ru_stride > 0, &rr);
                if (rr) {
                    record_failure(p.failures, p.index_base + i + 1, 0, rr);
                    m = qnan<T>();
                }
            }
            s_mult[row] = m;
            s_bad[row] = 0;
        }
        __syncthreads();
        if (row < rows) {
            const T m = s_mult[row];
            const bool scaled = p.family == ISSM_STUDENT_T;
            bool valid = true;
            for (int r0 = lo; r0 < hi; r0 += 4) {
                T v0 = mus[r0], v1 = mus[r0 + 1], v2 = mus[r0 + 2], v3 = mus[r0 + 3];
                for (int q0 = 0; q0 <= r0; q0 += 4) {
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int q = q0 + u;
                        const T z = scaled ? zT[q * LR + row] * m : zT[q * LR + row];
                        const T *col = Lc + q * LC + r0;
                        v0 += col[0] * z;
                        v1 += col[1] * z;
                        v2 += col[2] * z;
                        v3 += col[3] * z;
                    }
                }
                T *xr = xs + row * LX + r0;
                xr[0] = v0; xr[1] = v1; xr[2] = v2; xr[3] = v3;
                if (r0 < d) valid &= (bool)isfinite(v0);
                if (r0 + 1 < d) valid &= (bool)isfinite(v1);
                if (r0 + 2 < d) valid &= (bool)isfinite(v2);
                if (r0 + 3 < d) valid &= (bool)isfinite(v3);
            }
            if (!valid) s_bad[row] = 1;
        }
        __syncthreads();
        if (part == 0 && row < rows && s_bad[row])
            record_failure(p.failures, p.index_base + row0 + row + 1, 0, ISSM_REASON_GENERATED_NONFINITE);
        T *out = p.samples_out + row0 * d;
        if (vec) {
            constexpr int V = 16 / sizeof(T);
            const int dv = d / V;
            for (int e = tid; e < rows * dv; e += blockDim.x) {
                const int r = e / dv, c = e - r * dv;
                *reinterpret_cast<uint4 *>(out + (size_t)e * V) = *reinterpret_cast<const uint4 *>(xs + r * LX + c * V);
            }
        } else {
            for (int e = tid; e < rows * d; e += blockDim.x) {
                const int r = e / d, c = e - r * d;
                out[e] = xs[r * LX + c];
            }
        }
        __syncthreads();
    }
}

template <typename T, int D, bool FACTOR>
static int launch_simt(MixParams<T> p, cudaStream_t stream) {
    if (FACTOR && p.mode == kModeDraw && p.slots == nullptr && p.samples_out != nullptr) {
        const size_t smem = sizeof(T) * ((size_t)D * (D + 4) + D + (size_t)D * (kDrawRows + 4) +
                                         (size_t)kDrawRows * (D + 4));
        auto kern = draw_fixed_kernel<T, D>;
        if (smem > 48 * 1024) {
            const int e = allow_dynamic_smem((const void *)kern);
            if (e) return e;
        }
        const int64_t tiles = (p.n + kDrawRows - 1) / kDrawRows;
        const int blocks = (int)min(tiles, (int64_t)device_sms() * 64);
        if (blocks < 1) return 0;
        { kern<<<blocks, kDrawRows * kDrawParts, smem, stream>>>(p); note_launch(); }
        return (int)cudaGetLastError();
    }
    using Ly = Layout<D, FACTOR>;
    const size_t per = (size_t)Ly::kStride * sizeof(T);
    const size_t budget = 96 * 1024;
    int range = p.last_slot - p.first_slot + 1;
    if (p.mode == kModeDraw) range = p.slots == nullptr ? 1 : 0;  // fixed-slot draws stage one component
    int chunk = range > 0 ? (int)(budget / per) : 1;
    if (chunk < 1) chunk = 1;
    if (chunk > range && range > 0) chunk = range;
    p.chunk = chunk;
    size_t smem = range > 0 ? (size_t)chunk * per : 16;
    auto kern = mixture_simt_kernel<T, D, FACTOR>;
    if (smem > 48 * 1024) {
        const int e = allow_dynamic_smem((const void *)kern);
        if (e) return e;
    }
    const int threads = 128;
    int64_t blocks = (p.n + threads - 1) / threads;
    if (blocks < 1) return 0;
    { kern<<<(unsigned)blocks, threads, smem, stream>>>(p); note_launch(); }
    return (int)cudaGetLastError();
}

template <typename T>
static int dispatch_simt(const MixParams<T> &p, cudaStream_t stream) {
    const bool factor = p.scale_kind == ISSM_SCALE_FACTOR;
    const int d = p.d;
#define ISSM_DISPATCH(DD)                                                   \
    if (d <= DD) return factor ? launch_simt<T, DD, true>(p, stream)        \
                               : launch_simt<T, DD, false>(p, stream);
    ISSM_DISPATCH(4)
    ISSM_DISPATCH(16)
    ISSM_DISPATCH(32)
    ISSM_DISPATCH(64)
#undef ISSM_DISPATCH
    return ISSM_E_UNSUPPORTED;
}

template <typename T>
static MixParams<T> params_from(const issm_bank *b, const issm_denominator *den) {
    MixParams<T> p{};
    p.d = b->dim;
    p.k = b->count;
    p.family = b->family;
    p.scale_kind = b->scale_kind;
    p.loc = (const T *)b->locations;
    p.scales = (const T *)b->scales;
    p.lognorm = (const T *)b->lognormalizers;
    p.dofs = (const T *)b->dofs;
    p.range_risk = b->range_risk;
    p.first_slot = 0;
    p.last_slot = b->count - 1;
    if (den) {
        p.den_kind = den->kind;
        p.terms = den->terms;
        p.coef = (const T *)den->logcoefficients;
        p.group = den->group_of_slot;
        if (den->kind == ISSM_DENOM_PREFIX) p.last_slot = den->terms - 1;
    } else {
        p.den_kind = ISSM_DENOM_GENERATING;
    }
    return p;
}

int simt_mixture(const issm_bank *b, const issm_denominator *den, const void *x, int64_t n,
                 const int32_t *slots, int32_t fixed_slot, void *out_logden, void *out_generating,
                 uint64_t *failures, int64_t index_base, cudaStream_t stream) {
    if (b->dtype == ISSM_F32) {
        auto p = params_from<float>(b, den);
        p.n = n; p.x = (const float *)x; p.slots = slots; p.fixed_slot = fixed_slot;
        p.out_logden = (float *)out_logden; p.out_generating = (float *)out_generating;
        p.failures = failures; p.index_base = index_base; p.mode = kModeDenominator;
        return dispatch_simt(p, stream);
    }
    auto p = params_from<double>(b, den);
    p.n = n; p.x = (const double *)x; p.slots = slots; p.fixed_slot = fixed_slot;
    p.out_logden = (double *)out_logden; p.out_generating = (double *)out_generating;
    p.failures = failures; p.index_base = index_base; p.mode = kModeDenominator;
    return dispatch_simt(p, stream);
}

template <typename T>
static int simt_round_t(const issm_bank *b, const issm_denominator *den, const int32_t *slots, int fixed_slot,
                        const void *normals, const void *rn, int rn_stride, const void *ru, int ru_stride,
                        const void *logtargets, int64_t n, void *samples, void *logweights,
                        const int64_t *proposal_ids, int64_t *proposal_ids_out, uint64_t *failures,
                        int64_t index_base, int mode, cudaStream_t stream) {
    auto p = params_from<T>(b, den);
    p.n = n; p.slots = slots; p.fixed_slot = fixed_slot;
    p.normals = (const T *)normals; p.rnormals = (const T *)rn; p.rn_stride = rn_stride;
    p.runiforms = (const T *)ru; p.ru_stride = ru_stride;
    p.logtargets = (const T *)logtargets; p.samples_out = (T *)samples; p.logweights = (T *)logweights;
    p.proposal_ids = proposal_ids; p.proposal_ids_out = proposal_ids_out;
    p.failures = failures; p.index_base = index_base; p.mode = mode;
    return dispatch_simt(p, stream);
}

int simt_round(const issm_bank *b, const issm_denominator *den, const int32_t *slots, const void *normals,
               const void *rn, int rn_stride, const void *ru, int ru_stride, const void *logtargets,
               int64_t n, void *samples, void *logweights, const int64_t *proposal_ids,
               int64_t *proposal_ids_out, uint64_t *failures, cudaStream_t stream) {
    if (b->dtype == ISSM_F32)
        return simt_round_t<float>(b, den, slots, 0, normals, rn, rn_stride, ru, ru_stride, logtargets, n,
                                   samples, logweights, proposal_ids, proposal_ids_out, failures, 0,
                                   kModeRound, stream);
    return simt_round_t<double>(b, den, slots, 0, normals, rn, rn_stride, ru, ru_stride, logtargets, n,
                                samples, logweights, proposal_ids, proposal_ids_out, failures, 0,
                                kModeRound, stream);
}

int simt_draw(const issm_bank *b, const int32_t *slots, int32_t fixed_slot, const void *normals,
              const void *rn, int rn_stride, const void *ru, int ru_stride, int64_t n, void *samples,
              uint64_t *failures, int64_t index_base, cudaStream_t stream) {
    if (b->dtype == ISSM_F32)
        return simt_round_t<float>(b, nullptr, slots, fixed_slot, normals, rn, rn_stride, ru, ru_stride,
                                   nullptr, n, samples, nullptr, nullptr, nullptr, failures, index_base,
                                   kModeDraw, stream);
    return simt_round_t<double>(b, nullptr, slots, fixed_slot, normals, rn, rn_stride, ru, ru_stride,
                                nullptr, n, samples, nullptr, nullptr, nullptr, failures, index_base,
                                kModeDraw, stream);
}

template <typename T>
static int simt_draw_fused_t(const issm_bank *b, int fixed_slot, uint64_t seed, const uint64_t *counter,
                             uint64_t offset, const void *rn, int rn_stride, const void *ru, int ru_stride,
                             int64_t n, void *samples, uint64_t *failures, int64_t index_base,
                             cudaStream_t stream) {
    auto p = params_from<T>(b, nullptr);
    p.n = n; p.slots = nullptr; p.fixed_slot = fixed_slot;
    p.rnormals = (const T *)rn; p.rn_stride = rn_stride;
    p.runiforms = (const T *)ru; p.ru_stride = ru_stride;
    p.samples_out = (T *)samples;
    p.failures = failures; p.index_base = index_base; p.mode = kModeDraw;
    p.fused = 1; p.nseed = seed; p.nbase = counter; p.noffset = offset;
    return dispatch_simt(p, stream);
}

int simt_draw_fused(const issm_bank *b, int32_t fixed_slot, uint64_t seed, const uint64_t *counter,
                    uint64_t offset, const void *rn, int rn_stride, const void *ru, int ru_stride, int64_t n,
                    void *samples, uint64_t *failures, int64_t index_base, cudaStream_t stream) {
    if (b->scale_kind != ISSM_SCALE_FACTOR) return ISSM_E_UNSUPPORTED;
    if (b->dtype == ISSM_F32)
        return simt_draw_fused_t<float>(b, fixed_slot, seed, counter, offset, rn, rn_stride, ru, ru_stride, n,
                                        samples, failures, index_base, stream);
    return simt_draw_fused_t<double>(b, fixed_slot, seed, counter, offset, rn, rn_stride, ru, ru_stride, n,
                                     samples, failures, index_base, stream);
}

template <typename T>
static int simt_append_t(const issm_bank *b, int slot, const void *logcounts, const void *x, int64_t n,
                         void *lognum, uint64_t *failures, cudaStream_t stream) {
    auto p = params_from<T>(b, nullptr);
    p.den_kind = ISSM_DENOM_FULL;
    p.coef = (const T *)logcounts;
    p.first_slot = slot;
    p.last_slot = slot;
    p.n = n; p.x = (const T *)x; p.fixed_slot = slot;
    p.lognum = (T *)lognum; p.failures = failures; p.mode = kModeAppend;
    return dispatch_simt(p, stream);
}

int simt_append(const issm_bank *b, int slot, const void *logcounts, const void *x, int64_t n, void *lognum,
                uint64_t *failures, cudaStream_t stream) {
    if (b->dtype == ISSM_F32) return simt_append_t<float>(b, slot, logcounts, x, n, lognum, failures, stream);
    return simt_append_t<double>(b, slot, logcounts, x, n, lognum, failures, stream);
}

}  // namespace issm
