// group.cu — one launch per phase for every in-flight AMIS run of a serving
// loop: the rounds of many independent posterior runs (uneven dimension,
// sample budget and round) advance together, one round per run per step, so
// the host issues a fixed handful of launches per step whatever the number of
// runs (the per-run sequence is _launch_prefilled_amis_round!,
// src/amis_execution.jl:261-357, then the moment fit,
// src/adaptive_gaussian_execution.jl:348-425).
//
// A step's runs are rows of a descriptor table (GroupRun, device memory).
// Each kernel's blocks are assigned to (run, tile) pairs through per-run
// cumulative block counts (a binary search per block): a run's blocks only
// touch that run's arrays, and every per-run reduction runs in a fixed
// order, so a run's results are bitwise the same alone and in any mix.
//
// Per step, for every run r in its round t:
//   group_draw       x = mu_t + L_t z, z from the counter-based normal stream
//                    (Philox-4x32-10, the run's seed and offset);
//   group_target     the linear-regression log posterior kernel in its exact
//                    mode-centred form log p(y, b) = c0 - |U (b - b_hat)|^2 / 2
//                    (U^T U = X^T X / sigma^2 + I / prior_var, b_hat the mode,
//                    c0 = log p(y, b_hat); formed from X^T X, X^T y, y^T y on
//                    admission) — the same function as the likelihood summed
//                    over the observations;
//   group_mixture    new samples: log sum_{s<=t} n_s q_s(x); retained ones:
//                    logaddexp with n_t q_t(x) (the AMIS recurrence), by
//                    forward substitution in FP32;
//   group_form       log weights log pi - log mixture + log N_t and per-block
//                    (max, S, S2) partials;
//   group_summary    one block per run: the partials merged in order;
//   group_moments    per-block sums of w (x - c) and w (x - c)(x - c)^T about
//                    the previous location c (compensated FP32, stored FP64);
//   group_fit        one block per run: the sums merged in order, mean and
//                    covariance, the ridge sqrt(eps(Float32)) tr(L L^T) / d,
//                    an FP64 Cholesky and the next slot (or the candidate).
#include "issm_device.cuh"
#include "issm_internal.h"
#include "rng.cuh"

namespace issm {

using GroupRun = issm_group_run;
static_assert(sizeof(GroupRun) == 8 * 31, "issm_group_run is 31 eight-byte fields");

constexpr int kGTile = ISSM_GROUP_TILE;                       // samples per block of the per-sample kernels
constexpr int kGMomTiles = ISSM_GROUP_MOMENT_SAMPLES / kGTile;  // tiles per moment block
constexpr int kMomWords = ISSM_GROUP_MOMENT_WORDS;            // S0, S1, lower S2
static_assert(kMomWords == 1 + 64 + 64 * 65 / 2, "moment partial layout");

__device__ __forceinline__ int find_run(const GroupRun *runs, int nruns, int64_t blk, int which) {
    int lo = 0, hi = nruns - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        const int64_t b0 = which == 0 ? runs[mid].blk_new0 : which == 1 ? runs[mid].blk_all0 : runs[mid].blk_mom0;
        if (b0 <= blk) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// log q of one Gaussian factor slot: lognorm - |L^-1 (x - mu)|^2 / 2
__device__ __forceinline__ float group_logq(const float *x, const float *mu, const float *L, float lognorm, int d) {
    float z[64];
    float r2 = 0.f;
    for (int r = 0; r < d; ++r) {
        float s = x[r] - mu[r];
        for (int c = 0; c < r; ++c) s = fmaf(-L[r + c * d], z[c], s);
        s /= L[r + r * d];
        z[r] = s;
        r2 = fmaf(s, s, r2);
    }
    return lognorm - 0.5f * r2;
}

__global__ void group_draw_kernel(const GroupRun *__restrict__ runs, int nruns) {
    const int j = find_run(runs, nruns, blockIdx.x, 0);
    const GroupRun &R = runs[j];
    const int64_t i = (int64_t)(blockIdx.x - R.blk_new0) * kGTile + threadIdx.x;
    if (i >= R.n_round) return;
    const int d = (int)R.d, t = (int)R.round;
    const float *mu = R.loc + (size_t)t * d;
    const float *L = R.fac + (size_t)t * d * d;
    float z[64];
    // elements normal_offset + i d + e of the run's FP32 normal stream
    const uint64_t e0 = R.normal_offset + (uint64_t)i * d;
    for (int e = 0; e < d;) {
        const uint64_t el = e0 + e, blk = el >> 2;
        float v[4];
        NormalBlock<float>::eval(blk, R.seed, v);
        for (int q = (int)(el & 3); q < 4 && e < d; ++q, ++e) z[e] = v[q];
    }
    float *x = R.samples + (size_t)(R.n_old + i) * d;
    for (int r = 0; r < d; ++r) {
        float s = mu[r];
        for (int c = 0; c <= r; ++c) s = fmaf(L[r + c * d], z[c], s);
        x[r] = s;
    }
}

__global__ void group_target_kernel(const GroupRun *__restrict__ runs, int nruns) {
    const int j = find_run(runs, nruns, blockIdx.x, 0);
    const GroupRun &R = runs[j];
    const int64_t i = (int64_t)(blockIdx.x - R.blk_new0) * kGTile + threadIdx.x;
    if (i >= R.n_round) return;
    const int d = (int)R.d;
    const float *x = R.samples + (size_t)(R.n_old + i) * d;
    float dl[64];
    for (int c = 0; c < d; ++c) dl[c] = x[c] - R.t_mode[c];
    float q = 0.f;
    for (int r = 0; r < d; ++r) {
        float u = 0.f;
        for (int c = r; c < d; ++c) u = fmaf(R.t_chol[r + c * d], dl[c], u);
        q = fmaf(u, u, q);
    }
    const float v = (float)R.t_const - 0.5f * q;
    R.logtargets[R.n_old + i] = v;
    if (isnan(v) || v == INFINITY)
        record_failure(R.failures + 3 * R.round, R.n_old + i + 1, 0,
                       isnan(v) ? ISSM_REASON_TARGET_NAN : ISSM_REASON_TARGET_POS_INF);
}

__global__ void group_mixture_kernel(const GroupRun *__restrict__ runs, int nruns) {
    const int j = find_run(runs, nruns, blockIdx.x, 1);
    const GroupRun &R = runs[j];
    const int64_t i = (int64_t)(blockIdx.x - R.blk_all0) * kGTile + threadIdx.x;
    const int64_t ntot = R.n_old + R.n_round;
    if (i >= ntot) return;
    const int d = (int)R.d, t = (int)R.round;
    const float *x = R.samples + (size_t)i * d;
    const float lc = (float)R.logcount;
    float out;
    if (i >= R.n_old) {  // a new sample: every slot so far
        LseState<float> lse;
        for (int s = 0; s <= t; ++s)
            lse.add(lc + group_logq(x, R.loc + (size_t)s * d, R.fac + (size_t)s * d * d, R.lognorm[s], d));
        out = lse.value();
    } else {  // a retained sample gains slot t
        out = logaddexp(R.lognum[i], lc + group_logq(x, R.loc + (size_t)t * d, R.fac + (size_t)t * d * d,
                                                     R.lognorm[t], d));
    }
    R.lognum[i] = out;
    if (isnan(out) || out == -INFINITY)
        record_failure(R.failures + 3 * R.round, i + 1, 0, ISSM_REASON_PROPOSAL_INVALID);
}

__global__ void group_form_kernel(const GroupRun *__restrict__ runs, int nruns) {
    const int j = find_run(runs, nruns, blockIdx.x, 1);
    const GroupRun &R = runs[j];
    const int64_t blk = blockIdx.x - R.blk_all0;
    const int64_t i = blk * kGTile + threadIdx.x;
    const int64_t ntot = R.n_old + R.n_round;
    const double logtotal = log((double)ntot);
    float l = -INFINITY;
    if (i < ntot) {
        l = (float)((double)R.logtargets[i] - (double)R.lognum[i] + logtotal);
        R.logweights[i] = l;
        if (isnan(l) || l == INFINITY) record_failure(R.failures + 3 * R.round, i + 1, 0, ISSM_REASON_LOGWEIGHT_INVALID);
    }
    // block (max, sum e^{l-m}, sum e^{2(l-m)}) in FP64, merged in a fixed tree order
    __shared__ double sm[kGTile], ss[kGTile], sq[kGTile];
    sm[threadIdx.x] = (double)l;
    __syncthreads();
    for (int o = kGTile / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sm[threadIdx.x] = fmax(sm[threadIdx.x], sm[threadIdx.x + o]);
        __syncthreads();
    }
    const double m = sm[0];
    const double w = (l == -INFINITY || m == -INFINITY) ? 0.0 : exp((double)l - m);
    ss[threadIdx.x] = w;
    sq[threadIdx.x] = w * w;
    __syncthreads();
    for (int o = kGTile / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            ss[threadIdx.x] += ss[threadIdx.x + o];
            sq[threadIdx.x] += sq[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        R.partial[3 * blk] = m;
        R.partial[3 * blk + 1] = ss[0];
        R.partial[3 * blk + 2] = sq[0];
    }
}

// one block per run: merge the form partials in block order
__global__ void group_summary_kernel(const GroupRun *__restrict__ runs) {
    const GroupRun &R = runs[blockIdx.x];
    if (threadIdx.x != 0) return;
    const int64_t nb = (R.n_old + R.n_round + kGTile - 1) / kGTile;
    double m = -INFINITY;
    for (int64_t b = 0; b < nb; ++b) m = fmax(m, R.partial[3 * b]);
    double s = 0.0, s2 = 0.0;
    if (m != -INFINITY)
        for (int64_t b = 0; b < nb; ++b) {
            const double bm = R.partial[3 * b];
            if (bm == -INFINITY) continue;
            const double f = exp(bm - m);
            s += R.partial[3 * b + 1] * f;
            s2 += R.partial[3 * b + 2] * f * f;
        }
    double *o = R.summaries + 3 * R.round;
    o[0] = m;
    o[1] = s;
    o[2] = s2;
}

// per block of up to kGMomTiles tiles: S0, S1 = sum w (x - c) and the lower
// S2 = sum w (x - c)(x - c)^T, each summed in compensated FP32 (Kahan) and
// stored as FP64 for the fixed-order FP64 merge of the fit. FP64 arithmetic
// here would run on this GPU's narrow FP64 pipe (a warp-instruction holds it
// for about 16 SM cycles whatever the active lanes): two FP64 operations per
// (entry, sample) made this kernel most of a serving step.
__global__ void __launch_bounds__(256) group_moments_kernel(const GroupRun *__restrict__ runs, int nruns) {
    const int j = find_run(runs, nruns, blockIdx.x, 2);
    const GroupRun &R = runs[j];
    const int64_t mb = blockIdx.x - R.blk_mom0;
    const int d = (int)R.d, t = (int)R.round;
    const int64_t ntot = R.n_old + R.n_round;
    const double *sum = R.summaries + 3 * t;
    const double m = sum[0], inv = 1.0 / sum[1];
    const float *c = R.loc + (size_t)t * d;
    __shared__ float zt[32][65];
    __shared__ float wt[32];
    const int tri = d * (d + 1) / 2;
    constexpr int kPer = 9;  // lower-triangle entries per thread (d <= 64: 2080 / 256 < 9)
    float acc[kPer], cmp[kPer], s1 = 0.f, c1 = 0.f, s0 = 0.f, c0 = 0.f;
    int er[kPer], ec[kPer];
    for (int u = 0; u < kPer; ++u) {
        acc[u] = cmp[u] = 0.f;
        const int q = threadIdx.x + u * 256;
        int r = 0, cc = 0;
        if (q < tri) {
            r = (int)((sqrtf(8.f * (float)q + 1.f) - 1.f) * 0.5f);
            if ((r + 1) * (r + 2) / 2 <= q) ++r;
            if (r * (r + 1) / 2 > q) --r;
            cc = q - r * (r + 1) / 2;
        }
        er[u] = r;
        ec[u] = cc;
    }
    // Kahan step: sum += v with the running compensation
    auto kahan = [](float &s, float &k, float v) {
        const float y = v - k;
        const float tt = s + y;
        k = (tt - s) - y;
        s = tt;
    };
    const int64_t i0 = mb * kGMomTiles * kGTile, i1 = min(ntot, i0 + (int64_t)kGMomTiles * kGTile);
    for (int64_t s0i = i0; s0i < i1; s0i += 32) {
        const int rows = (int)min((int64_t)32, i1 - s0i);
        __syncthreads();
        for (int e = threadIdx.x; e < rows * d; e += blockDim.x) {
            const int r = e / d, cc = e - r * d;
            zt[r][cc] = R.samples[(s0i + r) * d + cc] - c[cc];
        }
        for (int r = threadIdx.x; r < rows; r += blockDim.x) {
            const double l = (double)R.logweights[s0i + r];
            wt[r] = l == -INFINITY ? 0.f : (float)(exp(l - m) * inv);
        }
        __syncthreads();
        for (int r = 0; r < rows; ++r) {
            const float w = wt[r];
            if (w == 0.f) continue;
#pragma unroll
            for (int u = 0; u < kPer; ++u)
                if (threadIdx.x + u * 256 < tri) kahan(acc[u], cmp[u], w * zt[r][er[u]] * zt[r][ec[u]]);
            if (threadIdx.x < d) kahan(s1, c1, w * zt[r][threadIdx.x]);
            if (threadIdx.x == 0) kahan(s0, c0, w);
        }
    }
    double *out = R.mpartial + (size_t)mb * kMomWords;
    if (threadIdx.x == 0) out[0] = (double)s0 - (double)c0;
    if (threadIdx.x < d) out[1 + threadIdx.x] = (double)s1 - (double)c1;
#pragma unroll
    for (int u = 0; u < kPer; ++u)
        if (threadIdx.x + u * 256 < tri) out[1 + 64 + threadIdx.x + u * 256] = (double)acc[u] - (double)cmp[u];
}

// one block per run: merge the moment partials, mean and covariance, ridge,
// FP64 Cholesky, and the next proposal (slot t + 1, or the candidate)
__global__ void __launch_bounds__(256) group_fit_kernel(const GroupRun *__restrict__ runs) {
    const GroupRun &R = runs[blockIdx.x];
    const int d = (int)R.d, t = (int)R.round;
    __shared__ double A[64][65];
    __shared__ double s1[64];
    __shared__ double s_ridge, s_s0;
    __shared__ int s_bad;
    const int tri = d * (d + 1) / 2;
    const float *c = R.loc + (size_t)t * d;
    // merged sums (fixed block order)
    for (int q = threadIdx.x; q < tri + d + 1; q += blockDim.x) {
        const int w = q < 1 ? 0 : q < 1 + d ? q : 1 + 64 + (q - 1 - d);
        double s = 0.0;
        for (int64_t b = 0; b < R.nmom; ++b) s += R.mpartial[(size_t)b * kMomWords + w];
        if (q == 0) s_s0 = s;
        else if (q < 1 + d) s1[q - 1] = s;
        else {
            const int e = q - 1 - d;
            int r = (int)((sqrtf(8.f * (float)e + 1.f) - 1.f) * 0.5f);
            if ((r + 1) * (r + 2) / 2 <= e) ++r;
            if (r * (r + 1) / 2 > e) --r;
            const int cc = e - r * (r + 1) / 2;
            A[r][cc] = s;
        }
    }
    if (threadIdx.x == 0) {
        // ridge: sqrt(eps(Float32)) tr(L_t L_t^T) / d
        double tr = 0.0;
        const float *L = R.fac + (size_t)t * d * d;
        for (int e = 0; e < d * d; ++e) tr += (double)L[e] * (double)L[e];
        s_ridge = 3.4526698300124393e-04 * tr / (double)d;
        s_bad = 0;
    }
    __syncthreads();
    const double inv0 = 1.0 / s_s0;
    for (int q = threadIdx.x; q < d; q += blockDim.x) R.mean[q] = (double)c[q] + s1[q] * inv0;
    for (int e = threadIdx.x; e < tri; e += blockDim.x) {
        int r = (int)((sqrtf(8.f * (float)e + 1.f) - 1.f) * 0.5f);
        if ((r + 1) * (r + 2) / 2 <= e) ++r;
        if (r * (r + 1) / 2 > e) --r;
        const int cc = e - r * (r + 1) / 2;
        double v = A[r][cc] * inv0 - (s1[r] * inv0) * (s1[cc] * inv0);
        R.cov[r + (size_t)cc * d] = v;
        R.cov[cc + (size_t)r * d] = v;
        if (r == cc) v += s_ridge;
        A[r][cc] = v;
    }
    __syncthreads();
    for (int jc = 0; jc < d; ++jc) {
        if (threadIdx.x == 0) {
            double piv = A[jc][jc];
            for (int q = 0; q < jc; ++q) piv -= A[jc][q] * A[jc][q];
            if (isfinite(piv) && piv > 0.0) A[jc][jc] = sqrt(piv);
            else s_bad = 1;
        }
        __syncthreads();
        if (s_bad) break;
        const double dj = A[jc][jc];
        for (int r = jc + 1 + threadIdx.x; r < d; r += blockDim.x) {
            double v = A[r][jc];
            for (int q = 0; q < jc; ++q) v -= A[r][q] * A[jc][q];
            A[r][jc] = v / dj;
        }
        __syncthreads();
    }
    __syncthreads();
    const bool last = t + 1 >= R.rounds;
    float *oloc = last ? R.cand_loc : R.loc + (size_t)(t + 1) * d;
    float *ofac = last ? R.cand_fac : R.fac + (size_t)(t + 1) * d * d;
    float *oln = last ? R.cand_lognorm : R.lognorm + (t + 1);
    if (s_bad) {
        if (threadIdx.x == 0)
            record_failure(R.failures + 3 * t, R.n_old + R.n_round + 1, 0, ISSM_REASON_MOMENT_FIT_INVALID);
        return;
    }
    for (int q = threadIdx.x; q < d; q += blockDim.x) oloc[q] = (float)R.mean[q];
    for (int e = threadIdx.x; e < d * d; e += blockDim.x) {
        const int r = e % d, cc = e / d;
        ofac[e] = r >= cc ? (float)A[r][cc] : 0.f;
    }
    if (threadIdx.x == 0) {
        // Gaussian lognormalizer of the stored FP32 factor
        double ld = 0.0;
        for (int q = 0; q < d; ++q) ld += log((double)(float)A[q][q]);
        *oln = (float)(-0.5 * (double)d * log(2.0 * 3.14159265358979323846) - ld);
    }
}

int group_step(const void *runs, int nruns, int64_t blocks_new, int64_t blocks_all, int64_t blocks_mom,
               cudaStream_t stream) {
    const GroupRun *R = (const GroupRun *)runs;
    if (blocks_new > 0) {
        group_draw_kernel<<<(unsigned)blocks_new, kGTile, 0, stream>>>(R, nruns);
        note_launch();
        group_target_kernel<<<(unsigned)blocks_new, kGTile, 0, stream>>>(R, nruns);
        note_launch();
    }
    group_mixture_kernel<<<(unsigned)blocks_all, kGTile, 0, stream>>>(R, nruns);
    note_launch();
    group_form_kernel<<<(unsigned)blocks_all, kGTile, 0, stream>>>(R, nruns);
    note_launch();
    group_summary_kernel<<<nruns, 32, 0, stream>>>(R);
    note_launch();
    group_moments_kernel<<<(unsigned)blocks_mom, 256, 0, stream>>>(R, nruns);
    note_launch();
    group_fit_kernel<<<nruns, 256, 0, stream>>>(R);
    note_launch();
    return (int)cudaGetLastError();
}

}  // namespace issm

extern "C" size_t issm_group_run_bytes(void) { return sizeof(issm_group_run); }

extern "C" int issm_group_step(const issm_group_run *runs, int32_t nruns, int64_t blocks_new, int64_t blocks_all,
                               int64_t blocks_mom, issm_stream_t stream) {
    if (nruns < 1 || blocks_all < 1 || blocks_new < 0 || blocks_mom < 1) return ISSM_E_SIZE;
    if (!runs) return ISSM_E_NULL;
    if (blocks_new > 0x7fffffff || blocks_all > 0x7fffffff || blocks_mom > 0x7fffffff) return ISSM_E_SIZE;
    return issm::group_step(runs, nruns, blocks_new, blocks_all, blocks_mom, (cudaStream_t)stream);
}
