// run.cu — one AMIS run issued from native code: every launch of every
// round, stream-ordered, no host synchronisation, in one C call. It performs
// the same sequence of library calls as the Python round loop
// (sampler.py::_moment_body), so its results are bitwise the same; the point
// is the host cost: one call instead of a dozen interpreted calls per round,
// which is what bounds a serving loop of many small runs.
//
// Reference counterpart: one AMIS round (_launch_prefilled_amis_round!,
// src/amis_execution.jl:261-357: draw, target, retrospective append, prefix
// mixture, weights and summary) followed by the moment fit
// (_fit_moment_proposal!, src/adaptive_gaussian_execution.jl:348-425), for
// every round.
#include <cmath>
#include <cstddef>
#include <cstring>

#include "issm_device.cuh"
#include "issm_internal.h"

namespace issm {

template <typename T> __global__ void to_f64_kernel(const T *__restrict__ src, int n, double *__restrict__ dst) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = (double)src[i];
}

static size_t round_up(size_t v) { return (v + 255) & ~(size_t)255; }

#define ISSM_TRY(expr)            \
    do {                          \
        int _st = (expr);         \
        if (_st != 0) return _st; \
    } while (0)

}  // namespace issm

using namespace issm;

extern "C" {

size_t issm_amis_run_desc_bytes(void) { return sizeof(issm_amis_run_desc); }
size_t issm_amis_run_desc_workspace_offset(void) { return offsetof(issm_amis_run_desc, workspace_bytes); }

size_t issm_amis_run_workspace_bytes(int32_t d, int64_t total, int32_t rounds) {
    if (d < 1 || total < 1 || rounds < 1) return 0;
    return round_up(issm_tc_workspace_bytes(rounds, d)) + round_up(issm_moments_workspace_bytes(total, d)) +
           round_up(issm_reduce_workspace_bytes(total));
}

int issm_amis_run(const issm_amis_run_desc *r, issm_stream_t stream) {
    if (!r || (!r->target && !r->target_bank) || !r->round_sizes) return ISSM_E_NULL;
    if (r->target_bank && !r->target_den) return ISSM_E_NULL;
    const issm_bank &h = r->history;
    const int d = h.dim, rounds = r->rounds;
    if (d < 1 || d > 64 || rounds < 1 || h.count < rounds) return ISSM_E_SIZE;
    if (h.family != ISSM_GAUSSIAN || h.scale_kind != ISSM_SCALE_FACTOR) return ISSM_E_UNSUPPORTED;
    if (h.dtype != ISSM_F32 && h.dtype != ISSM_F64) return ISSM_E_DTYPE;
    if (!h.locations || !h.scales || !h.lognormalizers) return ISSM_E_NULL;
    const bool tc = r->precision != ISSM_PREC_NATIVE;
    if (tc && (h.dtype != ISSM_F32 || !h.inverse_factors)) return ISSM_E_UNSUPPORTED;
    if (r->target_operand && h.dtype != ISSM_F32) return ISSM_E_DTYPE;  // the tensor-core likelihood reads FP32
    if (!r->samples || !r->logtargets || !r->lognum || !r->logweights || !r->round_ids || !r->round_ids_init ||
        !r->summaries || !r->round_failures || !r->mean || !r->cov || !r->shift || !r->cand_location ||
        !r->cand_factor || !r->cand_lognormalizer || !r->initial_location || !r->initial_factor ||
        !r->initial_lognormalizer || !r->logcounts || !r->workspace)
        return ISSM_E_NULL;
    int64_t total = 0;
    for (int t = 0; t < rounds; ++t) {
        if (r->round_sizes[t] < 1) return ISSM_E_SIZE;
        total += r->round_sizes[t];
    }
    if (r->workspace_bytes < issm_amis_run_workspace_bytes(d, total, rounds)) return ISSM_E_WORKSPACE;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t es = h.dtype == ISSM_F32 ? 4 : 8;
    const int dp = d <= 16 ? 16 : d <= 32 ? 32 : 64;
    char *ws = (char *)r->workspace;
    const size_t tc_bytes = round_up(issm_tc_workspace_bytes(rounds, d));
    const size_t mom_bytes = round_up(issm_moments_workspace_bytes(total, d));
    const size_t red_bytes = round_up(issm_reduce_workspace_bytes(total));
    char *ws_tc = ws, *ws_mom = ws + tc_bytes, *ws_red = ws + tc_bytes + mom_bytes;
    char *samples = (char *)r->samples, *logtargets = (char *)r->logtargets, *lognum = (char *)r->lognum;
    char *loc = (char *)h.locations, *fac = (char *)h.scales, *lnorm = (char *)h.lognormalizers;
    uint64_t *fail_all = (uint64_t *)r->round_failures;

    // scratch reset: the sticky timeout words and last-block counters sit at
    // offsets that depend on (rounds, d, total), so a workspace reused by
    // runs of another shape must not keep the earlier run's bytes there
    ISSM_TRY((int)cudaMemsetAsync(ws, 0, tc_bytes + mom_bytes + red_bytes, s));
    // slot 0 <- the committed proposal; state reset
    ISSM_TRY((int)cudaMemcpyAsync(loc, r->initial_location, d * es, cudaMemcpyDeviceToDevice, s));
    ISSM_TRY((int)cudaMemcpyAsync(fac, r->initial_factor, (size_t)d * d * es, cudaMemcpyDeviceToDevice, s));
    ISSM_TRY((int)cudaMemcpyAsync(lnorm, r->initial_lognormalizer, es, cudaMemcpyDeviceToDevice, s));
    if (tc) ISSM_TRY(issm_invert_factors(&h, 0, 1, (float *)h.inverse_factors, stream));
    ISSM_TRY((int)cudaMemsetAsync(fail_all, 0, sizeof(uint64_t) * 3 * rounds, s));
    ISSM_TRY((int)cudaMemcpyAsync(r->round_ids, r->round_ids_init, sizeof(int64_t) * total, cudaMemcpyDeviceToDevice,
                                  s));
    uint64_t offset = r->normal_offset;
    int64_t n_old = 0;
    for (int t = 0; t < rounds; ++t) {
        const int64_t n_new = r->round_sizes[t], n_tot = n_old + n_new;
        uint64_t *fail = fail_all + 3 * t;
        issm_bank view = h;
        view.count = t + 1;
        char *x_new = samples + (size_t)n_old * d * es;
        // draw (normals generated in the kernel) and target
        ISSM_TRY(issm_draw_philox(&view, t, r->seed, r->counter, offset, nullptr, 0, nullptr, 0, n_new, x_new, fail, 0,
                                  stream));
        offset += (uint64_t)n_new * d + 8;
        if (r->target_bank) {  // a radial-mixture target: the proposals' density kernels
            if (r->target_bank_precision != ISSM_PREC_NATIVE)
                ISSM_TRY(issm_mixture_logdensity_ws(r->target_bank, r->target_den, x_new, n_new, nullptr, 0,
                                                    logtargets + (size_t)n_old * es, nullptr, nullptr, 0,
                                                    r->target_bank_precision, ws_tc, tc_bytes, stream));
            else
                ISSM_TRY(issm_mixture_logdensity(r->target_bank, r->target_den, x_new, n_new, nullptr, 0,
                                                 logtargets + (size_t)n_old * es, nullptr, nullptr, 0,
                                                 ISSM_PREC_NATIVE, stream));
        } else if (r->target_operand)  // X beta on the tensor cores, the likelihood in the epilogue
            ISSM_TRY(issm_glm_logdensity(r->target, r->target_precision, r->target_operand, (const float *)x_new, n_new,
                                         (float *)(logtargets + (size_t)n_old * es),
                                         (int32_t *)(ws_tc + tc_bytes - 64), stream));
        else
            ISSM_TRY(issm_target_logdensity(r->target, x_new, n_new, logtargets + (size_t)n_old * es, stream));
        ISSM_TRY(issm_check_target_values(logtargets + (size_t)n_old * es, n_new, h.dtype, r->round_ids + n_old, fail,
                                          0, stream));
        // retrospective append over the retained samples, then the prefix mixture of the new ones
        if (n_old > 0) {
            if (tc)
                ISSM_TRY(issm_amis_append_ws(&view, t, r->logcounts, samples, n_old, lognum, fail, r->precision, ws_tc,
                                             tc_bytes, stream));
            else
                ISSM_TRY(issm_amis_append(&view, t, r->logcounts, samples, n_old, lognum, fail, r->precision, stream));
        }
        const issm_denominator den{ISSM_DENOM_PREFIX, t + 1, r->logcounts, nullptr};
        if (tc)
            ISSM_TRY(issm_mixture_logdensity_ws(&view, &den, x_new, n_new, nullptr, t, lognum + (size_t)n_old * es,
                                                nullptr, fail, 0, r->precision, ws_tc, tc_bytes, stream));
        else
            ISSM_TRY(issm_mixture_logdensity(&view, &den, x_new, n_new, nullptr, t, lognum + (size_t)n_old * es, nullptr,
                                             fail, 0, r->precision, stream));
        double *summary = r->summaries + 3 * t;
        ISSM_TRY(issm_amis_form_summary(logtargets, lognum, r->round_ids, std::log((double)n_tot), n_tot, h.dtype,
                                        r->logweights, fail, summary, ws_red, red_bytes, stream));
        // moments about the previous location, then the FP64 fit into slot t + 1 (or the candidate)
        if (h.dtype == ISSM_F32) {
            to_f64_kernel<float><<<1, 64, 0, s>>>((const float *)(loc + (size_t)t * d * es), d, r->shift);
        } else {
            to_f64_kernel<double><<<1, 64, 0, s>>>((const double *)(loc + (size_t)t * d * es), d, r->shift);
        }
        note_launch();
        ISSM_TRY((int)cudaGetLastError());
        const void *prev = fac + (size_t)t * d * d * es;
        ISSM_TRY(issm_weighted_moments_ws(samples, d, n_tot, r->logweights, h.dtype, summary, r->shift,
                                          h.dtype == ISSM_F32 ? prev : nullptr, r->mean, r->cov, r->precision, ws_mom,
                                          mom_bytes, stream));
        const bool last = t + 1 == rounds;
        void *out_loc = last ? r->cand_location : (void *)(loc + (size_t)(t + 1) * d * es);
        void *out_fac = last ? r->cand_factor : (void *)(fac + (size_t)(t + 1) * d * d * es);
        void *out_ln = last ? r->cand_lognormalizer : (void *)(lnorm + (size_t)(t + 1) * es);
        float *out_inv = (!last && tc) ? (float *)h.inverse_factors + (size_t)(t + 1) * dp * dp : nullptr;
        ISSM_TRY(issm_fit_factor_ex(r->mean, r->cov, d, prev, 0.0, r->logconstant, h.dtype, out_loc, out_fac, out_ln,
                                    out_inv, fail, n_tot + 1, stream));
        n_old = n_tot;
    }
    if (r->counter) ISSM_TRY(issm_counter_advance(r->counter, offset - r->normal_offset, stream));
    return ISSM_OK;
}

}  // extern "C"
