"""WeightedSamples and its statistics (src/results.jl, src/statistics.jl,
src/resampling.jl). Results stay on the device; reductions transfer only
their few FP64 summary words."""
import numpy as np
import torch

from . import native, ops
from .methods import MultinomialResampling, SystematicResampling


class AllZeroWeightsError(Exception):
    """Every raw log weight is -Inf (src/results.jl:133-144)."""

    def __str__(self):
        return "normalized weights are undefined because all raw weights are zero"


class SamplerExecutionError(Exception):
    """A sample-level failure decoded from the device failure record
    (src/native_execution.jl:832-882)."""

    def __init__(self, phase, index, reason_bits, count):
        self.phase, self.index, self.reason_bits, self.count = phase, index, reason_bits, count
        super().__init__(f"sampler failed during {phase} at sample {index} (reason 0x{reason_bits:04x}, "
                         f"{count} failures)")


class RoundError(Exception):
    def __init__(self, method, rnd, phase, cause, diagnostics=None):
        self.round, self.phase, self.cause, self.diagnostics = rnd, phase, cause, diagnostics or {}
        super().__init__(f"{method} failed in round {rnd} during {phase}: {cause}")


class AMISRoundError(RoundError):
    def __init__(self, *a, **k):
        super().__init__("AMIS", *a, **k)


class DMPMCRoundError(RoundError):
    def __init__(self, *a, **k):
        super().__init__("DM-PMC", *a, **k)


class NPMCRoundError(RoundError):
    def __init__(self, *a, **k):
        super().__init__("NPMC", *a, **k)


def phase_of(reason_bits):
    if reason_bits & (native.REASON_TARGET_NAN | native.REASON_TARGET_POS_INF):
        return "target"
    if reason_bits & (native.REASON_GENERATED_NONFINITE | native.REASON_DRAW_EXHAUSTED):
        return "proposal_draw"
    if reason_bits & native.REASON_PROPOSAL_INVALID:
        return "proposal_logdensity"
    if reason_bits & native.REASON_LOGWEIGHT_INVALID:
        return "logweight"
    if reason_bits & native.REASON_MOMENT_FIT_INVALID:
        return "factorization"
    return "unknown"


class WeightedSamples:
    """samples: (n, d) device tensor (the reference's d x n column-major
    layout), logweights: (n,), provenance / diagnostics: dicts."""

    def __init__(self, samples, logweights, provenance=None, diagnostics=None):
        if samples.shape[0] != logweights.shape[0]:
            raise ValueError("sample and weight counts must match")
        self.samples = samples
        self.logweights = logweights
        self.provenance = provenance or {}
        self.diagnostics = diagnostics or {}
        self._summary = None

    def __len__(self):
        return self.logweights.shape[0]

    def summary(self):
        if self._summary is None:
            self._summary = ops.logweight_summary(self.logweights)
        return self._summary

    def summary_host(self):
        return self.summary().cpu().numpy()


def _ess_logz(sm, n):
    m, s, s2 = (float(v) for v in sm)
    if s == 0.0:
        return 0.0, -np.inf
    return s * s / s2, m + np.log(s) - np.log(float(n))


def lognormalizer(result):
    """logsumexp(logweights) - log n (src/results.jl:560-567)."""
    return _ess_logz(result.summary_host(), len(result))[1]


def effective_sample_size(result):
    """(sum w)^2 / sum w^2 (src/execution.jl:175-186)."""
    return _ess_logz(result.summary_host(), len(result))[0]


def normalized_weights(result):
    """exp(l - max) / S on the device (src/results.jl:589-598)."""
    sm = result.summary()
    if float(sm[1]) == 0.0:
        raise AllZeroWeightsError()
    return ops.normalize(result.logweights, sm)


def mean(result):
    w = normalized_weights(result)
    x = result.samples
    if x.dim() == 1:
        return float(torch.dot(w.double(), x.double()))
    return (w.double()[None, :] @ x.double()).reshape(-1)


def var(result):
    w = normalized_weights(result).double()
    x = result.samples.double()
    mu = mean(result)
    return ((x - mu) ** 2 * (w[:, None] if x.dim() == 2 else w)).sum(0)


def cov(result):
    """Weighted covariance through the native two-pass moment kernel."""
    x = result.samples
    if x.dim() != 2:
        raise ValueError("covariance requires vector-valued samples")
    sm = result.summary()
    if float(sm[1]) == 0.0:
        raise AllZeroWeightsError()
    shift = torch.zeros(x.shape[1], dtype=torch.float64, device=x.device)
    _, c = ops.weighted_moments(x, result.logweights, sm, shift)
    return c


class UnweightedSamples:
    def __init__(self, samples, ancestors=None):
        self.samples = samples
        self.ancestors = ancestors

    def __len__(self):
        return self.samples.shape[0]


def resample(seed, result, count=None, method=None, cdf="exact"):
    """resample(rng, result, count; method) (src/resampling.jl:245-283).

    Multinomial draws `count` device uniforms from the seed; systematic draws
    one, u_i = (i + u) / count.

    cdf="exact" (default) selects on the exact 64-bit fixed-point CDF: the
    ancestors depend only on the weights and uniforms, bit-identical on any
    device and in any scan order. cdf="reference" builds the CDF the way the
    reference does, cumsum(exp(l - max)) / total in the weights' type
    (_resampling_cdf!, src/resampling.jl:199-225), and selects with its
    strict-< search and -Inf plateau repair (:92-118). The two rules pick
    different ancestors only for a uniform within the reference CDF's
    rounding of a boundary."""
    count = len(result) if count is None else int(count)
    if count <= 0:
        raise ValueError("resampling count must be positive")
    if cdf not in ("exact", "reference"):
        raise ValueError('cdf must be "exact" or "reference"')
    method = method or MultinomialResampling()
    sm = result.summary()
    if float(sm[1]) == 0.0:
        raise AllZeroWeightsError()
    dev = result.logweights.device
    lw = result.logweights
    if isinstance(method, SystematicResampling):
        u = float(ops.fill_uniforms(1, torch.float64, dev, seed).item())
        if cdf == "exact":
            anc = ops.resample_systematic(lw, u, count)
        else:
            grid = (torch.arange(count, dtype=torch.float64, device=dev) + u) / count
            anc = ops.resample_select(ops.resampling_cdf(lw), lw, grid.to(lw.dtype))
    elif isinstance(method, MultinomialResampling):
        u = ops.fill_uniforms(count, torch.float64, dev, seed)
        if cdf == "exact":
            anc = ops.resample_multinomial(lw, u)
        else:
            anc = ops.resample_select(ops.resampling_cdf(lw), lw, u.to(lw.dtype))
    else:
        raise TypeError("unknown resampling method")
    x = result.samples
    out = ops.gather(x if x.dim() == 2 else x.reshape(-1, 1), anc)
    if x.dim() == 1:
        out = out.reshape(-1)
    return UnweightedSamples(out, anc)
