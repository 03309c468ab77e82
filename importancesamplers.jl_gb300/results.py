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
    layout), or a dict of named (n, ...) device tensors (the reference's
    NamedTuple samples); logweights: (n,); provenance / diagnostics: dicts."""

    def __init__(self, samples, logweights, provenance=None, diagnostics=None):
        counts = [t.shape[0] for t in samples.values()] if isinstance(samples, dict) else [samples.shape[0]]
        if any(c != logweights.shape[0] for c in counts):
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


def _checked_summary(result):
    sm = result.summary()
    if float(sm[1]) == 0.0:
        raise AllZeroWeightsError()
    return sm


def _functional_values(f, result):
    """f's value for every sample, on the device: f maps the (n, d) sample
    tensor (or a dict of named (n, ...) tensors) to one number per sample
    (_device_functional_values, src/statistics.jl:15-34)."""
    v = f(result.samples)
    if not isinstance(v, torch.Tensor) or v.shape != (len(result),):
        raise ValueError("device functionals must return one concrete number per sample")
    if not v.dtype.is_floating_point:
        v = v.double()
    return v.contiguous()


def mean(result, f=None):
    """Self-normalised weighted mean (Statistics.mean(result),
    src/statistics.jl:11-16), or the weighted expectation of the scalar
    function f (mean(f, result), :18-33): one device pass, FP64 sums for FP64
    data and compensated FP32 sums merged in FP64 for FP32 data. Named (dict)
    samples give a dict of means."""
    sm = _checked_summary(result)
    if f is not None:
        v = _functional_values(f, result)
        return float(ops.weighted_sum(v, result.logweights, sm).item())
    x = result.samples
    if isinstance(x, dict):
        return {k: _mean_of(t, result.logweights, sm) for k, t in x.items()}
    return _mean_of(x, result.logweights, sm)


def _mean_of(x, lw, sm):
    if x.dim() == 1:
        return float(ops.weighted_sum(x, lw, sm).item())
    return ops.weighted_sum(x.reshape(x.shape[0], -1).contiguous(), lw, sm).reshape(x.shape[1:])


def var(result, f=None, corrected=False):
    """Uncorrected weighted variance (Statistics.var(result),
    src/statistics.jl:35-63), of the samples or of f's values;
    corrected=True is unsupported, as in the reference."""
    if corrected:
        raise ValueError("corrected moments are undefined for importance weights")
    sm = _checked_summary(result)
    x = _functional_values(f, result) if f is not None else result.samples
    mu = ops.weighted_sum(x, result.logweights, sm)
    dev = (x.double() - (mu if x.dim() == 2 else mu[0])) ** 2
    v = ops.weighted_sum(dev.contiguous(), result.logweights, sm)
    return float(v.item()) if x.dim() == 1 else v


def std(result, f=None, corrected=False):
    v = var(result, f, corrected)
    return float(np.sqrt(v)) if isinstance(v, float) else torch.sqrt(v)


def quantile(result, probabilities):
    """Component-wise weighted quantiles with the StatsBase generic-weight
    interpolation rule (Statistics.quantile, src/statistics.jl:106-154), on
    the device: a scalar probability gives (d,), a list gives (len, d); 1-D
    samples give floats. The reference requires a host result for this; here
    the device result is used as it is."""
    scalar = np.ndim(probabilities) == 0
    probs = [float(probabilities)] if scalar else [float(p) for p in probabilities]
    if not probs:
        raise ValueError("quantile probabilities cannot be empty")
    if not all(0.0 <= p <= 1.0 for p in probs):
        raise ValueError("quantile probabilities must lie in [0, 1]")
    sm = _checked_summary(result)
    x = result.samples
    if isinstance(x, dict):
        return {k: quantile(WeightedSamples(t, result.logweights), probabilities) for k, t in x.items()}
    q = ops.weighted_quantile(x.contiguous(), result.logweights, sm, probs)
    if x.dim() == 1:
        vals = q[:, 0].cpu().numpy()
        return float(vals[0]) if scalar else vals
    return q[0] if scalar else q


def median(result):
    return quantile(result, 0.5)


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
        if isinstance(self.samples, dict):
            return next(iter(self.samples.values())).shape[0]
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
    if isinstance(x, dict):  # named samples: every field gathered by the same ancestors
        return UnweightedSamples({k: _gather_rows(t, anc) for k, t in x.items()}, anc)
    return UnweightedSamples(_gather_rows(x, anc), anc)


def _gather_rows(x, anc):
    """Rows anc - 1 of an (n, ...) device tensor (_gather_resampled_samples!,
    src/resampling.jl:120-164): trailing dimensions flattened into one row of
    the gather kernel."""
    flat = x.reshape(x.shape[0], -1).contiguous()
    out = ops.gather(flat, anc)
    return out.reshape((anc.numel(),) + tuple(x.shape[1:]))
