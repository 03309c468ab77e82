"""Tensor-level wrappers over the C ABI: each function takes torch CUDA
tensors, checks shapes, and calls one libissm103.so entry point on the current
stream. Results stay on the device."""
import ctypes

import torch

from . import native

_U = native


def _dt(t):
    return native.dtype_code(t.dtype)


def _s(stream=None):
    return native.stream_ptr(stream)


def new_failures(device):
    return torch.zeros(3, dtype=torch.int64, device=device)


def denominator(kind, coef=None, terms=0, groups=None):
    d = native.Denominator(kind, int(terms), native.ptr(coef), native.ptr(groups))
    d._keep = (coef, groups)
    return d


def fill_normals(n, dtype, device, seed, offset=0, out=None):
    out = torch.empty(int(n), dtype=dtype, device=device) if out is None else out
    native.call("issm_fill_normals", int(seed) & (2 ** 64 - 1), int(offset), int(n), native.ptr(out),
                native.dtype_code(dtype), _s())
    return out


def fill_uniforms(n, dtype, device, seed, offset=0, out=None):
    out = torch.empty(int(n), dtype=dtype, device=device) if out is None else out
    native.call("issm_fill_uniforms", int(seed) & (2 ** 64 - 1), int(offset), int(n), native.ptr(out),
                native.dtype_code(dtype), _s())
    return out


def fill_normals_at(n, dtype, device, seed, counter, offset=0, out=None):
    """Normals at Philox offset counter[0] + offset, with the counter read on
    the device when the kernel runs (graph replays see the advanced value)."""
    out = torch.empty(int(n), dtype=dtype, device=device) if out is None else out
    native.call("issm_fill_normals_at", int(seed) & (2 ** 64 - 1), native.ptr(counter), int(offset), int(n),
                native.ptr(out), native.dtype_code(dtype), _s())
    return out


def fill_uniforms_at(n, dtype, device, seed, counter, offset=0, out=None):
    out = torch.empty(int(n), dtype=dtype, device=device) if out is None else out
    native.call("issm_fill_uniforms_at", int(seed) & (2 ** 64 - 1), native.ptr(counter), int(offset), int(n),
                native.ptr(out), native.dtype_code(dtype), _s())
    return out


def counter_advance(counter, increment):
    native.call("issm_counter_advance", native.ptr(counter), int(increment), _s())


def static_assign(cdf, uniforms, stratified=True, out=None):
    n = uniforms.numel()
    out = torch.empty(n, dtype=torch.int32, device=uniforms.device) if out is None else out
    native.call("issm_static_assign", native.ptr(cdf), cdf.numel(), native.ptr(uniforms), n, int(stratified),
                native.ptr(out), _dt(cdf), _s())
    return out


def draw(bank, normals, n, slots=None, fixed_slot=0, radial_normals=None, rn_stride=0, radial_uniforms=None,
         ru_stride=0, failures=None, index_base=0, out=None, bank_ref=None):
    out = torch.empty(int(n), bank.d, dtype=bank.dtype, device=normals.device) if out is None else out
    native.call("issm_draw", bank_ref or bank.ref(), native.ptr(slots), int(fixed_slot), native.ptr(normals),
                native.ptr(radial_normals), int(rn_stride), native.ptr(radial_uniforms), int(ru_stride), int(n),
                native.ptr(out), native.ptr(failures), int(index_base), _s())
    return out


def draw_philox(bank, n, seed, counter=None, offset=0, fixed_slot=0, radial_normals=None, rn_stride=0,
                radial_uniforms=None, ru_stride=0, failures=None, index_base=0, out=None, bank_ref=None):
    """draw() from a factor bank with the standard normals generated in the
    kernel: element offset (+ counter[0]) + i d + e of the `seed` normal
    stream (fill_normals_at) for row i, coordinate e. Bitwise equal to
    fill_normals_at followed by draw()."""
    out = torch.empty(int(n), bank.d, dtype=bank.dtype, device=bank.locations.device) if out is None else out
    native.call("issm_draw_philox", bank_ref or bank.ref(), int(fixed_slot), int(seed) & (2 ** 64 - 1),
                native.ptr(counter), int(offset), native.ptr(radial_normals), int(rn_stride),
                native.ptr(radial_uniforms), int(ru_stride), int(n), native.ptr(out), native.ptr(failures),
                int(index_base), _s())
    return out


def _tc_workspace(count, d, device):
    nb = native.lib().issm_tc_workspace_bytes(int(count), int(d))
    # the error word sits in the last 64 bytes of whatever buffer is passed: size it exactly
    buf = native.workspace(max(nb, 1 << 20), device, "tc", zero=True)
    return buf


def mixture_logdensity(bank, den, x, slots=None, fixed_slot=0, failures=None, generating=False, index_base=0,
                       precision=native.PREC_NATIVE, out=None, bank_ref=None):
    n = x.shape[0]
    out = torch.empty(n, dtype=bank.dtype, device=x.device) if out is None else out
    gen = torch.empty(n, dtype=bank.dtype, device=x.device) if generating else None
    if precision == native.PREC_NATIVE:
        native.call("issm_mixture_logdensity", bank_ref or bank.ref(), ctypes.byref(den), native.ptr(x), n,
                    native.ptr(slots), int(fixed_slot), native.ptr(out), native.ptr(gen), native.ptr(failures),
                    int(index_base), int(precision), _s())
    else:
        ws = _tc_workspace(bank.count, bank.d, x.device)
        native.call("issm_mixture_logdensity_ws", bank_ref or bank.ref(), ctypes.byref(den), native.ptr(x), n,
                    native.ptr(slots), int(fixed_slot), native.ptr(out), native.ptr(gen), native.ptr(failures),
                    int(index_base), int(precision), native.ptr(ws), ws.numel(), _s())
    return (out, gen) if generating else out


def mis_round(bank, den, slots, normals, logtargets=None, radial_normals=None, rn_stride=0, radial_uniforms=None,
              ru_stride=0, failures=None, precision=native.PREC_NATIVE, samples=None, logweights=None,
              proposal_ids_out=None):
    n = slots.numel()
    dev = slots.device
    samples = torch.empty(n, bank.d, dtype=bank.dtype, device=dev) if samples is None else samples
    logweights = torch.empty(n, dtype=bank.dtype, device=dev) if logweights is None else logweights
    pid = torch.empty(n, dtype=torch.int64, device=dev) if proposal_ids_out is None else proposal_ids_out
    native.call("issm_mis_round", bank.ref(), ctypes.byref(den), native.ptr(slots), native.ptr(normals),
                native.ptr(radial_normals), int(rn_stride), native.ptr(radial_uniforms), int(ru_stride),
                native.ptr(logtargets), n, native.ptr(samples), native.ptr(logweights),
                native.ptr(bank.proposal_ids), native.ptr(pid), native.ptr(failures), int(precision), _s())
    return samples, logweights, pid


def add_target_values(logweights, values, failures=None, index_base=0):
    native.call("issm_add_target_values", native.ptr(logweights), native.ptr(values), logweights.numel(),
                _dt(logweights), native.ptr(failures), int(index_base), _s())
    return logweights


def check_target_values(values, round_ids=None, failures=None, index_base=0):
    native.call("issm_check_target_values", native.ptr(values), values.numel(), _dt(values), native.ptr(round_ids),
                native.ptr(failures), int(index_base), _s())


def subtract_logweights(logtargets, logden, failures=None, index_base=0, out=None):
    out = torch.empty_like(logtargets) if out is None else out
    native.call("issm_subtract_logweights", native.ptr(logtargets), native.ptr(logden), logtargets.numel(),
                _dt(logtargets), native.ptr(out), native.ptr(failures), int(index_base), _s())
    return out


def amis_append(history_ref, slot, logcounts, x, lognum, failures=None, precision=native.PREC_NATIVE, count=None):
    if precision == native.PREC_NATIVE:
        native.call("issm_amis_append", history_ref, int(slot), native.ptr(logcounts), native.ptr(x), x.shape[0],
                    native.ptr(lognum), native.ptr(failures), int(precision), _s())
    else:
        ws = _tc_workspace(count or (int(slot) + 1), x.shape[1], x.device)
        native.call("issm_amis_append_ws", history_ref, int(slot), native.ptr(logcounts), native.ptr(x),
                    x.shape[0], native.ptr(lognum), native.ptr(failures), int(precision), native.ptr(ws), ws.numel(),
                    _s())
    return lognum


def amis_form(logtargets, lognum, logtotal, logweights, round_ids=None, failures=None):
    native.call("issm_amis_form", native.ptr(logtargets), native.ptr(lognum), native.ptr(round_ids),
                float(logtotal), logtargets.numel(), _dt(logtargets), native.ptr(logweights), native.ptr(failures),
                _s())
    return logweights


def amis_form_summary(logtargets, lognum, logtotal, logweights, out, round_ids=None, failures=None):
    """amis_form and logweight_summary in one pass (summary of the weights written)."""
    n = logtargets.numel()
    nb = native.lib().issm_reduce_workspace_bytes(n)
    ws = native.workspace(nb, logtargets.device, "reduce")
    native.call("issm_amis_form_summary", native.ptr(logtargets), native.ptr(lognum), native.ptr(round_ids),
                float(logtotal), n, _dt(logtargets), native.ptr(logweights), native.ptr(failures), native.ptr(out),
                native.ptr(ws), ws.numel(), _s())
    return out


def logweight_summary(logweights, out=None):
    n = logweights.numel()
    out = torch.empty(3, dtype=torch.float64, device=logweights.device) if out is None else out
    nb = native.lib().issm_reduce_workspace_bytes(n)
    ws = native.workspace(nb, logweights.device, "reduce")
    native.call("issm_logweight_summary", native.ptr(logweights), n, _dt(logweights), native.ptr(out),
                native.ptr(ws), ws.numel(), _s())
    return out


def normalize(logweights, summary, out=None):
    out = torch.empty_like(logweights) if out is None else out
    native.call("issm_normalize", native.ptr(logweights), logweights.numel(), _dt(logweights), native.ptr(summary),
                native.ptr(out), _s())
    return out


def resampling_cdf(logweights, out=None):
    n = logweights.numel()
    out = torch.empty_like(logweights) if out is None else out
    nb = native.lib().issm_reduce_workspace_bytes(n)
    ws = native.workspace(nb, logweights.device, "cdf")
    native.call("issm_resampling_cdf", native.ptr(logweights), n, _dt(logweights), native.ptr(out), native.ptr(ws),
                ws.numel(), _s())
    return out


def resample_select(cdf, logweights, uniforms, out=None):
    count = uniforms.numel()
    out = torch.empty(count, dtype=torch.int64, device=cdf.device) if out is None else out
    native.call("issm_resample_select", native.ptr(cdf), native.ptr(logweights), cdf.numel(), native.ptr(uniforms),
                count, _dt(cdf), native.ptr(out), _s())
    return out


def resample_multinomial(logweights, uniforms, out=None):
    n = logweights.numel()
    count = uniforms.numel()
    out = torch.empty(count, dtype=torch.int64, device=logweights.device) if out is None else out
    nb = native.lib().issm_resample_workspace_bytes(n)
    ws = native.workspace(nb, logweights.device, "resample")
    native.call("issm_resample_multinomial", native.ptr(logweights), n, _dt(logweights), native.ptr(uniforms),
                count, native.ptr(out), native.ptr(ws), ws.numel(), _s())
    return out


def resample_systematic(logweights, u, count, out=None):
    n = logweights.numel()
    out = torch.empty(int(count), dtype=torch.int64, device=logweights.device) if out is None else out
    nb = native.lib().issm_resample_workspace_bytes(n)
    ws = native.workspace(nb, logweights.device, "resample")
    native.call("issm_resample_systematic", native.ptr(logweights), n, _dt(logweights), float(u), int(count),
                native.ptr(out), native.ptr(ws), ws.numel(), _s())
    return out


def gather(src, ancestors, out=None):
    d = src.shape[1] if src.dim() == 2 else 1
    count = ancestors.numel()
    shape = (count, d) if src.dim() == 2 else (count,)
    out = torch.empty(shape, dtype=src.dtype, device=src.device) if out is None else out
    native.call("issm_gather", native.ptr(src), d, src.shape[0], native.ptr(ancestors), count, _dt(src),
                native.ptr(out), _s())
    return out


def local_resample(logweights, counts, uniforms, samples=None, ancestors=None, destination=None):
    k = counts.numel()
    d = samples.shape[1] if samples is not None else 1
    anc = torch.empty(k, dtype=torch.int64, device=logweights.device) if ancestors is None else ancestors
    if samples is not None and destination is None:
        destination = torch.empty(k, d, dtype=samples.dtype, device=samples.device)
    native.call("issm_local_resample", native.ptr(logweights), native.ptr(counts), k, native.ptr(uniforms),
                native.ptr(samples), d, _dt(logweights), native.ptr(anc), native.ptr(destination), _s())
    return anc, destination


def weighted_moments(x, logweights, summary, shift, mean=None, cov=None, precision=native.PREC_NATIVE,
                     prev_factor=None):
    n, d = x.shape
    dev = x.device
    mean = torch.empty(d, dtype=torch.float64, device=dev) if mean is None else mean
    cov = torch.empty(d, d, dtype=torch.float64, device=dev) if cov is None else cov
    nb = native.lib().issm_moments_workspace_bytes(n, d)
    ws = native.workspace(nb, dev, "moments", zero=True)
    native.call("issm_weighted_moments_ws", native.ptr(x), d, n, native.ptr(logweights), _dt(x),
                native.ptr(summary), native.ptr(shift), native.ptr(prev_factor), native.ptr(mean), native.ptr(cov),
                int(precision),
                native.ptr(ws), ws.numel(), _s())
    return mean, cov


def fit_factor(mean, cov, previous_factor, out_location, out_factor, out_lognorm, dof=0.0, logconstant=0.0,
               failures=None, failure_index=0, out_inverse=None, regularization=None):
    """FP64 ridge + Cholesky fit into a history slot. regularization=None
    keeps the reference's sqrt(eps(T)) of the factor type."""
    d = mean.numel()
    reg = -1.0 if regularization is None else float(regularization)
    native.call("issm_fit_factor_reg", native.ptr(mean), native.ptr(cov), d, native.ptr(previous_factor), float(dof),
                float(logconstant), _dt(out_factor), reg, native.ptr(out_location), native.ptr(out_factor),
                native.ptr(out_lognorm), native.ptr(out_inverse), native.ptr(failures), int(failure_index), _s())


def _same_dtype(x, logweights):
    """The statistics kernels read the values and the log weights in one
    type: when they differ, both are read in FP64."""
    if x.dtype != logweights.dtype:
        x, logweights = x.double(), logweights.double()
    return x.contiguous(), logweights.contiguous()


def weighted_sum(x, logweights, summary, out=None):
    """sum_i w_i x_i per column (FP64) with the self-normalised weights of
    the summary; x is (n,) or (n, d)."""
    x, logweights = _same_dtype(x, logweights)
    n = x.shape[0]
    d = x.shape[1] if x.dim() == 2 else 1
    out = torch.empty(d, dtype=torch.float64, device=x.device) if out is None else out
    nb = native.lib().issm_weighted_sum_workspace_bytes(n, d)
    ws = native.workspace(nb, x.device, "wsum")
    native.call("issm_weighted_sum", native.ptr(x), d, n, native.ptr(logweights), _dt(x), native.ptr(summary),
                native.ptr(out), native.ptr(ws), ws.numel(), _s())
    return out


def weighted_quantile(x, logweights, summary, probabilities):
    """Component-wise weighted quantiles: (len(probabilities), d) FP64."""
    x, logweights = _same_dtype(x, logweights)
    n = x.shape[0]
    d = x.shape[1] if x.dim() == 2 else 1
    probs = torch.tensor([float(p) for p in probabilities], dtype=torch.float64, device=x.device)
    out = torch.empty(probs.numel(), d, dtype=torch.float64, device=x.device)
    nb = native.lib().issm_weighted_quantile_workspace_bytes(d, probs.numel())
    ws = native.workspace(nb, x.device, "quantile")
    native.call("issm_weighted_quantile", native.ptr(x), d, n, native.ptr(logweights), _dt(x), native.ptr(summary),
                native.ptr(probs), probs.numel(), native.ptr(out), native.ptr(ws), ws.numel(), _s())
    return out


def glm_operand(target_struct, precision, device):
    """The observations' tensor-core operand form of a LINREG / LOGISTIC
    target (built once per target and precision)."""
    nb = native.lib().issm_glm_operand_bytes(target_struct.count, target_struct.dim, int(precision))
    ops_buf = torch.empty(max(int(nb), 16), dtype=torch.uint8, device=device)
    native.call("issm_glm_prepare", ctypes.byref(target_struct), int(precision), native.ptr(ops_buf),
                ops_buf.numel(), _s())
    return ops_buf


def glm_logdensity(target_struct, precision, operand, x, out=None):
    """Regression log target of n FP32 samples: X beta on the tensor cores
    with the likelihood reduced in the epilogue."""
    n = x.shape[0]
    out = torch.empty(n, dtype=torch.float32, device=x.device) if out is None else out
    err = native.workspace(64, x.device, "glm", zero=True)
    native.call("issm_glm_logdensity", ctypes.byref(target_struct), int(precision), native.ptr(operand),
                native.ptr(x), n, native.ptr(out), native.ptr(err), _s())
    return out


def select_kth(values, k, out=None):
    """The k-th smallest (1-based) of `values` into a device scalar (NaN last)."""
    out = torch.empty(1, dtype=values.dtype, device=values.device) if out is None else out
    ws = native.workspace(native.lib().issm_select_workspace_bytes(), values.device, "select")
    native.call("issm_select_kth", native.ptr(values), values.numel(), int(k), _dt(values), native.ptr(out),
                native.ptr(ws), ws.numel(), _s())
    return out


def npmc_clip(raw, out=None, threshold=None):
    """min(raw, (n - isqrt(n) + 1)-th smallest of raw), on the device."""
    out = torch.empty_like(raw) if out is None else out
    threshold = torch.empty(1, dtype=raw.dtype, device=raw.device) if threshold is None else threshold
    ws = native.workspace(native.lib().issm_select_workspace_bytes(), raw.device, "select")
    native.call("issm_npmc_clip", native.ptr(raw), raw.numel(), _dt(raw), native.ptr(out), native.ptr(threshold),
                native.ptr(ws), ws.numel(), _s())
    return out, threshold


def population_local_weights(local_logweights, starts, counts, thresholds, samples=None, tolerance=1e-6,
                             max_iterations=60, raw_means=True):
    """Per-slot normalised weights, local ESS, tempering power and status of a
    population whose slot k owns samples starts[k] .. starts[k] + counts[k] - 1
    (device int64 tensors; thresholds a device float64 tensor), and the
    untempered weighted raw means (d x K as (K, d)) when `samples` is given."""
    k = starts.numel()
    dev, dt = local_logweights.device, local_logweights.dtype
    weights = torch.zeros_like(local_logweights)
    ess = torch.zeros(k, dtype=dt, device=dev)
    powers = torch.zeros(k, dtype=dt, device=dev)
    status = torch.zeros(k, dtype=torch.uint8, device=dev)
    d = samples.shape[1] if samples is not None else 1
    means = torch.zeros(k, d, dtype=dt, device=dev) if (raw_means and samples is not None) else None
    native.call("issm_population_local_weights", native.ptr(local_logweights), native.ptr(samples), d, _dt(weights),
                native.ptr(starts), native.ptr(counts), native.ptr(thresholds), k, float(tolerance),
                int(max_iterations), native.ptr(weights), native.ptr(ess), native.ptr(powers), native.ptr(status),
                native.ptr(means), _s())
    return weights, ess, powers, status, means


def population_covariances(samples, weights, powers, status, bank, starts, counts):
    """Per-slot centres (K, d) and covariances (K, d, d) (symmetric, so the
    column-major d x d x K layout reads the same)."""
    k = starts.numel()
    n, d = samples.shape
    centres = torch.empty(k, d, dtype=samples.dtype, device=samples.device)
    covs = torch.empty(k, d, d, dtype=samples.dtype, device=samples.device)
    native.call("issm_population_covariances", native.ptr(samples), d, _dt(samples), native.ptr(weights),
                native.ptr(powers), native.ptr(status), native.ptr(bank.locations), bank.ref(), native.ptr(starts),
                native.ptr(counts), k, native.ptr(centres), native.ptr(covs), _s())
    return centres, covs


def population_factors(covariances, status, dofs=None):
    """Lower Cholesky factors of the ready slots (column-major: element
    (r, c) of slot k at factors[k].reshape(-1)[r + c d]) and potrf's info per
    slot; Student-t scaling when `dofs` is given."""
    k, d, _ = covariances.shape
    factors = torch.zeros_like(covariances)
    info = torch.zeros(k, dtype=torch.int32, device=covariances.device)
    native.call("issm_population_factors", native.ptr(covariances), d, k, _dt(covariances), native.ptr(status),
                native.ptr(dofs), native.ptr(factors), native.ptr(info), _s())
    return factors, info


def target_logdensity(target_struct, x, out=None):
    n = x.shape[0]
    out = torch.empty(n, dtype=x.dtype, device=x.device) if out is None else out
    native.call("issm_target_logdensity", ctypes.byref(target_struct), native.ptr(x), n, native.ptr(out), _s())
    return out


def check_tensor_core_errors(device):
    """Raise if a tensor-core kernel reported a timed-out completion wait (the
    sticky words at the end of the tc and moments workspaces)."""
    for tag in ("tc", "moments"):
        buf = native.scoped_workspace(device, tag)
        if buf is not None and int(buf[-64:-60].view(torch.int32).item()) != 0:
            raise RuntimeError(f"a tensor-core kernel ({tag}) timed out waiting for MMA completion")


def decode_failure(words):
    """_decode_native_failure (src/execution.jl:701-717) on the 3-word record."""
    w = [int(v) & (2 ** 64 - 1) for v in words]

    def dec(count, packed):
        if count == 0:
            return dict(count=0, first_logical_index=0, first_block=0, reason_bits=0)
        inv_index = (packed >> 32) & 0xFFFFFFFF
        inv_block = (packed >> 16) & 0xFFFF
        return dict(count=count, first_logical_index=(0xFFFFFFFF - inv_index + 1) & 0xFFFFFFFF,
                    first_block=(0xFFFF - inv_block + 1) & 0xFFFF, reason_bits=packed & 0xFFFF)

    return dec(w[0], w[1]), dec(1 if w[2] else 0, w[2])
