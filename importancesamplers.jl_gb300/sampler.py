"""prepare_sampler / importance_sample! / importance_sample
(src/methods/importance_sampling.jl:357-440, 857-935).

A prepared sampler owns every device buffer of its method, its counter-based
random stream and per-round failure records. A whole call is a host-driven
sequence of stream-ordered launches with no synchronisation until the end,
where the per-round summaries and failure words are read back in one copy.
The reference instead synchronises after nearly every launch
(src/mis_execution.jl:840) and reads scalars every round.
"""
import ctypes
import math
from fractions import Fraction

import numpy as np
import torch

from . import native, ops
from .bank import DeviceHistory, pack
from .methods import (AMIS, NPMC, DeterministicMixturePMC, ImportanceSampling, LocalResampling,
                      PartialDeterministicMixture, RandomMixture, StandardMIS)
from .proposals import GAUSSIAN, STUDENT_T
from .results import (AMISRoundError, DMPMCRoundError, NPMCRoundError, SamplerExecutionError, WeightedSamples,
                      phase_of)

GAMMA_DRAW_ATTEMPTS = 8


class SamplerBusyError(RuntimeError):
    """A prepared sampler is non-reentrant (src/methods/importance_sampling.jl:105-116)."""


def _radial_strides(dofs):
    """_radial_normal_stride / _radial_uniform_stride over a packed family
    (src/proposal_banks.jl:205-223)."""
    if dofs is None:
        return 0, 0
    rn = max(1 if float(v) == 1.0 else GAMMA_DRAW_ATTEMPTS for v in dofs)
    ru = max(0 if float(v) == 1.0 else GAMMA_DRAW_ATTEMPTS + (1 if float(v) < 2 else 0) for v in dofs)
    return rn, ru


def compile_partial_denominator(bank, ids, logmasses, groups):
    """_compile_partial_denominator (src/methods/static_mis.jl:241-303):
    group id per active slot and each member's log mass within its group."""
    nprop = len(bank.proposals)
    seen = [False] * nprop
    slot_of = {pid: s for s, pid in enumerate(ids)}
    group_of_slot = [0] * len(ids)
    coef = np.zeros(len(ids), dtype=logmasses.dtype)
    g = 0
    for group in groups:
        if len(group) == 0:
            raise ValueError("partial-MIS groups cannot be empty")
        members = []
        for pid in group:
            if isinstance(pid, bool) or not isinstance(pid, (int, np.integer)):
                raise ValueError("partial-MIS proposal IDs must be integers")
            if not 1 <= pid <= nprop:
                raise ValueError(f"partial-MIS proposal ID {pid} is out of range")
            if seen[pid - 1]:
                raise ValueError(f"partial-MIS proposal ID {pid} appears more than once")
            seen[pid - 1] = True
            if pid in slot_of:
                members.append(slot_of[pid])
        if not members:
            continue
        g += 1
        lm = [float(logmasses[s]) for s in members]
        mx = max(lm)
        glog = mx + math.log(sum(math.exp(v - mx) for v in lm))
        for s in members:
            group_of_slot[s] = g
            coef[s] = logmasses[s] - logmasses.dtype.type(glog)
    if not all(seen):
        raise ValueError("partial-MIS groups must include every proposal ID exactly once")
    return np.array(group_of_slot, dtype=np.int32), coef


def deterministic_allocation_plan(active_masses, schedule):
    """_deterministic_allocation_plan (src/population_preparation.jl:266-367):
    exact largest-remainder counts with rotating tie order, contiguous
    assignments per slot, and log(count / round_size) coefficients."""
    exact = [Fraction(float(m)) for m in active_masses]
    total = sum(exact)
    exact = [m / total for m in exact]
    k = len(exact)
    rounds = len(schedule)
    counts = np.zeros((k, rounds), dtype=np.int64)
    for r, size in enumerate(schedule):
        quota = [m * size for m in exact]
        c = [math.floor(q) for q in quota]
        rem = [q - f for q, f in zip(quota, c)]
        remaining = size - sum(c)
        if not 0 <= remaining < k:
            raise RuntimeError("invalid DM-PMC allocation remainder")
        first_tie = r % k  # mod1(round, K) with 1-based rounds -> 0-based slot r % K
        order = sorted(range(k), key=lambda s: (-rem[s], (s - first_tie) % k))
        for s in order[:remaining]:
            c[s] += 1
        if not all(v > 0 for v in c):
            raise ValueError(f"round {r + 1} of size {size} cannot allocate at least one sample to every "
                             "positive-mass proposal")
        counts[:, r] = c
    offsets = np.concatenate([[0], np.cumsum(schedule)])
    return counts, offsets


class _Span:
    """CUDA events around one launch group on the current stream (profiling)."""

    def __init__(self, sampler, name, nbytes):
        self.sampler, self.name, self.nbytes = sampler, name, nbytes

    def __enter__(self):
        if self.sampler.profile is not None:
            self.start = torch.cuda.Event(enable_timing=True)
            self.start.record()
        return self

    def __exit__(self, *exc):
        if self.sampler.profile is not None:
            end = torch.cuda.Event(enable_timing=True)
            end.record()
            self.sampler.profile.append((self.name, self.start, end, self.nbytes))
        return False


class PreparedSampler:
    def __init__(self, seed, target, algorithm, device, precision, graphs=True, regularization=None,
                 target_precision=None):
        self.profile = None  # list of (name, start, end, algorithmic bytes) when profiling
        self.regularization = regularization
        self.target_precision = precision if target_precision is None else target_precision
        self.seed = int(seed) & (2 ** 64 - 1)
        self.offset = 0
        self.target = target
        self.algorithm = algorithm
        self.device = device
        self.precision = precision
        self.busy = False
        self.calls = 0
        self.counter = None  # device uint64 Philox base (moment methods)
        self.graphs = graphs
        self.graph = None

    # counter-based stream: disjoint (seed, offset) ranges per draw. With a
    # device counter the offsets are relative to counter[0], which the run
    # advances on the device at its end (so a replayed graph draws new numbers).
    def normals(self, n, dtype):
        if self.counter is not None:
            out = ops.fill_normals_at(n, dtype, self.device, self.seed, self.counter, self.offset)
        else:
            out = ops.fill_normals(n, dtype, self.device, self.seed, self.offset)
        self.offset += int(n) + 8
        return out

    def normal_stream(self, n):
        """(seed, device counter or None, offset) of the next n standard
        normals, advanced as normals(n) would be; None when normals() has been
        replaced on the instance (prefilled batches), so callers take the
        buffer path."""
        if "normals" in self.__dict__:
            return None
        out = (self.seed, self.counter, self.offset)
        self.offset += int(n) + 8
        return out

    def uniforms(self, n, dtype):
        if self.counter is not None:
            out = ops.fill_uniforms_at(n, dtype, self.device, self.seed, self.counter, self.offset)
        else:
            out = ops.fill_uniforms(n, dtype, self.device, self.seed, self.offset)
        self.offset += int(n) + 8
        return out


def prepare_sampler(seed, target, algorithm, device="cuda", precision=native.PREC_NATIVE, graphs=True,
                    regularization=None, target_precision=None):
    """prepare_sampler(rng, logtarget, alg) with the device applied: packs the
    proposal(s) and allocates every buffer on the device.

    graphs=True lets an AMIS sampler with a native target record its whole
    run as one CUDA graph on the second call and replay it afterwards (the
    first call runs eagerly and sizes every workspace).

    regularization: the moment fit's ridge coefficient. None keeps the
    reference's sqrt(eps(T)) of the sample type; an FP64 sampler given
    sqrt(eps(Float32)) fits exactly as an FP32 one would, which is how an FP64
    run is compared with a reduced-precision run on the same draws.

    precision: PREC_NATIVE (the SIMT drop-in), PREC_TF32 or PREC_BF16 for
    the AMIS / N-PMC density, moment and target kernels. Static MIS and
    DM-PMC rounds (draw + every slot's density fused) run the SIMT kernel in
    every form. target_precision (default: precision) is the form of the
    built-in regression targets' X beta likelihood: PREC_BF16 (bf16 x3),
    PREC_TF32, PREC_BF16X1 (one bf16 product) or PREC_NATIVE (SIMT)."""
    native.require()
    device = torch.device(device)
    s = PreparedSampler(seed, target, algorithm, device, precision, graphs, regularization, target_precision)
    if isinstance(algorithm, ImportanceSampling):
        _prepare_static(s)
    elif isinstance(algorithm, (AMIS, NPMC)):
        _prepare_moment(s)
    elif isinstance(algorithm, DeterministicMixturePMC):
        _prepare_dmpmc(s)
    else:
        raise TypeError(f"{type(algorithm).__name__} is not supported")
    return s


def importance_sample_(sampler):
    """importance_sample!(sampler): one complete run; raises on failures."""
    if sampler.busy:
        raise SamplerBusyError("prepared sampler is already running")
    sampler.busy = True
    try:
        alg = sampler.algorithm
        if isinstance(alg, ImportanceSampling):
            return _run_static(sampler)
        if isinstance(alg, (AMIS, NPMC)):
            return _run_moment(sampler)
        return _run_dmpmc(sampler)
    finally:
        sampler.busy = False
        sampler.calls += 1


def importance_sample(seed, target, algorithm, device="cuda", precision=native.PREC_NATIVE, graphs=True):
    return importance_sample_(prepare_sampler(seed, target, algorithm, device, precision, graphs))


# ---- static MIS ------------------------------------------------------------------
def _prepare_static(s):
    alg = s.algorithm
    db = pack(alg.bank, s.device)
    s.bank = db
    s.dtype = db.dtype
    scheme = alg.mis_scheme
    if isinstance(scheme, StandardMIS):
        s.den = ops.denominator(native.DENOM_GENERATING)
    elif isinstance(scheme, PartialDeterministicMixture):
        grp, coef = compile_partial_denominator(alg.bank, db.host_ids, db.host_logmasses, scheme.groups)
        s.den = ops.denominator(native.DENOM_PARTIAL, torch.tensor(coef, device=s.device),
                                groups=torch.tensor(grp, device=s.device))
    else:
        s.den = ops.denominator(native.DENOM_FULL, db.logmasses)
    s.stratified = not isinstance(scheme, RandomMixture)
    dofs = None if db.dofs is None else db.dofs.cpu().numpy()
    s.rn_stride, s.ru_stride = _radial_strides(dofs)
    s.bound_target = s.target.bind(s.device, db.dtype)


def _raise_failures(words, error=None, rnd=None):
    fail, _ = ops.decode_failure(words)
    if fail["count"] == 0:
        return
    cause = SamplerExecutionError(phase_of(fail["reason_bits"]), fail["first_logical_index"], fail["reason_bits"],
                                  fail["count"])
    if error is None:
        raise cause
    raise error(rnd, cause.phase, cause)


def _radial_buffers(s, n, dtype):
    rn = s.normals(n * s.rn_stride, dtype) if s.rn_stride else None
    ru = s.uniforms(n * s.ru_stride, dtype) if s.ru_stride else None
    return rn, ru


def _run_static(s):
    alg, db = s.algorithm, s.bank
    n, d, dt = alg.nsamples, db.d, db.dtype
    fail = ops.new_failures(s.device)
    u = s.uniforms(n, dt)
    slots = ops.static_assign(db.cdf, u, s.stratified)
    normals = s.normals(n * d, dt)
    rn, ru = _radial_buffers(s, n, dt)
    # the fused round (draw + every slot's density + log weight) is the SIMT
    # kernel; the target runs in the sampler's target precision
    samples, lw, pid = ops.mis_round(db, s.den, slots, normals, None, rn, s.rn_stride, ru, s.ru_stride, fail,
                                     native.PREC_NATIVE)
    values = s.bound_target.evaluate(samples, precision=s.target_precision)
    ops.add_target_values(lw, values, fail)
    _raise_failures(fail.cpu().numpy())
    scheme = type(alg.mis_scheme).__name__
    return WeightedSamples(samples, lw, provenance={"proposal_id": pid},
                           diagnostics={"method": "importance_sampling", "mis_scheme": scheme,
                                        "nsamples": n, "failures": 0})


# ---- AMIS / NPMC ------------------------------------------------------------------
def _prepare_moment(s):
    alg = s.algorithm
    p = alg.proposal
    s.proposal = p
    s.dtype = torch.float32 if p.dtype == np.float32 else torch.float64
    s.rounds = alg.rounds
    s.schedule = list(alg.round_size)
    s.offsets = np.concatenate([[0], np.cumsum(s.schedule)])
    s.history = DeviceHistory.allocate(p, s.rounds, s.device)
    uniform = len(set(s.schedule)) == 1
    if uniform:  # no host-to-device copy (a blocking copy synchronises the stream)
        s.logcounts = torch.full((s.rounds,), math.log(s.schedule[0]), dtype=s.dtype, device=s.device)
    else:
        s.logcounts = torch.tensor(np.log(np.array(s.schedule, dtype=np.float64)), dtype=s.dtype, device=s.device)
    total = int(s.offsets[-1])
    d = p.dimension
    dev, dt = s.device, s.dtype
    s.samples = torch.empty(total, d, dtype=dt, device=dev)
    s.logtargets = torch.empty(total, dtype=dt, device=dev)
    s.lognum = torch.empty(total, dtype=dt, device=dev)
    s.logweights = torch.empty(total, dtype=dt, device=dev)
    # the small per-run state in three zeroed blocks (each part 256-byte aligned)
    s.summaries, s.mean, s.cov, s.shift = _carve(torch.float64, dev, (s.rounds, 3), (d,), (d, d), (d,))
    s.round_failures, s.counter = _carve(torch.int64, dev, (s.rounds, 3), (1,))
    s.cand_loc, s.cand_factor, s.cand_lognorm = _carve(dt, dev, (d,), (d, d), (1,))
    if isinstance(alg, NPMC):  # clipped weights of one round, the clip thresholds, the fit summaries
        s.clipped = torch.empty(max(s.schedule), dtype=dt, device=dev)
        s.clip_thresholds = torch.empty(s.rounds, dtype=dt, device=dev)
        s.fit_summaries = torch.zeros(s.rounds, 3, dtype=torch.float64, device=dev)
    s.committed = (s.history.locations[0].clone(), s.history.scales[0].clone(), s.history.lognormalizers[0].clone())
    dofs = None if p.family != STUDENT_T else [float(p.dof)]
    s.rn_stride, s.ru_stride = _radial_strides(dofs)
    s.bound_target = s.target.bind(s.device, dt)
    if uniform:  # 1-based round of each sample, with no host-to-device copy
        s.round_ids_init = torch.arange(total, device=dev) // s.schedule[0] + 1
    else:
        s.round_ids_init = torch.repeat_interleave(torch.arange(1, s.rounds + 1, device=dev),
                                                   torch.tensor(s.schedule, device=dev),
                                                   output_size=total).contiguous()
    s.round_ids = s.round_ids_init.clone()


def _carve(dtype, device, *shapes):
    """Zeroed tensors of the given shapes carved from one allocation, each
    starting on a 256-byte boundary (vectorised kernels read them)."""
    es = torch.empty((), dtype=dtype).element_size()
    step = 256 // es
    sizes = [int(np.prod(sh)) for sh in shapes]
    starts, o = [], 0
    for n in sizes:
        starts.append(o)
        o += (n + step - 1) // step * step
    buf = torch.zeros(o, dtype=dtype, device=device)
    return [buf[a:a + n].view(*sh) for a, n, sh in zip(starts, sizes, shapes)]


def _graph_eligible(s):
    """Whole-run graph capture needs a run with no host decisions: AMIS (NPMC
    clips through a selection), a native target, no per-span profiling and
    the sampler's own random stream."""
    from .targets import _Bound, _BoundBank

    return (s.graphs and isinstance(s.algorithm, AMIS) and s.profile is None
            and isinstance(s.bound_target, (_Bound, _BoundBank))
            and "normals" not in s.__dict__ and "uniforms" not in s.__dict__)


def _run_moment(s):
    is_npmc = isinstance(s.algorithm, NPMC)
    # an eligible AMIS run is issued by one issm_amis_run call (the same
    # library calls as the round loop, bitwise the same results)
    if not is_npmc and native_body_eligible(s):
        def body():
            _native_body(s)
    else:
        def body():
            _moment_body(s, is_npmc)
    if _graph_eligible(s) and s.calls >= 1:
        if s.graph is None:
            g = torch.cuda.CUDAGraph()
            torch.cuda.synchronize(s.device)
            l0 = native.lib().issm_kernel_launches()
            with torch.cuda.graph(g):
                body()
            s.graph_launches = int(native.lib().issm_kernel_launches() - l0)
            native.note_replay(-s.graph_launches)  # captured, not run
            s.graph = g
        s.graph.replay()
        native.note_replay(s.graph_launches)
    else:
        body()
    return _finish_moment(s, is_npmc)


def _moment_body(s, is_npmc):
    """Every launch of one AMIS/NPMC run, stream-ordered, no host reads."""
    h = s.history
    d, dt = h.d, h.dtype
    s.offset = 0
    loc0, fac0, ln0 = s.committed
    h.locations[0].copy_(loc0)
    h.scales[0].copy_(fac0)
    h.lognormalizers[0].copy_(ln0)
    h.attach_inverse_factors(0, 1)
    s.round_failures.zero_()
    s.round_ids.copy_(s.round_ids_init)
    for t in range(s.rounds):
        n_old, n_new = int(s.offsets[t]), int(s.schedule[t])
        n_tot = n_old + n_new
        fail = s.round_failures[t]
        view = h.view(t + 1)
        es = h.scales.element_size()
        with _Span(s, "draw", n_new * d * es):
            # standard normals generated inside the draw kernel (no normal buffer)
            stream = s.normal_stream(n_new * d)
            normals = s.normals(n_new * d, dt) if stream is None else None
            rn, ru = _radial_buffers(s, n_new, dt)
            x_new = s.samples[n_old:n_tot]
            if stream is None:
                ops.draw(h, normals, n_new, fixed_slot=t, radial_normals=rn, rn_stride=s.rn_stride,
                         radial_uniforms=ru, ru_stride=s.ru_stride, failures=fail, out=x_new, bank_ref=view)
            else:
                ops.draw_philox(h, n_new, stream[0], stream[1], stream[2], fixed_slot=t, radial_normals=rn,
                                rn_stride=s.rn_stride, radial_uniforms=ru, ru_stride=s.ru_stride, failures=fail,
                                out=x_new, bank_ref=view)
        with _Span(s, "target", n_new * (d + 1) * es):
            s.bound_target.evaluate(x_new, out=s.logtargets[n_old:n_tot], precision=s.target_precision)
            ops.check_target_values(s.logtargets[n_old:n_tot], s.round_ids[n_old:n_tot], fail)
        if is_npmc:
            den = ops.denominator(native.DENOM_GENERATING)
            lq = ops.mixture_logdensity(h, den, x_new, fixed_slot=t, failures=fail, out=s.lognum[n_old:n_tot],
                                        bank_ref=view, precision=s.precision)
            ops.subtract_logweights(s.logtargets[n_old:n_tot], lq, fail, out=s.logweights[n_old:n_tot])
            # clip the isqrt(n) largest weights on the device (src/npmc_execution.jl:22-33)
            lw_fit, _ = ops.npmc_clip(s.logweights[n_old:n_tot], out=s.clipped[:n_new],
                                      threshold=s.clip_thresholds[t:t + 1])
            x_fit = x_new
            ops.logweight_summary(s.logweights[n_old:n_tot], out=s.summaries[t])
            fit_summary = ops.logweight_summary(lw_fit, out=s.fit_summaries[t])
        else:
            if n_old > 0:
                with _Span(s, "amis_append", n_old * (d + 2) * es):
                    ops.amis_append(view, t, s.logcounts, s.samples[:n_old], s.lognum[:n_old], fail, s.precision)
            den = ops.denominator(native.DENOM_PREFIX, s.logcounts, terms=t + 1)
            with _Span(s, "mixture_new", n_new * (d + 1) * es + (t + 1) * d * d * es):
                ops.mixture_logdensity(h, den, x_new, fixed_slot=t, failures=fail, out=s.lognum[n_old:n_tot],
                                       bank_ref=view, precision=s.precision)
            with _Span(s, "form_summary", n_tot * (3 * es + 8)):
                fit_summary = ops.amis_form_summary(s.logtargets[:n_tot], s.lognum[:n_tot], math.log(n_tot),
                                                    s.logweights[:n_tot], s.summaries[t],
                                                    round_ids=s.round_ids[:n_tot], failures=fail)
                lw_fit = s.logweights[:n_tot]
                x_fit = s.samples[:n_tot]
        # algorithmic bytes: one read of the samples and weights (tensor-core
        # form), two (the native two-pass form)
        passes = 1 if s.precision != native.PREC_NATIVE else 2
        with _Span(s, "moments", passes * x_fit.shape[0] * (d + 1) * es):
            s.shift.copy_(h.locations[t])
            prev = h.scales[t] if h.scales[t].dim() == 2 and h.scales.dtype == torch.float32 else None
            ops.weighted_moments(x_fit, lw_fit, fit_summary, s.shift, s.mean, s.cov, precision=s.precision,
                                 prev_factor=prev)
        last = t + 1 == s.rounds
        out_loc = s.cand_loc if last else h.locations[t + 1]
        out_fac = s.cand_factor if last else h.scales[t + 1]
        out_ln = s.cand_lognorm if last else h.lognormalizers[t + 1:t + 2]
        with _Span(s, "fit", 3 * d * d * 8):
            inv = None
            if not last and s.precision != native.PREC_NATIVE and getattr(h, "inverse_factors", None) is not None:
                inv = h.inverse_factors[t + 1]
            ops.fit_factor(s.mean, s.cov, h.scales[t], out_loc, out_fac, out_ln, dof=h.dof,
                           logconstant=h.logconstant, failures=fail, failure_index=n_tot + 1, out_inverse=inv,
                           regularization=s.regularization)
    ops.counter_advance(s.counter, s.offset)


def native_body_eligible(s):
    """issm_amis_run covers AMIS with a Gaussian factor history, a native
    target, generated normals and no per-span profiling."""
    from .targets import _Bound, _BoundBank

    h = getattr(s, "history", None)
    return (isinstance(s.algorithm, AMIS) and h is not None and h.family == GAUSSIAN and h.d <= 64
            and h.scale_kind == native.SCALE_FACTOR and isinstance(s.bound_target, (_Bound, _BoundBank))
            and s.profile is None
            and "normals" not in s.__dict__ and "uniforms" not in s.__dict__
            and (s.precision == native.PREC_NATIVE or h.dtype == torch.float32))


def _native_body(s):
    """Every launch of one AMIS run through one issm_amis_run call: the same
    library calls as _moment_body, issued from native code."""
    h = s.history
    if s.precision != native.PREC_NATIVE:
        h.attach_inverse_factors(0, 0)  # allocate; the run inverts slot 0 itself
    d, total = h.d, int(s.offsets[-1])
    nb = native.lib().issm_amis_run_workspace_bytes(d, total, s.rounds)
    ws = native.workspace(nb, s.device, "run", zero=True)
    s.run_workspace = ws
    sizes = (ctypes.c_int64 * s.rounds)(*[int(v) for v in s.schedule])
    bank = h.view(h.count)._obj
    loc0, fac0, ln0 = s.committed
    from .targets import _BoundBank

    radial = isinstance(s.bound_target, _BoundBank)
    target_ptr = None if radial else ctypes.cast(ctypes.byref(s.bound_target.struct), ctypes.c_void_p)
    desc = native.AmisRunDesc(bank, target_ptr, s.rounds,
                              int(s.precision), ctypes.cast(sizes, ctypes.c_void_p), float(h.logconstant), s.seed, 0,
                              native.ptr(s.counter), native.ptr(s.logcounts), native.ptr(s.round_ids_init),
                              native.ptr(loc0), native.ptr(fac0), native.ptr(ln0), native.ptr(s.samples),
                              native.ptr(s.logtargets), native.ptr(s.lognum), native.ptr(s.logweights),
                              native.ptr(s.round_ids), native.ptr(s.summaries), native.ptr(s.round_failures),
                              native.ptr(s.mean), native.ptr(s.cov), native.ptr(s.shift), native.ptr(s.cand_loc),
                              native.ptr(s.cand_factor), native.ptr(s.cand_lognorm), native.ptr(ws), ws.numel())
    # the same target form as the host round loop's evaluate()
    if radial:
        tb = s.bound_target
        desc.target_bank = ctypes.addressof(tb.bank.struct)
        desc.target_den = ctypes.addressof(tb.den)
        desc.target_bank_precision = tb.effective_precision(s.target_precision, h.dtype)
    else:
        operand = s.bound_target.tensor_operand(s.target_precision, h.dtype, s.device)
        if operand is not None:
            desc.target_operand, desc.target_precision = native.ptr(operand), int(s.target_precision)
    native.call("issm_amis_run", ctypes.byref(desc), native.stream_ptr())
    s.offset = sum(int(v) * d + 8 for v in s.schedule)


def _run_workspace_errors(s):
    """The sticky timeout words of the tensor-core and moments regions of the
    run workspace (issm_amis_run_desc layout)."""
    ws = getattr(s, "run_workspace", None)
    if ws is None:
        return
    lib = native.lib()
    d, total = s.history.d, int(s.offsets[-1])
    up = lambda v: (int(v) + 255) // 256 * 256  # noqa: E731
    tc_end = up(lib.issm_tc_workspace_bytes(s.rounds, d))
    mom_end = tc_end + up(lib.issm_moments_workspace_bytes(total, d))
    for end in (tc_end, mom_end):
        if int(ws[end - 64:end - 60].view(torch.int32).item()) != 0:
            raise RuntimeError("a tensor-core kernel timed out waiting for MMA completion")


def _finish_moment_summary(s):
    """The serving form of _finish_moment for AMIS: one packed device-to-host
    read of the failure records, the per-round summaries and the posterior
    mean (the last round's FP64 moment pass runs over every retained sample
    with the final weights, so its mean is the weighted posterior mean);
    raises on the first failed round; returns (posterior mean, log Z, ESS)
    of the final round. The samples stay on the device, uncopied."""
    packed = torch.cat([s.round_failures.view(torch.float64).reshape(-1), s.summaries.reshape(-1), s.mean]).cpu()
    words = packed[:3 * s.rounds].view(torch.int64).numpy().reshape(s.rounds, 3)
    summaries = packed[3 * s.rounds:6 * s.rounds].numpy().reshape(s.rounds, 3)
    if s.precision != native.PREC_NATIVE:
        if getattr(s, "run_workspace", None) is not None:
            _run_workspace_errors(s)
        else:
            ops.check_tensor_core_errors(s.device)
    for t in range(s.rounds):
        if words[t][0] != 0:
            _raise_failures(words[t], AMISRoundError, t + 1)
    m, sm, s2 = summaries[-1]
    n = int(s.offsets[-1])
    ess = 0.0 if sm == 0 else sm * sm / s2
    logz = -np.inf if sm == 0 else m + np.log(sm) - np.log(n)
    return packed[6 * s.rounds:].numpy().copy(), float(logz), float(ess)


def _finish_moment(s, is_npmc):
    """Read the failure records, the per-round summaries and the last fit's
    FP64 weighted mean back in one copy, raise on the first failed round and
    build the result.

    The result's `samples` is a view of the sampler's retained-sample buffer
    (at d = 64, 40 x 50,000 samples that buffer is 512 MB, and copying it
    would double the run's HBM traffic beyond the moments pass): it stays
    valid until the sampler's next run, which overwrites it. Clone it to keep
    it longer. The log weights and round ids are copies, as in the reference
    (src/adaptive_gaussian_execution.jl:1090-1100 copies the log weights)."""
    packed = torch.cat([s.round_failures.view(torch.float64).reshape(-1), s.summaries.reshape(-1), s.mean]).cpu()
    words = packed[:3 * s.rounds].view(torch.int64).numpy().reshape(s.rounds, 3)
    summaries = packed[3 * s.rounds:6 * s.rounds].numpy().reshape(s.rounds, 3)
    moment_mean = packed[6 * s.rounds:].numpy().copy()
    if s.precision != native.PREC_NATIVE:
        if getattr(s, "run_workspace", None) is not None:
            _run_workspace_errors(s)
        else:
            ops.check_tensor_core_errors(s.device)
    err = NPMCRoundError if is_npmc else AMISRoundError
    for t in range(s.rounds):
        if words[t][0] != 0:
            _raise_failures(words[t], err, t + 1)
    total = int(s.offsets[-1])
    ess = np.zeros(s.rounds)
    logz = np.zeros(s.rounds)
    for t in range(s.rounds):
        m, sm, s2 = summaries[t]
        n_t = int(s.schedule[t]) if is_npmc else int(s.offsets[t + 1])
        ess[t] = 0.0 if sm == 0 else sm * sm / s2
        logz[t] = -np.inf if sm == 0 else m + np.log(sm) - np.log(n_t)
    for dst, src in zip(s.committed, (s.cand_loc, s.cand_factor, s.cand_lognorm[0])):
        dst.copy_(src)
    # AMIS: the last round's moment pass runs over every retained sample with
    # the final weights, so its mean is the weighted posterior mean. NPMC fits
    # on the last round's clipped weights, so its mean is that fit's centre.
    diagnostics = {"method": "npmc" if is_npmc else "amis", "rounds": s.rounds, "round_sizes": list(s.schedule),
                   "round_ess": ess, "round_lognormalizers": logz, "target_evaluations": total,
                   "proposal_evaluations": total if is_npmc else s.rounds * total, "failures": 0,
                   "moment_mean": moment_mean}
    if is_npmc:  # _moment_extra_diagnostics(::NPMC) (src/npmc_execution.jl:5-6)
        fit = s.fit_summaries.cpu().numpy()
        diagnostics["adaptation_ess"] = np.array([0.0 if f[1] == 0 else f[1] * f[1] / f[2] for f in fit])
        diagnostics["clipped_counts"] = [math.isqrt(int(v)) for v in s.schedule]
    return WeightedSamples(s.samples, s.logweights.clone(), provenance={"round": s.round_ids.clone()},
                           diagnostics=diagnostics)


def reweigh_amis(sampler, precision=native.PREC_NATIVE, dtype=None):
    """The final AMIS weights of a completed run, recomputed from scratch in
    another precision form on the same retained samples and the same proposal
    history: the full deterministic mixture log sum_t n_t q_t(x) over all T
    slots (the closed form of the append recurrence,
    src/amis_execution.jl:12-35), the weights log pi - log mixture + log N_T,
    their summary, and the weighted mean.

    This is the comparison of precision forms with the adaptation held fixed:
    a whole adaptive run amplifies any difference in a fit into the next
    round's draws, so two runs from the same draws part ways by more than
    their arithmetic; re-weighing one run's samples under its own history
    isolates the arithmetic. dtype: the sample/bank type of the form
    (float32 for the tensor-core forms; default: the run's own).

    Returns (log Z, FP64 weighted mean (d,), log weights (N,))."""
    h = sampler.history
    dtype = h.dtype if dtype is None else dtype
    if precision != native.PREC_NATIVE and dtype != torch.float32:
        raise ValueError("the tensor-core forms take float32 samples and proposals")
    rounds, d, dev = sampler.rounds, h.d, sampler.device
    total = int(sampler.offsets[-1])
    bank = h.__class__(d, rounds, h.family, h.scale_kind, dtype, h.locations.to(dtype).contiguous(),
                       h.scales.to(dtype).contiguous(), h.lognormalizers.to(dtype).contiguous(),
                       None if h.dofs is None else h.dofs.to(dtype).contiguous(), h.range_risk)
    if precision != native.PREC_NATIVE:
        bank.attach_inverse_factors()
    x = sampler.samples if sampler.samples.dtype == dtype else sampler.samples.to(dtype)
    logtargets = sampler.target.bind(dev, dtype).evaluate(x, precision=precision)
    logcounts = sampler.logcounts.to(dtype)
    den = ops.denominator(native.DENOM_PREFIX, logcounts, terms=rounds)
    lognum = ops.mixture_logdensity(bank, den, x, fixed_slot=rounds - 1, precision=precision)
    lw = torch.empty(total, dtype=dtype, device=dev)
    summary = torch.zeros(3, dtype=torch.float64, device=dev)
    ops.amis_form_summary(logtargets, lognum, math.log(total), lw, summary)
    shift = h.locations[rounds - 1].double().contiguous()
    mean, _ = ops.weighted_moments(x, lw, summary, shift, precision=precision)
    m, s, _ = summary.cpu().numpy()
    logz = -math.inf if s == 0 else float(m + np.log(s) - np.log(total))
    return logz, mean.cpu().numpy(), lw


def share_normal_stream(sampler, dtype=torch.float32):
    """Make `sampler` draw its standard normals from the `dtype` normal stream
    of its own seed, converted to its sample type.

    FP32 and FP64 normal streams of one seed are different numbers (an FP32
    Philox block yields four 24-bit uniforms, an FP64 block two 53-bit ones).
    An FP64 sampler set up this way draws, call for call, the same normals as
    an FP32 or tensor-core sampler with the same seed, so the two runs differ
    only by their arithmetic: this is how a reduced-precision run is compared
    with an FP64 run on the same draws. The normals pass through a device
    buffer, so the sampler runs its rounds eagerly (no whole-run graph)."""
    def normals(n, dt):
        if sampler.counter is not None:
            out = ops.fill_normals_at(n, dtype, sampler.device, sampler.seed, sampler.counter, sampler.offset)
        else:
            out = ops.fill_normals(n, dtype, sampler.device, sampler.seed, sampler.offset)
        sampler.offset += int(n) + 8
        return out.to(dt)

    sampler.normals = normals
    return sampler


def current_proposal(sampler):
    """The committed (learned) proposal of a moment sampler as host arrays."""
    loc, fac, ln = sampler.committed
    return loc.cpu().numpy(), fac.cpu().numpy().T.copy(), float(ln)


# ---- DM-PMC ------------------------------------------------------------------------
def _prepare_dmpmc(s):
    alg = s.algorithm
    db = pack(alg.bank, s.device)
    s.bank = db
    s.dtype = db.dtype
    s.schedule = list(alg.round_size)
    active = np.array([alg.bank.masses[i - 1] for i in db.host_ids])
    counts, offsets = deterministic_allocation_plan(active, s.schedule)
    s.counts_host, s.offsets = counts, offsets
    s.counts = torch.tensor(counts.T.copy(), device=s.device)  # rounds x K
    rounds = len(s.schedule)
    s.rounds = rounds
    s.slots = []
    s.coefs = []
    for r in range(rounds):
        sl = np.repeat(np.arange(db.count, dtype=np.int32), counts[:, r])
        s.slots.append(torch.tensor(sl, device=s.device))
        coef = np.log(counts[:, r].astype(np.float64) / float(s.schedule[r]))
        s.coefs.append(torch.tensor(coef, dtype=db.dtype, device=s.device))
    s.committed_locations = db.locations.clone()
    dofs = None if db.dofs is None else db.dofs.cpu().numpy()
    s.rn_stride, s.ru_stride = _radial_strides(dofs)
    s.bound_target = s.target.bind(s.device, db.dtype)
    total = int(offsets[-1])
    s.summaries = torch.zeros(rounds, 3, dtype=torch.float64, device=s.device)
    s.round_failures = torch.zeros(rounds, 3, dtype=torch.int64, device=s.device)
    s.samples = torch.empty(total, db.d, dtype=db.dtype, device=s.device)
    s.logweights = torch.empty(total, dtype=db.dtype, device=s.device)
    s.proposal_ids = torch.empty(total, dtype=torch.int64, device=s.device)
    # locations in force during each round and the uniforms each resampling
    # step consumed (device-side provenance, read only by diagnostics)
    s.location_history = torch.empty(rounds, db.count, db.d, dtype=db.dtype, device=s.device)
    s.resample_uniform_history = [None] * rounds


def _run_dmpmc(s):
    db = s.bank
    d, dt = db.d, db.dtype
    db.locations.copy_(s.committed_locations)
    s.round_failures.zero_()
    local = isinstance(s.algorithm.resampling, LocalResampling)
    for r in range(s.rounds):
        lo, hi = int(s.offsets[r]), int(s.offsets[r + 1])
        n = hi - lo
        fail = s.round_failures[r]
        s.location_history[r].copy_(db.locations)
        normals = s.normals(n * d, dt)
        rn, ru = _radial_buffers(s, n, dt)
        den = ops.denominator(native.DENOM_FULL, s.coefs[r])
        x, lw, pid = ops.mis_round(db, den, s.slots[r], normals, None, rn, s.rn_stride, ru, s.ru_stride, fail,
                                   native.PREC_NATIVE, samples=s.samples[lo:hi], logweights=s.logweights[lo:hi],
                                   proposal_ids_out=s.proposal_ids[lo:hi])
        s.bound_target.evaluate(x, out=_scratch(s, n, dt), precision=s.target_precision)
        ops.add_target_values(lw, s._scratch[:n], fail)
        ops.logweight_summary(lw, out=s.summaries[r])
        if local:
            u = s.uniforms(db.count, dt)
            _, dst = ops.local_resample(lw, s.counts[r], u, x)
        else:
            u = s.uniforms(db.count, torch.float64)
            anc = ops.resample_multinomial(lw, u)
            dst = ops.gather(x, anc)
        s.resample_uniform_history[r] = u
        db.locations.copy_(dst)
    words = s.round_failures.cpu().numpy()
    summaries = s.summaries.cpu().numpy()
    for r in range(s.rounds):
        if words[r][0] != 0:
            _raise_failures(words[r], DMPMCRoundError, r + 1)
        if summaries[r][1] == 0.0:
            from .results import AllZeroWeightsError

            raise DMPMCRoundError(r + 1, "resampling", AllZeroWeightsError())
    ess = np.array([sm[1] ** 2 / sm[2] for sm in summaries])
    logz = np.array([sm[0] + np.log(sm[1]) - np.log(s.schedule[r]) for r, sm in enumerate(summaries)])
    s.committed_locations = db.locations.clone()
    round_ids = torch.repeat_interleave(torch.arange(1, s.rounds + 1, device=s.device),
                                        torch.tensor(s.schedule, device=s.device), output_size=int(sum(s.schedule)))
    return WeightedSamples(s.samples.clone(), s.logweights.clone(),
                           provenance={"round": round_ids, "proposal_id": s.proposal_ids.clone()},
                           diagnostics={"method": "deterministic_mixture_pmc", "rounds": s.rounds,
                                        "round_sizes": list(s.schedule), "round_ess": ess,
                                        "round_lognormalizers": logz,
                                        "resampling": "local" if local else "global", "failures": 0})


def _scratch(s, n, dt):
    buf = getattr(s, "_scratch", None)
    if buf is None or buf.numel() < n:
        s._scratch = torch.empty(n, dtype=dt, device=s.device)
    return s._scratch[:n]
