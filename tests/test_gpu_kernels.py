"""Parity of every libissm103.so kernel with the FP64 oracle and with the
reference's golden vectors, called through the C ABI.

Tolerances: FP64 kernels within 64 eps relative (the reference's own static-MIS
parity bar is 32-64 eps); FP32 kernels within 2e-5 relative of the oracle
value scaled by max(1, |value|); integer outputs (slots, ancestors,
failure words) bit-exact.
"""
import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

EPS64 = np.finfo(np.float64).eps
F32_PREV1 = float(np.nextafter(np.float32(1), np.float32(0)))


def tdt(np_dtype):
    return torch.float32 if np_dtype == np.float32 else torch.float64


def make_bank(issm, orc, rng, d, k, family, kind, dtype, dev, spread=2.0):
    props = []
    for _ in range(k):
        mu = (rng.normal(size=d) * spread).astype(dtype)
        if kind == "factor":
            A = rng.normal(size=(d, d))
            L = np.linalg.cholesky(A @ A.T / d + 0.1 * np.eye(d)).astype(dtype)
            sc = L
        elif kind == "diagonal":
            sc = np.exp(rng.normal(size=d) * 0.3).astype(dtype)
        else:
            sc = dtype(np.exp(rng.normal() * 0.3))
        if family == "gaussian":
            f = {"factor": issm.FactorGaussian, "diagonal": issm.DiagonalGaussian, "spherical": issm.SphericalGaussian}
            props.append(f[kind](mu, sc))
        else:
            f = {"factor": issm.FactorStudentT, "diagonal": issm.DiagonalStudentT, "spherical": issm.SphericalStudentT}
            props.append(f[kind](dtype(rng.choice([3.0, 5.0, 7.5])), mu, sc))
    masses = rng.dirichlet(np.ones(k))
    bank = issm.ProposalBank(props, masses)
    db = issm.pack(bank, dev)
    return bank, db, oracle_bank(orc, db)


def oracle_bank(orc, db):
    fam = orc.STUDENT_T if db.family == 1 else orc.GAUSSIAN
    dofs = None if db.dofs is None else db.dofs.double().cpu().numpy()
    rr = None if db.range_risk is None else db.range_risk.cpu().numpy()
    return orc.BankView(db.d, fam, db.scale_kind, db.locations.double().cpu().numpy(),
                        db.scales.double().cpu().numpy(), db.lognormalizers.double().cpu().numpy(), dofs, rr)


def assert_close(got, exp, dtype, scale_eps=64):
    got = np.asarray(got, dtype=np.float64)
    exp = np.asarray(exp, dtype=np.float64)
    assert got.shape == exp.shape
    same_inf = (np.isinf(got) & np.isinf(exp) & (np.sign(got) == np.sign(exp)))
    fin = ~same_inf
    if dtype == np.float64:
        tol = scale_eps * EPS64 * np.maximum(1.0, np.abs(exp[fin]))
    else:
        tol = 2e-5 * np.maximum(1.0, np.abs(exp[fin]))
    err = np.abs(got[fin] - exp[fin])
    assert np.all(err <= tol), f"max err {err.max():.3e} at {np.argmax(err - tol)}"


# ---- golden densities -----------------------------------------------------------
def _single_bank(issm, c, dtype, dev):
    loc = np.asarray(c["location"], dtype=dtype)
    if c["kind"] == "factor":
        sc = np.asarray(c["scale"], dtype=dtype)
    elif c["kind"] == "diagonal":
        sc = np.asarray(c["scale"], dtype=dtype)
    else:
        sc = dtype(c["scale"][0])
    if "dof" in c:
        f = {"factor": issm.FactorStudentT, "diagonal": issm.DiagonalStudentT, "spherical": issm.SphericalStudentT}
        p = f[c["kind"]](dtype(c["dof"]), loc, sc)
    else:
        f = {"factor": issm.FactorGaussian, "diagonal": issm.DiagonalGaussian, "spherical": issm.SphericalGaussian}
        p = f[c["kind"]](loc, sc)
    return issm.pack(issm.ProposalBank([p]), dev)


@pytest.mark.parametrize("name", ["native_gaussian_analytic", "native_gaussian_range",
                                  "native_student_t_analytic", "native_student_t_subnormal"])
def test_golden_component_densities(issm, cuda, golden, name):
    c = golden[name]
    for sub in c["cases"]:
        dtype = np.float32 if sub.get("dtype", c.get("dtype")) == "f32" else np.float64
        rtol = sub.get("rtol_eps", c["rtol_eps"]) * float(np.finfo(dtype).eps)
        db = _single_bank(issm, sub, dtype, cuda)
        x = torch.tensor(np.asarray(sub["x"], dtype=dtype).reshape(1, -1), device=cuda)
        den = issm.ops.denominator(issm.native.DENOM_GENERATING)
        fail = issm.ops.new_failures(cuda)
        out, gen = issm.ops.mixture_logdensity(db, den, x, fixed_slot=0, failures=fail, generating=True)
        got = float(gen.double().item())
        assert got == pytest.approx(sub["expected"], rel=max(rtol, 4 * float(np.finfo(dtype).eps)), abs=1e-300), sub


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_golden_packed_factor_primitives(issm, cuda, golden, dtype):
    c = golden["packed_factor_primitives"]
    p = issm.FactorGaussian(np.asarray(c["location"], dtype=dtype), np.asarray(c["factor"], dtype=dtype))
    db = issm.pack(issm.ProposalBank([p]), cuda)
    normals = torch.tensor(np.asarray(c["normals"], dtype=dtype), device=cuda)
    x = issm.ops.draw(db, normals, 1, fixed_slot=0)
    assert x.double().cpu().numpy().reshape(-1).tolist() == c["expected_sample"]
    den = issm.ops.denominator(issm.native.DENOM_GENERATING)
    _, gen = issm.ops.mixture_logdensity(db, den, x, fixed_slot=0, generating=True)
    assert float(gen.item()) == pytest.approx(c["expected_logdensity"], rel=8 * float(np.finfo(dtype).eps))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_golden_realized_denominator(issm, cuda, golden, dtype):
    c = golden["realized_mixture_denominator"]
    props = [issm.SphericalGaussian(dtype(m), dtype(s)) for m, s in zip(c["locations"], c["scales"])]
    db = issm.pack_proposals(props, cuda)
    coef = np.asarray(c["coefficients"], dtype=dtype)
    x = torch.tensor([[dtype(c["x"][0])]], device=cuda)
    for r in range(2):
        den = issm.ops.denominator(issm.native.DENOM_FULL, torch.tensor(coef[:, r].copy(), device=cuda))
        out, gen = issm.ops.mixture_logdensity(db, den, x, slots=torch.zeros(1, dtype=torch.int32, device=cuda),
                                               generating=True)
        assert float(out.item()) == pytest.approx(c["expected"][r], rel=16 * float(np.finfo(dtype).eps))
        assert float(gen.item()) == pytest.approx(c["expected_generating"], rel=16 * float(np.finfo(dtype).eps))


# ---- random banks vs oracle ------------------------------------------------------------
CASES = [
    (1, 1, "gaussian", "spherical"), (3, 5, "gaussian", "factor"), (5, 3, "student", "factor"),
    (16, 64, "gaussian", "factor"), (7, 9, "gaussian", "diagonal"), (4, 6, "student", "diagonal"),
    (33, 4, "gaussian", "factor"), (64, 3, "student", "factor"), (2, 2, "student", "spherical"),
]


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("d,k,family,kind", CASES)
@pytest.mark.parametrize("denom", ["full", "generating", "partial", "prefix"])
def test_mixture_logdensity_vs_oracle(issm, orc, cuda, dtype, d, k, family, kind, denom):
    rng = np.random.default_rng(hash((d, k, family, kind, denom)) & 0xFFFF)
    bank, db, ob = make_bank(issm, orc, rng, d, k, family, kind, dtype, cuda)
    n = int(rng.choice([1, 37, 1001, 4099]))
    slots = rng.integers(0, k, size=n).astype(np.int32)
    x = np.stack([db.locations[s].double().cpu().numpy() for s in slots]) + rng.normal(size=(n, d)) * 1.5
    x = x.astype(dtype)
    coef = db.logmasses.double().cpu().numpy()
    groups = None
    terms = 0
    if denom == "full":
        kind_c = issm.native.DENOM_FULL
    elif denom == "generating":
        kind_c = issm.native.DENOM_GENERATING
    elif denom == "partial":
        kind_c = issm.native.DENOM_PARTIAL
        groups = (np.arange(k) % 2).astype(np.int32)
    else:
        kind_c = issm.native.DENOM_PREFIX
        terms = max(1, k - 1)
        slots = np.minimum(slots, terms - 1).astype(np.int32)
    den = issm.ops.denominator(kind_c, torch.tensor(coef.astype(dtype), device=cuda), terms=terms,
                               groups=None if groups is None else torch.tensor(groups, device=cuda))
    fail = issm.ops.new_failures(cuda)
    out, gen = issm.ops.mixture_logdensity(db, den, torch.tensor(x, device=cuda),
                                           slots=torch.tensor(slots, device=cuda), failures=fail, generating=True)
    eo, eg, rs = orc.mixture_logdensity(ob, x.astype(np.float64).reshape(-1), kind_c, coef, terms=terms,
                                        group_of_slot=groups, slots=slots)
    assert_close(out.cpu().numpy(), eo, dtype)
    assert_close(gen.cpu().numpy(), eg, dtype)
    assert int(fail[0].item()) == int(np.count_nonzero(rs))


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("family", ["gaussian", "student"])
def test_mis_round_vs_oracle(issm, orc, cuda, dtype, family):
    rng = np.random.default_rng(5)
    d, k, n = 6, 7, 3001
    bank, db, ob = make_bank(issm, orc, rng, d, k, family, "factor", dtype, cuda)
    slots = np.sort(rng.integers(0, k, size=n)).astype(np.int32)
    normals = rng.normal(size=n * d).astype(dtype)
    rn_stride, ru_stride = (8, 8) if family == "student" else (0, 0)
    rn = rng.normal(size=n * 8).astype(dtype) if family == "student" else None
    ru = rng.random(size=n * 8).astype(dtype) if family == "student" else None
    logt = (rng.normal(size=n) * 3).astype(dtype)
    den = issm.ops.denominator(issm.native.DENOM_FULL, db.logmasses)
    fail = issm.ops.new_failures(cuda)
    T = lambda a: None if a is None else torch.tensor(a, device=cuda)  # noqa: E731
    x, lw, pid = issm.ops.mis_round(db, den, T(slots), T(normals), T(logt), T(rn), rn_stride, T(ru), ru_stride, fail)
    ex, rs = orc.draw(ob, normals.astype(np.float64), slots=slots, radial_normals=None if rn is None else rn.astype(np.float64),
                      rn_stride=rn_stride, radial_uniforms=None if ru is None else ru.astype(np.float64),
                      ru_stride=ru_stride)
    assert_close(x.cpu().numpy().reshape(-1), ex, dtype)
    eo, _, _ = orc.mixture_logdensity(ob, x.double().cpu().numpy().reshape(-1), orc.DENOM_FULL,
                                      db.logmasses.double().cpu().numpy(), slots=slots)
    assert_close(lw.cpu().numpy(), logt.astype(np.float64) - eo, dtype)
    ids = db.proposal_ids.cpu().numpy()
    assert np.array_equal(pid.cpu().numpy(), ids[slots])
    assert int(fail[0].item()) == int(np.count_nonzero(rs))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("d", [1, 3, 5, 16, 64])
@pytest.mark.parametrize("family", ["gaussian", "student"])
def test_draw_philox_matches_fill_then_draw(issm, orc, cuda, dtype, d, family):
    """Normals generated inside the draw kernel give bitwise the samples of
    fill_normals_at + draw, for stream offsets that split Philox blocks, with
    and without a device counter, over several 128-row tiles and a ragged one."""
    rng = np.random.default_rng(d)
    _, db, _ = make_bank(issm, orc, rng, d, 3, family, "factor", dtype, cuda)
    n, seed = 1000, 0xC0FFEE
    rn_stride, ru_stride = (8, 8) if family == "student" else (0, 0)
    T = lambda a: None if a is None else torch.tensor(a, device=cuda)  # noqa: E731
    rn = T(rng.normal(size=n * 8).astype(dtype)) if family == "student" else None
    ru = T(rng.random(size=n * 8).astype(dtype)) if family == "student" else None
    for counter_value, offset in ((None, 0), (None, 3), (7, 5), (4096, 0)):
        counter = None if counter_value is None else torch.tensor([counter_value], dtype=torch.int64, device=cuda)
        f1, f2 = issm.ops.new_failures(cuda), issm.ops.new_failures(cuda)
        if counter is None:
            normals = issm.ops.fill_normals(n * d, tdt(dtype), cuda, seed=seed, offset=offset)
        else:
            normals = issm.ops.fill_normals_at(n * d, tdt(dtype), cuda, seed, counter, offset)
        a = issm.ops.draw(db, normals, n, fixed_slot=1, radial_normals=rn, rn_stride=rn_stride,
                          radial_uniforms=ru, ru_stride=ru_stride, failures=f1)
        b = issm.ops.draw_philox(db, n, seed, counter, offset, fixed_slot=1, radial_normals=rn,
                                 rn_stride=rn_stride, radial_uniforms=ru, ru_stride=ru_stride, failures=f2)
        assert torch.equal(a, b), (counter_value, offset)
        assert torch.equal(f1, f2)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_amis_append_and_form_vs_oracle(issm, orc, cuda, dtype, golden):
    c = golden["amis_retrospective_mixture"]
    props = [issm.SphericalGaussian(dtype(m), dtype(s)) for m, s in zip(c["history_means"], c["history_scales"])]
    h = issm.pack_proposals(props, cuda)
    # a spherical history is packed as spherical; the recurrence is scale-form agnostic
    logcounts = torch.tensor(np.log(np.asarray(c["schedule"], dtype=np.float64)).astype(dtype), device=cuda)
    n1 = torch.tensor(np.asarray(c["normals"][0], dtype=dtype), device=cuda)
    n2 = torch.tensor(np.asarray(c["normals"][1], dtype=dtype), device=cuda)
    x = torch.empty(5, 1, dtype=tdt(dtype), device=cuda)
    lognum = torch.empty(5, dtype=tdt(dtype), device=cuda)
    fail = issm.ops.new_failures(cuda)
    issm.ops.draw(h, n1, 2, fixed_slot=0, out=x[:2])
    issm.ops.mixture_logdensity(h, issm.ops.denominator(issm.native.DENOM_PREFIX, logcounts, terms=1), x[:2],
                                fixed_slot=0, out=lognum[:2], failures=fail)
    issm.ops.draw(h, n2, 3, fixed_slot=1, out=x[2:])
    issm.ops.amis_append(h.ref(), 1, logcounts, x[:2], lognum[:2], fail)
    issm.ops.mixture_logdensity(h, issm.ops.denominator(issm.native.DENOM_PREFIX, logcounts, terms=2), x[2:],
                                fixed_slot=1, out=lognum[2:], failures=fail)
    lt = -(x[:, 0] ** 2) / 3
    lw = torch.empty_like(lt)
    issm.ops.amis_form(lt, lognum, math.log(5), lw, failures=fail)
    eps = float(np.finfo(dtype).eps)
    assert np.allclose(x.double().cpu().numpy().reshape(-1), c["expected_samples"], rtol=16 * eps)
    assert np.allclose(lognum.double().cpu().numpy(), c["expected_lognumerators"], rtol=16 * eps)
    assert np.allclose(lw.double().cpu().numpy(), c["expected_logweights"], rtol=16 * eps, atol=16 * eps)
    assert int(fail[0].item()) == 0


# ---- reductions -----------------------------------------------------------------------------
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_golden_ess_extremes(issm, cuda, golden, dtype):
    big = float(np.finfo(dtype).max)
    vals = {"max": big, "-max": -big, "-inf": -np.inf}
    for case in golden["ess_extremes"]["cases"]:
        lw = torch.tensor(np.array([vals[v] for v in case["lw"]], dtype=dtype), device=cuda)
        res = issm.WeightedSamples(lw.reshape(-1, 1), lw)
        assert issm.effective_sample_size(res) == case["ess"]
        logz = issm.lognormalizer(res)
        assert (logz == -np.inf) if case.get("logz") == "-inf" else np.isfinite(logz)


def test_golden_stable_lognormalizer(issm, cuda, golden):
    c = golden["stable_lognormalizer"]
    lw = torch.tensor([-np.inf if v == "-inf" else v for v in c["logweights"]], dtype=torch.float64, device=cuda)
    res = issm.WeightedSamples(torch.tensor([[1.0], [2.0], [3.0]], dtype=torch.float64, device=cuda), lw)
    assert issm.lognormalizer(res) == pytest.approx(c["expected_logz"], rel=4 * EPS64)
    assert np.allclose(issm.normalized_weights(res).cpu().numpy(), c["expected_weights"], rtol=4 * EPS64)
    sh = issm.WeightedSamples(torch.tensor([[1.0], [3.0]], dtype=torch.float64, device=cuda),
                              torch.tensor(c["shifted"], dtype=torch.float64, device=cuda))
    assert issm.normalized_weights(sh).cpu().numpy().tolist() == c["shifted_weights"]
    assert float(issm.mean(sh)[0]) == c["shifted_mean"]


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("n", [1, 2, 255, 4097, 1_000_003])
def test_summary_and_normalize_vs_oracle(issm, orc, cuda, dtype, n):
    rng = np.random.default_rng(n)
    lw = (rng.normal(size=n) * 4).astype(dtype)
    lw[rng.random(n) < 0.1] = -np.inf
    if n > 1:
        lw[0] = 3.0
    t = torch.tensor(lw, device=cuda)
    sm = issm.ops.logweight_summary(t).cpu().numpy()
    ref = orc.logweight_summary(lw.astype(np.float64))
    assert sm[0] == ref[0]
    rt = 1e-12 if dtype == np.float64 else 2e-6
    assert sm[1] == pytest.approx(ref[1], rel=rt) and sm[2] == pytest.approx(ref[2], rel=rt)
    w = issm.ops.normalize(t, torch.tensor(sm, device=cuda)).double().cpu().numpy()
    assert np.allclose(w, orc.normalize(lw.astype(np.float64)), rtol=rt * 10, atol=1e-300 if dtype == np.float64 else 1e-30)


def test_summary_full_size_properties(issm, cuda):
    """4M+ samples: the summary is invariant to permutation and to a shift of
    every log weight (max and sums move together)."""
    n = 4_194_304 + 17
    g = torch.Generator(device=cuda).manual_seed(3)
    lw = torch.randn(n, device=cuda, generator=g) * 5
    a = issm.ops.logweight_summary(lw).cpu().numpy()
    b = issm.ops.logweight_summary(lw[torch.randperm(n, device=cuda, generator=g)]).cpu().numpy()
    c = issm.ops.logweight_summary(lw + 7.0).cpu().numpy()
    # FP32 exponentials are taken about per-thread running maxima, so the
    # grouping changes them at the 1e-7 level; the FP64 sums add nothing more.
    assert a[0] == b[0] and a[1] == pytest.approx(b[1], rel=1e-6) and a[2] == pytest.approx(b[2], rel=1e-6)
    assert c[0] == pytest.approx(a[0] + 7.0, rel=1e-7)
    assert c[1] == pytest.approx(a[1], rel=1e-5)


# ---- resampling ---------------------------------------------------------------------------------
def test_golden_multinomial_select(issm, cuda, golden):
    c = golden["multinomial_select"]
    for dtype in (np.float32, np.float64):
        cdf = torch.tensor(np.asarray(c["cdf"], dtype=dtype), device=cuda)
        lw = torch.log(torch.tensor(np.asarray(c["weights"], dtype=dtype), device=cuda))
        u = torch.tensor(np.asarray(c["uniforms"], dtype=dtype), device=cuda)
        anc = issm.ops.resample_select(cdf, lw, u)
        assert anc.cpu().tolist() == c["expected"]
        samples = torch.tensor(np.asarray(c["samples"], dtype=dtype), device=cuda)
        cand = issm.ops.gather(samples, anc)
        assert torch.equal(cand, samples[anc - 1])


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_golden_multinomial_plateaus(issm, cuda, golden, dtype):
    from test_oracle_golden import _plateau_uniforms

    for case in golden["multinomial_plateaus"]["cases"]:
        cdf = np.array(case["cdf"], dtype=dtype)
        with np.errstate(divide="ignore"):
            lw = np.log(np.diff(np.concatenate([[0], cdf]))).astype(dtype)
        u = np.array(_plateau_uniforms(case["uniforms"], dtype), dtype=dtype)
        anc = issm.ops.resample_select(torch.tensor(cdf, device=cuda), torch.tensor(lw, device=cuda),
                                       torch.tensor(u, device=cuda))
        assert anc.cpu().tolist() == case["expected"]


def test_golden_zero_mass_support(issm, orc, cuda, golden):
    c = golden["zero_mass_support"]
    lw = np.array([-np.inf if v == "-inf" else v for v in c["logweights"]], dtype=np.float32)
    cdf = issm.ops.resampling_cdf(torch.tensor(lw, device=cuda))
    assert np.array_equal(cdf.cpu().numpy(), orc.resampling_cdf(lw, np.float32))
    u = torch.tensor([0.0, 0.5, F32_PREV1], dtype=torch.float32, device=cuda)
    anc = issm.ops.resample_select(cdf, torch.tensor(lw, device=cuda), u)
    assert anc.cpu().tolist() == c["expected"]
    t = golden["zero_mass_tail"]
    lw = np.full(t["n"], -np.inf, dtype=np.float32)
    for k, v in t["finite"].items():
        lw[int(k) - 1] = np.float32(v)
    tl = torch.tensor(lw, device=cuda)
    cdf = issm.ops.resampling_cdf(tl)
    sel = issm.ops.resample_select(cdf, tl, torch.tensor([F32_PREV1], device=cuda)).item()
    assert np.isfinite(lw[sel - 1])


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("n", [1, 3, 1000, 65537, 300_001])
def test_fixed_point_resampling_bit_exact(issm, orc, cuda, dtype, n):
    rng = np.random.default_rng(n + 1)
    lw = (rng.normal(size=n) * 3).astype(dtype)
    lw[rng.random(n) < 0.05] = -np.inf
    lw[n // 2] = 1.0
    t = torch.tensor(lw, device=cuda)
    u = rng.random(size=max(1, n // 3))
    anc = issm.ops.resample_multinomial(t, torch.tensor(u, device=cuda)).cpu().numpy()
    assert np.array_equal(anc, orc.resample_multinomial_fixed(lw.astype(np.float64), u))
    us = float(rng.random())
    sys_anc = issm.ops.resample_systematic(t, us, n).cpu().numpy()
    assert np.array_equal(sys_anc, orc.resample_systematic_fixed(lw.astype(np.float64), us, n))
    assert np.all(np.isfinite(lw[anc - 1])) and np.all(np.diff(sys_anc) >= 0)


def test_systematic_full_size_properties(issm, cuda):
    """N = 4,194,304: ancestors sorted, every zero-weight sample unselected,
    each sample's count within one of its expected share n w_i."""
    n = 4_194_304
    g = torch.Generator(device=cuda).manual_seed(9)
    lw = torch.randn(n, device=cuda, generator=g, dtype=torch.float32) * 2
    lw[::1000] = -float("inf")
    anc = issm.ops.resample_systematic(lw, 0.6180339887, n)
    assert bool(torch.all(anc[1:] >= anc[:-1]))
    counts = torch.bincount(anc - 1, minlength=n).double()
    sm = issm.ops.logweight_summary(lw)
    w = issm.ops.normalize(lw, sm).double()
    assert float((counts - w * n).abs().max()) <= 1.0 + 1e-6
    assert int(counts[::1000].sum()) == 0


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_local_resample_vs_oracle(issm, orc, cuda, dtype):
    rng = np.random.default_rng(11)
    counts = np.array([1, 5, 300, 17, 1000, 2], dtype=np.int64)
    n = int(counts.sum())
    lw = (rng.normal(size=n) * 2).astype(dtype)
    lw[:1] = -np.inf  # first slot: no positive weight -> ancestor 0
    u = rng.random(size=counts.size).astype(dtype)
    x = rng.normal(size=(n, 3)).astype(dtype)
    anc, dst = issm.ops.local_resample(torch.tensor(lw, device=cuda), torch.tensor(counts, device=cuda),
                                       torch.tensor(u, device=cuda), torch.tensor(x, device=cuda))
    exp = orc.local_resample(lw.astype(np.float64), counts, u.astype(np.float64))
    assert np.array_equal(anc.cpu().numpy(), exp)
    ok = exp > 0
    assert np.array_equal(dst.cpu().numpy()[ok], x[exp[ok] - 1])


# ---- moments and fit ----------------------------------------------------------------------------
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_golden_literal_moments(issm, orc, cuda, golden, dtype):
    c = golden["amis_literal_moments"]["vector"]
    X = np.array(c["samples"], dtype=dtype)  # n x d
    lw = np.array(c["logweights"], dtype=dtype)
    tx, tl = torch.tensor(X, device=cuda), torch.tensor(lw, device=cuda)
    sm = issm.ops.logweight_summary(tl)
    mean, cov = issm.ops.weighted_moments(tx, tl, sm, torch.zeros(2, dtype=torch.float64, device=cuda))
    em, ec, _ = orc.weighted_moments(X.astype(np.float64).reshape(-1), 2, lw.astype(np.float64))
    eps = float(np.finfo(dtype).eps)
    assert np.allclose(mean.cpu().numpy(), em, rtol=32 * eps)
    assert np.allclose(cov.cpu().numpy(), ec, rtol=64 * eps, atol=64 * eps)
    P = np.array(c["previous_factor"], dtype=dtype)
    prev = torch.tensor(np.ascontiguousarray(P.T), device=cuda)
    loc = torch.empty(2, dtype=tdt(dtype), device=cuda)
    fac = torch.empty(2, 2, dtype=tdt(dtype), device=cuda)
    ln = torch.empty(1, dtype=tdt(dtype), device=cuda)
    fail = issm.ops.new_failures(cuda)
    issm.ops.fit_factor(mean, cov, prev, loc, fac, ln, failures=fail)
    L = fac.double().cpu().numpy().T
    reg = math.sqrt(eps)
    expected_cov = ec + reg * np.trace(P.astype(np.float64) @ P.T.astype(np.float64)) / 2 * np.eye(2)
    assert np.allclose(L @ L.T, expected_cov, rtol=64 * eps, atol=64 * eps)
    assert int(fail[0].item()) == 0


@pytest.mark.parametrize("d", [1, 5, 9, 16, 33, 47, 64])
def test_moments_and_fit_vs_oracle(issm, orc, cuda, d):
    rng = np.random.default_rng(d)
    n = 20011
    A = rng.normal(size=(d, d))
    X = rng.normal(size=(n, d)) @ A.T + 3.0
    lw = rng.normal(size=n)
    tx, tl = torch.tensor(X, device=cuda), torch.tensor(lw, device=cuda)
    sm = issm.ops.logweight_summary(tl)
    shift = torch.full((d,), 2.5, dtype=torch.float64, device=cuda)
    mean, cov = issm.ops.weighted_moments(tx, tl, sm, shift)
    em, ec, _ = orc.weighted_moments(X.reshape(-1), d, lw)
    assert np.allclose(mean.cpu().numpy(), em, rtol=1e-11, atol=1e-11)
    assert np.allclose(cov.cpu().numpy(), ec, rtol=1e-10, atol=1e-10)
    prev = np.linalg.cholesky(np.cov(X.T).reshape(d, d) + np.eye(d)) if d > 1 else np.array([[1.3]])
    for dof in (0.0, 5.0):
        st, L, ln = orc.fit_factor(em, ec, prev, dof=dof,
                                   logconstant=orc.student_t_logconstant(dof, d) if dof else 0.0)
        loc = torch.empty(d, dtype=torch.float64, device=cuda)
        fac = torch.empty(d, d, dtype=torch.float64, device=cuda)
        lnt = torch.empty(1, dtype=torch.float64, device=cuda)
        issm.ops.fit_factor(mean, cov, torch.tensor(np.ascontiguousarray(prev.T), device=cuda), loc, fac, lnt,
                            dof=dof, logconstant=orc.student_t_logconstant(dof, d) if dof else 0.0)
        assert st == 0
        assert np.allclose(fac.cpu().numpy().T, L, rtol=1e-9, atol=1e-10)
        assert float(lnt.item()) == pytest.approx(ln, rel=1e-10)


def test_fit_failure_is_recorded(issm, cuda):
    d = 3
    mean = torch.zeros(d, dtype=torch.float64, device=cuda)
    cov = -torch.eye(d, dtype=torch.float64, device=cuda)  # not positive definite
    prev = torch.eye(d, dtype=torch.float64, device=cuda) * 1e-12
    loc = torch.empty(d, dtype=torch.float64, device=cuda)
    fac = torch.empty(d, d, dtype=torch.float64, device=cuda)
    ln = torch.empty(1, dtype=torch.float64, device=cuda)
    fail = issm.ops.new_failures(cuda)
    issm.ops.fit_factor(mean, cov, prev, loc, fac, ln, failures=fail, failure_index=42)
    f, _ = issm.ops.decode_failure(fail.cpu().numpy())
    assert f["count"] == 1 and f["first_logical_index"] == 42 and f["reason_bits"] == 0x2000


# ---- random streams, assignment and failures ------------------------------------------------------
def test_philox_normals_match_oracle(issm, orc, cuda):
    out = issm.ops.fill_normals(10001, torch.float64, cuda, seed=123, offset=77).cpu().numpy()
    exp = orc.philox_normals(123, 77, 10001)
    assert np.allclose(out, exp, rtol=1e-13, atol=1e-13)
    u = issm.ops.fill_uniforms(1001, torch.float64, cuda, seed=5, offset=3).cpu().numpy()
    assert np.array_equal(u, orc.philox_uniforms(5, 3, 1001))
    f = issm.ops.fill_normals(1 << 20, torch.float32, cuda, seed=9).double()
    assert abs(float(f.mean())) < 5e-3 and abs(float(f.std()) - 1.0) < 5e-3


def test_device_counter_offsets(issm, orc, cuda):
    """fill_*_at reads its Philox base from device memory; counter_advance
    moves it on the stream."""
    ctr = torch.tensor([70], dtype=torch.int64, device=cuda)
    out = issm.ops.fill_normals_at(4097, torch.float64, cuda, 123, ctr, offset=7).cpu().numpy()
    assert np.allclose(out, orc.philox_normals(123, 77, 4097), rtol=1e-13, atol=1e-13)
    issm.ops.counter_advance(ctr, 1000)
    assert int(ctr.item()) == 1070
    u = issm.ops.fill_uniforms_at(333, torch.float64, cuda, 5, ctr, offset=3).cpu().numpy()
    assert np.array_equal(u, orc.philox_uniforms(5, 1073, 333))
    f = issm.ops.fill_normals_at(1001, torch.float32, cuda, 9, ctr, offset=0)
    g = issm.ops.fill_normals(1001, torch.float32, cuda, seed=9, offset=1070)
    assert torch.equal(f, g)


@pytest.mark.parametrize("stratified", [True, False])
def test_static_assign_vs_oracle(issm, orc, cuda, stratified):
    rng = np.random.default_rng(2)
    cdf = np.cumsum(rng.dirichlet(np.ones(13)))
    cdf[-1] = 1.0
    u = rng.random(5000)
    slots = issm.ops.static_assign(torch.tensor(cdf, device=cuda), torch.tensor(u, device=cuda), stratified)
    assert np.array_equal(slots.cpu().numpy(), orc.static_assign(cdf, u, stratified))


def test_failure_records_target_and_weight(issm, cuda):
    lw = torch.zeros(6, dtype=torch.float64, device=cuda)
    vals = torch.tensor([0.0, float("nan"), float("inf"), 1.0, 2.0, -3.0], dtype=torch.float64, device=cuda)
    fail = issm.ops.new_failures(cuda)
    issm.ops.add_target_values(lw, vals, fail)
    f, draw = issm.ops.decode_failure(fail.cpu().numpy())
    assert f["count"] == 2 and f["first_logical_index"] == 2 and f["reason_bits"] == 0x0100
    assert draw["count"] == 0
    assert torch.isinf(lw[1]) and torch.isinf(lw[2]) and float(lw[3]) == 1.0


def test_student_t_draw_exhausted_is_recorded(issm, cuda):
    p = issm.FactorStudentT(5.0, np.zeros(2), np.eye(2))
    db = issm.pack(issm.ProposalBank([p]), cuda)
    n = 4
    normals = torch.zeros(n * 2, dtype=torch.float64, device=cuda)
    rn = torch.full((n * 8,), -100.0, dtype=torch.float64, device=cuda)  # every candidate rejected
    ru = torch.full((n * 8,), 0.5, dtype=torch.float64, device=cuda)
    fail = issm.ops.new_failures(cuda)
    issm.ops.draw(db, normals, n, fixed_slot=0, radial_normals=rn, rn_stride=8, radial_uniforms=ru, ru_stride=8,
                  failures=fail)
    f, draw = issm.ops.decode_failure(fail.cpu().numpy())
    assert f["count"] == 2 * n
    assert draw["count"] == 1 and draw["first_logical_index"] == 1
