"""Pin the FP64 oracle to the reference's own known-answer tests.

Every case comes from tests/golden/reference_vectors.json, which re-enters the
literal inputs and expected outputs of the cited reference test.
"""
import math

import numpy as np
import pytest

EPS64 = np.finfo(np.float64).eps
F32_PREV1 = float(np.nextafter(np.float32(1), np.float32(0)))


def _bank_from_case(orc, c, dtype_max=None):
    d = len(c["location"])
    kind = c["kind"]
    family = orc.STUDENT_T if "dof" in c else orc.GAUSSIAN
    if kind == "factor":
        L = np.array(c["scale"], dtype=np.float64)
        logabsdet = float(np.sum(np.log(np.diag(L))))
        scales = L.reshape(-1, order="F")
        sk = orc.SCALE_FACTOR
    elif kind == "diagonal":
        s = np.array(c["scale"], dtype=np.float64)
        logabsdet = float(np.sum(np.log(s)))
        scales = s
        sk = orc.SCALE_DIAGONAL
    else:
        s = float(c["scale"][0])
        logabsdet = d * math.log(s)
        scales = np.array([s])
        sk = orc.SCALE_SPHERICAL
    if family == orc.STUDENT_T:
        lognorm = orc.student_t_logconstant(c["dof"], d) - logabsdet
        dofs = [c["dof"]]
        rr = None
        if kind == "factor":
            rr = [orc.range_risk_f(orc.factor_exponent_bound(np.array(c["scale"])), np.float64)]
    else:
        lognorm = orc.gaussian_lognormalizer(d, logabsdet)
        dofs, rr = None, None
    return orc.BankView(d, family, sk, c["location"], scales, [lognorm], dofs, rr)


def test_log_mixture_accumulator(orc, golden):
    c = golden["log_mixture_accumulator"]
    num = -math.inf
    for logcoef, q in c["steps"]:
        num = orc.lib().orc_logaddexp(num, logcoef + math.log(q))
    assert num == pytest.approx(c["expected_numerator"], rel=8 * EPS64)
    lw = c["logtarget"] - num + c["logtotal"]
    assert lw == pytest.approx(c["expected_logweight"], rel=8 * EPS64)


def test_packed_factor_primitives(orc, golden):
    c = golden["packed_factor_primitives"]
    L = np.array(c["factor"])
    lognorm = orc.gaussian_lognormalizer(2, float(np.sum(np.log(np.diag(L)))))
    bank = orc.BankView(2, orc.GAUSSIAN, orc.SCALE_FACTOR, c["location"], L.reshape(-1, order="F"), [lognorm])
    x, reasons = orc.draw(bank, c["normals"], fixed_slot=0)
    assert list(x) == c["expected_sample"]
    assert reasons[0] == 0
    lq = orc.component_logdensity(bank, 0, x)
    assert lq == pytest.approx(c["expected_logdensity"], rel=8 * EPS64)


@pytest.mark.parametrize("name", ["native_gaussian_analytic", "native_gaussian_range",
                                  "native_student_t_analytic", "native_student_t_subnormal"])
def test_native_densities(orc, golden, name):
    c = golden[name]
    for sub in c["cases"]:
        rtol = sub.get("rtol_eps", c["rtol_eps"]) * EPS64
        bank = _bank_from_case(orc, sub)
        got = orc.component_logdensity(bank, 0, sub["x"])
        assert got == pytest.approx(sub["expected"], rel=rtol, abs=1e-300), sub


def test_realized_mixture_denominator(orc, golden):
    c = golden["realized_mixture_denominator"]
    lognorm = orc.gaussian_lognormalizer(1, 0.0)
    bank = orc.BankView(1, orc.GAUSSIAN, orc.SCALE_SPHERICAL, c["locations"], c["scales"], [lognorm, lognorm])
    coef = np.array(c["coefficients"])  # rows = slots, columns = rounds
    for r in range(2):
        out, gen, rs = orc.mixture_logdensity(bank, c["x"], orc.DENOM_FULL, coef[:, r], slots=[0])
        assert out[0] == pytest.approx(c["expected"][r], rel=16 * EPS64)
        assert gen[0] == pytest.approx(c["expected_generating"], rel=16 * EPS64)
        assert rs[0] == 0


def test_multinomial_select(orc, golden):
    c = golden["multinomial_select"]
    anc = orc.resample_select(c["cdf"], np.log(c["weights"]), c["uniforms"])
    assert list(anc) == c["expected"]


def _plateau_uniforms(tag, dtype):
    nf = lambda v: float(np.nextafter(dtype(v), dtype(0)))  # noqa: E731
    up = lambda v: float(np.nextafter(dtype(v), dtype(1)))  # noqa: E731
    if tag == "plateau_a":
        return [0.0, nf(0.5), 0.5, nf(1.0)]
    if tag == "plateau_b":
        return [0.0, 0.25, up(0.25), nf(1.0)]
    return [1.0]


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_multinomial_plateaus(orc, golden, dtype):
    for case in golden["multinomial_plateaus"]["cases"]:
        cdf = np.array(case["cdf"], dtype=dtype)
        with np.errstate(divide="ignore"):
            lw = np.log(np.diff(np.concatenate([[0], cdf])))
        u = np.array(_plateau_uniforms(case["uniforms"], dtype), dtype=dtype)
        anc = orc.resample_select(cdf.astype(np.float64), lw.astype(np.float64), u.astype(np.float64))
        assert list(anc) == case["expected"]


def test_zero_mass_support(orc, golden):
    c = golden["zero_mass_support"]
    lw = np.array([-np.inf if v == "-inf" else v for v in c["logweights"]], dtype=np.float32)
    cdf = orc.resampling_cdf(lw, np.float32)
    u = np.array([0.0, 0.5, F32_PREV1], dtype=np.float32)
    anc = orc.resample_select(cdf.astype(np.float64), lw.astype(np.float64), u.astype(np.float64))
    assert list(anc) == c["expected"]
    t = golden["zero_mass_tail"]
    lw = np.full(t["n"], -np.inf, dtype=np.float32)
    for k, v in t["finite"].items():
        lw[int(k) - 1] = np.float32(v)
    cdf = orc.resampling_cdf(lw, np.float32)
    sel = orc.resample_select(cdf.astype(np.float64), lw.astype(np.float64), [F32_PREV1])[0]
    assert np.isfinite(lw[sel - 1])


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_ess_extremes(orc, golden, dtype):
    big = float(np.finfo(dtype).max)
    vals = {"max": big, "-max": -big, "-inf": -np.inf}
    for case in golden["ess_extremes"]["cases"]:
        lw = [vals[v] for v in case["lw"]]
        ess, logz = orc.summary_to_ess_logz(orc.logweight_summary(lw), len(lw))
        assert ess == case["ess"]
        if case.get("logz") == "-inf":
            assert logz == -np.inf
        else:
            assert np.isfinite(logz)


def test_stable_lognormalizer(orc, golden):
    c = golden["stable_lognormalizer"]
    lw = [-np.inf if v == "-inf" else v for v in c["logweights"]]
    ess, logz = orc.summary_to_ess_logz(orc.logweight_summary(lw), len(lw))
    assert logz == pytest.approx(c["expected_logz"], rel=4 * EPS64)
    assert np.allclose(orc.normalize(lw), c["expected_weights"], rtol=4 * EPS64, atol=0)
    w = orc.normalize(c["shifted"])
    assert list(w) == c["shifted_weights"]
    mean, cov, _ = orc.weighted_moments(c["shifted_samples"], 1, c["shifted"])
    # the moment fit scales deviations by sqrt(w) (src/adaptive_gaussian_execution.jl:268-273);
    # statistics.jl's var multiplies by w instead, hence a few ulps here.
    assert mean[0] == c["shifted_mean"]
    assert cov[0, 0] == pytest.approx(c["shifted_var"], rel=4 * EPS64)


def _spherical_history(orc, means, scales):
    lognorm = [orc.gaussian_lognormalizer(1, math.log(s)) for s in scales]
    return orc.BankView(1, orc.GAUSSIAN, orc.SCALE_SPHERICAL, means, scales, lognorm)


def test_amis_retrospective_mixture(orc, golden):
    """Round-by-round recurrence of src/amis_execution.jl:261-357 on fed draws."""
    c = golden["amis_retrospective_mixture"]
    hist = _spherical_history(orc, c["history_means"], c["history_scales"])
    logcounts = np.log(np.array(c["schedule"], dtype=np.float64))
    x1, _ = orc.draw(hist, c["normals"][0], fixed_slot=0)
    num1, _, _ = orc.mixture_logdensity(hist, x1, orc.DENOM_PREFIX, logcounts, terms=1, fixed_slot=0)
    x2, _ = orc.draw(hist, c["normals"][1], fixed_slot=1)
    old, _, _ = orc.mixture_logdensity(hist, x1, orc.DENOM_GENERATING, slots=[1, 1])
    num1 = np.array([orc.lib().orc_logaddexp(a, logcounts[1] + b) for a, b in zip(num1, old)])
    num2, _, _ = orc.mixture_logdensity(hist, x2, orc.DENOM_PREFIX, logcounts, terms=2, fixed_slot=1)
    xs = np.concatenate([x1, x2])
    nums = np.concatenate([num1, num2])
    lw = -(xs ** 2) / 3 - (nums - math.log(5))
    assert np.allclose(xs, c["expected_samples"], rtol=16 * EPS64, atol=0)
    assert np.allclose(nums, c["expected_lognumerators"], rtol=16 * EPS64, atol=0)
    assert np.allclose(lw, c["expected_logweights"], rtol=16 * EPS64, atol=0)


def test_amis_round_diagnostics(orc, golden):
    c = golden["amis_round_diagnostics"]
    tgt = orc.TargetView(orc.TARGET_STD_NORMAL, 1)
    normals = np.concatenate(c["normals"])
    out = orc.amis_run(tgt, 1, [c["proposal"]["location"]], [[c["proposal"]["scale"]]],
                       [c["round_size"]] * c["rounds"], normals)
    assert out["status"] == 0
    assert np.allclose(out["round_ess"], c["f64"]["ess"], rtol=16 * EPS64, atol=0)
    assert np.allclose(out["round_logz"], c["f64"]["logz"], rtol=16 * EPS64, atol=1e-16)


def test_amis_literal_moments(orc, golden):
    c = golden["amis_literal_moments"]
    sc = c["scalar"]
    mean, cov, w = orc.weighted_moments(sc["samples"], 1, sc["logweights"])
    ex = np.exp(np.array(sc["logweights"]) - max(sc["logweights"]))
    ex /= ex.sum()
    assert np.allclose(w, ex, rtol=8 * EPS64)
    m = float(np.dot(ex, sc["samples"]))
    var = float(np.dot(ex, (np.array(sc["samples"]) - m) ** 2)) + math.sqrt(EPS64) * sc["previous_scale"] ** 2
    st, L, ln = orc.fit_factor(mean, cov, [[sc["previous_scale"]]])
    assert st == 0
    assert mean[0] == pytest.approx(m, rel=8 * EPS64)
    assert L[0, 0] ** 2 == pytest.approx(var, rel=16 * EPS64)
    vc = c["vector"]
    X = np.array(vc["samples"]).T  # d x n
    mean, cov, w = orc.weighted_moments(X.reshape(-1, order="F"), 2, vc["logweights"])
    ex = np.exp(np.array(vc["logweights"]) - max(vc["logweights"]))
    ex /= ex.sum()
    mu = X @ ex
    Cm = ((X - mu[:, None]) * ex) @ (X - mu[:, None]).T
    P = np.array(vc["previous_factor"])
    Cm += math.sqrt(EPS64) * np.trace(P @ P.T) / 2 * np.eye(2)
    st, L, ln = orc.fit_factor(mean, cov, P)
    assert st == 0
    assert np.allclose(mean, mu, rtol=16 * EPS64)
    assert np.allclose(L @ L.T, Cm, rtol=32 * EPS64)
    assert ln == pytest.approx(orc.gaussian_lognormalizer(2, float(np.sum(np.log(np.diag(L))))))


def test_amis_complete_cpu(orc, golden):
    """Final retrospective weights of a 2-round scalar AMIS, restated in numpy."""
    c = golden["amis_complete_cpu"]
    mu0, s0 = c["proposal"]["location"], c["proposal"]["scale"]
    target = lambda x: -((x - 0.75) ** 2) / 3  # noqa: E731
    n1, n2 = np.array(c["normals"][0]), np.array(c["normals"][1])
    x1 = mu0 + s0 * n1
    logq = lambda x, m, s: -math.log(s) - 0.5 * math.log(2 * math.pi) - 0.5 * ((x - m) / s) ** 2  # noqa: E731
    lw1 = target(x1) - logq(x1, mu0, s0)
    w = np.exp(lw1 - lw1.max())
    w /= w.sum()
    m2 = float(np.dot(w, x1))
    v2 = float(np.dot(w, (x1 - m2) ** 2)) + math.sqrt(EPS64) * s0 ** 2
    s2 = math.sqrt(v2)
    x2 = m2 + s2 * n2
    xs = np.concatenate([x1, x2])
    den = np.logaddexp(math.log(3) + logq(xs, mu0, s0), math.log(3) + logq(xs, m2, s2)) - math.log(6)
    expected = target(xs) - den
    tgt = orc.TargetView(orc.TARGET_QUADRATIC, 1, a=[0.75], p0=3.0)
    out = orc.amis_run(tgt, 1, [mu0], [[s0]], c["schedule"], np.concatenate([n1, n2]))
    assert out["status"] == 0
    assert np.allclose(out["samples"], xs, rtol=8 * EPS64)
    assert np.allclose(out["logweights"], expected, rtol=64 * EPS64, atol=1e-14)


def test_det_exp_accuracy(orc):
    xs = np.concatenate([-np.logspace(-8, 2.8, 500), [0.0, -1e-300, -700.0]])
    got = np.array([orc.det_exp(x) for x in xs])
    ref = np.exp(xs)
    assert np.allclose(got, ref, rtol=4e-16, atol=0)


def test_fixed_cdf_properties(orc):
    rng = np.random.default_rng(3)
    lw = rng.normal(size=10001) * 3
    lw[::97] = -np.inf
    prefix = orc.fixed_prefix(lw)
    assert np.all(np.diff(prefix.astype(np.float64)) >= 0)
    u = rng.random(4000)
    anc = orc.resample_multinomial_fixed(lw, u)
    assert np.all(np.isfinite(lw[anc - 1]))
    sys_anc = orc.resample_systematic_fixed(lw, 0.37, 10001)
    assert np.all(np.diff(sys_anc) >= 0)
    assert np.all(np.isfinite(lw[sys_anc - 1]))
    # systematic counts stay within one of the expected share
    w = np.exp(lw - lw.max())
    w /= w.sum()
    counts = np.bincount(sys_anc - 1, minlength=lw.size)
    assert np.all(np.abs(counts - w * lw.size) <= 1.0 + 1e-9)


def _quantile_rule(values, weights, probabilities):
    """The StatsBase generic-weight interpolation rule as
    src/statistics.jl:247-283 states it, restated with numpy for one
    coordinate: NaN anywhere gives NaN; positive weights only, sorted by value
    (stable); threshold p (W - w_first) + w_first against the cumulative
    weights; linear interpolation between the bracketing values."""
    if np.any(np.isnan(values)):
        return np.full(len(probabilities), np.nan)
    keep = np.flatnonzero(weights != 0)
    order = keep[np.argsort(values[keep], kind="stable")]
    v, w = values[order], weights[order]
    cw = np.cumsum(w)
    total, first = cw[-1], w[0]
    out = []
    for p in probabilities:
        threshold = p * (total - first) + first
        upper = int(np.searchsorted(cw, threshold, side="right"))  # 0-based index of the first cw > threshold
        if upper >= len(v):
            out.append(v[-1])
            continue
        lower = upper - 1
        frac = (threshold - cw[lower]) / (cw[upper] - cw[lower])
        if frac == 0:
            out.append(v[lower])
            continue
        diff = v[upper] - v[lower]
        out.append(v[lower] + frac * diff if np.isfinite(diff) else (1 - frac) * v[lower] + frac * v[upper])
    return np.array(out)


def test_weighted_quantile_matches_the_rule(orc):
    """The oracle's weighted quantile (sort-based, FP64) equals an
    independent numpy restatement of the reference's rule: random weights,
    zero weights, ties, a NaN coordinate and the end probabilities."""
    rng = np.random.default_rng(12)
    n, d = 3000, 4
    x = rng.normal(size=(n, d))
    x[:, 1] = np.round(x[:, 1], 1)  # many ties
    x[5, 3] = np.nan
    w = rng.exponential(size=n)
    w[rng.random(n) < 0.2] = 0.0
    w /= w.sum()
    probs = [0.0, 0.01, 0.25, 0.5, 0.9, 0.999, 1.0]
    got = orc.weighted_quantile(x.reshape(-1), d, w, probs)
    for c in range(d):
        exp = _quantile_rule(x[:, c], w, probs)
        if c == 3:
            assert np.all(np.isnan(got[:, c]))
        else:
            assert np.allclose(got[:, c], exp, rtol=1e-12, atol=1e-12), (c, got[:, c], exp)
