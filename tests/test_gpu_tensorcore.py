"""tcgen05 descriptor encodings, pinned by exact small-integer GEMMs, and the
tensor-core forms of the mixture density against the FP64 oracle."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("layout", [0, 1])
@pytest.mark.parametrize("kind", ["bf16", "tf32"])
@pytest.mark.parametrize("n,k", [(16, 16), (64, 32), (80, 64), (128, 48), (192, 64), (256, 64)])
def test_tc_gemm_selftest_exact(issm, cuda, kind, n, k, layout):
    _selftest(issm, cuda, kind, n, k, layout)


@pytest.mark.parametrize("n,k", [(16, 16), (80, 64), (80, 128), (256, 48)])
def test_tc_gemm_selftest_mn_major(issm, cuda, n, k):
    """MN-major bf16 staging (the weighted-moments kernel's layout): leading
    byte offset = K-group stride, stride byte offset = row-group stride."""
    _selftest(issm, cuda, "bf16", n, k, 2)


def _selftest(issm, cuda, kind, n, k, layout):
    prec = (issm.native.PREC_BF16 if kind == "bf16" else issm.native.PREC_TF32) | (layout << 8)
    g = torch.Generator(device=cuda).manual_seed(n * 131 + k)
    a = torch.randint(-4, 5, (128, k), generator=g, device=cuda).float()
    b = torch.randint(-4, 5, (n, k), generator=g, device=cuda).float()
    c = torch.full((128, n), float("nan"), device=cuda)
    status = torch.zeros(1, dtype=torch.int32, device=cuda)
    issm.native.call("issm_tc_selftest", issm.native.ptr(a), issm.native.ptr(b), issm.native.ptr(c), n, k, prec,
                     issm.native.ptr(status), issm.native.stream_ptr())
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    assert torch.equal(c, a @ b.T)


def _factor_bank(issm, rng, d, k, family, cuda, spread=1.5):
    props = []
    for _ in range(k):
        A = rng.normal(size=(d, d))
        L = np.linalg.cholesky(A @ A.T / d + 0.1 * np.eye(d)).astype(np.float32)
        mu = (rng.normal(size=d) * spread).astype(np.float32)
        if family == "gaussian":
            props.append(issm.FactorGaussian(mu, L))
        else:
            props.append(issm.FactorStudentT(np.float32(5.0), mu, L))
    return issm.pack_proposals(props, cuda)


# relative to max(1, |value|): TF32 keeps ~11 bits per product, bf16 x3 ~16
TOL = {"tf32": 4e-3, "bf16": 5e-5}


@pytest.mark.parametrize("prec", ["tf32", "bf16"])
@pytest.mark.parametrize("d,k,family", [(5, 3, "gaussian"), (16, 8, "gaussian"), (33, 5, "student"),
                                        (64, 12, "gaussian"), (64, 40, "student")])
@pytest.mark.parametrize("denom", ["prefix", "full", "generating"])
def test_tc_mixture_vs_oracle(issm, orc, cuda, prec, d, k, family, denom):
    from test_gpu_kernels import oracle_bank

    rng = np.random.default_rng(d * 100 + k)
    db = _factor_bank(issm, rng, d, k, family, cuda)
    ob = oracle_bank(orc, db)
    slot = k - 1 if denom == "prefix" else k // 2
    n = 3001
    L = db.scales[slot].double().cpu().numpy().T
    x = (db.locations[slot].double().cpu().numpy() + rng.normal(size=(n, d)) @ L.T).astype(np.float32)
    coef = torch.log(torch.softmax(torch.tensor(rng.normal(size=k), device=cuda), 0)).float().contiguous()
    kind = {"prefix": issm.native.DENOM_PREFIX, "full": issm.native.DENOM_FULL,
            "generating": issm.native.DENOM_GENERATING}[denom]
    terms = k if denom == "prefix" else 0
    den = issm.ops.denominator(kind, coef, terms=terms)
    precision = issm.native.PREC_TF32 if prec == "tf32" else issm.native.PREC_BF16
    fail = issm.ops.new_failures(cuda)
    out, gen = issm.ops.mixture_logdensity(db, den, torch.tensor(x, device=cuda), fixed_slot=slot, failures=fail,
                                           generating=True, precision=precision)
    torch.cuda.synchronize()
    issm.ops.check_tensor_core_errors(cuda)
    eo, eg, _ = orc.mixture_logdensity(ob, x.astype(np.float64).reshape(-1), kind, coef.double().cpu().numpy(),
                                       terms=terms, fixed_slot=slot)
    got = out.double().cpu().numpy()
    err = np.abs(got - eo) / np.maximum(1.0, np.abs(eo))
    assert err.max() <= TOL[prec], err.max()
    gerr = np.abs(gen.double().cpu().numpy() - eg) / np.maximum(1.0, np.abs(eg))
    assert gerr.max() <= TOL[prec]
    assert int(fail[0].item()) == 0


@pytest.mark.parametrize("prec", ["tf32", "bf16"])
@pytest.mark.parametrize("d", [8, 64])
def test_tc_amis_append_vs_oracle(issm, orc, cuda, prec, d):
    from test_gpu_kernels import oracle_bank

    rng = np.random.default_rng(d)
    k = 6
    db = _factor_bank(issm, rng, d, k, "gaussian", cuda)
    ob = oracle_bank(orc, db)
    n = 70001
    x = (rng.normal(size=(n, d)) * 2).astype(np.float32)
    lognum = (rng.normal(size=n) - 50).astype(np.float32)
    logcounts = torch.tensor(np.log(np.arange(1, k + 1, dtype=np.float32)), device=cuda)
    slot = 4
    t = torch.tensor(lognum, device=cuda)
    precision = issm.native.PREC_TF32 if prec == "tf32" else issm.native.PREC_BF16
    issm.ops.amis_append(db.ref(), slot, logcounts, torch.tensor(x, device=cuda), t, precision=precision,
                         count=k)
    torch.cuda.synchronize()
    issm.ops.check_tensor_core_errors(cuda)
    lq, _, _ = orc.mixture_logdensity(ob, x.astype(np.float64).reshape(-1), orc.DENOM_GENERATING, slots=None,
                                      fixed_slot=slot)
    exp = np.logaddexp(lognum.astype(np.float64), float(logcounts[slot]) + lq)
    err = np.abs(t.double().cpu().numpy() - exp) / np.maximum(1.0, np.abs(exp))
    assert err.max() <= TOL[prec]


@pytest.mark.parametrize("prec", ["tf32", "bf16"])
@pytest.mark.parametrize("d,n", [(3, 1000), (16, 100003), (64, 262145)])
def test_tc_moments_vs_oracle(issm, orc, cuda, prec, d, n):
    rng = np.random.default_rng(n)
    A = rng.normal(size=(d, d)) / np.sqrt(d)
    X = (rng.normal(size=(n, d)) @ A.T + 1.0).astype(np.float32)
    lw = (rng.normal(size=n) * 0.5).astype(np.float32)
    tx, tl = torch.tensor(X, device=cuda), torch.tensor(lw, device=cuda)
    sm = issm.ops.logweight_summary(tl)
    shift = torch.full((d,), 0.9, dtype=torch.float64, device=cuda)
    precision = issm.native.PREC_TF32 if prec == "tf32" else issm.native.PREC_BF16
    mean, cov = issm.ops.weighted_moments(tx, tl, sm, shift, precision=precision)
    torch.cuda.synchronize()
    issm.ops.check_tensor_core_errors(cuda)
    em, ec, _ = orc.weighted_moments(X.astype(np.float64).reshape(-1), d, lw.astype(np.float64))
    scale = np.sqrt(np.outer(np.diag(ec), np.diag(ec)))
    # both forms contract bf16 x3 splits (about 16 bits per product) with FP32
    # accumulation in tensor memory
    tol = 2e-4
    assert np.max(np.abs(mean.cpu().numpy() - em) / np.sqrt(np.diag(ec))) < tol
    assert np.max(np.abs(cov.cpu().numpy() - ec) / scale) < tol


@pytest.mark.parametrize("d", [9, 33, 64])
def test_tc_moments_far_centre_and_low_ess(issm, orc, cuda, d):
    """A centre hundreds of standard deviations from the weighted mean (the
    one-pass sums cancel; the centred second pass must take over) and a
    weighted covariance of rank below d (a handful of samples carry the
    weight): the covariance matches the oracle on the spread's scale and
    stays semidefinite to FP32 rounding of the Gram sums."""
    rng = np.random.default_rng(d)
    n = 40_000
    X = (rng.normal(size=(n, d)) * 0.02 + 0.7).astype(np.float32)
    for case in ("far", "low_ess"):
        lw = (rng.normal(size=n) * 0.5).astype(np.float32)
        if case == "low_ess":
            lw = np.full(n, -60.0, dtype=np.float32)
            lw[rng.choice(n, d // 3 + 1, replace=False)] = rng.normal(size=d // 3 + 1).astype(np.float32)
        tx, tl = torch.tensor(X, device=cuda), torch.tensor(lw, device=cuda)
        sm = issm.ops.logweight_summary(tl)
        shift = torch.full((d,), -8.0 if case == "far" else 0.7, dtype=torch.float64, device=cuda)
        mean, cov = issm.ops.weighted_moments(tx, tl, sm, shift, precision=issm.native.PREC_BF16)
        torch.cuda.synchronize()
        issm.ops.check_tensor_core_errors(cuda)
        em, ec, _ = orc.weighted_moments(X.astype(np.float64).reshape(-1), d, lw.astype(np.float64))
        c = cov.cpu().numpy()
        spread = float(np.trace(ec)) / d
        assert np.max(np.abs(mean.cpu().numpy() - em)) < 2e-4 * np.sqrt(spread), case
        assert np.max(np.abs(c - ec)) < 2e-4 * spread, case
        assert np.linalg.eigvalsh(0.5 * (c + c.T)).min() > -1e-5 * spread, case


@pytest.mark.parametrize("prec", ["tf32", "bf16"])
def test_tc_amis_matches_native_form(issm, cuda, prec):
    """Same draws, FP32 SIMT vs tensor-core forms: log Z and the posterior
    mean agree to well inside the estimator's own error."""
    rng = np.random.default_rng(5)
    d = 16
    Lt = np.tril(rng.normal(size=(d, d)) * 0.3, -1) + np.diag(1 + np.abs(rng.normal(size=d)))
    target = issm.StudentTTarget(np.zeros(d), Lt, 5.0)
    p = issm.FactorGaussian(np.zeros(d, dtype=np.float32), (2.5 * np.eye(d)).astype(np.float32))
    out = {}
    for name, precision in (("native", issm.native.PREC_NATIVE),
                            (prec, issm.native.PREC_TF32 if prec == "tf32" else issm.native.PREC_BF16)):
        s = issm.prepare_sampler(7, target, issm.AMIS(p, rounds=8, round_size=20000), device=cuda,
                                 precision=precision)
        r = issm.importance_sample_(s)
        out[name] = (r.diagnostics["round_lognormalizers"][-1], issm.mean(r).cpu().numpy())
    assert abs(out["native"][0] - out[prec][0]) < 2e-2
    assert np.max(np.abs(out["native"][1] - out[prec][1])) < 5e-2


@pytest.mark.parametrize("d", [3, 16, 40, 64])
def test_fit_factor_writes_inverse(issm, orc, cuda, d):
    """The FP64 blocked Cholesky matches the oracle and the FP32 inverse it
    writes for the tensor-core forms inverts the stored factor."""
    rng = np.random.default_rng(d + 1)
    A = rng.normal(size=(d, d))
    cov = A @ A.T / d + 0.3 * np.eye(d)
    mean = rng.normal(size=d)
    prev = np.linalg.cholesky(cov + np.eye(d)).astype(np.float32)
    st, L, ln = orc.fit_factor(mean, cov, prev.astype(np.float64), regularization=float(np.sqrt(np.finfo(np.float32).eps)))
    dp = 16 if d <= 16 else 32 if d <= 32 else 64
    loc = torch.empty(d, dtype=torch.float32, device=cuda)
    fac = torch.empty(d, d, dtype=torch.float32, device=cuda)
    lnt = torch.empty(1, dtype=torch.float32, device=cuda)
    inv = torch.full((dp, dp), float("nan"), dtype=torch.float32, device=cuda)
    fail = issm.ops.new_failures(cuda)
    issm.ops.fit_factor(torch.tensor(mean, device=cuda), torch.tensor(cov, device=cuda),
                        torch.tensor(np.ascontiguousarray(prev.T), device=cuda), loc, fac, lnt, failures=fail,
                        out_inverse=inv)
    torch.cuda.synchronize()
    assert st == 0 and int(fail[0].item()) == 0
    Lg = fac.double().cpu().numpy().T
    assert np.allclose(Lg, L, rtol=1e-6, atol=1e-6)
    W = inv.double().cpu().numpy()
    assert np.all(W[d:, :] == 0) and np.all(W[:, d:] == 0)
    assert np.allclose(W[:d, :d] @ Lg, np.eye(d), atol=1e-4)
