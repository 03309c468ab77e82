"""The reference benchmark configurations other than the headline, as parity
cases: plain AMIS on a 5-D Gaussian mixture (FP64), the static-MIS
microbench at full size (N = 4,194,304, d = 16, K = 64), and DM-PMC on a
logistic-regression posterior (256 proposals x 64 samples). Inputs are seeded
synthetic data of the configurations' shapes and distributions."""
import math

import numpy as np
import pytest
import torch

from test_gpu_api import Prefilled
from test_gpu_kernels import oracle_bank

pytestmark = pytest.mark.gpu


def test_plain_amis_gaussian_mixture_d5(issm, orc, cuda):
    """20 rounds x 2,000 on an equal-weight mixture of three N(mu_j, I)
    (mu_j ~ N(0, 3^2 I)), initial SphericalGaussian(0, 3): the sampler matches
    the oracle on the same draws, and log Z-hat is close to the analytic 0."""
    d, rounds, size = 5, 20, 2000
    rng = np.random.default_rng(2026)
    means = rng.normal(scale=3.0, size=(3, d))
    target = issm.GaussianMixtureTarget(means)
    p = issm.SphericalGaussian(np.zeros(d), 3.0)
    s = issm.prepare_sampler(0, target, issm.AMIS(p, rounds=rounds, round_size=size), device=cuda)
    normals = rng.normal(size=(rounds, size * d))
    Prefilled(s, list(normals))
    res = issm.importance_sample_(s)
    tgt = orc.TargetView(orc.TARGET_GAUSS_MIX, d, j=3, a=means.T)
    out = orc.amis_run(tgt, d, np.zeros(d), 3.0 * np.eye(d), [size] * rounds, normals.reshape(-1),
                       regularization=math.sqrt(np.finfo(np.float64).eps))
    assert np.allclose(res.samples.cpu().numpy().reshape(-1), out["samples"], rtol=1e-9, atol=1e-9)
    assert np.allclose(res.logweights.cpu().numpy(), out["logweights"], rtol=1e-9, atol=1e-9)
    logz = float(res.diagnostics["round_lognormalizers"][-1])
    assert logz == pytest.approx(out["round_logz"][-1], rel=1e-9, abs=1e-9)
    assert abs(logz) < 0.3  # analytic log Z = 0; the estimate's sampling error at 40,000 samples


def test_static_mis_microbench_full_size(issm, orc, cuda):
    """N = 4,194,304 samples, d = 16, K = 64 full-covariance Gaussians
    (mu_k ~ N(0, 2^2 I), Sigma_k = A A^T / d + 0.1 I, alpha ~ Dirichlet(1)):
    balance-heuristic log q for every sample by the FP32 path and the BF16x3
    tensor-core form, agreeing everywhere; a 20,000-sample subset against the
    FP64 oracle; normalisation; systematic resampling of all N with one seeded
    uniform, bit-exact against the oracle."""
    n, d, k = 4_194_304, 16, 64
    rng = np.random.default_rng(16)
    props = []
    for _ in range(k):
        A = rng.normal(size=(d, d))
        L = np.linalg.cholesky(A @ A.T / d + 0.1 * np.eye(d))
        props.append(issm.FactorGaussian(rng.normal(scale=2.0, size=d).astype(np.float32), L.astype(np.float32)))
    alpha = rng.dirichlet(np.ones(k))
    db = issm.pack(issm.ProposalBank(props, alpha), cuda)
    u = issm.ops.fill_uniforms(n, torch.float32, cuda, seed=7)
    slots = issm.ops.static_assign(db.cdf, u, stratified=True)
    normals = issm.ops.fill_normals(n * d, torch.float32, cuda, seed=8)
    den = issm.ops.denominator(issm.native.DENOM_FULL, db.logmasses)
    fail = issm.ops.new_failures(cuda)
    x, lw, _ = issm.ops.mis_round(db, den, slots, normals, failures=fail)
    logq = -lw  # no target: log weights are -log q
    tc = issm.ops.mixture_logdensity(db, den, x, fixed_slot=0, failures=fail, precision=issm.native.PREC_BF16)
    torch.cuda.synchronize()
    issm.ops.check_tensor_core_errors(cuda)
    assert int(fail[0].item()) == 0
    err = ((tc.double() - logq.double()).abs() / logq.double().abs().clamp(min=1.0)).max().item()
    assert err < 5e-5, err
    # FP64 oracle on a subset (in the bank's packed slot order)
    idx = np.sort(rng.choice(n, 20_000, replace=False))
    xs = x[torch.tensor(idx, device=cuda)].double().cpu().numpy()
    ob = oracle_bank(orc, db)
    eo, _, _ = orc.mixture_logdensity(ob, xs.reshape(-1), orc.DENOM_FULL, db.logmasses.double().cpu().numpy())
    got = logq[torch.tensor(idx, device=cuda)].double().cpu().numpy()
    assert np.allclose(got, eo, rtol=2e-6, atol=2e-6)
    # normalisation and systematic resampling of all N
    sm = issm.ops.logweight_summary(lw)
    w = issm.ops.normalize(lw, sm)
    assert float(w.double().sum().item()) == pytest.approx(1.0, rel=1e-5)
    useed = 0.3183098861837907
    nb = issm.native.lib().issm_resample_workspace_bytes(n)
    ws = torch.empty(nb, dtype=torch.uint8, device=cuda)
    anc = torch.empty(n, dtype=torch.int64, device=cuda)
    issm.native.call("issm_resample_systematic", issm.native.ptr(lw), n, issm.native.F32, useed, n,
                     issm.native.ptr(anc), issm.native.ptr(ws), nb, issm.native.stream_ptr())
    a = anc.cpu().numpy()
    assert np.all(np.diff(a) >= 0) and a[0] >= 1 and a[-1] <= n
    assert np.array_equal(a, orc.resample_systematic_fixed(lw.double().cpu().numpy(), useed, n))


def test_dm_pmc_logistic_regression(issm, orc, cuda):
    """DM-PMC on a Bernoulli-logit posterior (n_obs = 10,000, p = 32,
    X ~ N(0,1), beta* ~ N(0, 1/p), prior N(0, 10 I)) with 256 spherical
    proposals x 64 samples per round, three rounds, global resampling: each
    round's log weights against the oracle's target and realized-mixture
    denominator, and the next locations against the oracle's selection."""
    n_obs, p, k, per = 10_000, 32, 256, 64
    rng = np.random.default_rng(3232)
    X = rng.normal(size=(n_obs, p))
    beta = rng.normal(scale=1 / np.sqrt(p), size=p)
    y = (rng.random(n_obs) < 1 / (1 + np.exp(-X @ beta))).astype(np.float64)
    target = issm.LogisticRegressionTarget(X, y, prior_var=10.0)
    centres = beta + rng.normal(scale=0.05, size=(k, p))
    bank = issm.ProposalBank([issm.SphericalGaussian(c, 0.05) for c in centres], np.ones(k))
    alg = issm.DeterministicMixturePMC(bank, rounds=3, round_size=k * per, resampling=issm.GlobalResampling())
    s = issm.prepare_sampler(5, target, alg, device=cuda)
    res = issm.importance_sample_(s)
    db = s.bank
    counts = s.counts_host
    x_all = res.samples.cpu().numpy()
    lw_all = res.logweights.cpu().numpy()
    locs = s.location_history.cpu().numpy()

    def log_target(xs):
        # Bernoulli-logit log likelihood plus the N(0, 10 I) log prior, in FP64 chunks
        out = np.empty(xs.shape[0])
        for i in range(0, xs.shape[0], 1024):
            eta = X @ xs[i:i + 1024].T
            ll = (y[:, None] * eta - np.logaddexp(0.0, eta)).sum(axis=0)
            out[i:i + 1024] = ll - 0.5 * p * np.log(2 * np.pi * 10.0) - (xs[i:i + 1024] ** 2).sum(axis=1) / 20.0
        return out
    for r in range(3):
        lo, hi = int(s.offsets[r]), int(s.offsets[r + 1])
        ob = orc.BankView(p, orc.GAUSSIAN, orc.SCALE_SPHERICAL, locs[r], db.scales.double().cpu().numpy(),
                          db.lognormalizers.double().cpu().numpy())
        slots = np.repeat(np.arange(k, dtype=np.int32), counts[:, r])
        coef = np.log(counts[:, r] / float(s.schedule[r]))
        x = x_all[lo:hi]
        den, _, _ = orc.mixture_logdensity(ob, x.reshape(-1), orc.DENOM_FULL, coef, slots=slots)
        tgt = log_target(x)
        assert np.allclose(lw_all[lo:hi], tgt - den, rtol=1e-9, atol=1e-7)
        u = s.resample_uniform_history[r].cpu().numpy()
        anc = orc.resample_multinomial_fixed(lw_all[lo:hi], u)
        nxt = locs[r + 1] if r < 2 else s.committed_locations.cpu().numpy()
        assert np.array_equal(nxt, x[anc - 1])
