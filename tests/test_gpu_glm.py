"""The regression targets' likelihood on the tensor cores (issm_glm_*):
X beta for every (sample, observation) pair as a tcgen05 GEMM with the
Bernoulli-logit or Gaussian log-likelihood reduced in the epilogue, against
the same log target in FP64 (numpy) and against the SIMT kernel. The batch
callback it replaces is src/batched_targets.jl:54-214 with the user batch of
examples/batched_linear_regression.jl:18-37."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

# largest |error| / max(1, |log target|) per form: bf16 x3 keeps about 16
# bits per product, tf32 11, one bf16 product 8. The Gaussian likelihood
# squares the residual y - x'beta, which doubles the relative error of a
# small residual, and the FP32 sum over observations adds about 1e-6
# (the SIMT FP32 path is held to 1e-5 for the same reason)
TOL = {"bf16": 1e-5, "tf32": 2e-3, "bf16x1": 1e-2}


def _fp64_logtarget(kind, X, y, B, sigma, prior_var):
    eta = B @ X.T  # (n, nobs)
    d = X.shape[1]
    prior = -0.5 * d * (np.log(2 * np.pi) + np.log(prior_var)) - np.sum(B * B, axis=1) / (2 * prior_var)
    if kind == "logistic":
        ll = np.sum(y[None, :] * eta - np.logaddexp(0.0, eta), axis=1)
        return ll + prior
    r = y[None, :] - eta
    nobs = X.shape[0]
    return -0.5 * nobs * (np.log(2 * np.pi) + 2 * np.log(sigma)) - np.sum(r * r, axis=1) / (2 * sigma ** 2) + prior


@pytest.mark.parametrize("form", ["bf16", "tf32", "bf16x1"])
@pytest.mark.parametrize("kind", ["logistic", "linreg"])
@pytest.mark.parametrize("d,nobs,n", [(3, 50, 1), (16, 257, 129), (32, 10_000, 5000), (64, 700, 300)])
def test_glm_tensor_core_vs_fp64(issm, cuda, form, kind, d, nobs, n):
    rng = np.random.default_rng(d * 1000 + nobs)
    X = rng.normal(size=(nobs, d))
    beta_true = rng.normal(size=d) / np.sqrt(d)
    if kind == "logistic":
        y = (rng.random(nobs) < 1 / (1 + np.exp(-X @ beta_true))).astype(np.float64)
        target = issm.LogisticRegressionTarget(X, y, prior_var=10.0)
        sigma, pv = 1.0, 10.0
    else:
        y = X @ beta_true + 0.5 * rng.normal(size=nobs)
        target = issm.LinearRegressionTarget(X, y, sigma=0.5, prior_var=1.0)
        sigma, pv = 0.5, 1.0
    B = (beta_true + rng.normal(size=(n, d)) * 0.2).astype(np.float32)
    prec = {"bf16": issm.native.PREC_BF16, "tf32": issm.native.PREC_TF32, "bf16x1": issm.native.PREC_BF16X1}[form]
    bound = target.bind(cuda, torch.float32)
    tb = torch.tensor(B, device=cuda)
    got = bound.evaluate(tb, precision=prec)
    simt = bound.evaluate(tb, precision=issm.native.PREC_NATIVE)
    torch.cuda.synchronize()
    err_word = issm.native.scoped_workspace(cuda, "glm")
    assert err_word is not None and int(err_word[:4].view(torch.int32).item()) == 0
    # the device computes in the FP32-rounded X, y and samples
    X32, y32 = X.astype(np.float32).astype(np.float64), y.astype(np.float32).astype(np.float64)
    exp = _fp64_logtarget(kind, X32, y32, B.astype(np.float64), sigma, pv)
    g = got.double().cpu().numpy()
    rel = np.abs(g - exp) / np.maximum(1.0, np.abs(exp))
    assert rel.max() <= TOL[form], f"{form} {kind}: max rel err {rel.max():.3e}"
    srel = np.abs(simt.double().cpu().numpy() - exp) / np.maximum(1.0, np.abs(exp))
    assert srel.max() <= 1e-5


def test_dm_pmc_logistic_c3_shape(issm, cuda):
    """DM-PMC on the Bernoulli-logit posterior at the C3 shape (n_obs =
    10,000, p = 32, 256 factor-Gaussian proposals x 64 samples, 50 rounds,
    global resampling) with the likelihood on the tensor cores (BF16 x3),
    beside the same run with the SIMT FP32 likelihood on the same draws:
    the per-round log Z and the final population agree to the likelihood's
    precision, and the posterior mean is close to the FP64 Laplace mode."""
    rng = np.random.default_rng(31)
    nobs, p, k, m, rounds = 10_000, 32, 256, 64, 50
    X = rng.normal(size=(nobs, p))
    beta = rng.normal(size=p) / np.sqrt(p)
    y = (rng.random(nobs) < 1 / (1 + np.exp(-X @ beta))).astype(np.float64)
    target = issm.LogisticRegressionTarget(X, y, prior_var=10.0)
    # proposals: centres from the prior, a fixed factor at the posterior scale
    scale = 1.0 / np.sqrt(nobs / 4.0)
    L = (scale * np.eye(p)).astype(np.float32)
    centres = rng.normal(size=(k, p)).astype(np.float32) * 0.3
    bank = issm.ProposalBank([issm.FactorGaussian(c, L) for c in centres])
    out = {}
    for form, tprec in (("bf16", issm.native.PREC_BF16), ("fp32", issm.native.PREC_NATIVE)):
        s = issm.prepare_sampler(5, target, issm.DeterministicMixturePMC(bank, rounds=rounds, round_size=k * m),
                                 device=cuda, target_precision=tprec)
        r = issm.importance_sample_(s)
        out[form] = (np.asarray(r.diagnostics["round_lognormalizers"]), s.committed_locations.double().cpu().numpy(),
                     issm.mean(r).cpu().numpy())
    dlz = np.abs(out["bf16"][0] - out["fp32"][0])
    # round 1 draws the same samples from the same bank: the two likelihood
    # forms differ by their arithmetic; later rounds resample, and tiny weight
    # differences pick other ancestors, so they agree statistically only
    assert dlz[0] < 0.05, dlz[0]
    assert np.all(np.isfinite(out["bf16"][0])) and np.median(dlz) < 1.0
    # the two posterior means agree within a few posterior standard deviations (about 0.02 here)
    assert np.max(np.abs(out["bf16"][2] - out["fp32"][2])) < 0.1
