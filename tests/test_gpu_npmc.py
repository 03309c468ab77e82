"""N-PMC (src/npmc_execution.jl) on the device against the FP64 oracle on
the same draws: per-round weights by the generating density, the clipping of
the isqrt(n) largest log weights to the (n - isqrt(n) + 1)-th smallest (a
device radix select, NaN last as Julia's sort), the clipped-weight ESS
(adaptation_ess) and the moment fits that follow."""
import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("n", [1, 2, 7, 1000, 65537])
def test_select_kth_and_clip_vs_sort(issm, cuda, dtype, n):
    rng = np.random.default_rng(n)
    v = rng.normal(size=n) * 10.0
    if n > 10:
        v[rng.choice(n, n // 10, replace=False)] = -np.inf
        v[rng.choice(n, 3, replace=False)] = np.inf
        v[rng.choice(n, 2, replace=False)] = np.nan
        v[:4] = [0.0, -0.0, 1e-40, -1e-40]  # signed zeros and subnormals order as values
    t = torch.tensor(v, dtype=dtype, device=cuda)
    host = t.double().cpu().numpy()
    order = np.sort(host)  # NaN last, as Julia's isless
    for k in sorted({1, n, (n + 1) // 2, n - math.isqrt(n) + 1}):
        got = float(issm.ops.select_kth(t, k).item())
        exp = order[k - 1]
        assert (np.isnan(got) and np.isnan(exp)) or got == exp, (k, got, exp)
    clipped, thr = issm.ops.npmc_clip(t)
    kth = order[n - math.isqrt(n)]
    assert float(thr.item()) == kth or (np.isnan(kth) and np.isnan(float(thr.item())))
    exp = np.where(np.isnan(host) | np.isnan(kth), np.nan, np.minimum(host, kth))
    got = clipped.double().cpu().numpy()
    assert np.array_equal(np.isnan(got), np.isnan(exp)) and np.array_equal(got[~np.isnan(got)],
                                                                            exp[~np.isnan(exp)])


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_npmc_vs_oracle(issm, orc, cuda, dtype):
    """Multi-round N-PMC (d = 6, Student-t target) on fed normals."""
    from test_gpu_api import Prefilled

    rng = np.random.default_rng(23)
    d, rounds, size = 6, 5, 4000
    Lt = np.tril(rng.normal(size=(d, d)) * 0.3, -1) + np.diag(1 + np.abs(rng.normal(size=d)))
    target = issm.StudentTTarget(np.zeros(d), Lt, 5.0)
    p = issm.FactorGaussian(np.full(d, 0.5, dtype=dtype), (2.0 * np.eye(d)).astype(dtype))
    s = issm.prepare_sampler(3, target, issm.NPMC(p, rounds=rounds, round_size=size), device=cuda)
    normals = [rng.normal(size=size * d) for _ in range(rounds)]
    Prefilled(s, normals)
    res = issm.importance_sample_(s)
    reg = float(np.sqrt(np.finfo(dtype).eps))
    tgt = orc.TargetView(orc.TARGET_STUDENT_T, d, a=np.zeros(d), b=Lt, p0=5.0)
    out = orc.npmc_run(tgt, d, np.full(d, 0.5), 2.0 * np.eye(d), [size] * rounds, np.concatenate(normals),
                       regularization=reg)
    assert out["status"] == 0
    tol = 1e-9 if dtype == np.float64 else 2e-4
    assert np.allclose(res.samples.double().cpu().numpy().reshape(-1), out["samples"], rtol=tol, atol=tol)
    assert np.allclose(res.logweights.double().cpu().numpy(), out["logweights"], rtol=tol, atol=tol)
    assert np.allclose(res.diagnostics["round_ess"], out["round_ess"], rtol=tol * 10)
    assert np.allclose(res.diagnostics["round_lognormalizers"], out["round_logz"], rtol=tol * 10, atol=tol * 10)
    assert np.allclose(res.diagnostics["adaptation_ess"], out["adaptation_ess"], rtol=tol * 10)
    assert res.diagnostics["clipped_counts"] == [math.isqrt(size)] * rounds
    # clipping raised the ESS the fit sees
    assert np.all(np.asarray(res.diagnostics["adaptation_ess"]) >= np.asarray(res.diagnostics["round_ess"]) - 1e-6)
