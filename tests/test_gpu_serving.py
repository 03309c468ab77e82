"""Serving mix (continuous batching of independent Bayesian linear-regression
posteriors of uneven dimension and budget): every run gives bitwise the same
result alone and in the mix, and matches the conjugate analytic posterior."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _requests(issm, spec, seed=0):
    rng = np.random.default_rng(seed)
    reqs, truth = [], {}
    for rid, (d, n_obs, budget) in enumerate(spec):
        X = rng.normal(size=(n_obs, d))
        beta = rng.normal(size=d)
        y = X @ beta + 0.5 * rng.normal(size=n_obs)
        target = issm.LinearRegressionTarget(X, y, sigma=0.5, prior_var=1.0)
        mean, logz = target.analytic()
        A = X.T @ X / 0.25 + np.eye(d)
        truth[rid] = (mean, np.sqrt(np.diag(np.linalg.inv(A))), logz)
        p = issm.FactorGaussian(np.zeros(d, dtype=np.float32), np.eye(d, dtype=np.float32))
        reqs.append(issm.serving.ServeRequest(rid, target, p, rounds=4, round_size=budget // 4, seed=1000 + rid))
    return reqs, truth


SPEC = [(2, 50, 4_000), (9, 400, 20_000), (16, 120, 8_000), (33, 300, 40_000), (64, 1000, 24_000), (5, 2000, 12_000)]


def test_serving_mix_matches_alone_and_analytic(issm, cuda):
    reqs, truth = _requests(issm, SPEC)
    alone = {}
    for r in reqs:
        out = issm.serving.ServeLoop(cuda, max_inflight=1).run([r])
        alone[r.rid] = out[0]
    reqs2, _ = _requests(issm, SPEC)
    mixed = {res.rid: res for res in issm.serving.ServeLoop(cuda, max_inflight=4).run(reqs2)}
    assert sorted(mixed) == sorted(alone)
    for rid, a in alone.items():
        m = mixed[rid]
        assert np.array_equal(a.posterior_mean, m.posterior_mean)
        assert a.logz == m.logz and a.ess == m.ess
        mean, sd, logz = truth[rid]
        assert np.max(np.abs(m.posterior_mean - mean) / sd) < 0.25, rid
        assert abs(m.logz - logz) < 0.1, (rid, m.logz, logz)


def test_serving_admission_respects_memory_budget(issm, cuda):
    reqs, _ = _requests(issm, SPEC[:4], seed=3)
    biggest = max(r.footprint() for r in reqs)
    loop = issm.serving.ServeLoop(cuda, memory_budget=biggest, max_inflight=4)
    out = loop.run(reqs)
    assert len(out) == 4
    # with room for one run at a time the runs cannot overlap
    spans = sorted((r.start, r.end) for r in out)
    assert all(spans[i][1] <= spans[i + 1][0] + 1e-3 for i in range(len(spans) - 1))
    with pytest.raises(ValueError):
        issm.serving.ServeLoop(cuda, memory_budget=biggest // 2).run(reqs[:1] if reqs[0].footprint() > biggest // 2
                                                                     else [max(reqs, key=lambda r: r.footprint())])
