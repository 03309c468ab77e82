"""Serving mix (continuous batching of independent Bayesian linear-regression
posteriors of uneven dimension and budget): every run gives bitwise the same
result alone and in the mix, and matches the conjugate analytic posterior."""
import numpy as np
import pytest
import torch

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
        post_cov = np.linalg.inv(A)
        truth[rid] = (mean, np.sqrt(np.diag(post_cov)), logz)
        # warm start: the posterior's Laplace form, displaced and widened by
        # 0.5/sqrt(d) of its scale so that the first round's ESS is a fair
        # fraction of the round in every dimension
        Lp = np.linalg.cholesky(post_cov)
        f = 0.5 / np.sqrt(d)
        p = issm.FactorGaussian((mean + f * Lp @ rng.normal(size=d)).astype(np.float32),
                                ((1 + f) * Lp).astype(np.float32))
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
    # at every admission the runs holding memory (admitted, not yet retired)
    # fit the budget together
    size = {r.rid: r.footprint() for r in reqs}
    for a in out:
        held = sum(size[b.rid] for b in out if b.start <= a.start < b.end)
        assert held <= biggest, (a.rid, held, biggest)
    with pytest.raises(ValueError):
        issm.serving.ServeLoop(cuda, memory_budget=biggest // 2).run(reqs[:1] if reqs[0].footprint() > biggest // 2
                                                                     else [max(reqs, key=lambda r: r.footprint())])


@pytest.mark.parametrize("d,n_obs,budget", [(33, 300, 40_000)])
def test_tc_amis_far_start_completes(issm, cuda, d, n_obs, budget):
    """AMIS in the BF16 tensor-core form from N(0, I) on a posterior whose
    scale is ~0.03: the weighted mean jumps hundreds of proposal scales and the
    early rounds carry an ESS below d. Every round's fit must succeed (the
    moments stay semidefinite and are re-centred when the one-pass sums
    cancel), and the result is a finite log evidence. (Further out, e.g.
    d = 64 at scale 0.016, three rounds of ESS ~ 1 shrink the FP32 ridge
    sqrt(eps(Float32)) tr(prev)/d below FP32 summation accuracy and the
    factorisation fails in any FP32 arithmetic, the reference's included.)"""
    rng = np.random.default_rng(d)
    X = rng.normal(size=(n_obs, d))
    y = X @ rng.normal(size=d) + 0.5 * rng.normal(size=n_obs)
    target = issm.LinearRegressionTarget(X, y, sigma=0.5, prior_var=1.0)
    p = issm.FactorGaussian(np.zeros(d, dtype=np.float32), np.eye(d, dtype=np.float32))
    s = issm.prepare_sampler(1000 + d, target, issm.AMIS(p, rounds=4, round_size=budget // 4), device=cuda,
                             precision=issm.native.PREC_BF16)
    res = issm.importance_sample_(s)
    issm.ops.check_tensor_core_errors(cuda)
    assert np.isfinite(float(res.diagnostics["round_lognormalizers"][-1]))


@pytest.mark.parametrize("kind", ["linreg", "student_t"])
@pytest.mark.parametrize("precision", ["native", "bf16"])
@pytest.mark.parametrize("d", [5, 33, 64])
def test_native_run_matches_host_round_loop(issm, cuda, precision, d, kind):
    """issm_amis_run issues the same library calls as the host round loop:
    samples, log weights, summaries and the final proposal are bitwise equal,
    for a target with its own kernel (linear regression: SIMT, or X beta on
    the tensor cores in the bf16 form) and for a radial-mixture target (a
    normalised Student-t, evaluated by the proposals' density kernels)."""
    rng = np.random.default_rng(d)
    X = rng.normal(size=(200, d))
    y = X @ rng.normal(size=d) + 0.5 * rng.normal(size=200)
    target = issm.LinearRegressionTarget(X, y, sigma=0.5, prior_var=1.0)
    mean, _ = target.analytic()
    L = np.linalg.cholesky(np.linalg.inv(X.T @ X / 0.25 + np.eye(d)))
    if kind == "student_t":
        target = issm.StudentTTarget(mean, L, 5.0)
    p = issm.FactorGaussian((mean + 0.1 * L @ rng.normal(size=d)).astype(np.float32), (1.2 * L).astype(np.float32))
    prec = issm.native.PREC_NATIVE if precision == "native" else issm.native.PREC_BF16
    out = []
    for native_run in (False, True):
        s = issm.prepare_sampler(77, target, issm.AMIS(p, rounds=4, round_size=[3000, 2000, 2500, 1999]),
                                 device=cuda, precision=prec, graphs=False)
        assert issm.sampler.native_body_eligible(s)
        s.busy = True
        if native_run:
            issm.sampler._native_body(s)
        else:
            issm.sampler._moment_body(s, False)
        res = issm.sampler._finish_moment(s, False)
        s.busy = False
        out.append((res.samples.cpu(), res.logweights.cpu(), s.summaries.cpu(), s.committed[0].cpu(),
                    s.committed[1].cpu(), s.offset))
    for a, b in zip(*out):
        if isinstance(a, torch.Tensor):
            assert torch.equal(a, b)
        else:
            assert a == b


def test_native_run_failure_matches_host_round_loop(issm, cuda):
    """A target that returns NaN fails round 1 with the same error through
    issm_amis_run as through the host round loop."""
    d = 4
    target = issm.QuadraticTarget(np.zeros(d), float("nan"))
    p = issm.FactorGaussian(np.zeros(d, dtype=np.float32), np.eye(d, dtype=np.float32))
    msgs = []
    for native_run in (False, True):
        s = issm.prepare_sampler(3, target, issm.AMIS(p, rounds=3, round_size=500), device=cuda, graphs=False)
        assert issm.sampler.native_body_eligible(s)
        s.busy = True
        (issm.sampler._native_body if native_run else (lambda x: issm.sampler._moment_body(x, False)))(s)
        with pytest.raises(issm.AMISRoundError) as e:
            issm.sampler._finish_moment_summary(s)
        s.busy = False
        msgs.append(str(e.value))
    assert msgs[0] == msgs[1] and "round 1" in msgs[0]


def test_serving_falls_back_for_student_t_proposals(issm, cuda):
    """Student-t proposal histories are not covered by issm_amis_run: the loop
    issues those runs from the host round loop, with the same results as a
    run alone."""
    rng = np.random.default_rng(9)
    d = 6
    X = rng.normal(size=(80, d))
    y = X @ rng.normal(size=d) + 0.5 * rng.normal(size=80)
    target = issm.LinearRegressionTarget(X, y, sigma=0.5, prior_var=1.0)
    mean, _ = target.analytic()
    L = np.linalg.cholesky(np.linalg.inv(X.T @ X / 0.25 + np.eye(d)))
    mk = lambda rid: issm.serving.ServeRequest(  # noqa: E731
        rid, target, issm.FactorStudentT(np.float32(7.0), mean.astype(np.float32), (1.3 * L).astype(np.float32)),
        rounds=3, round_size=2000, seed=40 + rid)
    s = issm.prepare_sampler(0, target, issm.AMIS(mk(0).proposal, rounds=3, round_size=2000), device=cuda)
    assert not issm.sampler.native_body_eligible(s)
    alone = issm.serving.ServeLoop(cuda, max_inflight=1).run([mk(0)])[0]
    mixed = {r.rid: r for r in issm.serving.ServeLoop(cuda, max_inflight=2).run([mk(0), mk(1)])}
    assert np.array_equal(alone.posterior_mean, mixed[0].posterior_mean) and alone.logz == mixed[0].logz
    assert np.all(np.isfinite(mixed[1].posterior_mean))


def test_failed_run_is_reported_and_the_loop_continues(issm, cuda):
    """A request whose target returns NaN fails in round 1: its result
    carries the AMISRoundError and NaN outputs, and the runs around it
    finish with the same numbers as alone."""
    reqs, _ = _requests(issm, SPEC[:3])
    d = 4
    bad = issm.serving.ServeRequest(99, issm.QuadraticTarget(np.zeros(d), float("nan")),
                                    issm.FactorGaussian(np.zeros(d, dtype=np.float32), np.eye(d, dtype=np.float32)),
                                    rounds=3, round_size=500, seed=5)
    out = {r.rid: r for r in issm.serving.ServeLoop(cuda, max_inflight=4).run(reqs[:1] + [bad] + reqs[1:])}
    assert isinstance(out[99].error, issm.AMISRoundError) and np.all(np.isnan(out[99].posterior_mean))
    reqs2, _ = _requests(issm, SPEC[:3])
    for r in reqs2:
        alone = issm.serving.ServeLoop(cuda, max_inflight=1).run([r])[0]
        assert out[r.rid].error is None
        assert np.array_equal(out[r.rid].posterior_mean, alone.posterior_mean) and out[r.rid].logz == alone.logz


def test_launch_failure_is_reported_and_the_loop_continues(issm, cuda):
    """A request that cannot be issued (its batch target raises while the
    run's launches are being queued) is reported with that error and NaN
    outputs; its slot and memory return to the loop and the other runs
    finish with their numbers alone."""
    reqs, _ = _requests(issm, SPEC[:2])
    d = 4

    def broken(samples):
        raise ValueError("target evaluation failed")

    bad = issm.serving.ServeRequest(77, issm.LogTarget(batch=broken),
                                    issm.FactorGaussian(np.zeros(d, dtype=np.float32), np.eye(d, dtype=np.float32)),
                                    rounds=2, round_size=500, seed=3)
    out = {r.rid: r for r in issm.serving.ServeLoop(cuda, max_inflight=2).run([bad] + reqs)}
    assert isinstance(out[77].error, ValueError) and np.all(np.isnan(out[77].posterior_mean))
    reqs2, _ = _requests(issm, SPEC[:2])
    for r in reqs2:
        alone = issm.serving.ServeLoop(cuda, max_inflight=1).run([r])[0]
        assert out[r.rid].error is None
        assert np.array_equal(out[r.rid].posterior_mean, alone.posterior_mean) and out[r.rid].logz == alone.logz


def test_grouped_serving_matches_alone_and_analytic(issm, cuda):
    """One launch per phase per step for every in-flight run
    (issm_group_step): each run gives bitwise the same numbers alone and in
    the mix (runs of d = 2..64 and budgets 4k..40k share every launch), and
    matches the conjugate analytic posterior."""
    reqs, truth = _requests(issm, SPEC)
    alone = {}
    for r in reqs:
        alone[r.rid] = issm.serving.GroupedServeLoop(cuda).run([r])[0]
    reqs2, _ = _requests(issm, SPEC)
    mixed = {res.rid: res for res in issm.serving.GroupedServeLoop(cuda).run(reqs2)}
    assert sorted(mixed) == sorted(alone)
    for rid, a in alone.items():
        m = mixed[rid]
        assert m.error is None and a.error is None
        assert np.array_equal(a.posterior_mean, m.posterior_mean)
        assert a.logz == m.logz and a.ess == m.ess
        mean, sd, logz = truth[rid]
        assert np.max(np.abs(m.posterior_mean - mean) / sd) < 0.25, rid
        assert abs(m.logz - logz) < 0.1, (rid, m.logz, logz)


def test_grouped_serving_staggered_arrivals(issm, cuda):
    """Requests arriving while others are mid-run join at the next step (the
    table holds runs in different rounds) and still give their alone
    numbers; the memory budget caps the admitted footprint."""
    reqs, truth = _requests(issm, SPEC * 3, seed=5)
    for k, r in enumerate(reqs):
        r.arrival = 0.002 * k
    loop = issm.serving.GroupedServeLoop(cuda, max_inflight=5)
    out = {res.rid: res for res in loop.run(reqs)}
    assert len(out) == len(reqs)
    reqs2, _ = _requests(issm, SPEC * 3, seed=5)
    for r in reqs2[::4]:
        a = issm.serving.GroupedServeLoop(cuda).run([r])[0]
        assert np.array_equal(a.posterior_mean, out[r.rid].posterior_mean) and a.logz == out[r.rid].logz
    for rid, res in out.items():
        mean, sd, logz = truth[rid]
        assert np.max(np.abs(res.posterior_mean - mean) / sd) < 0.25, rid
