"""End-to-end parity of the public API (prepare_sampler / importance_sample!)
with the FP64 oracle on fed draws, as the reference's prefilled-RNG tests do
(test/amis_kernel.jl:918-1051)."""
import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


class Prefilled:
    """Feeds fixed normal batches to a prepared sampler (AMISPrefilledRNG)."""

    def __init__(self, sampler, batches, uniform=None):
        self.batches = list(batches)
        self.uniform = uniform
        sampler.normals = self.normals
        if uniform is not None:
            sampler.uniforms = self.uniforms

    def normals(self, n, dtype):
        b = self.batches.pop(0)
        return torch.tensor(np.asarray(b[:n], dtype=np.float64), dtype=dtype, device="cuda")

    def uniforms(self, n, dtype):
        return torch.full((n,), self.uniform, dtype=dtype, device="cuda")


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_golden_amis_round_diagnostics(issm, cuda, golden, dtype):
    c = golden["amis_round_diagnostics"]
    p = issm.FactorGaussian(np.array([c["proposal"]["location"]], dtype=dtype),
                            np.array([[c["proposal"]["scale"]]], dtype=dtype))
    s = issm.prepare_sampler(0, issm.StandardNormalTarget(1), issm.AMIS(p, rounds=c["rounds"],
                                                                         round_size=c["round_size"]), device=cuda)
    Prefilled(s, c["normals"])
    res = issm.importance_sample_(s)
    exp = c["f64"] if dtype == np.float64 else c["f32"]
    eps = float(np.finfo(dtype).eps)
    assert np.allclose(res.diagnostics["round_ess"], exp["ess"], rtol=16 * eps)
    assert np.allclose(res.diagnostics["round_lognormalizers"], exp["logz"], rtol=16 * eps, atol=16 * eps)
    assert res.provenance["round"].cpu().tolist() == [1, 1, 2, 2]


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_golden_amis_complete(issm, orc, cuda, golden, dtype):
    c = golden["amis_complete_cpu"]
    p = issm.FactorGaussian(np.array([c["proposal"]["location"]], dtype=dtype),
                            np.array([[c["proposal"]["scale"]]], dtype=dtype))
    s = issm.prepare_sampler(0, issm.QuadraticTarget([0.75], 3.0),
                             issm.AMIS(p, rounds=2, round_size=c["schedule"]), device=cuda)
    Prefilled(s, c["normals"])
    res = issm.importance_sample_(s)
    tgt = orc.TargetView(orc.TARGET_QUADRATIC, 1, a=[0.75], p0=3.0)
    reg = math.sqrt(float(np.finfo(dtype).eps))
    out = orc.amis_run(tgt, 1, [c["proposal"]["location"]], [[c["proposal"]["scale"]]], c["schedule"],
                       np.concatenate(c["normals"]), regularization=reg)
    eps = float(np.finfo(dtype).eps)
    assert np.allclose(res.samples.double().cpu().numpy().reshape(-1), out["samples"], rtol=64 * eps)
    assert np.allclose(res.logweights.double().cpu().numpy(), out["logweights"], rtol=64 * eps, atol=64 * eps)
    # transactional reuse: the learned proposal seeds the next call
    loc, fac, _ = issm.current_proposal(s)
    Prefilled(s, [[-1.0, 0.0, 1.0], [0.5, -0.5, 1.5]])
    second = issm.importance_sample_(s)
    assert float(second.samples[0, 0]) == pytest.approx(float(loc[0]) + float(fac[0, 0]) * -1.0,
                                                        rel=8 * eps)


@pytest.mark.parametrize("family", ["gaussian", "student"])
def test_amis_vs_oracle_d8(issm, orc, cuda, family):
    """Multi-round factor AMIS (d=8, FP64) against the oracle on the same draws."""
    rng = np.random.default_rng(17)
    d, rounds, size = 8, 4, 3000
    Lt = np.tril(rng.normal(size=(d, d)) * 0.3, -1) + np.diag(1 + np.abs(rng.normal(size=d)))
    target = issm.StudentTTarget(np.zeros(d), Lt, 5.0)
    if family == "gaussian":
        p = issm.FactorGaussian(np.full(d, 0.5), 2.0 * np.eye(d))
        dof = 0.0
    else:
        p = issm.FactorStudentT(7.0, np.full(d, 0.5), 2.0 * np.eye(d))
        dof = 7.0
    s = issm.prepare_sampler(3, target, issm.AMIS(p, rounds=rounds, round_size=size), device=cuda)
    normals = [rng.normal(size=size * d) for _ in range(rounds)]
    rn = [rng.normal(size=size * 8) for _ in range(rounds)]
    ru = [rng.random(size=size * 8) for _ in range(rounds)]
    feed_n = list(normals)
    order = []
    for r in range(rounds):
        order.append(feed_n[r])
        if family == "student":
            order.append(rn[r])
    Prefilled(s, order)
    if family == "student":
        ruq = list(ru)
        s.uniforms = lambda n, dt: torch.tensor(ruq.pop(0)[:n], dtype=dt, device="cuda")
    res = issm.importance_sample_(s)
    tv = orc.TargetView(orc.TARGET_STUDENT_T, d, a=np.zeros(d), b=Lt, p0=5.0)
    out = orc.amis_run(tv, d, np.full(d, 0.5), 2.0 * np.eye(d), [size] * rounds, np.concatenate(normals),
                       family=orc.STUDENT_T if dof else orc.GAUSSIAN, dof=dof,
                       radial_normals=np.concatenate(rn) if dof else None, rn_stride=8 if dof else 0,
                       radial_uniforms=np.concatenate(ru) if dof else None, ru_stride=8 if dof else 0)
    assert out["status"] == 0
    assert np.allclose(res.samples.cpu().numpy().reshape(-1), out["samples"], rtol=1e-9, atol=1e-9)
    assert np.allclose(res.logweights.cpu().numpy(), out["logweights"], rtol=1e-9, atol=1e-9)
    assert np.allclose(res.diagnostics["round_ess"], out["round_ess"], rtol=1e-9)
    assert np.allclose(res.diagnostics["round_lognormalizers"], out["round_logz"], rtol=1e-9, atol=1e-12)


def test_static_mis_schemes_vs_oracle(issm, orc, cuda):
    rng = np.random.default_rng(23)
    d, k, n = 5, 6, 5000
    props = []
    for _ in range(k):
        A = rng.normal(size=(d, d))
        props.append(issm.FactorGaussian(rng.normal(size=d) * 2, np.linalg.cholesky(A @ A.T / d + 0.2 * np.eye(d))))
    bank = issm.ProposalBank(props, rng.dirichlet(np.ones(k)))
    for scheme in (issm.StratifiedMixture(), issm.RandomMixture(), issm.StandardMIS(),
                   issm.PartialDeterministicMixture([[1, 2, 3], [4, 5, 6]])):
        s = issm.prepare_sampler(5, issm.StandardNormalTarget(d), issm.ImportanceSampling(bank, n, scheme),
                                 device=cuda)
        res = issm.importance_sample_(s)
        db = s.bank
        from test_gpu_kernels import oracle_bank

        ob = oracle_bank(orc, db)
        x = res.samples.cpu().numpy()
        ids = db.proposal_ids.cpu().numpy()
        slot_of = {int(pid): i for i, pid in enumerate(ids)}
        slots = np.array([slot_of[int(v)] for v in res.provenance["proposal_id"].cpu().numpy()], dtype=np.int32)
        kind = {issm.StratifiedMixture: orc.DENOM_FULL, issm.RandomMixture: orc.DENOM_FULL,
                issm.StandardMIS: orc.DENOM_GENERATING, issm.PartialDeterministicMixture: orc.DENOM_PARTIAL}[type(scheme)]
        coef = db.logmasses.double().cpu().numpy()
        grp = None
        if kind == orc.DENOM_PARTIAL:
            coef = s.den._keep[0].double().cpu().numpy()
            grp = s.den._keep[1].cpu().numpy()
        den, _, _ = orc.mixture_logdensity(ob, x.reshape(-1), kind, coef, group_of_slot=grp, slots=slots)
        tgt = -0.5 * d * np.log(2 * np.pi) - 0.5 * np.sum(x * x, axis=1)
        assert np.allclose(res.logweights.cpu().numpy(), tgt - den, rtol=1e-11, atol=1e-11)
        if not isinstance(scheme, issm.RandomMixture):
            assert np.all(np.diff(slots) >= 0)  # stratified assignment is monotone


@pytest.mark.parametrize("resampling", ["global", "local"])
def test_dm_pmc_vs_oracle(issm, orc, cuda, resampling):
    """Each round's weights against the oracle's realized-mixture denominator
    at that round's locations, and each next location set against the oracle's
    selection (fixed-point multinomial or local) on the sampler's uniforms."""
    rng = np.random.default_rng(31)
    d, k = 3, 4
    props = [issm.SphericalGaussian(rng.normal(size=d) * 2, 1.0) for _ in range(k)]
    bank = issm.ProposalBank(props, [1.0, 2.0, 3.0, 2.0])
    alg = issm.DeterministicMixturePMC(bank, rounds=3, round_size=[40, 41, 40],
                                       resampling=issm.GlobalResampling() if resampling == "global"
                                       else issm.LocalResampling())
    s = issm.prepare_sampler(9, issm.StandardNormalTarget(d), alg, device=cuda)
    res = issm.importance_sample_(s)
    db = s.bank
    counts = s.counts_host
    x_all = res.samples.cpu().numpy()
    lw_all = res.logweights.cpu().numpy()
    locs = s.location_history.cpu().numpy()
    us = s.resample_uniform_history
    for r in range(3):
        lo, hi = int(s.offsets[r]), int(s.offsets[r + 1])
        ob = orc.BankView(d, orc.GAUSSIAN, orc.SCALE_SPHERICAL, locs[r], db.scales.double().cpu().numpy(),
                          db.lognormalizers.double().cpu().numpy())
        slots = np.repeat(np.arange(k, dtype=np.int32), counts[:, r])
        coef = np.log(counts[:, r] / float(s.schedule[r]))
        x = x_all[lo:hi]
        den, _, _ = orc.mixture_logdensity(ob, x.reshape(-1), orc.DENOM_FULL, coef, slots=slots)
        tgt = -0.5 * d * np.log(2 * np.pi) - 0.5 * np.sum(x * x, axis=1)
        assert np.allclose(lw_all[lo:hi], tgt - den, rtol=1e-11, atol=1e-11)
        u = us[r].cpu().numpy()
        if resampling == "global":
            anc = orc.resample_multinomial_fixed(lw_all[lo:hi], u)
        else:
            anc = orc.local_resample(lw_all[lo:hi], counts[:, r], u)
        nxt = locs[r + 1] if r < 2 else s.committed_locations.cpu().numpy()
        assert np.array_equal(nxt, x[anc - 1])


def test_resample_api_bit_exact(issm, orc, cuda):
    rng = np.random.default_rng(41)
    n = 20000
    x = torch.tensor(rng.normal(size=(n, 2)), device=cuda)
    lw = torch.tensor(rng.normal(size=n) * 2, device=cuda)
    res = issm.WeightedSamples(x, lw)
    draws = issm.resample(77, res, 500)
    u = issm.ops.fill_uniforms(500, torch.float64, cuda, 77).cpu().numpy()
    exp = orc.resample_multinomial_fixed(lw.cpu().numpy(), u)
    assert np.array_equal(draws.ancestors.cpu().numpy(), exp)
    assert torch.equal(draws.samples, x[draws.ancestors - 1])
    sys = issm.resample(78, res, n, method=issm.SystematicResampling())
    u1 = float(issm.ops.fill_uniforms(1, torch.float64, cuda, 78).item())
    assert np.array_equal(sys.ancestors.cpu().numpy(), orc.resample_systematic_fixed(lw.cpu().numpy(), u1, n))
    with pytest.raises(issm.AllZeroWeightsError):
        issm.resample(1, issm.WeightedSamples(x[:2], torch.full((2,), -float("inf"), dtype=torch.float64,
                                                                 device=cuda)), 2)


def test_amis_failure_raises_round_error(issm, cuda):
    p = issm.FactorGaussian(np.zeros(2), np.eye(2))
    bad = issm.LogTarget(lambda x: torch.where(x[:, 0] > 0, torch.full_like(x[:, 0], float("nan")),
                                               -0.5 * (x ** 2).sum(1)))
    s = issm.prepare_sampler(1, bad, issm.AMIS(p, rounds=2, round_size=64), device=cuda)
    with pytest.raises(issm.AMISRoundError) as e:
        issm.importance_sample_(s)
    assert e.value.round == 1 and e.value.phase == "target"
    # the committed proposal is unchanged by the failed call
    loc, fac, _ = issm.current_proposal(s)
    assert np.allclose(loc, 0.0) and np.allclose(fac, np.eye(2))


@pytest.mark.parametrize("precision", ["native", "tf32"])
def test_amis_graph_replay_matches_eager(issm, cuda, precision):
    """From its second call an AMIS sampler replays one recorded CUDA graph;
    the device Philox counter keeps the stream advancing, so graph and eager
    samplers with the same seed agree call for call."""
    prec = {"native": issm.native.PREC_NATIVE, "tf32": issm.native.PREC_TF32}[precision]
    rng = np.random.default_rng(3)
    d = 16
    Lt = np.tril(rng.normal(size=(d, d)) * 0.2, -1) + np.diag(1 + np.abs(rng.normal(size=d)))
    target = issm.StudentTTarget(np.zeros(d), Lt, 5.0)

    def sampler(graphs):
        p = issm.FactorGaussian(np.full(d, 0.3, dtype=np.float32), 2.0 * np.eye(d, dtype=np.float32))
        return issm.prepare_sampler(7, target, issm.AMIS(p, rounds=5, round_size=4000), device=cuda,
                                    precision=prec, graphs=graphs)

    g, e = sampler(True), sampler(False)
    for call in range(4):
        rg, re_ = issm.importance_sample_(g), issm.importance_sample_(e)
        assert (g.graph is not None) == (call >= 1) and e.graph is None
        assert torch.allclose(rg.samples, re_.samples, rtol=1e-6, atol=1e-6)
        assert torch.allclose(rg.logweights, re_.logweights, rtol=1e-5, atol=1e-5)
        assert np.allclose(rg.diagnostics["round_ess"], re_.diagnostics["round_ess"], rtol=1e-5)
    # successive calls draw fresh numbers (a result's samples view the
    # sampler's buffer until its next run, so keep a copy)
    first = rg.samples[:100].clone()
    assert not torch.equal(first, issm.importance_sample_(g).samples[:100])
    assert int(g.counter.item()) == int(e.counter.item()) + g.offset


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_resampling_rules_disagree_only_at_rounded_boundaries(issm, cuda, dtype):
    """The exact fixed-point rule and the reference's float CDF rule
    (src/resampling.jl:92-118,199-225) on 2^20 random weights and uniforms:
    they pick different ancestors only where a uniform lies within the float
    CDF's rounding of the interval boundaries between the two picks (a float
    CDF can merge several tiny-weight intervals into one rounding step). The
    measured disagreement rate is bounded by n times the CDF's rounding."""
    n = 1 << 20
    g = torch.Generator(device=cuda).manual_seed(11)
    lw = (torch.randn(n, generator=g, device=cuda, dtype=torch.float64) * 2.0).to(dtype)
    res = issm.WeightedSamples(torch.arange(n, device=cuda, dtype=dtype), lw)
    exact = issm.resample(5, res, n).ancestors.cpu().numpy()
    ref = issm.resample(5, res, n, cdf="reference").ancestors.cpu().numpy()
    u = issm.ops.fill_uniforms(n, torch.float64, cuda, 5).to(dtype).double().cpu().numpy()
    w = np.exp(lw.double().cpu().numpy() - float(lw.max()))
    cdf = np.cumsum(w) / w.sum()  # FP64 reference for the boundaries
    diff = np.nonzero(exact != ref)[0]
    eps = float(torch.finfo(dtype).eps)
    # FP64 disagreements come from the fixed-point CDF's own quantisation
    # (2^-42 of the largest weight per term at this n), not from the float CDF
    tol = max(8 * eps, 1e-11)
    rate = diff.size / n
    assert rate <= 4 * n * eps + 1e-5, rate
    for i in diff:
        lo, hi = sorted((int(exact[i]), int(ref[i])))
        # every boundary between the two picks (cdf[lo - 1] .. cdf[hi - 2],
        # 0-based) lies within the rounding of the uniform
        assert abs(u[i] - cdf[lo - 1]) <= tol, (i, u[i], cdf[lo - 1])
        assert abs(u[i] - cdf[hi - 2]) <= tol, (i, u[i], cdf[hi - 2])
    # systematic under both rules
    exact_s = issm.resample(6, res, n, method=issm.SystematicResampling()).ancestors.cpu().numpy()
    ref_s = issm.resample(6, res, n, method=issm.SystematicResampling(), cdf="reference").ancestors.cpu().numpy()
    assert np.mean(exact_s != ref_s) <= 4 * n * eps + 1e-5
