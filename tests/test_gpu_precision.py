"""Run-level parity of the precision forms on the d = 64 Student-t AMIS
workload (nu = 5 target with a seeded lower-triangular scale; Gaussian factor
proposals from N(0, 9 I); 40 rounds x 50,000 samples, 2M retained samples),
against FP64 on the same draws.

Two comparisons, because adaptation amplifies differences: each round's fit
sets the next round's proposal, and with heavy-tailed weights a perturbation
of a fit grows by a factor of about two per round, so two whole runs from the
same normals part ways by far more than their arithmetic (an FP64 device run
and the FP64 oracle, which differ only in summation order, drift to about
1e-3 in some round's log Z).

* Frozen proposals: every form re-weighs the FP64 run's 2M retained samples
  under the FP64 run's own 40-slot proposal history (reweigh_amis) — the
  final deterministic-mixture weights, log Z and posterior mean. This isolates
  the arithmetic of the forms and is held to BASELINE's accuracy gate
  (|d log Z| <= 1e-3, posterior-mean difference <= 1e-2) for BF16 x3 and
  FP32; TF32 keeps about 11 bits per product and gets a wider bound.
* Adaptive runs from the same draws (share_normal_stream, FP32 ridge): the
  first round, drawn from the same initial proposal, agrees to the forms'
  log-density tolerance; the FP64 device run matches the FP64 oracle
  restatement of the reference's CPU AMIS on the first rounds.

Reference behaviour: _launch_prefilled_amis_round! (src/amis_execution.jl:
261-357) on prefilled draws, as in test/amis_kernel.jl:918-1051."""
import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

D, ROUNDS, ROUND_SIZE, DOF = 64, 40, 50_000, 5.0
FP32_RIDGE = float(np.sqrt(np.finfo(np.float32).eps))

# frozen proposals: |log Zhat_form - log Zhat_fp64| and the largest
# coordinate difference of the posterior mean (measured on a GB300: BF16 x3
# 3.1e-5 / 8.2e-6, FP32 1.9e-6 / 1.9e-6, TF32 1.0e-3 / 7.4e-4)
FROZEN_BOUNDS = {"bf16": (1e-3, 1e-2), "fp32": (1e-3, 1e-2), "tf32": (3e-2, 5e-2)}
# first adaptive round (same proposal, same draws): |d log Z|
FIRST_ROUND_BOUNDS = {"bf16": 1e-3, "fp32": 1e-4, "tf32": 3e-2}


def _problem():
    rng = np.random.default_rng(20261203)
    return np.tril(rng.normal(scale=0.3, size=(D, D)), -1) + np.diag(1.0 + np.abs(rng.normal(size=D)))


def _codes(issm):
    return {"fp32": issm.native.PREC_NATIVE, "fp64": issm.native.PREC_NATIVE, "tf32": issm.native.PREC_TF32,
            "bf16": issm.native.PREC_BF16}


def _sampler(issm, cuda, form, seed, rounds=ROUNDS, round_size=ROUND_SIZE):
    target = issm.StudentTTarget(np.zeros(D), _problem(), DOF)
    dt = np.float64 if form == "fp64" else np.float32
    p = issm.FactorGaussian(np.zeros(D, dtype=dt), (3.0 * np.eye(D)).astype(dt))
    s = issm.prepare_sampler(seed, target, issm.AMIS(p, rounds=rounds, round_size=round_size), device=cuda,
                             precision=_codes(issm)[form], regularization=FP32_RIDGE if form == "fp64" else None)
    if form == "fp64":
        issm.share_normal_stream(s, torch.float32)
    return s


@pytest.fixture(scope="module")
def fp64_run(issm, cuda):
    s = _sampler(issm, cuda, "fp64", 4242)
    r = issm.importance_sample_(s)
    return s, np.asarray(r.diagnostics["round_lognormalizers"])


def test_reweigh_reproduces_the_run(issm, cuda, fp64_run):
    """The closed-form final mixture (all 40 slots at once) reproduces the
    run's own final weights, built by the append recurrence, in FP64."""
    s, logz = fp64_run
    lz, mean, lw = issm.reweigh_amis(s)
    assert abs(lz - logz[-1]) < 1e-9
    assert torch.allclose(lw, s.logweights, rtol=1e-10, atol=1e-9)
    ref = issm.mean(issm.WeightedSamples(s.samples, s.logweights)).cpu().numpy()
    assert np.max(np.abs(mean - ref)) < 1e-9


@pytest.mark.parametrize("form", ["bf16", "fp32", "tf32"])
def test_amis_d64_form_vs_fp64_frozen_proposals(issm, cuda, fp64_run, form):
    """Each form re-weighs the FP64 run's samples under its proposals:
    log Z, posterior mean and log weights against FP64."""
    s, _ = fp64_run
    lz64, mean64, lw64 = issm.reweigh_amis(s)
    lz, mean, lw = issm.reweigh_amis(s, _codes(issm)[form], torch.float32)
    tol_logz, tol_mean = FROZEN_BOUNDS[form]
    dlz = abs(lz - lz64)
    dmean = float(np.max(np.abs(mean - mean64)))
    assert dlz <= tol_logz, f"{form}: |d log Z| = {dlz:.3e}"
    assert dmean <= tol_mean, f"{form}: posterior mean differs by {dmean:.3e}"
    # a log weight is the difference of two log densities of size ~100 at
    # d = 64, so its error is bounded in absolute terms: the forms' relative
    # log-density tolerances times that size, at most, and far less on
    # average over the normalised FP64 weights (which is what moves log Z)
    err = (lw.double() - lw64).abs()
    w = torch.softmax(lw64, 0)
    max_bound, mean_bound = {"bf16": (2e-2, 2e-3), "fp32": (2e-3, 2e-4), "tf32": (1.0, 5e-2)}[form]
    assert float(err.max()) <= max_bound, f"{form}: max |d log w| = {float(err.max()):.3e}"
    assert float((w * err).sum()) <= mean_bound, f"{form}: weighted |d log w| = {float((w * err).sum()):.3e}"


@pytest.mark.parametrize("form", ["bf16", "fp32", "tf32"])
def test_amis_d64_first_round_same_draws(issm, cuda, fp64_run, form):
    """Round 1 draws the same normals from the same proposal in every form,
    so its log Z differs from FP64's by the forms' arithmetic alone."""
    _, logz64 = fp64_run
    s = _sampler(issm, cuda, form, 4242, rounds=1)
    r = issm.importance_sample_(s)
    d1 = abs(float(r.diagnostics["round_lognormalizers"][0]) - logz64[0])
    assert d1 <= FIRST_ROUND_BOUNDS[form], f"{form}: round-1 |d log Z| = {d1:.3e}"


def test_amis_d64_fp64_device_vs_oracle_same_draws(issm, orc, cuda):
    """The FP64 device form against the FP64 oracle restatement of the
    reference's CPU AMIS on the same draws: 3 rounds x 50,000 samples (before
    adaptation has amplified summation-order differences)."""
    rounds = 3
    s = _sampler(issm, cuda, "fp64", 99, rounds=rounds)
    run = issm.importance_sample_(s)
    normals, offset = [], 0
    for _ in range(rounds):
        n = ROUND_SIZE * D
        normals.append(issm.ops.fill_normals(n, torch.float32, cuda, 99, offset).double().cpu().numpy())
        offset += n + 8
    tgt = orc.TargetView(orc.TARGET_STUDENT_T, D, a=np.zeros(D), b=_problem(), p0=DOF)
    out = orc.amis_run(tgt, D, np.zeros(D), 3.0 * np.eye(D), [ROUND_SIZE] * rounds, np.concatenate(normals),
                       regularization=FP32_RIDGE)
    assert out["status"] == 0
    assert np.allclose(run.diagnostics["round_lognormalizers"], out["round_logz"], rtol=1e-9, atol=1e-9)
    x = run.samples.cpu().numpy().reshape(-1)
    assert np.allclose(x, out["samples"], rtol=1e-9, atol=1e-9)
    assert np.allclose(run.logweights.cpu().numpy(), out["logweights"], rtol=1e-10, atol=1e-8)
    assert math.isfinite(float(run.diagnostics["round_lognormalizers"][-1]))
