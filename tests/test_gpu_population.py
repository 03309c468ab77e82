"""Population adaptation kernels (issm_population_local_weights /
_covariances / _factors) against the FP64 oracle restatement of
src/population_covariance.jl: ESS-tempered local weights (ready, tempered,
tempering-failed and all-zero slots), weighted covariances about the
tempered mean or the location, the current covariance kept for slots that
are not ready, and potrf's info convention for non-finite and indefinite
covariances."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _population(rng, d, k, m, spread=3.0):
    x = rng.normal(size=(k * m, d))
    lw = rng.normal(size=k * m) * spread
    starts = np.arange(k, dtype=np.int64) * m
    counts = np.full(k, m, dtype=np.int64)
    return x, lw, starts, counts


def _dev(a, dtype, cuda):
    return torch.tensor(np.ascontiguousarray(a), dtype=dtype, device=cuda)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("d,m", [(3, 150), (16, 700), (64, 1000)])
def test_population_local_weights_vs_oracle(issm, orc, cuda, dtype, d, m):
    rng = np.random.default_rng(d * 7 + m)
    k = 6
    x, lw, starts, counts = _population(rng, d, k, m)
    lw[starts[4]:starts[4] + m] = -np.inf  # all-zero slot
    # thresholds: reached, tempered twice, unreachable (tempering fails), all-zero, reached
    thr = np.array([2.0, 0.3 * m, 0.6 * m, 5.0 * m, 1.0, 1.0])
    if dtype == torch.float32:
        x, lw = x.astype(np.float32).astype(np.float64), lw.astype(np.float32).astype(np.float64)
    ew, eess, epw, est, emeans = orc.population_local_weights(lw, x.reshape(-1), d, starts, counts, thr)
    w, ess, pw, st, means = issm.ops.population_local_weights(
        _dev(lw, dtype, cuda), _dev(starts, torch.int64, cuda), _dev(counts, torch.int64, cuda),
        _dev(thr, torch.float64, cuda), samples=_dev(x, dtype, cuda))
    torch.cuda.synchronize()
    assert st.cpu().numpy().tolist() == est.tolist() == [0, 0, 0, 2, 1, 0]
    tol = 1e-10 if dtype == torch.float64 else 2e-6
    ready = est == 0
    assert np.allclose(pw.double().cpu().numpy(), epw, rtol=tol, atol=tol)
    assert np.allclose(ess.double().cpu().numpy(), eess, rtol=tol)
    mask = np.repeat(ready, m)
    assert np.allclose(w.double().cpu().numpy()[mask], ew[mask], rtol=tol, atol=tol * 1e-3)
    assert np.allclose(means.double().cpu().numpy()[ready | (est == 2)], emeans[ready | (est == 2)], rtol=tol,
                       atol=tol)
    # tempered slots reach their threshold at the power found
    assert 0.0 < epw[1] < 1.0 and eess[1] >= thr[1] and eess[2] >= thr[2]


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("d,family", [(3, "gaussian"), (16, "student"), (64, "gaussian")])
def test_population_covariances_and_factors_vs_oracle(issm, orc, cuda, dtype, d, family):
    rng = np.random.default_rng(d + (1 if family == "student" else 0))
    k, m = 5, 600
    x, lw, starts, counts = _population(rng, d, k, m, spread=1.0)
    thr = np.array([1.0, 0.5 * m, 1.0, 10.0 * m, 1.0])  # ready, tempered, ready, failed, ready
    npdt = np.float64 if dtype == torch.float64 else np.float32
    props = []
    for _ in range(k):
        A = rng.normal(size=(d, d))
        L = np.linalg.cholesky(A @ A.T / d + 0.3 * np.eye(d)).astype(npdt)
        loc = (rng.normal(size=d) * 0.2).astype(npdt)
        props.append(issm.FactorGaussian(loc, L) if family == "gaussian" else issm.FactorStudentT(npdt(6.0), loc, L))
    bank = issm.pack_proposals(props, cuda)
    x = x.astype(npdt)
    lw = lw.astype(npdt)
    tx, tl = _dev(x, dtype, cuda), _dev(lw, dtype, cuda)
    ts, tc_ = _dev(starts, torch.int64, cuda), _dev(counts, torch.int64, cuda)
    w, ess, pw, st, _ = issm.ops.population_local_weights(tl, ts, tc_, _dev(thr, torch.float64, cuda), samples=tx)
    centres, covs = issm.ops.population_covariances(tx, w, pw, st, bank, ts, tc_)
    dofs = bank.dofs if family == "student" else None
    factors, info = issm.ops.population_factors(covs, st, dofs=dofs)
    torch.cuda.synchronize()
    status = st.cpu().numpy()
    assert status.tolist() == [0, 0, 0, 2, 0]
    # the oracle on the device's weights (the local-weight step is pinned above)
    nu = None if dofs is None else dofs.double().cpu().numpy()
    ecen, ecov = orc.population_covariances(x.astype(np.float64).reshape(-1), d, w.double().cpu().numpy(),
                                            pw.double().cpu().numpy(), status,
                                            bank.locations.double().cpu().numpy(),
                                            bank.scales.double().cpu().numpy(), nu, starts, counts)
    tol = 1e-10 if dtype == torch.float64 else 2e-5
    assert np.allclose(centres.double().cpu().numpy(), ecen, rtol=tol, atol=tol)
    scale = np.max(np.abs(ecov))
    assert np.max(np.abs(covs.double().cpu().numpy() - ecov)) <= tol * scale
    ef, einfo = orc.population_factors(covs.double().cpu().numpy(), d, status, nu)
    assert info.cpu().numpy().tolist() == einfo.tolist() == [0] * k
    ready = status == 0
    assert np.allclose(factors.double().cpu().numpy()[ready], ef[ready], rtol=tol * 10, atol=tol * 10)
    # a ready factor reproduces its covariance (Student-t: scaled by (nu-2)/nu)
    f0 = factors[0].double().cpu().numpy().T  # column-major storage -> L
    c0 = covs[0].double().cpu().numpy()
    mult = 1.0 if nu is None else (nu[0] - 2.0) / nu[0]
    assert np.allclose(f0 @ f0.T, c0 * mult, rtol=1e-4, atol=1e-4 * scale)


def test_population_factors_info_convention(issm, orc, cuda):
    """potrf's info: -1 for a non-finite covariance, the failing column for
    an indefinite one, 0 (and nothing written) for slots that are not ready."""
    d = 4
    good = np.eye(d) * 2.0
    nonfinite = np.eye(d)
    nonfinite[2, 1] = nonfinite[1, 2] = np.inf
    indefinite = np.eye(d)
    indefinite[2, 2] = -1.0
    covs = np.stack([good, nonfinite, indefinite, good])
    status = np.array([0, 0, 0, 1], dtype=np.uint8)
    f, info = issm.ops.population_factors(_dev(covs, torch.float64, cuda), _dev(status, torch.uint8, cuda))
    torch.cuda.synchronize()
    ef, einfo = orc.population_factors(covs, d, status)
    assert info.cpu().numpy().tolist() == einfo.tolist() == [0, -1, 3, 0]
    got = f.cpu().numpy()
    assert np.allclose(got[0], ef[0]) and np.all(got[3] == 0.0)
