"""Result statistics on the device (src/statistics.jl): the weighted mean
and functional mean (one FP64 pass, bitwise reproducible), the weighted
variance, the component-wise weighted quantiles with the StatsBase
generic-weight interpolation rule (a weighted radix select on the device,
against the oracle's stable sort), and named (structured) samples through
mean and resample (src/resampling.jl:120-164)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

PROBS = [0.0, 0.1, 0.25, 0.5, 0.9, 1.0]


def _weights(lw):
    w = np.exp(lw - lw.max())
    return w / w.sum()


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("n,d", [(1, 3), (17, 1), (5000, 7), (200_001, 64)])
def test_weighted_quantile_vs_oracle(issm, orc, cuda, dtype, n, d):
    rng = np.random.default_rng(n + d)
    x = rng.normal(size=(n, d))
    if n > 100:
        x[: n // 3, 0] = np.round(x[: n // 3, 0], 1)  # ties
        x[5, 1 % d] = -0.0
    lw = rng.normal(size=n) * 2.0
    if n > 100:
        lw[rng.choice(n, n // 5, replace=False)] = -np.inf  # zero weights
    tx = torch.tensor(x, dtype=dtype, device=cuda)
    tl = torch.tensor(lw, dtype=dtype, device=cuda)
    res = issm.WeightedSamples(tx, tl)
    q = issm.quantile(res, PROBS)
    torch.cuda.synchronize()
    xs = tx.double().cpu().numpy()
    ws = _weights(tl.double().cpu().numpy())
    exp = orc.weighted_quantile(xs.reshape(-1), d, ws, PROBS)
    got = q.cpu().numpy()
    # the interpolation fraction divides a cumulative-weight difference by one
    # sample's weight: the sums' order (per-bin on the device, sequential in
    # the oracle) moves it by rounding / weight, a few 1e-9 at worst here
    tol = 1e-8 if dtype == torch.float64 else 1e-6
    assert np.allclose(got, exp, rtol=tol, atol=tol), np.max(np.abs(got - exp))
    assert np.allclose(issm.median(res).cpu().numpy(), exp[3], rtol=tol, atol=tol)


def test_weighted_quantile_nan_coordinate(issm, orc, cuda):
    x = np.array([[1.0, 2.0], [np.nan, 3.0], [0.5, 1.0]])
    lw = np.zeros(3)
    res = issm.WeightedSamples(torch.tensor(x, device=cuda), torch.tensor(lw, device=cuda))
    got = issm.quantile(res, [0.5]).cpu().numpy()
    exp = orc.weighted_quantile(x.reshape(-1), 2, _weights(lw), [0.5])
    assert np.isnan(got[0, 0]) and np.isnan(exp[0, 0]) and got[0, 1] == exp[0, 1]
    with pytest.raises(ValueError):
        issm.quantile(res, [1.5])


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_weighted_mean_var_and_functional_mean(issm, cuda, dtype):
    rng = np.random.default_rng(4)
    n, d = 300_000, 9
    x = rng.normal(size=(n, d)) * 2.0 + 1.0
    lw = rng.normal(size=n)
    tx, tl = torch.tensor(x, dtype=dtype, device=cuda), torch.tensor(lw, dtype=dtype, device=cuda)
    res = issm.WeightedSamples(tx, tl)
    xs, ws = tx.double().cpu().numpy(), _weights(tl.double().cpu().numpy())
    # FP32 log weights are summarised in FP32 (max, sum of expf), as the
    # reference sums FP32 weights; the weighted sums themselves are FP64
    tol = 1e-10 if dtype == torch.float64 else 2e-6
    m = issm.mean(res).cpu().numpy()
    assert np.allclose(m, ws @ xs, rtol=tol, atol=tol)
    # bitwise reproducible: the same reduction order every call
    assert np.array_equal(m, issm.mean(res).cpu().numpy())
    v = issm.var(res).cpu().numpy()
    assert np.allclose(v, ws @ (xs - ws @ xs) ** 2, rtol=10 * tol)
    f = lambda s: (s[:, 0] * s[:, 1]).double()  # noqa: E731
    fm = issm.mean(res, f)
    assert fm == pytest.approx(float(ws @ (xs[:, 0] * xs[:, 1])), rel=10 * tol, abs=tol)
    fv = issm.var(res, f)
    vals = xs[:, 0] * xs[:, 1]
    assert fv == pytest.approx(float(ws @ (vals - ws @ vals) ** 2), rel=100 * tol)
    assert issm.std(res, f) == pytest.approx(np.sqrt(fv))


def test_named_samples_mean_and_resample(issm, cuda):
    """NamedTuple-like samples: a dict of fields sharing one weight vector."""
    rng = np.random.default_rng(8)
    n = 4096
    fields = {"mu": torch.tensor(rng.normal(size=(n, 3)), device=cuda),
              "sigma": torch.tensor(rng.random(size=n) + 0.5, device=cuda),
              "L": torch.tensor(rng.normal(size=(n, 2, 2)), device=cuda)}
    lw = torch.tensor(rng.normal(size=n), device=cuda)
    res = issm.WeightedSamples(fields, lw)
    assert len(res) == n
    ws = _weights(lw.cpu().numpy())
    means = issm.mean(res)
    assert np.allclose(means["mu"].cpu().numpy(), ws @ fields["mu"].cpu().numpy())
    assert means["sigma"] == pytest.approx(float(ws @ fields["sigma"].cpu().numpy()))
    assert np.allclose(means["L"].cpu().numpy(), np.tensordot(ws, fields["L"].cpu().numpy(), axes=1))
    draws = issm.resample(3, res, 1000)
    anc = draws.ancestors.cpu().numpy() - 1
    for k, t in fields.items():
        assert torch.equal(draws.samples[k], t[torch.tensor(anc, device=cuda)])
    q = issm.quantile(res, 0.5)
    assert set(q) == set(fields) and q["mu"].shape == (3,)
