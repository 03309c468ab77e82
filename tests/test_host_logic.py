"""Host-side logic of the package (no GPU): proposal constants, bank
metadata, DM-PMC allocation plans and partial-MIS compilation, checked against
the reference's golden vectors and the oracle."""
import math

import numpy as np
import pytest


def test_student_t_logconstant_matches_oracle(issm, orc):
    for dof in (0.3, 1.0, 2.5, 5.0, 31.0, 40.0, 1e6):
        for d in (1, 2, 3, 5, 16, 64):
            assert issm.student_t_logconstant(dof, d) == pytest.approx(orc.student_t_logconstant(dof, d),
                                                                       rel=1e-14, abs=1e-12)


def test_student_t_logconstant_against_lgamma(issm):
    for dof in (1.5, 5.0, 12.0):
        for d in (1, 3, 4, 9):
            exact = math.lgamma((dof + d) / 2) - math.lgamma(dof / 2) - d / 2 * math.log(dof * math.pi)
            assert issm.student_t_logconstant(dof, d) == pytest.approx(exact, rel=1e-12)


def test_proposal_validation(issm):
    with pytest.raises(ValueError):
        issm.FactorGaussian(np.zeros(2), np.array([[1.0, 0.5], [0.0, 1.0]]))
    with pytest.raises(ValueError):
        issm.SphericalGaussian(np.zeros(2), -1.0)
    with pytest.raises(TypeError):
        issm.FactorGaussian(np.zeros(2, dtype=np.float32), np.eye(2))
    with pytest.raises(ValueError):
        issm.ProposalBank([])
    with pytest.raises(ValueError):
        issm.ProposalBank([issm.SphericalGaussian(0.0, 1.0)], [0.0])


def test_gaussian_lognormalizer(issm, golden):
    c = golden["packed_factor_primitives"]
    p = issm.FactorGaussian(np.array(c["location"]), np.array(c["factor"]))
    assert float(p.lognormalizer) == pytest.approx(-math.log(2 * math.pi) - math.log(2.0), rel=1e-15)


def test_bank_metadata_sorted_stably_by_mass(issm):
    props = [issm.SphericalGaussian(float(i), 1.0) for i in range(1, 5)]
    bank = issm.ProposalBank(props, [1, 3, 2, 0])
    ids, logm, cdf = bank.active_metadata()
    assert ids == [1, 3, 2]
    assert cdf[-1] == 1.0
    assert np.allclose(np.exp(logm), [1 / 6, 2 / 6, 3 / 6])
    ties = issm.ProposalBank(props[:3], [1, 1, 1]).active_metadata()[0]
    assert ties == [1, 2, 3]


def test_dm_pmc_allocation_oracle(issm, golden):
    c = golden["dm_pmc_allocation"]
    props = [issm.SphericalGaussian(float(i), 1.0) for i in range(1, 5)]
    bank = issm.ProposalBank(props, c["masses"])
    ids, _, _ = bank.active_metadata()
    assert ids == c["active_ids"]
    active = [bank.masses[i - 1] for i in ids]
    counts, offsets = issm.deterministic_allocation_plan(active, c["schedule"])
    by_id = np.zeros((4, 3), dtype=np.int64)
    for s, pid in enumerate(ids):
        by_id[pid - 1] = counts[s]
    assert by_id.tolist() == c["counts_by_id"]
    assert (offsets + 1).tolist() == c["offsets"]


def test_dm_pmc_rotating_ties(issm, golden):
    c = golden["dm_pmc_rotating_ties"]
    counts, _ = issm.deterministic_allocation_plan(c["masses"], c["schedule"])
    assert counts.tolist() == c["counts"]


def test_dm_pmc_large_float32_counts(issm, golden):
    c = golden["dm_pmc_large_f32_counts"]
    counts, _ = issm.deterministic_allocation_plan(np.float32(c["masses_f32"]), [c["round_size"]] * 2)
    assert counts[:, 0].tolist() == c["first_round"]
    assert counts[:, 1].tolist() == c["second_round"]


def test_dm_pmc_uncovered_proposal_rejected(issm):
    with pytest.raises(ValueError):
        issm.deterministic_allocation_plan([100.0, 1.0, 1.0], [10])


def test_partial_denominator_compile(issm):
    from issm.sampler import compile_partial_denominator

    props = [issm.SphericalGaussian(float(i), 1.0) for i in range(4)]
    bank = issm.ProposalBank(props, [1.0, 2.0, 3.0, 4.0])
    ids, logm, _ = bank.active_metadata()
    grp, coef = compile_partial_denominator(bank, ids, logm, [[1, 2], [3, 4]])
    # slots are ordered by mass: ids [1, 2, 3, 4]
    assert grp.tolist() == [1, 1, 2, 2]
    assert np.allclose(np.exp(coef), [1 / 3, 2 / 3, 3 / 7, 4 / 7])
    with pytest.raises(ValueError):
        compile_partial_denominator(bank, ids, logm, [[1, 2], [3]])
    with pytest.raises(ValueError):
        compile_partial_denominator(bank, ids, logm, [[1, 1], [2, 3, 4]])


def test_schedules(issm):
    p = issm.SphericalGaussian(0.0, 1.0)
    assert issm.AMIS(p, rounds=3, round_size=5).round_size == [5, 5, 5]
    assert issm.AMIS(p, rounds=2, round_size=[2, 3]).round_size == [2, 3]
    with pytest.raises(ValueError):
        issm.AMIS(p, rounds=2, round_size=[2])
    with pytest.raises(ValueError):
        issm.AMIS(issm.SphericalStudentT(2.0, 0.0, 1.0), rounds=2, round_size=2)


def test_failure_decoding(issm):
    idx, block, reason = 37, 0, 0x0400
    packed = (((0xFFFFFFFF - idx + 1) & 0xFFFFFFFF) << 32) | (((0xFFFF - block + 1) & 0xFFFF) << 16) | reason
    fail, draw = issm.ops.decode_failure([2, packed, 0])
    assert fail == dict(count=2, first_logical_index=37, first_block=0, reason_bits=0x0400)
    assert draw["count"] == 0


def test_no_cpu_fallback(issm):
    import torch

    if torch.cuda.is_available():
        pytest.skip("has a GPU")
    with pytest.raises(RuntimeError):
        issm.prepare_sampler(0, issm.StandardNormalTarget(1),
                             issm.ImportanceSampling(issm.SphericalGaussian(np.zeros(1), 1.0), nsamples=8))


def test_carved_state_is_aligned_and_zero(issm):
    """The small per-run state is carved from one allocation per dtype; every
    part starts on a 256-byte boundary (vectorised kernels read it) and is
    zeroed."""
    import torch

    parts = issm.sampler._carve(torch.float64, torch.device("cpu"), (5, 3), (33,), (33, 33), (33,))
    assert [tuple(p.shape) for p in parts] == [(5, 3), (33,), (33, 33), (33,)]
    base = parts[0].data_ptr()
    for p in parts:
        assert (p.data_ptr() - base) % 256 == 0 and p.is_contiguous()
        assert float(p.abs().sum()) == 0.0
    ends = sorted((p.data_ptr(), p.data_ptr() + p.numel() * 8) for p in parts)
    assert all(ends[i][1] <= ends[i + 1][0] for i in range(len(ends) - 1))


def test_serve_footprint_grows_with_the_run(issm):
    import numpy as np

    def req(d, rounds, size):
        p = issm.FactorGaussian(np.zeros(d, dtype=np.float32), np.eye(d, dtype=np.float32))
        return issm.serving.ServeRequest(0, None, p, rounds=rounds, round_size=size, seed=0)

    a = req(8, 4, 1000).footprint()
    assert req(8, 4, 2000).footprint() > a
    assert req(16, 4, 1000).footprint() > a
    assert req(8, 8, 1000).footprint() > a
    assert req(8, 4, 1000).footprint() >= 4 * 1000 * 8 * 4  # at least the retained samples


def test_grouped_table_offsets_and_layout(issm):
    """The grouped serving step's descriptor table: 31 eight-byte fields in
    issm_group_run order (the library's own size), each run's block ranges
    the exclusive prefix sums of its block counts, its retained count and
    normal-stream position set by its round, and the fixed fields left as
    admitted."""
    sv = issm.serving
    assert len(sv._RUN_FIELDS) * 8 == issm.native.lib().issm_group_run_bytes()

    class Fake:
        def __init__(self, d, n, rnd):
            self.row = np.zeros(len(sv._RUN_FIELDS), dtype=np.int64)
            self.row[sv._COL["d"]], self.row[sv._COL["n_round"]], self.row[sv._COL["rounds"]] = d, n, 4
            self.row[sv._COL["samples"]] = 1000 + d
            self.row.view(np.float64)[sv._COL["t_const"]] = -1.5
            self.round = rnd

    runs = [Fake(5, 300, 0), Fake(64, 128, 2), Fake(2, 5000, 3)]
    t, bn, ba, bm = sv.GroupedServeLoop._table(runs)
    col = sv._COL
    assert t.shape == (3, len(sv._RUN_FIELDS))
    assert list(t[:, col["round"]]) == [0, 2, 3]
    assert list(t[:, col["n_old"]]) == [0, 256, 15000]
    assert list(t[:, col["normal_offset"]]) == [0, 2 * (128 * 64 + 8), 3 * (5000 * 2 + 8)]
    new = [3, 1, 40]
    alln = [3, 3, 157]          # ceil(300 / 128), ceil(384 / 128), ceil(20000 / 128)
    mom = [1, 1, 10]            # ceil(n_all / 2048)
    assert list(t[:, col["blk_new0"]]) == [0, 3, 4] and bn == sum(new)
    assert list(t[:, col["blk_all0"]]) == [0, 3, 6] and ba == sum(alln)
    assert list(t[:, col["blk_mom0"]]) == [0, 1, 2] and bm == sum(mom)
    assert list(t[:, col["nmom"]]) == mom
    assert list(t[:, col["samples"]]) == [1005, 1064, 1002]
    assert np.all(t.view(np.float64)[:, col["t_const"]] == -1.5)
    # the fixed rows are not modified by building a table
    assert runs[1].row[col["round"]] == 0


def test_grouped_run_preparation_layout(issm):
    """A grouped run's host preparation: one allocation of 256-byte aligned,
    non-overlapping slices in the issm_group_run order the step kernels read,
    an admission head holding the target's mode and upper factor (column
    major) and the history's slot 0, and the mode-centred target constant
    equal to the log joint density at the mode."""
    rng = np.random.default_rng(2)
    d, n_obs = 7, 90
    X = rng.normal(size=(n_obs, d))
    y = X @ rng.normal(size=d) + 0.5 * rng.normal(size=n_obs)
    tgt = issm.LinearRegressionTarget(X, y, sigma=0.5, prior_var=1.0)
    p = issm.FactorGaussian(rng.normal(size=d).astype(np.float32), (0.3 * np.eye(d)).astype(np.float32))
    req = issm.serving.ServeRequest(0, tgt, p, rounds=4, round_size=1000, seed=3)
    prep = issm.serving._Prep(req)
    offs = sorted(prep.off.items(), key=lambda kv: kv[1])
    assert all(o % 256 == 0 for _, o in offs)
    assert [k for k, _ in offs[:6]] == ["failures", "t_mode", "t_chol", "lognorm", "loc", "fac"]
    assert offs[-1][1] < prep.nbytes
    head = prep.head
    assert head.size == prep.off["fac"] + 4 * d * d
    f32 = head.view(np.float32)
    # failure words are zero; the head's other slots hold what the kernels read
    assert not head[prep.off["failures"]:prep.off["failures"] + 24 * 4].any()
    A = X.T @ X / 0.25 + np.eye(d)
    mode = np.linalg.solve(A, X.T @ y / 0.25)
    o = prep.off["t_mode"] // 4
    assert np.allclose(f32[o:o + d], mode, rtol=1e-6)
    o = prep.off["t_chol"] // 4
    U = f32[o:o + d * d].reshape(d, d).T  # column-major
    assert np.allclose(U.T @ U, A, rtol=1e-5) and np.allclose(np.tril(U, -1), 0)
    o = prep.off["loc"] // 4
    assert np.array_equal(f32[o:o + d], p.location)
    # t_const = log N(y | X mode, s2 I) + log N(mode | 0, I)
    r = y - X @ mode
    c0 = (-0.5 * n_obs * np.log(2 * np.pi * 0.25) - 0.5 * r @ r / 0.25 - 0.5 * d * np.log(2 * np.pi)
          - 0.5 * mode @ mode)
    assert prep.t_const == pytest.approx(c0, rel=1e-12)


def test_factor_exponent_bound_matches_the_entrywise_rule(issm):
    """The vectorised bound equals the entry-by-entry rule of
    src/student_t_range.jl:21-31 (max |e|, |e - 1| over the nonzero
    lower-triangle binary exponents; 2^62 for a non-finite entry; the upper
    triangle ignored)."""
    import math
    import sys

    bound = sys.modules["issm.proposals"].factor_exponent_bound

    def entrywise(f):
        b = 0
        for c in range(f.shape[0]):
            for r in range(c, f.shape[0]):
                v = float(f[r, c])
                if v == 0.0:
                    continue
                if not math.isfinite(v):
                    return 1 << 62
                e = math.frexp(v)[1]
                b = max(b, abs(e), abs(e - 1))
        return b

    rng = np.random.default_rng(8)
    cases = [np.tril(rng.normal(size=(k, k)) * 10.0 ** rng.integers(-60, 60)) for k in (1, 2, 9, 64)]
    cases += [np.zeros((3, 3)), np.diag([1e-310, 1.0, 1e308]), np.tril(rng.normal(size=(6, 6))).astype(np.float32)]
    bad = np.eye(4)
    bad[2, 1] = np.inf
    upper = np.eye(4)
    upper[0, 3] = np.nan
    cases += [bad, upper]
    for f in cases:
        assert bound(f) == entrywise(f)


def test_linear_regression_evidence_in_d_dimensions(issm):
    """The conjugate evidence in d x d form (determinant lemma and Woodbury)
    equals the n-dimensional Gaussian marginal of y."""
    rng = np.random.default_rng(9)
    for n, d in ((40, 3), (300, 12)):
        X = rng.normal(size=(n, d))
        y = X @ rng.normal(size=d) + 0.7 * rng.normal(size=n)
        t = issm.LinearRegressionTarget(X, y, sigma=0.7, prior_var=2.0)
        _, logz = t.analytic()
        C = 0.49 * np.eye(n) + 2.0 * X @ X.T
        ref = -0.5 * (n * np.log(2 * np.pi) + np.linalg.slogdet(C)[1] + y @ np.linalg.solve(C, y))
        assert logz == pytest.approx(ref, rel=1e-11, abs=1e-9)
