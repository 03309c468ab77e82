"""Generate tests/golden/reference_vectors.json.

The reference (ImportanceSamplers.jl) is Julia, and no Julia is installed
where these fixtures are made, so its known-answer tests are read as
specifications: each case below re-enters the literal inputs of one reference
test (cited file:line) and its expected output, either the literal the test
asserts or the closed form the test compares against, evaluated here in
120-bit mpmath arithmetic.

Run:  python tests/golden/make_golden.py [--check-source REFERENCE_ROOT]

--check-source verifies that every cited reference line still contains the
quoted literal snippet (provenance check; needs the reference checkout).
"""
import argparse
import json
import os
import sys

import mpmath as mp

mp.mp.prec = 120

F32_MAX = float.fromhex("0x1.fffffep+127")
F64_MAX = sys.float_info.max


def f(x):
    return float(x)


def log2pi():
    return mp.log(2 * mp.pi)


def student_t_logconstant(nu, d):
    nu = mp.mpf(nu)
    return (mp.loggamma((nu + d) / 2) - mp.loggamma(nu / 2)
            - mp.mpf(d) / 2 * mp.log(nu * mp.pi))


CASES = []


def case(name, source, snippet, **data):
    CASES.append({"name": name, "source": source, "snippet": snippet, **data})


def build():
    # -- log-mixture accumulator ------------------------------------------
    a = mp.log(2) + mp.log(mp.mpf("0.25"))
    b = mp.log(3) + mp.log(mp.mpf("0.5"))
    num = mp.log(mp.e ** a + mp.e ** b)
    case("log_mixture_accumulator", "test/log_mixture_accumulator.jl:9-16",
         "numerator = IS._append_logmixture(T(-Inf), log(T(2)), log(T(0.25)))",
         steps=[[f(mp.log(2)), 0.25], [f(mp.log(3)), 0.5]],
         expected_numerator=f(num),
         logtarget=f(mp.log(4)), logtotal=f(mp.log(5)),
         expected_logweight=f(mp.log(4) - num + mp.log(5)), rtol_eps=8)

    # -- packed factor draw and density -------------------------------------
    case("packed_factor_primitives", "test/static_mis_kernel.jl:268-296",
         "factor = T[1 0; 0.25 2]",
         location=[2.0, 2.0], factor=[[1.0, 0.0], [0.25, 2.0]], normals=[1.0, 2.0],
         expected_sample=[3.0, 6.25],
         expected_logdensity=f(-mp.log(2 * mp.pi) - mp.log(2) - mp.mpf("2.5")),
         rtol_eps=8)

    # -- native Gaussian analytic densities --------------------------------
    gauss = []
    gauss.append(dict(kind="spherical", location=[1.25], scale=[2.5], x=[-0.75],
                      expected=f(-mp.mpf("0.5") * ((mp.mpf("-0.75") - mp.mpf("1.25")) / mp.mpf("2.5")) ** 2
                                 - mp.log(mp.mpf("2.5")) - log2pi() / 2)))
    gauss.append(dict(kind="spherical", location=[1, -1, 2], scale=[2.0], x=[3, -5, 8],
                      expected=f(-mp.mpf("0.5") * 14 - 3 * mp.log(2) - mp.mpf("1.5") * log2pi())))
    gauss.append(dict(kind="diagonal", location=[1, -1, 2], scale=[2, 4, 0.5], x=[3, 3, 3],
                      expected=f(-mp.mpf("0.5") * 6 - mp.log(4) - mp.mpf("1.5") * log2pi())))
    gauss.append(dict(kind="factor", location=[0, 0], scale=[[2, 0], [0.5, 1.5]], x=[2, 2],
                      expected=f(-log2pi() - mp.log(3) - 1)))
    case("native_gaussian_analytic", "test/native_proposals.jl:179-200",
         "diagonal = DiagonalGaussian(Float64[1, -1, 2], Float64[2, 4, 0.5])",
         dtype="f64", cases=gauss, rtol_eps=16)

    # -- representable range, Float64 and Float32 ---------------------------
    rng = []
    for dtype, magnitude, tail, largest in (("f64", 1e308, 1.5e154, F64_MAX),
                                            ("f32", _f32(2e38), _f32(2e19), F32_MAX)):
        for (location, scale, point) in ((-magnitude, magnitude, magnitude), (0.0, 1.0, tail)):
            radius = ((mp.mpf(point) - mp.mpf(location)) / mp.mpf(scale)) ** 2
            vec = f(-2 * mp.log(mp.mpf(scale)) - log2pi() - radius / 2)
            for kind, sc in (("spherical", [scale]), ("diagonal", [scale, scale]),
                             ("factor", [[scale, 0.0], [0.0, scale]])):
                rng.append(dict(dtype=dtype, kind=kind, location=[location, 0.0], scale=sc,
                                x=[point, 0.0], expected=vec))
        rng.append(dict(dtype=dtype, kind="factor", location=[0.0, 0.0],
                        scale=[[1.0, 0.0], [largest, largest]], x=[2.0, 0.0],
                        expected=f(-mp.log(mp.mpf(largest)) - log2pi() - 4)))
        point = _f32(0.75 * float(mp.sqrt(largest))) if dtype == "f32" else 0.75 * float(mp.sqrt(largest))
        rng.append(dict(dtype=dtype, kind="spherical", location=[0.0, 0.0], scale=[1.0],
                        x=[point, point], expected=f(-log2pi() - 2 * mp.mpf(point) ** 2 / 2)))
    case("native_gaussian_range", "test/native_proposals.jl:202-232",
         "for (T, magnitude, tail) in ((Float32, 2f38, 2f19), (Float64, 1e308, 1.5e154))",
         cases=rng, rtol_eps=8)

    # -- native Student-t analytic densities --------------------------------
    st = []
    for (location, scale, point) in ((0.0, 1e-200, 1e200), (-1e308, 1.0, 1e308)):
        z = (mp.mpf(point) - mp.mpf(location)) / mp.mpf(scale)
        st.append(dict(kind="spherical", dof=1.0, location=[location], scale=[scale], x=[point],
                       expected=f(-mp.log(mp.pi) - mp.log(mp.mpf(scale)) - mp.log1p(z ** 2))))
    # factor Student-t with extreme entries (test/native_proposals.jl:243-256)
    eta = float.fromhex("0x0.0000000000001p-1022")
    fac4 = [[1.0, 0, 0, 0], [0, 1e-200, 0, 0], [1e300, 0, 1e-300, 0], [0, 0, 1e300, 1e-300]]
    for L, point in (([[1e-200, 0.0], [1e-200, 1.0]], [1e200, 1e200]),
                     (fac4, [1e-300, 1e200, 0.0, 0.0]),
                     ([[1e200, 0.0], [1e300, 1e-300]], [1e-200, 0.0]),
                     ([[1.0, 0.0], [2e-124, eta]], [1e-200, eta])):
        d = len(point)
        z = []
        for r in range(d):
            v = mp.mpf(point[r]) - sum(mp.mpf(L[r][c]) * z[c] for c in range(r))
            z.append(v / mp.mpf(L[r][r]))
        radius = sum(z[i] ** 2 for i in range(d))
        logdet = sum(mp.log(mp.mpf(L[i][i])) for i in range(d))
        at_location = student_t_logconstant(1, d) - logdet
        st.append(dict(kind="factor", dof=1.0, location=[0.0] * d, scale=L, x=point,
                       expected=f(at_location - (d + 1) / mp.mpf(2) * mp.log1p(radius))))
    for nu, point, dtype in ((1.0, 1e200, "f64"), (1e308, 2e154, "f64")):
        st.append(dict(kind="spherical", dof=nu, location=[0.0], scale=[1.0], x=[point], dtype=dtype,
                       expected=f(student_t_logconstant(nu, 1) - (mp.mpf(nu) + 1) / 2 * mp.log1p(mp.mpf(point) ** 2 / mp.mpf(nu)))))
    for kind, sc in (("spherical", [1.0]), ("diagonal", [1.0, 1.0]), ("factor", [[1.0, 0.0], [0.0, 1.0]])):
        st.append(dict(kind=kind, dof=1.0, location=[0.0, 0.0], scale=sc, x=[1e200, -1e200],
                       expected=f(-mp.log(2 * mp.pi) - mp.mpf("1.5") * mp.log1p(2 * mp.mpf(1e200) ** 2))))
    st.append(dict(kind="spherical", dof=1.0, location=[1.25], scale=[2.5], x=[-0.75],
                   expected=f(-mp.log(mp.pi) - mp.log(mp.mpf("2.5")) - mp.log1p(((mp.mpf("-0.75") - mp.mpf("1.25")) / mp.mpf("2.5")) ** 2))))
    st.append(dict(kind="spherical", dof=1.0, location=[1, -1], scale=[2.0], x=[3, -5],
                   expected=f(-log2pi() - 2 * mp.log(2) - mp.mpf("1.5") * mp.log1p(5))))
    st.append(dict(kind="diagonal", dof=3.0, location=[1, -1], scale=[2, 4], x=[3, 3],
                   expected=f(-log2pi() - mp.log(8) - mp.mpf("2.5") * mp.log1p(mp.mpf(2) / 3))))
    st.append(dict(kind="factor", dof=2.0, location=[0, 0], scale=[[2, 0], [0.5, 1.5]], x=[2, 2],
                   expected=f(-log2pi() - mp.log(3) - 2 * mp.log1p(1))))
    st.append(dict(kind="spherical", dof=float(2 ** 52), location=[0, 0, 0], scale=[1.0], x=[0, 0, 0],
                   expected=f(-3 * log2pi() / 2), rtol_eps=8))
    tiny = eta
    st.append(dict(kind="spherical", dof=tiny, location=[0, 0, 0], scale=[1.0], x=[0, 0, 0],
                   expected=f(-mp.log(4 * mp.pi) - mp.log(mp.mpf(tiny)) / 2)))
    case("native_student_t_analytic", "test/native_proposals.jl:234-300",
         "factor = FactorStudentT(2.0, Float64[0, 0], Float64[2 0; 0.5 1.5])",
         dtype="f64", cases=st, rtol_eps=64)

    # -- Student-t subnormal radius ----------------------------------------
    sub = []
    for dtype, dof in (("f64", float.fromhex("0x0.0000000000001p-1022")),):
        for point in (float(mp.sqrt(dof)) / 2, 1.25 * float(mp.sqrt(dof))):
            exp_ = f(-log2pi() - (mp.mpf(dof) + 2) / 2 * mp.log1p(mp.mpf(point) ** 2 / mp.mpf(dof)))
            for kind, sc in (("spherical", [1.0]), ("diagonal", [1.0, 1.0]), ("factor", [[1.0, 0.0], [0.0, 1.0]])):
                sub.append(dict(dtype=dtype, kind=kind, dof=dof, location=[0.0, 0.0], scale=sc,
                                x=[point, 0.0], expected=exp_))
    case("native_student_t_subnormal", "test/native_proposals.jl:302-317",
         "dof = nextfloat(zero(T))", cases=sub, rtol_eps=8)

    # -- realized mixture denominator ----------------------------------------
    ln = -log2pi() / 2
    case("realized_mixture_denominator", "test/dm_pmc_kernel.jl:15-75",
         "logcoefficients = T[",
         locations=[-1.0, 1.0], scales=[1.0, 1.0],
         coefficients=[[f(mp.log(mp.mpf(3) / 4)), f(mp.log(mp.mpf(1) / 4))],
                       [f(mp.log(mp.mpf(1) / 4)), f(mp.log(mp.mpf(3) / 4))]],
         x=[-1.0], generating_slot=0,
         expected=[f(ln + mp.log(mp.mpf(3) / 4 + mp.exp(-2) / 4)),
                   f(ln + mp.log(mp.mpf(1) / 4 + 3 * mp.exp(-2) / 4))],
         expected_generating=f(ln), rtol_eps=16)

    # -- multinomial select -------------------------------------------------
    case("multinomial_select", "test/dm_pmc_kernel.jl:205-233",
         "uniforms = T[0.1, 0.2, 0.2001, 0.95]",
         cdf=[0.2, 0.5, 0.9, 1.0], weights=[0.2, 0.3, 0.4, 0.1],
         uniforms=[0.1, 0.2, 0.2001, 0.95], expected=[1, 2, 2, 4],
         samples=[[1, 2], [3, 4], [11, 12], [13, 14]])
    case("multinomial_plateaus", "test/dm_pmc_kernel.jl:235-272",
         "cdf=T[0, 0, 0.5, 1],",
         cases=[dict(cdf=[0.0, 0.0, 0.5, 1.0], uniforms="plateau_a", expected=[3, 3, 4, 4]),
                dict(cdf=[0.25, 1.0, 1.0, 1.0], uniforms="plateau_b", expected=[1, 2, 2, 2]),
                dict(cdf=[0.25, 0.5, 0.75, 1.0], uniforms="one", expected=[4])])

    # -- zero-mass support through the Float32 CDF ----------------------------
    lw = [-1e999] + [0.0] * 6 + [-1e999] + [0.0] * 6 + [-1e999]
    case("zero_mass_support", "test/resampling.jl:54-59",
         "@test resample(BoundaryUniformRNG(uniforms), result, 3).samples == [2, 9, 14]",
         logweights=["-inf" if v < -1e300 else v for v in lw],
         uniforms_f32=["0", "0.5", "prevfloat1"], expected=[2, 9, 14])
    case("zero_mass_tail", "test/resampling.jl:61-65",
         "logweights[2] = logweights[66] = Float32(-24log(2))",
         n=259, finite={"1": 0.0, "2": f(-24 * mp.log(2)), "66": f(-24 * mp.log(2))},
         uniform_f32="prevfloat1")

    # -- ESS extremes --------------------------------------------------------
    case("ess_extremes", "test/dm_pmc_kernel.jl:274-296",
         "concentrated = DMPMCKernelIS._logweight_summary(",
         cases=[dict(lw=["max", "max"], ess=2.0, logz_finite=True),
                dict(lw=["-max", "-max"], ess=2.0, logz_finite=True),
                dict(lw=["max", "-max"], ess=1.0, logz_finite=True),
                dict(lw=["-inf", "-inf"], ess=0.0, logz="-inf")])

    # -- stable log normaliser -------------------------------------------------
    case("stable_lognormalizer", "test/results.jl:357-388",
         "extreme_logs = [1000.0, 999.0, -Inf]",
         logweights=[1000.0, 999.0, "-inf"],
         expected_logz=f(1000 + mp.log1p(mp.exp(-1)) - mp.log(3)),
         expected_weights=[f(1 / (1 + mp.exp(-1))), f(1 / (1 + mp.exp(1))), 0.0],
         shifted=[1e20, 1e20], shifted_weights=[0.5, 0.5], shifted_samples=[1.0, 3.0],
         shifted_mean=2.0, shifted_var=1.0)

    # -- AMIS retrospective mixture ------------------------------------------
    x1 = [mp.mpf(-1) + v for v in (mp.mpf("-0.5"), mp.mpf("0.75"))]
    x2 = [1 + mp.mpf("1.5") * v for v in (mp.mpf(-1), mp.mpf("0.25"), mp.mpf(1))]
    xs = x1 + x2

    def lq(x, m, s):
        return -mp.log(s) - log2pi() / 2 - ((x - m) / s) ** 2 / 2

    nums = [mp.log(2 * mp.e ** lq(x, -1, 1) + 3 * mp.e ** lq(x, 1, mp.mpf("1.5"))) for x in xs]
    case("amis_retrospective_mixture", "test/amis_kernel.jl:203-262,423-477",
         "first_normals = T[-0.5, 0.75]",
         schedule=[2, 3], history_means=[-1.0, 1.0], history_scales=[1.0, 1.5],
         normals=[[-0.5, 0.75], [-1.0, 0.25, 1.0]], target="neg_x2_over_3",
         expected_samples=[f(x) for x in xs], expected_lognumerators=[f(v) for v in nums],
         expected_logweights=[f(-(x ** 2) / 3 - v + mp.log(5)) for x, v in zip(xs, nums)],
         round_ids=[1, 1, 2, 2, 2], rtol_eps=16)

    # -- AMIS diagnostics --------------------------------------------------------
    case("amis_round_diagnostics", "test/amis_kernel.jl:918-967",
         "ess=Float64[2.0, 3.473043499457537],",
         proposal=dict(location=0.0, scale=1.0), rounds=2, round_size=2,
         normals=[[-2.0, 2.0], [0.0, 1.0]], target="std_normal",
         f64=dict(ess=[2.0, 3.473043499457537], logz=[0.0, -0.2279354492780643]),
         f32=dict(ess=[2.0, 3.472985029220581], logz=[0.0, -0.22794675827026367]),
         rtol_eps=16)

    # -- literal two-pass moments -------------------------------------------------
    case("amis_literal_moments", "test/amis.jl:218-247,305-372",
         "vector_samples = T[-2 0 3 5; 4 -1 2 7]",
         scalar=dict(samples=[-3.0, -0.25, 1.5, 4.0], logweights=[-1000.0, -3.0, -1.0, -2.0],
                     previous_scale=1.75),
         vector=dict(samples=[[-2.0, 4.0], [0.0, -1.0], [3.0, 2.0], [5.0, 7.0]],
                     logweights=[-900.0, -2.0, -0.5, -4.0], previous_factor=[[2.0, 0.0], [-0.5, 1.25]]),
         rtol_eps=32)

    # -- complete CPU AMIS: retrospective final weights --------------------------
    case("amis_complete_cpu", "test/amis_kernel.jl:969-1051",
         "proposal = SphericalGaussian(T(-0.5), T(1.25))",
         schedule=[3, 3], proposal=dict(location=-0.5, scale=1.25),
         normals=[[-1.0, 0.25, 1.5], [-0.75, 1.25, 9.0]], target="neg_sq_x_minus_0.75_over_3",
         rtol_eps=64)

    # -- DM-PMC allocation ---------------------------------------------------------
    case("dm_pmc_allocation", "test/dm_pmc.jl:71-118",
         "expected_counts = [",
         masses=[1, 3, 2, 0], schedule=[13, 14, 13], active_ids=[1, 3, 2],
         counts_by_id=[[2, 2, 2], [7, 7, 7], [4, 5, 4], [0, 0, 0]], offsets=[1, 14, 28, 41])
    case("dm_pmc_rotating_ties", "test/dm_pmc.jl:120-137",
         "DeterministicMixturePMC(bank; rounds=3, round_size=[4, 4, 4])",
         masses=[1, 1, 1], schedule=[4, 4, 4], counts=[[2, 1, 1], [1, 2, 1], [1, 1, 2]])
    case("dm_pmc_large_f32_counts", "test/dm_pmc.jl:139-151",
         "@test first_round == [8_388_610, 8_388_609]",
         masses_f32=[0.5, 0.5], round_size=2 ** 24 + 3,
         first_round=[8388610, 8388609], second_round=[8388609, 8388610])


def _f32(v):
    import struct
    return struct.unpack("f", struct.pack("f", v))[0]


def check_source(root):
    bad = []
    for c in CASES:
        path, _, span = c["source"].partition(":")
        lines = open(os.path.join(root, path)).read().splitlines()
        ranges = []
        for part in span.split(","):
            lo, _, hi = part.partition("-")
            ranges.append((int(lo), int(hi or lo)))
        text = "\n".join("\n".join(lines[lo - 1:hi]) for lo, hi in ranges)
        if c["snippet"] not in text:
            bad.append(c["name"])
    return bad


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--check-source", default=None)
    args = ap.parse_args()
    build()
    if args.check_source:
        bad = check_source(args.check_source)
        if bad:
            raise SystemExit(f"provenance check failed for: {bad}")
        print("provenance check passed for", len(CASES), "cases")
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_vectors.json")
    with open(out, "w") as fh:
        json.dump({"generator": "tests/golden/make_golden.py", "cases": CASES}, fh, indent=1)
    print("wrote", out, len(CASES), "cases")


if __name__ == "__main__":
    main()
