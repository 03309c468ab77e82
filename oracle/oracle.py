"""ctypes view of the FP64 C oracle (oracle/issm_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline / reference arm of bench.py. The product never imports it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SOURCE = os.path.join(HERE, "issm_oracle.c")
LIBRARY = os.path.join(HERE, "liboracle.so")

GAUSSIAN, STUDENT_T = 0, 1
SCALE_FACTOR, SCALE_DIAGONAL, SCALE_SPHERICAL = 0, 1, 2
DENOM_FULL, DENOM_GENERATING, DENOM_PARTIAL, DENOM_PREFIX = 0, 1, 2, 3
TARGET_GAUSS_MIX, TARGET_STUDENT_T, TARGET_LINREG, TARGET_LOGISTIC, TARGET_STD_NORMAL, TARGET_QUADRATIC = range(6)


def build(force=False):
    """Compile the oracle with gcc (-ffp-contract=off keeps rounding explicit)."""
    if not force and os.path.exists(LIBRARY) and os.path.getmtime(LIBRARY) >= os.path.getmtime(SOURCE):
        return LIBRARY
    cmd = ["gcc", "-O2", "-std=gnu11", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           "-o", LIBRARY, SOURCE, "-lm"]
    subprocess.run(cmd, check=True)
    return LIBRARY


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIBRARY)
        _declare(_lib)
    return _lib


class Bank(C.Structure):
    _fields_ = [("d", C.c_int), ("k", C.c_int), ("family", C.c_int), ("scale_kind", C.c_int),
                ("loc", C.c_void_p), ("scales", C.c_void_p), ("lognorm", C.c_void_p),
                ("dofs", C.c_void_p), ("range_risk", C.c_void_p)]


class Target(C.Structure):
    _fields_ = [("kind", C.c_int), ("d", C.c_int), ("j", C.c_int),
                ("a", C.c_void_p), ("b", C.c_void_p), ("c", C.c_void_p),
                ("p0", C.c_double), ("p1", C.c_double)]


def _declare(L):
    d, i32, i64, p = C.c_double, C.c_int, C.c_int64, C.c_void_p
    L.orc_student_t_logconstant.restype = d
    L.orc_student_t_logconstant.argtypes = [d, i32]
    L.orc_gaussian_lognormalizer.restype = d
    L.orc_gaussian_lognormalizer.argtypes = [i32, d]
    L.orc_factor_exponent_bound.restype = i32
    L.orc_factor_exponent_bound.argtypes = [p, i32]
    L.orc_logaddexp.restype = d
    L.orc_logaddexp.argtypes = [d, d]
    L.orc_component_logdensity.restype = d
    L.orc_component_logdensity.argtypes = [C.POINTER(Bank), i32, p, p, p]
    L.orc_mixture_logdensity.argtypes = [C.POINTER(Bank), i32, i32, p, p, p, i64, p, i32, p, p, p]
    L.orc_draw.argtypes = [C.POINTER(Bank), p, i32, p, p, i32, p, i32, i64, p, p]
    L.orc_static_assign.argtypes = [p, i32, p, i64, i32, p]
    L.orc_target_logdensity.restype = d
    L.orc_target_logdensity.argtypes = [C.POINTER(Target), p]
    L.orc_logweight_summary.argtypes = [p, i64, p]
    L.orc_normalize.argtypes = [p, i64, p]
    L.orc_resampling_cdf_f32.argtypes = [p, i64, p]
    L.orc_resampling_cdf_f64.argtypes = [p, i64, p]
    L.orc_resample_select.argtypes = [p, p, i64, p, i64, p]
    L.orc_det_exp.restype = d
    L.orc_det_exp.argtypes = [d]
    L.orc_fixed_scale_bits.restype = i32
    L.orc_fixed_scale_bits.argtypes = [i64]
    L.orc_fixed_prefix.restype = i32
    L.orc_fixed_prefix.argtypes = [p, i64, p]
    L.orc_resample_multinomial_fixed.argtypes = [p, i64, p, i64, p]
    L.orc_resample_systematic_fixed.argtypes = [p, i64, d, i64, p]
    L.orc_local_resample.argtypes = [p, p, i32, p, p]
    L.orc_weighted_moments.argtypes = [p, i32, i64, p, p, p, p]
    L.orc_fit_factor.restype = i32
    L.orc_fit_factor.argtypes = [p, p, i32, p, d, d, d, p, p]
    L.orc_philox_normals.argtypes = [C.c_uint64, C.c_uint64, i64, p]
    L.orc_philox_uniforms.argtypes = [C.c_uint64, C.c_uint64, i64, p]
    L.orc_amis_run.restype = i32
    L.orc_amis_run.argtypes = [C.POINTER(Target), i32, i32, d, p, p, i32, p, p, p, i32, p, i32, d,
                               p, p, p, p, p, p, p, p, p, p]
    L.orc_set_threads.argtypes = [i32]
    L.orc_num_threads.restype = i32
    L.orc_weighted_quantile.argtypes = [p, i32, i64, p, p, i32, p]
    L.orc_npmc_run.restype = i32
    L.orc_npmc_run.argtypes = [C.POINTER(Target), i32, i32, d, p, p, i32, p, p, p, i32, p, i32, d,
                               p, p, p, p, p, p, p, p]
    L.orc_population_local_weights.argtypes = [p, p, i32, p, p, p, i32, d, i32, p, p, p, p, p]
    L.orc_population_covariances.argtypes = [p, i32, p, p, p, p, p, p, p, p, i32, p, p]
    L.orc_population_factors.argtypes = [p, i32, i32, p, p, p, p]


def _f64(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


def _ptr(a):
    return None if a is None else a.ctypes.data


class BankView:
    """Holds FP64 copies alive while the C struct points at them."""

    def __init__(self, d, family, scale_kind, locations, scales, lognormalizers, dofs=None, range_risk=None):
        self.loc = _f64(locations).reshape(-1)
        self.scales = _f64(scales).reshape(-1)
        self.lognorm = _f64(lognormalizers).reshape(-1)
        self.k = self.lognorm.size
        self.dofs = None if dofs is None else _f64(dofs).reshape(-1)
        self.rr = None if range_risk is None else np.ascontiguousarray(range_risk, dtype=np.uint8)
        self.struct = Bank(d, self.k, family, scale_kind, _ptr(self.loc), _ptr(self.scales),
                           _ptr(self.lognorm), _ptr(self.dofs), _ptr(self.rr))


def set_threads(n):
    lib().orc_set_threads(int(n))


def num_threads():
    return lib().orc_num_threads()


def student_t_logconstant(dof, d):
    return lib().orc_student_t_logconstant(float(dof), int(d))


def gaussian_lognormalizer(d, logabsdet):
    return lib().orc_gaussian_lognormalizer(int(d), float(logabsdet))


def factor_exponent_bound(factor):
    f = np.asfortranarray(_f64(factor))
    return lib().orc_factor_exponent_bound(f.ctypes.data, f.shape[0])


def range_risk_f(bound, dtype):
    """_factor_range_risk (src/student_t_range.jl:35-36)."""
    emin = 126 if dtype == np.float32 else 1022
    return bound >= emin // 2


def component_logdensity(bank, slot, x):
    x = _f64(x)
    vals = np.zeros(bank.struct.d)
    exps = np.zeros(bank.struct.d, dtype=np.int32)
    return lib().orc_component_logdensity(C.byref(bank.struct), int(slot), x.ctypes.data,
                                          vals.ctypes.data, exps.ctypes.data)


def mixture_logdensity(bank, x, kind=DENOM_FULL, coef=None, terms=0, group_of_slot=None,
                       slots=None, fixed_slot=0):
    x = _f64(x)
    n = x.size // bank.struct.d
    coef = None if coef is None else _f64(coef)
    grp = None if group_of_slot is None else np.ascontiguousarray(group_of_slot, dtype=np.int32)
    sl = None if slots is None else np.ascontiguousarray(slots, dtype=np.int32)
    out = np.empty(n)
    gen = np.empty(n)
    rs = np.empty(n, dtype=np.uint32)
    lib().orc_mixture_logdensity(C.byref(bank.struct), kind, int(terms), _ptr(coef), _ptr(grp),
                                 x.ctypes.data, n, _ptr(sl), int(fixed_slot), out.ctypes.data,
                                 gen.ctypes.data, rs.ctypes.data)
    return out, gen, rs


def draw(bank, normals, slots=None, fixed_slot=0, radial_normals=None, rn_stride=0,
         radial_uniforms=None, ru_stride=0):
    nz = _f64(normals)
    n = nz.size // bank.struct.d
    sl = None if slots is None else np.ascontiguousarray(slots, dtype=np.int32)
    rn = None if radial_normals is None else _f64(radial_normals)
    ru = None if radial_uniforms is None else _f64(radial_uniforms)
    out = np.empty(n * bank.struct.d)
    rs = np.empty(n, dtype=np.uint32)
    lib().orc_draw(C.byref(bank.struct), _ptr(sl), int(fixed_slot), nz.ctypes.data, _ptr(rn),
                   int(rn_stride), _ptr(ru), int(ru_stride), n, out.ctypes.data, rs.ctypes.data)
    return out, rs


def static_assign(cdf, uniforms, stratified=True):
    cdf = _f64(cdf)
    u = _f64(uniforms)
    out = np.empty(u.size, dtype=np.int32)
    lib().orc_static_assign(cdf.ctypes.data, cdf.size, u.ctypes.data, u.size, int(stratified),
                            out.ctypes.data)
    return out


def logweight_summary(lw):
    lw = _f64(lw)
    out = np.empty(3)
    lib().orc_logweight_summary(lw.ctypes.data, lw.size, out.ctypes.data)
    return out


def summary_to_ess_logz(sm, n):
    m, s, s2 = sm
    if s == 0.0:
        return 0.0, -np.inf
    return s * s / s2, m + np.log(s) - np.log(float(n))


def normalize(lw):
    lw = _f64(lw)
    out = np.empty(lw.size)
    lib().orc_normalize(lw.ctypes.data, lw.size, out.ctypes.data)
    return out


def resampling_cdf(lw, dtype=np.float32):
    if dtype == np.float32:
        a = np.ascontiguousarray(lw, dtype=np.float32)
        out = np.empty(a.size, dtype=np.float32)
        lib().orc_resampling_cdf_f32(a.ctypes.data, a.size, out.ctypes.data)
    else:
        a = _f64(lw)
        out = np.empty(a.size)
        lib().orc_resampling_cdf_f64(a.ctypes.data, a.size, out.ctypes.data)
    return out


def resample_select(cdf, lw, uniforms):
    cdf = _f64(cdf)
    lw = _f64(lw)
    u = _f64(uniforms)
    out = np.empty(u.size, dtype=np.int64)
    lib().orc_resample_select(cdf.ctypes.data, lw.ctypes.data, cdf.size, u.ctypes.data, u.size,
                              out.ctypes.data)
    return out


def det_exp(x):
    return lib().orc_det_exp(float(x))


def fixed_prefix(lw):
    lw = _f64(lw)
    out = np.empty(lw.size, dtype=np.uint64)
    st = lib().orc_fixed_prefix(lw.ctypes.data, lw.size, out.ctypes.data)
    return None if st != 0 else out


def resample_multinomial_fixed(lw, uniforms):
    lw = _f64(lw)
    u = _f64(uniforms)
    out = np.zeros(u.size, dtype=np.int64)
    lib().orc_resample_multinomial_fixed(lw.ctypes.data, lw.size, u.ctypes.data, u.size, out.ctypes.data)
    return out


def resample_systematic_fixed(lw, u, count):
    lw = _f64(lw)
    out = np.zeros(int(count), dtype=np.int64)
    lib().orc_resample_systematic_fixed(lw.ctypes.data, lw.size, float(u), int(count), out.ctypes.data)
    return out


def local_resample(lw, counts, uniforms):
    lw = _f64(lw)
    counts = np.ascontiguousarray(counts, dtype=np.int64)
    u = _f64(uniforms)
    out = np.zeros(counts.size, dtype=np.int64)
    lib().orc_local_resample(lw.ctypes.data, counts.ctypes.data, counts.size, u.ctypes.data, out.ctypes.data)
    return out


def weighted_moments(x, d, lw):
    x = _f64(x)
    lw = _f64(lw)
    n = lw.size
    mean = np.empty(d)
    cov = np.empty(d * d)
    w = np.empty(n)
    lib().orc_weighted_moments(x.ctypes.data, int(d), n, lw.ctypes.data, mean.ctypes.data,
                               cov.ctypes.data, w.ctypes.data)
    return mean, cov.reshape(d, d, order="F"), w


def fit_factor(mean, cov, prev_factor, dof=0.0, logconstant=0.0, regularization=None):
    d = len(mean)
    mean = _f64(mean)
    cov = np.asfortranarray(_f64(cov)).reshape(-1, order="F").copy()
    prev = np.asfortranarray(_f64(prev_factor)).reshape(-1, order="F").copy()
    reg = np.sqrt(np.finfo(np.float64).eps) if regularization is None else regularization
    L = np.empty(d * d)
    ln = C.c_double()
    st = lib().orc_fit_factor(mean.ctypes.data, cov.ctypes.data, d, prev.ctypes.data, float(dof),
                              float(logconstant), float(reg), L.ctypes.data, C.addressof(ln))
    return st, L.reshape(d, d, order="F"), ln.value


def weighted_quantile(x, d, w, probs):
    """(len(probs), d) weighted quantiles of x (n x d) under weights w."""
    x, w, pr = _f64(x), _f64(w), _f64(probs)
    n = w.size
    out = np.empty(pr.size * d)
    lib().orc_weighted_quantile(x.ctypes.data, int(d), n, w.ctypes.data, pr.ctypes.data, pr.size, out.ctypes.data)
    return out.reshape(pr.size, d)


def npmc_run(target, d, loc0, factor0, schedule, normals, family=GAUSSIAN, dof=0.0, regularization=None):
    """Complete N-PMC on fed draws. Returns a dict of FP64 arrays."""
    schedule = np.ascontiguousarray(schedule, dtype=np.int64)
    rounds = schedule.size
    total = int(schedule.sum())
    loc0 = _f64(loc0)
    f0 = np.asfortranarray(_f64(factor0)).reshape(-1, order="F").copy()
    nz = _f64(normals)
    reg = np.sqrt(np.finfo(np.float64).eps) if regularization is None else regularization
    out = dict(samples=np.empty(total * d), logweights=np.empty(total), round_ess=np.empty(rounds),
               round_logz=np.empty(rounds), adaptation_ess=np.empty(rounds), hist_loc=np.zeros(rounds * d),
               hist_factor=np.zeros(rounds * d * d), hist_lognorm=np.zeros(rounds))
    st = lib().orc_npmc_run(C.byref(target.struct), int(d), int(family), float(dof), loc0.ctypes.data,
                            f0.ctypes.data, rounds, schedule.ctypes.data, nz.ctypes.data, None, 0, None, 0,
                            float(reg), out["samples"].ctypes.data, out["logweights"].ctypes.data,
                            out["round_ess"].ctypes.data, out["round_logz"].ctypes.data,
                            out["adaptation_ess"].ctypes.data, out["hist_loc"].ctypes.data,
                            out["hist_factor"].ctypes.data, out["hist_lognorm"].ctypes.data)
    out["status"] = st
    return out


def population_local_weights(lw, x, d, starts, counts, thresholds, tolerance=1e-6, max_iterations=60):
    """Returns (weights, local_ess, powers, status, raw_means (K, d))."""
    lw = _f64(lw)
    x = _f64(x)
    starts = np.ascontiguousarray(starts, dtype=np.int64)
    counts = np.ascontiguousarray(counts, dtype=np.int64)
    thr = _f64(thresholds)
    k = starts.size
    w = np.zeros(lw.size)
    ess, pw = np.zeros(k), np.zeros(k)
    st = np.zeros(k, dtype=np.uint8)
    means = np.zeros(k * d)
    lib().orc_population_local_weights(lw.ctypes.data, x.ctypes.data, int(d), starts.ctypes.data, counts.ctypes.data,
                                       thr.ctypes.data, k, float(tolerance), int(max_iterations), w.ctypes.data,
                                       ess.ctypes.data, pw.ctypes.data, st.ctypes.data, means.ctypes.data)
    return w, ess, pw, st, means.reshape(k, d)


def population_covariances(x, d, weights, powers, status, locations, factors, dofs, starts, counts):
    """factors: (K, d, d) with factors[k] the column-major storage (row-major
    L^T); returns (centres (K, d), covariances (K, d, d))."""
    x, w, pw, loc = _f64(x), _f64(weights), _f64(powers), _f64(locations)
    fac = _f64(factors)
    st = np.ascontiguousarray(status, dtype=np.uint8)
    starts = np.ascontiguousarray(starts, dtype=np.int64)
    counts = np.ascontiguousarray(counts, dtype=np.int64)
    nu = None if dofs is None else _f64(dofs)
    k = starts.size
    cen = np.zeros(k * d)
    cov = np.zeros(k * d * d)
    lib().orc_population_covariances(x.ctypes.data, int(d), w.ctypes.data, pw.ctypes.data, st.ctypes.data,
                                     loc.ctypes.data, fac.ctypes.data, _ptr(nu), starts.ctypes.data,
                                     counts.ctypes.data, k, cen.ctypes.data, cov.ctypes.data)
    return cen.reshape(k, d), cov.reshape(k, d, d)


def population_factors(covs, d, status, dofs=None):
    """covs: (K, d, d) (symmetric); returns (factors (K, d, d) in the same
    column-major storage, info (K,))."""
    c = _f64(covs)
    k = c.shape[0]
    st = np.ascontiguousarray(status, dtype=np.uint8)
    nu = None if dofs is None else _f64(dofs)
    f = np.zeros(k * d * d)
    info = np.zeros(k, dtype=np.int32)
    lib().orc_population_factors(c.ctypes.data, int(d), k, st.ctypes.data, _ptr(nu), f.ctypes.data,
                                 info.ctypes.data)
    return f.reshape(k, d, d), info


def philox_normals(seed, offset, n):
    out = np.empty(int(n))
    lib().orc_philox_normals(int(seed), int(offset), int(n), out.ctypes.data)
    return out


def philox_uniforms(seed, offset, n):
    out = np.empty(int(n))
    lib().orc_philox_uniforms(int(seed), int(offset), int(n), out.ctypes.data)
    return out


class TargetView:
    def __init__(self, kind, d, j=0, a=None, b=None, c=None, p0=0.0, p1=0.0):
        # matrices are stored column-major, as the reference's Julia arrays
        flat = lambda v: None if v is None else np.ascontiguousarray(np.asarray(v, dtype=np.float64).ravel(order="F"))  # noqa: E731
        self.a, self.b, self.c = flat(a), flat(b), flat(c)
        self.struct = Target(kind, d, j, _ptr(self.a), _ptr(self.b), _ptr(self.c), float(p0), float(p1))


def target_logdensity(target, x):
    x = _f64(x)
    return lib().orc_target_logdensity(C.byref(target.struct), x.ctypes.data)


def amis_run(target, d, loc0, factor0, schedule, normals, family=GAUSSIAN, dof=0.0,
             radial_normals=None, rn_stride=0, radial_uniforms=None, ru_stride=0,
             regularization=None):
    """Complete AMIS on fed draws. Returns a dict of FP64 arrays."""
    schedule = np.ascontiguousarray(schedule, dtype=np.int64)
    rounds = schedule.size
    total = int(schedule.sum())
    loc0 = _f64(loc0)
    f0 = np.asfortranarray(_f64(factor0)).reshape(-1, order="F").copy()
    nz = _f64(normals)
    rn = None if radial_normals is None else _f64(radial_normals)
    ru = None if radial_uniforms is None else _f64(radial_uniforms)
    reg = np.sqrt(np.finfo(np.float64).eps) if regularization is None else regularization
    out = dict(samples=np.empty(total * d), logtargets=np.empty(total), lognum=np.empty(total),
               logweights=np.empty(total), round_ess=np.empty(rounds), round_logz=np.empty(rounds),
               hist_loc=np.zeros(rounds * d), hist_factor=np.zeros(rounds * d * d),
               hist_lognorm=np.zeros(rounds), reasons=np.zeros(total, dtype=np.uint32))
    st = lib().orc_amis_run(C.byref(target.struct), int(d), int(family), float(dof), loc0.ctypes.data,
                            f0.ctypes.data, rounds, schedule.ctypes.data, nz.ctypes.data, _ptr(rn),
                            int(rn_stride), _ptr(ru), int(ru_stride), float(reg),
                            out["samples"].ctypes.data, out["logtargets"].ctypes.data,
                            out["lognum"].ctypes.data, out["logweights"].ctypes.data,
                            out["round_ess"].ctypes.data, out["round_logz"].ctypes.data,
                            out["hist_loc"].ctypes.data, out["hist_factor"].ctypes.data,
                            out["hist_lognorm"].ctypes.data, out["reasons"].ctypes.data)
    out["status"] = st
    return out
