"""Native radial proposals: Gaussian and Student-t in spherical, diagonal and
lower-triangular factor forms (src/proposals.jl).

Construction validates like the reference and precomputes the normalised
log-density constant; parameters live on the host as numpy arrays of the
proposal's float type (float32 or float64) until a bank is packed onto the
device.
"""
import math

import numpy as np

GAUSSIAN, STUDENT_T = 0, 1
SPHERICAL, DIAGONAL, FACTOR = "spherical", "diagonal", "factor"


def _float_type(location):
    a = np.asarray(location)
    if a.dtype not in (np.float32, np.float64):
        raise TypeError("native parameter must be a Float32 or Float64 scalar or vector")
    return a.dtype.type


def _validated_location(location):
    dt = _float_type(location)
    a = np.array(location, dtype=dt, copy=True)
    if a.ndim > 1 or a.size == 0:
        raise ValueError("native parameter must be nonempty")
    if not np.all(np.isfinite(a)):
        raise ValueError("native parameter must contain only finite values")
    return a, dt


def gaussian_lognormalizer(dt, dimension, logabsdet):
    """_gaussian_lognormalizer (src/proposals.jl:237-240)."""
    logtwopi = math.log(2.0 * math.pi)
    return dt(-0.5 * dimension * logtwopi - float(logabsdet))


def student_t_logconstant(dof, dimension):
    """_student_t_logconstant (src/proposals.jl:413-437): log Gamma((nu+d)/2) -
    log Gamma(nu/2) - d/2 log(nu pi) - ... evaluated through the shifted
    gamma-ratio recurrence and six Stirling terms for odd d."""
    dof = float(dof)
    value = -dimension * math.log(2.0 * math.pi) / 2.0
    if dimension % 2 == 1:
        shifted, correction = dof, 0.0
        while shifted < 32.0:
            if shifted < 1.0:
                correction += (math.log(shifted) + math.log(shifted + 2.0)) / 2.0 - math.log1p(shifted)
            else:
                correction += math.log1p(-(1.0 / (shifted + 1.0)) ** 2) / 2.0
            shifted += 2.0
        r = 1.0 / shifted
        coeffs = (-1.0 / 4.0, 1.0 / 24.0, -1.0 / 20.0, 17.0 / 112.0, -31.0 / 36.0, 691.0 / 88.0)
        poly = 0.0
        for c in reversed(coeffs):
            poly = poly * (r * r) + c
        correction += r * poly
        value += correction
    start = 1 if dimension % 2 == 1 else 0
    for offset in range(start, dimension - 1, 2):
        x = float(offset)
        value += math.log1p(x / dof) if x <= dof else math.log(x) + math.log1p(dof / x) - math.log(dof)
    return value


def factor_exponent_bound(factor):
    """_factor_exponent_bound (src/student_t_range.jl:21-31): the largest
    |e| or |e - 1| over the binary exponents e (v = m 2^e, m in [0.5, 1)) of
    the nonzero lower-triangle entries; 2^62 when one is not finite."""
    f = np.asarray(factor, dtype=np.float64)
    v = f[np.tril_indices(f.shape[0])]
    v = v[v != 0.0]
    if v.size == 0:
        return 0
    if not np.all(np.isfinite(v)):
        return 1 << 62
    e = np.frexp(v)[1].astype(np.int64)
    return int(max(np.abs(e).max(), np.abs(e - 1).max()))


def factor_range_risk(bound, dt):
    """_factor_range_risk (src/student_t_range.jl:35-36)."""
    emin = 126 if dt == np.float32 else 1022
    return bound >= emin // 2


class RadialProposal:
    """One native radial proposal (_GaussianProposal / _StudentTProposal)."""

    def __init__(self, family, location, scale_kind, scale, logabsdet, dof=None):
        loc, dt = _validated_location(location)
        self.scalar = np.ndim(location) == 0
        self.dtype = dt
        self.location = loc.reshape(-1)
        self.dimension = self.location.size
        self.family = family
        self.scale_kind = scale_kind
        self.scale = scale
        if family == STUDENT_T:
            if not (isinstance(dof, (float, np.floating)) and math.isfinite(dof) and dof > 0):
                raise ValueError("degrees of freedom must be finite and positive")
            self.dof = dt(dof)
            self.logconstant = dt(student_t_logconstant(float(self.dof), self.dimension))
            self.lognormalizer = dt(float(self.logconstant) - float(logabsdet))
        else:
            self.dof = None
            self.logconstant = None
            self.lognormalizer = gaussian_lognormalizer(dt, self.dimension, logabsdet)

    # dense lower-triangular factor of the scale (covariance for Gaussians)
    def factor_matrix(self):
        d = self.dimension
        if self.scale_kind == FACTOR:
            return np.array(self.scale, dtype=self.dtype)
        if self.scale_kind == DIAGONAL:
            return np.diag(np.asarray(self.scale, dtype=self.dtype))
        return np.eye(d, dtype=self.dtype) * self.dtype(self.scale)

    def exponent_bound(self):
        return factor_exponent_bound(self.factor_matrix()) if self.scale_kind == FACTOR else 0

    def __repr__(self):
        fam = "Gaussian" if self.family == GAUSSIAN else f"StudentT(nu={float(self.dof)})"
        return f"{self.scale_kind.capitalize()}{fam}(d={self.dimension}, {self.dtype.__name__})"


def _positive_scale(scale, dt):
    s = np.asarray(scale)
    if s.dtype != dt:
        raise TypeError("scale must have the same Float32 or Float64 type as location")
    if not (np.all(np.isfinite(s)) and np.all(s > 0)):
        raise ValueError("scale must be finite and positive")
    return s


def _factor(factor, location):
    dt = _float_type(location)
    L = np.array(factor, copy=True)
    if L.dtype != dt:
        raise TypeError("factor must have the same floating type as location")
    d = np.asarray(location).size
    if L.shape != (d, d):
        raise ValueError("factor must be square and match the location length")
    if not np.all(np.isfinite(L)):
        raise ValueError("factor must contain only finite values")
    if np.any(np.triu(L, 1) != 0):
        raise ValueError("factor must be lower triangular")
    if not np.all(np.diag(L) > 0):
        raise ValueError("factor diagonal must be positive")
    return L


def SphericalGaussian(location, scale):
    """N(location, scale^2 I) (src/proposals.jl:242-268)."""
    dt = _float_type(location)
    s = _positive_scale(scale, dt)
    d = np.asarray(location).size
    return RadialProposal(GAUSSIAN, location, SPHERICAL, dt(s), d * math.log(float(s)))


def DiagonalGaussian(location, scales):
    """N(location, diag(scales)^2) (src/proposals.jl:285-315)."""
    if np.ndim(location) == 0:
        raise ValueError("DiagonalGaussian requires a vector location")
    dt = _float_type(location)
    s = _positive_scale(scales, dt).reshape(-1)
    if s.size != np.asarray(location).size:
        raise ValueError("diagonal scales must match the location length")
    return RadialProposal(GAUSSIAN, location, DIAGONAL, s.copy(), float(np.sum(np.log(s.astype(np.float64)))))


def FactorGaussian(location, factor):
    """N(location, L L^T) with lower-triangular L (src/proposals.jl:367-393)."""
    if np.ndim(location) == 0:
        raise ValueError("FactorGaussian requires a vector location")
    L = _factor(factor, location)
    return RadialProposal(GAUSSIAN, location, FACTOR, L, float(np.sum(np.log(np.diag(L).astype(np.float64)))))


def SphericalStudentT(dof, location, scale):
    """Student-t with spherical elliptical scale (src/proposals.jl:453-475)."""
    dt = _float_type(location)
    s = _positive_scale(scale, dt)
    d = np.asarray(location).size
    return RadialProposal(STUDENT_T, location, SPHERICAL, dt(s), d * math.log(float(s)), dof=dt(dof))


def DiagonalStudentT(dof, location, scales):
    """Student-t with diagonal elliptical scale (src/proposals.jl:477-503)."""
    if np.ndim(location) == 0:
        raise ValueError("DiagonalStudentT requires a vector location")
    dt = _float_type(location)
    s = _positive_scale(scales, dt).reshape(-1)
    return RadialProposal(STUDENT_T, location, DIAGONAL, s.copy(), float(np.sum(np.log(s.astype(np.float64)))),
                          dof=dt(dof))


def FactorStudentT(dof, location, factor):
    """Student-t with scale matrix L L^T (src/proposals.jl:505-529)."""
    if np.ndim(location) == 0:
        raise ValueError("FactorStudentT requires a vector location")
    dt = _float_type(location)
    L = _factor(factor, location)
    return RadialProposal(STUDENT_T, location, FACTOR, L, float(np.sum(np.log(np.diag(L).astype(np.float64)))),
                          dof=dt(dof))
