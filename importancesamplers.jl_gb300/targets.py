"""Targets: a user batch callback (LogTarget, src/targets.jl:65-76 with the
batch path of src/batched_targets.jl) or one of the built-in native targets the
benchmark workloads use. Every target maps an (n, d) device tensor of samples
to n log densities on the device."""
import numpy as np
import torch

from . import native, ops
from .proposals import student_t_logconstant


class LogTarget:
    """LogTarget(batch=f): f(samples (n, d) tensor) -> (n,) tensor of log densities."""

    def __init__(self, batch):
        if not callable(batch):
            raise TypeError("batch must be callable")
        self.batch = batch

    def bind(self, device, dtype):
        return self

    def evaluate(self, samples, out=None):
        v = self.batch(samples)
        if not isinstance(v, torch.Tensor) or v.shape != (samples.shape[0],):
            raise ValueError("a batch target must return one log density per sample")
        v = v.to(dtype=samples.dtype)
        if out is not None:
            out.copy_(v)
            return out
        return v


class _NativeTarget:
    kind = None

    def __init__(self, d, count=0, a=None, b=None, p0=0.0, p1=0.0):
        self.d, self.count, self.p0, self.p1 = d, count, float(p0), float(p1)
        self.host = (a, b)
        self._bound = {}

    def bind(self, device, dtype):
        key = (str(device), dtype)
        if key not in self._bound:
            a, b = self.host
            ta = None if a is None else torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device=device)
            tb = None if b is None else torch.as_tensor(np.ascontiguousarray(b), dtype=dtype, device=device)
            s = native.Target(self.kind, self.d, self.count, native.dtype_code(dtype), native.ptr(ta),
                              native.ptr(tb), None, self.p0, self.p1)
            self._bound[key] = (s, ta, tb)
        bound = _Bound(self, *self._bound[key])
        return bound


class _Bound:
    def __init__(self, target, struct, ta, tb):
        self.target, self.struct, self.keep = target, struct, (ta, tb)

    def evaluate(self, samples, out=None):
        return ops.target_logdensity(self.struct, samples, out)


def _colmajor(a):
    """Reference matrices are column-major: store A^T row-major."""
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).T)


class StandardNormalTarget(_NativeTarget):
    kind = native.TARGET_STD_NORMAL

    def __init__(self, d):
        super().__init__(d)


class QuadraticTarget(_NativeTarget):
    """-|x - center|^2 / divisor."""
    kind = native.TARGET_QUADRATIC

    def __init__(self, center, divisor):
        c = np.atleast_1d(np.asarray(center, dtype=np.float64))
        super().__init__(c.size, a=c, p0=divisor)


class GaussianMixtureTarget(_NativeTarget):
    """Equal-weight mixture of N(mean_j, I); means is (J, d)."""
    kind = native.TARGET_GAUSS_MIX

    def __init__(self, means):
        m = np.atleast_2d(np.asarray(means, dtype=np.float64))
        super().__init__(m.shape[1], count=m.shape[0], a=m)


class StudentTTarget(_NativeTarget):
    """Normalised multivariate t with location, lower scale factor L and nu."""
    kind = native.TARGET_STUDENT_T

    def __init__(self, location, factor, dof):
        loc = np.asarray(location, dtype=np.float64).reshape(-1)
        L = np.asarray(factor, dtype=np.float64)
        d = loc.size
        logc = student_t_logconstant(float(dof), d) - float(np.sum(np.log(np.diag(L))))
        super().__init__(d, a=loc, b=_colmajor(L), p0=dof, p1=logc)
        self.location, self.factor, self.dof = loc, L, float(dof)


class LinearRegressionTarget(_NativeTarget):
    """N(y | X beta, sigma^2 I) N(beta | 0, prior_var I) (unnormalised posterior,
    normalised joint: its log evidence is the analytic conjugate value)."""
    kind = native.TARGET_LINREG

    def __init__(self, X, y, sigma, prior_var=1.0):
        X = np.asarray(X, dtype=np.float64)
        super().__init__(X.shape[1], count=X.shape[0], a=_colmajor(X), b=np.asarray(y, dtype=np.float64),
                         p0=sigma, p1=prior_var)
        self.X, self.y, self.sigma, self.prior_var = X, np.asarray(y, dtype=np.float64), float(sigma), float(prior_var)

    def analytic(self):
        """Posterior mean and log evidence of the conjugate model."""
        X, y, s2, pv = self.X, self.y, self.sigma ** 2, self.prior_var
        n, d = X.shape
        A = X.T @ X / s2 + np.eye(d) / pv
        b = X.T @ y / s2
        mean = np.linalg.solve(A, b)
        cov_y = s2 * np.eye(n) + pv * X @ X.T
        sign, logdet = np.linalg.slogdet(cov_y)
        logz = -0.5 * (n * np.log(2 * np.pi) + logdet + y @ np.linalg.solve(cov_y, y))
        return mean, logz


class LogisticRegressionTarget(_NativeTarget):
    """Bernoulli-logit(y | X beta) N(beta | 0, prior_var I)."""
    kind = native.TARGET_LOGISTIC

    def __init__(self, X, y, prior_var=10.0):
        X = np.asarray(X, dtype=np.float64)
        super().__init__(X.shape[1], count=X.shape[0], a=_colmajor(X), b=np.asarray(y, dtype=np.float64),
                         p1=prior_var)
