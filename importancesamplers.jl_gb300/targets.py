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

    def evaluate(self, samples, out=None, precision=None):
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
        self.operands = {}  # tensor-core operand form of a regression target, per precision

    def tensor_operand(self, precision, dtype, device):
        """The observations' tensor-core operand form when this target runs
        its X beta on the tensor cores at `precision` for samples of `dtype`
        (a regression target, a reduced-precision form, FP32, d <= 64), built
        once per precision; else None (the SIMT kernel)."""
        prec = native.PREC_NATIVE if precision is None else int(precision)
        s = self.struct
        if not (prec != native.PREC_NATIVE and s.kind in (native.TARGET_LINREG, native.TARGET_LOGISTIC)
                and dtype == torch.float32 and s.dtype == native.F32 and s.dim <= 64):
            return None
        if prec not in self.operands:
            self.operands[prec] = ops.glm_operand(s, prec, device)
        return self.operands[prec]

    def evaluate(self, samples, out=None, precision=None):
        """The regression targets run their X beta on the tensor cores in the
        reduced-precision forms (FP32 samples, d <= 64); every other case is
        the SIMT kernel in the target's type."""
        operand = self.tensor_operand(precision, samples.dtype, samples.device)
        if operand is not None:
            return ops.glm_logdensity(self.struct, int(precision), operand, samples, out)
        return ops.target_logdensity(self.struct, samples, out)


class _BoundBank:
    """A normalised target that is itself a radial mixture: evaluated by the
    same balance-heuristic kernels as the proposals (SIMT or tensor core)."""

    def __init__(self, bank, coef):
        self.bank, self.coef = bank, coef
        kind = native.DENOM_GENERATING if coef is None else native.DENOM_FULL
        self.den = ops.denominator(kind, coef)

    def effective_precision(self, precision, dtype):
        """The form the density kernels run in: a tensor-core form only for a
        factor bank and FP32 samples, else the SIMT form."""
        prec = native.PREC_NATIVE if precision is None else int(precision)
        if prec != native.PREC_NATIVE and (self.bank.scale_kind != native.SCALE_FACTOR or dtype != torch.float32):
            prec = native.PREC_NATIVE
        return prec

    def evaluate(self, samples, out=None, precision=None):
        prec = self.effective_precision(precision, samples.dtype)
        return ops.mixture_logdensity(self.bank, self.den, samples, fixed_slot=0, precision=prec, out=out)


def _bank_target(key_store, key, proposals, coef_value, device, dtype):
    if key not in key_store:
        from .bank import pack_proposals

        npdt = np.float32 if dtype == torch.float32 else np.float64
        props = [p(npdt) for p in proposals]
        bank = pack_proposals(props, device)
        bank.attach_inverse_factors()
        coef = None
        if coef_value is not None:
            coef = torch.full((bank.count,), coef_value, dtype=dtype, device=device)
        key_store[key] = _BoundBank(bank, coef)
    return key_store[key]


def _colmajor(a):
    """Reference matrices are column-major: store A^T row-major."""
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).T)


class StandardNormalTarget(_NativeTarget):
    """N(0, I), normalised: evaluated as a one-slot factor bank."""
    kind = native.TARGET_STD_NORMAL

    def __init__(self, d):
        super().__init__(d)

    def bind(self, device, dtype):
        from .proposals import FactorGaussian

        d = self.d
        return _bank_target(self._bound, ("bank", str(device), dtype),
                            [lambda t: FactorGaussian(np.zeros(d, dtype=t), np.eye(d, dtype=t))], None, device, dtype)


class QuadraticTarget(_NativeTarget):
    """-|x - center|^2 / divisor."""
    kind = native.TARGET_QUADRATIC

    def __init__(self, center, divisor):
        c = np.atleast_1d(np.asarray(center, dtype=np.float64))
        super().__init__(c.size, a=c, p0=divisor)


class GaussianMixtureTarget(_NativeTarget):
    """Equal-weight mixture of N(mean_j, I); means is (J, d). Evaluated as a
    balance-heuristic bank with coefficients -log J."""
    kind = native.TARGET_GAUSS_MIX

    def __init__(self, means):
        m = np.atleast_2d(np.asarray(means, dtype=np.float64))
        super().__init__(m.shape[1], count=m.shape[0], a=m)
        self.means = m

    def bind(self, device, dtype):
        from .proposals import FactorGaussian

        d = self.d
        props = [lambda t, mu=mu: FactorGaussian(mu.astype(t), np.eye(d, dtype=t)) for mu in self.means]
        return _bank_target(self._bound, ("bank", str(device), dtype), props, -float(np.log(len(self.means))),
                            device, dtype)


class StudentTTarget(_NativeTarget):
    """Normalised multivariate t with location, lower scale factor L and nu:
    a one-slot factor Student-t bank."""
    kind = native.TARGET_STUDENT_T

    def __init__(self, location, factor, dof):
        loc = np.asarray(location, dtype=np.float64).reshape(-1)
        L = np.asarray(factor, dtype=np.float64)
        d = loc.size
        logc = student_t_logconstant(float(dof), d) - float(np.sum(np.log(np.diag(L))))
        super().__init__(d, a=loc, b=_colmajor(L), p0=dof, p1=logc)
        self.location, self.factor, self.dof = loc, L, float(dof)

    def bind(self, device, dtype):
        from .proposals import FactorStudentT

        loc, L, nu = self.location, self.factor, self.dof
        return _bank_target(self._bound, ("bank", str(device), dtype),
                            [lambda t: FactorStudentT(t(nu), loc.astype(t), L.astype(t))], None, device, dtype)


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
        # y ~ N(0, C), C = s2 I_n + pv X X^T, in d x d form: det C = s2^n
        # pv^d det A (determinant lemma) and y^T C^-1 y = (y^T y - y^T X
        # A^-1 X^T y / s2) / s2 (Woodbury)
        L = np.linalg.cholesky(A)
        logdet = n * np.log(s2) + d * np.log(pv) + 2.0 * np.sum(np.log(np.diag(L)))
        quad = (y @ y - b @ mean * s2) / s2
        logz = -0.5 * (n * np.log(2 * np.pi) + logdet + quad)
        return mean, logz


class LogisticRegressionTarget(_NativeTarget):
    """Bernoulli-logit(y | X beta) N(beta | 0, prior_var I)."""
    kind = native.TARGET_LOGISTIC

    def __init__(self, X, y, prior_var=10.0):
        X = np.asarray(X, dtype=np.float64)
        super().__init__(X.shape[1], count=X.shape[0], a=_colmajor(X), b=np.asarray(y, dtype=np.float64),
                         p1=prior_var)
