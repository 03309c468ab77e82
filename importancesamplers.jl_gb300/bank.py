"""ProposalBank and its packed device form (src/proposal_banks.jl).

`ProposalBank` validates and normalises masses like the reference; `pack()`
builds the device bank the kernels read: slots are the positive-mass
proposals sorted stably by mass (the order that defines the assignment CDF),
stored as the reference's column-major arrays in torch tensors.
"""
import math

import numpy as np
import torch

from . import native
from .proposals import DIAGONAL, FACTOR, GAUSSIAN, SPHERICAL, STUDENT_T, factor_range_risk


class ProposalBank:
    """Explicit proposal population with normalised nonnegative masses
    (ProposalBank, src/proposal_banks.jl:40-95)."""

    def __init__(self, proposals, masses=None):
        proposals = list(proposals)
        if not proposals:
            raise ValueError("a proposal bank cannot be empty")
        if masses is None:
            dt = proposals[0].dtype
            masses = np.ones(len(proposals), dtype=dt)
        masses = np.asarray(masses)
        if masses.size != len(proposals):
            raise ValueError("proposal and mass counts must match")
        if masses.dtype == np.bool_:
            raise TypeError("mass element type must be a concrete non-Bool real type")
        ft = np.promote_types(masses.dtype if masses.dtype.kind == "f" else np.float64, np.float32)
        fm = masses.astype(ft)
        if np.any((masses > 0) & ~(fm > 0)):
            raise ValueError("positive masses must stay positive through floating conversion")
        if not np.all(np.isfinite(fm)):
            raise ValueError("masses must be finite")
        if np.any(fm < 0):
            raise ValueError("masses must be nonnegative")
        mx = fm.max()
        if not mx > 0:
            raise ValueError("at least one mass must be positive")
        scaled = fm / mx
        normalized = scaled / scaled.sum()
        if np.any((scaled > 0) & ~(normalized > 0)):
            raise ValueError("positive masses must stay positive through final normalization")
        self.proposals = proposals
        self.masses = normalized

    def __len__(self):
        return len(self.proposals)

    def active_metadata(self):
        """_prepare_active_proposal_metadata (src/proposal_banks.jl:301-326):
        1-based ids of positive masses sorted stably by mass, the assignment
        CDF and the normalised log masses."""
        ids = [i + 1 for i in np.flatnonzero(self.masses != 0)]
        ids.sort(key=lambda pid: self.masses[pid - 1])  # Python sort is stable
        dt = self.masses.dtype.type
        m = np.array([self.masses[i - 1] for i in ids], dtype=dt)
        m = m / m.sum()
        cdf = np.cumsum(m, dtype=dt)
        cdf[-1] = dt(1)
        logm = np.empty_like(cdf)
        prev = dt(0)
        for s in range(cdf.size):
            if not cdf[s] > prev:
                raise ValueError("every positive proposal mass must retain a positive assignment interval")
            logm[s] = np.log(cdf[s] - prev)
            prev = cdf[s]
        mx = logm.max()
        logm = logm - dt(mx + np.log(np.sum(np.exp(logm - mx))))
        return ids, logm, cdf


class DeviceBank:
    """Packed device bank (_PackedFactorBank / _PackedDiagonalBank) plus the
    C-ABI struct that points into it."""

    def __init__(self, d, count, family, scale_kind, dtype, locations, scales, lognormalizers, dofs=None,
                 range_risk=None, proposal_ids=None, logmasses=None, cdf=None):
        self.d, self.count, self.family, self.scale_kind, self.dtype = d, count, family, scale_kind, dtype
        self.locations, self.scales, self.lognormalizers = locations, scales, lognormalizers
        self.dofs, self.range_risk = dofs, range_risk
        self.proposal_ids, self.logmasses, self.cdf = proposal_ids, logmasses, cdf
        self.refresh()

    def refresh(self):
        self.struct = native.Bank(self.d, self.count, self.family, self.scale_kind, native.dtype_code(self.dtype),
                                  0, native.ptr(self.locations), native.ptr(self.scales),
                                  native.ptr(self.lognormalizers), native.ptr(self.dofs),
                                  native.ptr(self.range_risk), native.ptr(getattr(self, "inverse_factors", None)))
        return self

    def attach_inverse_factors(self, first=0, count=None):
        """Allocate (once) and fill the FP32 inverse factors W_k = L_k^-1 the
        tensor-core forms read (issm_bank.inverse_factors)."""
        if self.scale_kind != native.SCALE_FACTOR or self.dtype != torch.float32 or self.d > 64:
            return self
        dp = 16 if self.d <= 16 else 32 if self.d <= 32 else 64
        if getattr(self, "inverse_factors", None) is None:
            self.inverse_factors = torch.zeros(self.count, dp, dp, dtype=torch.float32, device=self.locations.device)
            self.refresh()
            self.__dict__.pop("_views", None)
        count = self.count - first if count is None else count
        if count > 0:
            native.call("issm_invert_factors", self.ref(), int(first), int(count), native.ptr(self.inverse_factors),
                        native.stream_ptr())
        return self

    def ref(self):
        import ctypes

        return ctypes.byref(self.struct)


def _scale_kind_code(kind):
    return {FACTOR: native.SCALE_FACTOR, DIAGONAL: native.SCALE_DIAGONAL, SPHERICAL: native.SCALE_SPHERICAL}[kind]


def pack_proposals(proposals, device, dtype=None):
    """Pack homogeneous radial proposals into a DeviceBank (one slot each)."""
    first = proposals[0]
    dt = first.dtype
    for p in proposals:
        if p.family != first.family or p.dtype != dt:
            raise ValueError("a packed proposal bank requires one radial family and floating type")
        if p.dimension != first.dimension:
            raise ValueError("positive-mass native Gaussian proposals must have one common dimension")
    kinds = {p.scale_kind for p in proposals}
    kind = FACTOR if FACTOR in kinds else (DIAGONAL if DIAGONAL in kinds else SPHERICAL)
    d, k = first.dimension, len(proposals)
    tdt = torch.float32 if dt == np.float32 else torch.float64
    loc = np.stack([p.location for p in proposals]).astype(dt)
    if kind == FACTOR:
        # slot k holds L_k column-major: the row-major storage of L_k^T
        sc = np.stack([p.factor_matrix().T for p in proposals]).astype(dt)
    elif kind == DIAGONAL:
        sc = np.stack([np.broadcast_to(np.asarray(p.scale, dtype=dt), (d,)) for p in proposals]).astype(dt)
    else:
        sc = np.array([p.scale for p in proposals], dtype=dt)
    lnorm = np.array([p.lognormalizer for p in proposals], dtype=dt)
    dofs = rr = None
    if first.family == STUDENT_T:
        dofs = torch.tensor(np.array([p.dof for p in proposals], dtype=dt), device=device)
        if kind == FACTOR:
            rr = torch.tensor([1 if factor_range_risk(p.exponent_bound(), dt) else 0 for p in proposals],
                              dtype=torch.uint8, device=device)
    # torch.tensor keeps numpy strides; the kernels read raw C-order memory
    return DeviceBank(d, k, native.STUDENT_T if first.family == STUDENT_T else native.GAUSSIAN,
                      _scale_kind_code(kind), tdt,
                      torch.tensor(np.ascontiguousarray(loc), device=device).contiguous(),
                      torch.tensor(np.ascontiguousarray(sc), device=device).contiguous(),
                      torch.tensor(np.ascontiguousarray(lnorm), device=device).contiguous(), dofs, rr)


def pack(bank, device):
    """Pack the active slots of a ProposalBank."""
    ids, logm, cdf = bank.active_metadata()
    proposals = [bank.proposals[i - 1] for i in ids]
    db = pack_proposals(proposals, device)
    db.proposal_ids = torch.tensor(ids, dtype=torch.int64, device=device)
    db.logmasses = torch.tensor(logm.astype(proposals[0].dtype), device=device)
    db.cdf = torch.tensor(cdf.astype(proposals[0].dtype), device=device)
    db.host_ids, db.host_logmasses, db.host_cdf = ids, logm, cdf
    db.attach_inverse_factors()
    return db


class DeviceHistory(DeviceBank):
    """AMIS proposal history: `rounds` factor slots filled as rounds adapt
    (_FactorProposalHistory, src/adaptive_gaussian.jl:53-59,102-123)."""

    @classmethod
    def allocate(cls, proposal, rounds, device):
        d = proposal.dimension
        dt = proposal.dtype
        tdt = torch.float32 if dt == np.float32 else torch.float64
        loc = torch.zeros(rounds, d, dtype=tdt, device=device)
        sc = torch.zeros(rounds, d, d, dtype=tdt, device=device)
        lnorm = torch.zeros(rounds, dtype=tdt, device=device)
        # slot 0 in one host-to-device copy
        host = np.concatenate([np.asarray(proposal.location, dtype=dt).reshape(-1),
                               np.ascontiguousarray(proposal.factor_matrix().T, dtype=dt).reshape(-1),
                               np.asarray([proposal.lognormalizer], dtype=dt)])
        first = torch.from_numpy(host).to(device)
        loc[0].copy_(first[:d])
        sc[0].copy_(first[d:d + d * d].view(d, d))
        lnorm[0:1].copy_(first[d + d * d:])
        dofs = rr = None
        fam = native.GAUSSIAN
        if proposal.family == STUDENT_T:
            fam = native.STUDENT_T
            dofs = torch.full((rounds,), float(proposal.dof), dtype=tdt, device=device)
            rr = torch.zeros(rounds, dtype=torch.uint8, device=device)
        h = cls(d, rounds, fam, native.SCALE_FACTOR, tdt, loc, sc, lnorm, dofs, rr)
        h.logconstant = 0.0 if proposal.family != STUDENT_T else float(proposal.logconstant)
        h.dof = 0.0 if proposal.family != STUDENT_T else float(proposal.dof)
        h.attach_inverse_factors(0, 1)
        return h

    def view(self, slots):
        """A bank struct over the first `slots` history slots."""
        import ctypes

        views = self.__dict__.setdefault("_views", {})
        if slots not in views:
            views[slots] = native.Bank(self.d, slots, self.family, self.scale_kind, native.dtype_code(self.dtype), 0,
                                       native.ptr(self.locations), native.ptr(self.scales),
                                       native.ptr(self.lognormalizers), native.ptr(self.dofs),
                                       native.ptr(self.range_risk),
                                       native.ptr(getattr(self, "inverse_factors", None)))
        return ctypes.byref(views[slots])


def log_sum_exp(values):
    m = max(values)
    return m + math.log(sum(math.exp(v - m) for v in values))
