"""Algorithm configurations (src/methods/*.jl): typed, validated at
construction, and independent of the device they later run on."""
import math

from .bank import ProposalBank
from .proposals import RadialProposal


class AbstractMISScheme:
    pass


class StratifiedMixture(AbstractMISScheme):
    """Stratified assignment + full balance-heuristic mixture (src/methods/static_mis.jl)."""


class RandomMixture(AbstractMISScheme):
    """Independent assignment + full mixture."""


class StandardMIS(AbstractMISScheme):
    """Stratified assignment + generating-proposal denominator."""


class PartialDeterministicMixture(AbstractMISScheme):
    """Stratified assignment + mixture restricted to the generating proposal's group."""

    def __init__(self, groups):
        self.groups = [list(g) for g in groups]


def _schedule(rounds, round_size):
    """_validate_adaptive_schedule: positive Int rounds, Int or per-round sizes."""
    if not isinstance(rounds, int) or isinstance(rounds, bool) or rounds < 1:
        raise ValueError("rounds must be a positive Int")
    if isinstance(round_size, int) and not isinstance(round_size, bool):
        if round_size < 1:
            raise ValueError("round_size must be positive")
        return [round_size] * rounds
    sizes = list(round_size)
    if len(sizes) != rounds or not all(isinstance(s, int) and not isinstance(s, bool) and s > 0 for s in sizes):
        raise ValueError("round_size must be a positive Int or a positive Int vector with one entry per round")
    return sizes


class ImportanceSampling:
    """ImportanceSampling(proposal_or_bank; nsamples, mis_scheme)
    (src/methods/importance_sampling.jl:46-86)."""

    def __init__(self, proposal, nsamples, mis_scheme=None):
        if not isinstance(nsamples, int) or nsamples < 1:
            raise ValueError("nsamples must be a positive Int")
        if isinstance(proposal, ProposalBank):
            self.bank = proposal
            self.mis_scheme = mis_scheme or StratifiedMixture()
        elif isinstance(proposal, RadialProposal):
            if mis_scheme is not None:
                raise ValueError("a MIS scheme requires a ProposalBank")
            self.bank = ProposalBank([proposal])
            self.mis_scheme = StandardMIS()
        else:
            raise TypeError("proposal must be a native radial proposal or a ProposalBank")
        self.proposal = proposal
        self.nsamples = nsamples


class AMIS:
    """AMIS(proposal; rounds, round_size) (src/methods/amis.jl:42-47)."""

    def __init__(self, proposal, rounds, round_size):
        if not isinstance(proposal, RadialProposal):
            raise TypeError("AMIS requires a native Gaussian or Student-t proposal")
        if proposal.dof is not None and not float(proposal.dof) > 2:
            raise ValueError("covariance adaptation requires Student-t degrees of freedom > 2")
        self.proposal = proposal
        self.rounds = rounds
        self.round_size = _schedule(rounds, round_size)


class NPMC:
    """NPMC(proposal; rounds, round_size): standard-IS weights per round with
    sqrt(n) largest weights clipped before the moment fit (src/methods/npmc.jl)."""

    def __init__(self, proposal, rounds, round_size):
        if not isinstance(proposal, RadialProposal):
            raise TypeError("NPMC requires a native Gaussian or Student-t proposal")
        self.proposal = proposal
        self.rounds = rounds
        self.round_size = _schedule(rounds, round_size)


class GlobalResampling:
    """Resample all K locations from the round's weighted population."""


class LocalResampling:
    """Resample each proposal's next location from its own samples."""


class DeterministicMixturePMC:
    """DeterministicMixturePMC(bank; rounds, round_size, resampling)
    (src/methods/dm_pmc.jl:72-86)."""

    def __init__(self, bank, rounds, round_size, resampling=None):
        if not isinstance(bank, ProposalBank):
            raise TypeError("DM-PMC requires a ProposalBank")
        self.bank = bank
        self.rounds = rounds
        self.round_size = _schedule(rounds, round_size)
        self.resampling = resampling or GlobalResampling()


class MultinomialResampling:
    """Independent weighted draws with replacement (src/resampling.jl:8-13)."""


class SystematicResampling:
    """One uniform, evenly spaced draws: u_i = (i + u)/count."""


def isqrt(n):
    return math.isqrt(n)
