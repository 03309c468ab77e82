"""GB300-native importance-sampling hot path with the ImportanceSamplers.jl API.

The device work runs in libissm103.so (hand-written sm_103a CUDA behind the C
ABI of include/issm.h); this package is the host-side mirror of the
reference's public interface: proposals, banks, algorithm configurations,
prepare_sampler / importance_sample! / importance_sample, WeightedSamples and
its reductions and resampling.
"""
from . import native, ops, serving, shards
from .bank import DeviceBank, DeviceHistory, ProposalBank, pack, pack_proposals
from .methods import (AMIS, NPMC, DeterministicMixturePMC, GlobalResampling, ImportanceSampling, LocalResampling,
                      MultinomialResampling, PartialDeterministicMixture, RandomMixture, StandardMIS,
                      StratifiedMixture, SystematicResampling)
from .proposals import (DiagonalGaussian, DiagonalStudentT, FactorGaussian, FactorStudentT, SphericalGaussian,
                        SphericalStudentT, student_t_logconstant)
from .results import (AllZeroWeightsError, AMISRoundError, DMPMCRoundError, NPMCRoundError, SamplerExecutionError,
                      UnweightedSamples, WeightedSamples, cov, effective_sample_size, lognormalizer, mean, median,
                      normalized_weights, quantile, resample, std, var)
from .sampler import (SamplerBusyError, current_proposal, deterministic_allocation_plan, importance_sample,
                      importance_sample_, prepare_sampler, reweigh_amis, share_normal_stream)
from .targets import (GaussianMixtureTarget, LinearRegressionTarget, LogisticRegressionTarget, LogTarget,
                      QuadraticTarget, StandardNormalTarget, StudentTTarget)

__all__ = [n for n in dir() if not n.startswith("_")]
