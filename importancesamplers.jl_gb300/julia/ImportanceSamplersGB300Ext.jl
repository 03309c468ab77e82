# ImportanceSamplersGB300Ext — package extension of ImportanceSamplers.jl that
# runs the importance-sampling hot path through libissm103.so (include/issm.h)
# on a GB300 (sm_103a). It is loaded with CUDA.jl, like the package's own CUDA
# extension, and plugs into the execution-plan seam of the package:
#
#   _prepare_backend_execution(sampler)               (src/methods/importance_sampling.jl:279-297)
#   _execute_prepared_sampler!(sampler, plan, threaded)  (:932-935)
#   per-phase hooks with a plan argument           (src/adaptive_gaussian_execution.jl:855-874)
#
# Registration (the package's Project.toml):
#   [weakdeps]    CUDA = "052768ef-5323-5732-b1bb-66c8b64840ba"
#   [extensions]  ImportanceSamplersGB300Ext = "CUDA"
# and the library path in ENV["ISSM_LIBRARY"] (default "libissm103").
#
# Scope: AMIS with a factor Gaussian history on a CUDADevice (the round loop
# of src/amis_execution.jl:261-357 and the fit of
# src/adaptive_gaussian_execution.jl:348-425), the log-weight summary, and the
# resampling CDF (src/resampling.jl:199-225). Every other method keeps the
# package's own CUDA path (the plan is `nothing` for it).
#
# The library never synchronises and never frees caller memory; device
# arrays are the sampler's CuArrays, passed as raw pointers with the
# package's column-major layouts. Sample-level failures land in the package's
# own 3-word failure record, so `_device_failure_snapshot` decodes them as
# before.
#
# Julia is not available where this file was written; it mirrors the C ABI
# that the Python test-suite exercises through ctypes and has not itself been
# run.
module ImportanceSamplersGB300Ext

import CUDA
import ImportanceSamplers
import MLDataDevices

const IS = ImportanceSamplers
const LIB = get(ENV, "ISSM_LIBRARY", "libissm103")

# ---- C structs (field order of include/issm.h) -----------------------------------
const ISSM_F32, ISSM_F64 = Int32(0), Int32(1)
const ISSM_GAUSSIAN, ISSM_STUDENT_T = Int32(0), Int32(1)
const ISSM_SCALE_FACTOR = Int32(0)
const ISSM_DENOM_PREFIX = Int32(3)
const ISSM_PREC_NATIVE, ISSM_PREC_TF32, ISSM_PREC_BF16 = Int32(0), Int32(1), Int32(2)

struct IssmBank
    dim::Int32
    count::Int32
    family::Int32
    scale_kind::Int32
    dtype::Int32
    reserved::Int32
    locations::CUDA.CuPtr{Cvoid}
    scales::CUDA.CuPtr{Cvoid}
    lognormalizers::CUDA.CuPtr{Cvoid}
    dofs::CUDA.CuPtr{Cvoid}
    range_risk::CUDA.CuPtr{UInt8}
    inverse_factors::CUDA.CuPtr{Float32}
end

struct IssmDenominator
    kind::Int32
    terms::Int32
    logcoefficients::CUDA.CuPtr{Cvoid}
    group_of_slot::CUDA.CuPtr{Int32}
end

issm_dtype(::Type{Float32}) = ISSM_F32
issm_dtype(::Type{Float64}) = ISSM_F64

stream_handle() = CUDA.stream().handle

function issm_check(status, where)
    status == 0 && return nothing
    message = unsafe_string(ccall((:issm_status_string, LIB), Cstring, (Cint,), status))
    throw(ErrorException("$where: $message (status $status)"))
end

# ---- the plan ----------------------------------------------------------------------
# Device state the library needs beyond the package's own workspace: FP64
# moment scratch, the FP32 inverse factors of the history (tensor-core forms),
# the counter-based random stream's device base, per-round summaries and the
# library workspaces.
struct GB300MomentPlan{T}
    precision::Int32
    seed::UInt64
    counter::CUDA.CuVector{UInt64}
    inverse_factors::Union{Nothing,CUDA.CuArray{Float32,3}}
    mean::CUDA.CuVector{Float64}
    covariance::CUDA.CuMatrix{Float64}
    shift::CUDA.CuVector{Float64}
    summaries::CUDA.CuMatrix{Float64}       # 3 x rounds: (max, S, S2)
    tc_workspace::CUDA.CuVector{UInt8}
    moments_workspace::CUDA.CuVector{UInt8}
    reduce_workspace::CUDA.CuVector{UInt8}
    normal_offset::Base.RefValue{UInt64}
end

function _history_bank(plan::GB300MomentPlan{T}, history, count) where {T}
    d = size(history.means, 1)
    return IssmBank(Int32(d), Int32(count), ISSM_GAUSSIAN, ISSM_SCALE_FACTOR, issm_dtype(T), Int32(0),
        pointer(history.means), pointer(history.factors), pointer(history.lognormalizers),
        CUDA.CuPtr{Cvoid}(0), CUDA.CuPtr{UInt8}(0),
        plan.inverse_factors === nothing ? CUDA.CuPtr{Float32}(0) : pointer(plan.inverse_factors))
end

_factor_history(state) = state.history isa IS._FactorProposalHistory

# The plan applies to AMIS on a CUDA device with a factor Gaussian history of
# dimension <= 64; anything else keeps `nothing` (the package's own path).
function _gb300_plan(sampler, state::IS._PreparedMomentSampler)
    sampler.algorithm isa IS.AMIS || return nothing
    sampler.device isa MLDataDevices.CUDADevice || return nothing
    _factor_history(state) || return nothing
    history = state.history
    T = eltype(history.factors)
    d = size(history.means, 1)
    d <= 64 || return nothing
    rounds = length(state.schedule)
    total = sum(state.schedule)
    precision = T === Float32 ? ISSM_PREC_BF16 : ISSM_PREC_NATIVE
    dp = d <= 16 ? 16 : d <= 32 ? 32 : 64
    inverse = precision == ISSM_PREC_NATIVE ? nothing : CUDA.zeros(Float32, dp, dp, rounds)
    tc_bytes = ccall((:issm_tc_workspace_bytes, LIB), Csize_t, (Int32, Int32), rounds, d)
    moments_bytes = ccall((:issm_moments_workspace_bytes, LIB), Csize_t, (Int64, Int32), total, d)
    reduce_bytes = ccall((:issm_reduce_workspace_bytes, LIB), Csize_t, (Int64,), total)
    seed = rand(sampler.rng, UInt64)
    return GB300MomentPlan{T}(precision, seed, CUDA.zeros(UInt64, 1), inverse,
        CUDA.zeros(Float64, d), CUDA.zeros(Float64, d, d), CUDA.zeros(Float64, d),
        CUDA.zeros(Float64, 3, rounds), CUDA.zeros(UInt8, max(tc_bytes, 1 << 20)),
        CUDA.zeros(UInt8, moments_bytes), CUDA.zeros(UInt8, reduce_bytes), Ref(UInt64(0)))
end
_gb300_plan(sampler, state) = nothing

function IS._prepare_backend_execution(sampler::IS._PreparedImportanceSampler)
    plan = _gb300_plan(sampler, sampler.method_state)
    plan === nothing && return sampler
    return IS._PreparedImportanceSampler(sampler.rng, sampler.random_buffers, sampler.target,
        sampler.algorithm, sampler.method_state, sampler.device, sampler.factor_execution,
        sampler.threaded, sampler.running, sampler.executed, plan)
end

# The package's own moment round loop runs unchanged and calls the hooks
# below for its device phases.
IS._execute_prepared_sampler!(sampler, plan::GB300MomentPlan, threaded) =
    IS._importance_sample_cpu!(sampler, threaded)

IS._reset_prepared_moment_history!(plan::GB300MomentPlan, history, rounds, record) = begin
    plan.normal_offset[] = UInt64(0)
    IS._reset_moment_history!(history, rounds)
end

# ---- one AMIS round: draw, target, retrospective denominators, weights -------------
# _launch_prefilled_amis_round! (src/amis_execution.jl:261-357) with the
# normals generated inside the draw kernel (issm_draw_philox) instead of a
# prefilled buffer.
function IS._draw_moment_round!(sampler, plan::GB300MomentPlan{T}, state, round_ids, target, round,
                                execution) where {T}
    history = state.history
    workspace = state.workspace
    d = size(history.means, 1)
    first = state.offsets[round]
    n_new = state.offsets[round + 1] - first
    n_old = first - 1
    slot = Int32(round - 1)
    bank = Ref(_history_bank(plan, history, round))
    failures = sampler.random_buffers.failure_scratch.record.words
    samples = pointer(workspace.samples) + n_old * d * sizeof(T)
    st = ccall((:issm_draw_philox, LIB), Cint,
        (Ref{IssmBank}, Int32, UInt64, CUDA.CuPtr{UInt64}, UInt64, CUDA.CuPtr{Cvoid}, Int32, CUDA.CuPtr{Cvoid},
         Int32, Int64, CUDA.CuPtr{Cvoid}, CUDA.CuPtr{UInt64}, Int64, Ptr{Cvoid}),
        bank, slot, plan.seed, pointer(plan.counter), plan.normal_offset[], CUDA.CuPtr{Cvoid}(0), Int32(0),
        CUDA.CuPtr{Cvoid}(0), Int32(0), n_new, samples, pointer(failures), Int64(first), stream_handle())
    issm_check(st, "issm_draw_philox")
    plan.normal_offset[] += UInt64(n_new * d + 8)
    # the target: the package's batch hook (src/batched_targets.jl:92-126)
    # writes the new samples' log targets; a scalar target keeps the package path
    new_samples = view(workspace.samples, :, first:(first + n_new - 1))
    new_logtargets = view(workspace.logtargets, first:(first + n_new - 1))
    target isa IS._BoundBatchTarget ||
        throw(ArgumentError("the GB300 plan evaluates batch targets; scalar targets keep the package's CUDA path"))
    IS._invoke_batch_target!(target, new_logtargets, new_samples, failures, execution)
    st = ccall((:issm_check_target_values, LIB), Cint,
        (CUDA.CuPtr{Cvoid}, Int64, Int32, CUDA.CuPtr{Int64}, CUDA.CuPtr{UInt64}, Int64, Ptr{Cvoid}),
        pointer(new_logtargets), n_new, issm_dtype(T), pointer(round_ids) + n_old * sizeof(Int64),
        pointer(failures), Int64(first), stream_handle())
    issm_check(st, "issm_check_target_values")
    if plan.inverse_factors !== nothing
        st = ccall((:issm_invert_factors, LIB), Cint, (Ref{IssmBank}, Int32, Int32, CUDA.CuPtr{Float32}, Ptr{Cvoid}),
            bank, slot, Int32(1), pointer(plan.inverse_factors), stream_handle())
        issm_check(st, "issm_invert_factors")
    end
    lognum = pointer(workspace.lognumerators)
    if n_old > 0  # the old samples gain the newest component
        st = ccall((:issm_amis_append_ws, LIB), Cint,
            (Ref{IssmBank}, Int32, CUDA.CuPtr{Cvoid}, CUDA.CuPtr{Cvoid}, Int64, CUDA.CuPtr{Cvoid},
             CUDA.CuPtr{UInt64}, Int32, CUDA.CuPtr{Cvoid}, Csize_t, Ptr{Cvoid}),
            bank, slot, pointer(state.logcounts), pointer(workspace.samples), Int64(n_old), lognum,
            pointer(failures), plan.precision, pointer(plan.tc_workspace), sizeof(plan.tc_workspace),
            stream_handle())
        issm_check(st, "issm_amis_append_ws")
    end
    den = Ref(IssmDenominator(ISSM_DENOM_PREFIX, Int32(round), pointer(state.logcounts), CUDA.CuPtr{Int32}(0)))
    st = ccall((:issm_mixture_logdensity_ws, LIB), Cint,
        (Ref{IssmBank}, Ref{IssmDenominator}, CUDA.CuPtr{Cvoid}, Int64, CUDA.CuPtr{Int32}, Int32, CUDA.CuPtr{Cvoid},
         CUDA.CuPtr{Cvoid}, CUDA.CuPtr{UInt64}, Int64, Int32, CUDA.CuPtr{Cvoid}, Csize_t, Ptr{Cvoid}),
        bank, den, samples, Int64(n_new), CUDA.CuPtr{Int32}(0), slot, lognum + n_old * sizeof(T),
        CUDA.CuPtr{Cvoid}(0), pointer(failures), Int64(first), plan.precision, pointer(plan.tc_workspace),
        sizeof(plan.tc_workspace), stream_handle())
    issm_check(st, "issm_mixture_logdensity_ws")
    # weights of every retained sample, and their (max, S, S2) summary in the same pass
    n_tot = n_old + n_new
    st = ccall((:issm_amis_form_summary, LIB), Cint,
        (CUDA.CuPtr{Cvoid}, CUDA.CuPtr{Cvoid}, CUDA.CuPtr{Int64}, Float64, Int64, Int32, CUDA.CuPtr{Cvoid},
         CUDA.CuPtr{UInt64}, CUDA.CuPtr{Float64}, CUDA.CuPtr{Cvoid}, Csize_t, Ptr{Cvoid}),
        pointer(workspace.logtargets), lognum, pointer(round_ids), log(Float64(n_tot)), Int64(n_tot),
        issm_dtype(T), pointer(workspace.logweights), pointer(failures),
        pointer(plan.summaries) + 3 * (round - 1) * sizeof(Float64), pointer(plan.reduce_workspace),
        sizeof(plan.reduce_workspace), stream_handle())
    issm_check(st, "issm_amis_form_summary")
    return nothing
end

# ---- the round's summary: one 24-byte read ---------------------------------------
function IS._prepared_moment_summary(plan::GB300MomentPlan, algorithm, state, round, fit, transfers)
    words = Array(view(plan.summaries, :, round))
    IS._record_reported_transfer!(transfers, 1, sizeof(words), Val(:logweight_summary))
    m, s, s2 = words
    n = state.offsets[round + 1] - 1
    ess = iszero(s) ? 0.0 : s * s / s2
    logz = iszero(s) ? -Inf : m + log(s) - log(Float64(n))
    return (ess=ess, lognormalizer=logz)
end

# ---- the moment fit: weighted moments (tensor core or two-pass) and FP64 Cholesky --
# _fit_moment_proposal!(device, ...) (src/adaptive_gaussian_execution.jl:348-425,
# 530-639) for a factor history.
function IS._fit_prepared_moment_proposal!(plan::GB300MomentPlan{T}, workspace, history, round,
                                           sample_count, args...) where {T}
    d = size(history.means, 1)
    summary = pointer(plan.summaries) + 3 * (round - 1) * sizeof(Float64)
    previous = pointer(history.factors) + (round - 1) * d * d * sizeof(T)
    copyto!(plan.shift, Float64.(view(history.means, :, round)))
    st = ccall((:issm_weighted_moments_ws, LIB), Cint,
        (CUDA.CuPtr{Cvoid}, Int32, Int64, CUDA.CuPtr{Cvoid}, Int32, CUDA.CuPtr{Float64}, CUDA.CuPtr{Float64},
         CUDA.CuPtr{Cvoid}, CUDA.CuPtr{Float64}, CUDA.CuPtr{Float64}, Int32, CUDA.CuPtr{Cvoid}, Csize_t, Ptr{Cvoid}),
        pointer(workspace.samples), Int32(d), Int64(sample_count), pointer(workspace.logweights), issm_dtype(T),
        summary, pointer(plan.shift), T === Float32 ? previous : CUDA.CuPtr{Cvoid}(0), pointer(plan.mean),
        pointer(plan.covariance), plan.precision, pointer(plan.moments_workspace), sizeof(plan.moments_workspace),
        stream_handle())
    issm_check(st, "issm_weighted_moments_ws")
    # the candidate lands in the workspace; the package stores it into slot round + 1
    st = ccall((:issm_fit_factor_ex, LIB), Cint,
        (CUDA.CuPtr{Float64}, CUDA.CuPtr{Float64}, Int32, CUDA.CuPtr{Cvoid}, Float64, Float64, Int32,
         CUDA.CuPtr{Cvoid}, CUDA.CuPtr{Cvoid}, CUDA.CuPtr{Cvoid}, CUDA.CuPtr{Float32}, CUDA.CuPtr{UInt64}, Int64,
         Ptr{Cvoid}),
        pointer(plan.mean), pointer(plan.covariance), Int32(d), previous, 0.0, 0.0, issm_dtype(T),
        pointer(workspace.candidate_mean), pointer(workspace.candidate_scale),
        pointer(workspace.candidate_lognormalizer),
        plan.inverse_factors === nothing || round >= size(plan.inverse_factors, 3) ? CUDA.CuPtr{Float32}(0) :
            pointer(plan.inverse_factors) + round * size(plan.inverse_factors, 1)^2 * sizeof(Float32),
        pointer(IS._native_failure_scratch(workspace).record.words), Int64(sample_count + 1), stream_handle())
    issm_check(st, "issm_fit_factor_ex")
    return nothing
end

# ---- reference-rule resampling CDF on CuArrays --------------------------------------
# _resampling_cdf! (src/resampling.jl:199-225): exp(l - max) scan and divide,
# one launch sequence on the device, no host reads beyond the package's own
# all-zero check of the summary.
function IS._resampling_cdf!(cdf::CUDA.CuVector{T}, logweights::CUDA.CuVector{T},
                             transfers::IS._ResultTransferCounter=IS._ResultTransferCounter(0, 0)) where {T<:Union{Float32,Float64}}
    n = length(logweights)
    bytes = ccall((:issm_reduce_workspace_bytes, LIB), Csize_t, (Int64,), n)
    workspace = CUDA.zeros(UInt8, bytes)
    st = ccall((:issm_resampling_cdf, LIB), Cint,
        (CUDA.CuPtr{Cvoid}, Int64, Int32, CUDA.CuPtr{Cvoid}, CUDA.CuPtr{Cvoid}, Csize_t, Ptr{Cvoid}),
        pointer(logweights), Int64(n), issm_dtype(T), pointer(cdf), pointer(workspace), bytes, stream_handle())
    st == -5 && throw(IS.AllZeroWeightsError())  # ISSM_E_ALL_ZERO
    issm_check(st, "issm_resampling_cdf")
    return cdf
end

end # module
