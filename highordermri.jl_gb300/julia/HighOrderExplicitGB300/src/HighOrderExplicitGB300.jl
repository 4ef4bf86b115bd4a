"""
    HighOrderExplicitGB300

Julia front end of libhoexplicit.so: the GB300 (sm_103a) explicit
higher-order encoding operator as a third `HighOrderExplicitOp`
implementation beside HighOrderMRI's `:array` and `:kernel`.

`GB300ExplicitOp(grid, kspha, times; ...)` takes the constructor keywords of
`HighOrderExplicitOp` (fieldmap, csm, mask, concomitant, recon_terms,
k_nominal, kspha_dt, gpus).  Model preparation reuses HighOrderMRI's own
`prep_kspha`, `basisfunc_spha` and `prep_concomitant`, so both packages see
the same model.  Solver vectors are `CuVector{ComplexF32}` on the operator's
device; calls are ordered on `CUDA.stream()`.
"""
module HighOrderExplicitGB300

using CUDA
using LinearAlgebra
using LinearOperators
using LinearOperatorCollection
using ChainRulesCore
import HighOrderMRI
import HighOrderMRI: Grid, HighOrderExplicitOp, prep_kspha, basisfunc_spha, prep_concomitant

export GB300ExplicitOp, explicit_backward, encode, GB300Batch, set_kspha!

const libhoe = get(ENV, "HOE_LIBRARY",
    normpath(joinpath(@__DIR__, "..", "..", "..", "libhoexplicit.so")))

const HOE_ABI_VERSION = Int32(2)
const HOE_ENGINE_FP32_SIMT = Int32(0)
const HOE_ENGINE_TC_BF16X3 = Int32(1)
const HOE_ENGINE_AUTO = Int32(2)
const HOE_GRAD_KSPHA = Int32(1)
const HOE_GRAD_FIELDMAP = Int32(2)
const HOE_GRAD_T0_B0 = Int32(4)
const HOE_GRAD_T0_COEF = Int32(8)

# Field order and types match `hoe_desc` in include/hoexplicit.h.
struct HoeDesc
    abi_version::Int32
    nX::Int32; nY::Int32; nZ::Int32
    nSam::Int32; nCha::Int32; nTerm::Int32; has_concomitant::Int32; nVox::Int32
    engine::Int32; device::Int32; tc_plan::Int32; reserved::Int32; split_hint::Int32
    mask_idx::Ptr{Int32}
    bf::Ptr{Float64}
    kspha::Ptr{Float64}
    times::Ptr{Float64}
    fieldmap::Ptr{Float64}
    csm::Ptr{Float64}
    kspha_dt::Ptr{Float64}
end

last_error(h) = unsafe_string(ccall((:hoe_last_error, libhoe), Cstring, (Ptr{Cvoid},), h))

# Status codes -> the exception types the reference raises.
function check(rc::Cint, h=C_NULL)
    rc == 0 && return nothing
    msg = last_error(h)
    rc in (-1, -6, -7) && throw(ArgumentError(msg))
    rc == -2 && throw(DimensionMismatch(msg))
    rc == -3 && throw(OutOfMemoryError())
    error("libhoexplicit: [$rc] $msg")
end

mutable struct GB300ExplicitOp{T,F,G} <: HighOrderExplicitOp{Complex{T}}
    nrow::Int
    ncol::Int
    symmetric::Bool
    hermitian::Bool
    prod!::F
    tprod!::Nothing
    ctprod!::G
    nprod::Int
    ntprod::Int
    nctprod::Int
    Mv::CuVector{Complex{T}}
    Mtu::CuVector{Complex{T}}
    handle::Ptr{Cvoid}
    device::CuDevice
    nSam::Int
    nCha::Int
    nTermEff::Int
    derivative::Bool
    has_kdot::Bool
end

LinearOperators.storage_type(op::GB300ExplicitOp) = typeof(op.Mv)

function activate(op::GB300ExplicitOp)
    (op.handle == C_NULL || ccall((:hoe_is_closed, libhoe), Cint, (Ptr{Cvoid},), op.handle) != 0) &&
        throw(ArgumentError("operator is closed"))
    CUDA.device!(op.device)
    return op.handle
end

stream_handle() = CUDA.stream().handle

function forward!(op::GB300ExplicitOp, res, x)
    h = activate(op)
    rc = op.derivative ?
        ccall((:hoe_derivative, libhoe), Cint, (Ptr{Cvoid}, CuPtr{ComplexF32}, CuPtr{ComplexF32}, CUDA.CUstream),
              h, x, res, stream_handle()) :
        ccall((:hoe_forward, libhoe), Cint, (Ptr{Cvoid}, CuPtr{ComplexF32}, CuPtr{ComplexF32}, CUDA.CUstream),
              h, x, res, stream_handle())
    check(rc, h)
    return res
end

function adjoint!(op::GB300ExplicitOp, res, y)
    h = activate(op)
    check(ccall((:hoe_adjoint, libhoe), Cint, (Ptr{Cvoid}, CuPtr{ComplexF32}, CuPtr{ComplexF32}, CUDA.CUstream),
                h, y, res, stream_handle()), h)
    return res
end

"""
    GB300ExplicitOp(grid, kspha, times; fieldmap, csm, mask, concomitant=nothing,
        recon_terms=nothing, k_nominal=kspha[2:4,:], kspha_dt=nothing, kdot=nothing,
        gpus=nothing, engine=:auto)

The `:gb300` implementation of `HighOrderExplicitOp` (see
HighOrderExplicitOp.jl:44-51).  `engine=:tc` uses the tcgen05 tensor-core
contraction (split-BF16, FP32 accumulation), `engine=:fp32` the plain FP32
CUDA-core kernel, `engine=:auto` the tensor cores where the device and the
coil count (at most 64) allow them, else the FP32 kernel.  With `kspha_dt` the forward product evaluates the
derivative `B x` of the reference's kspha_dt mode and concomitant terms are
ignored (array_operator.jl:139, 159-166).  `kdot` (the same shape as `kspha`)
supplies dkspha/dt for the coefficient part of the t0 gradient without
switching the product to the derivative.  A plan whose residual phase bound
exceeds 1024 cycles runs on the FP32 kernel (`engine=:auto`) or is refused
(`engine=:tc`).
"""
function GB300ExplicitOp(grid::Grid{T}, kspha::AbstractMatrix{T}, times::AbstractVector{T};
    fieldmap=zeros(T, grid.matrixSize...), csm=ones(Complex{T}, grid.matrixSize..., 1),
    mask=trues(grid.matrixSize...), concomitant=nothing, recon_terms=nothing,
    k_nominal=kspha[2:4, :], kspha_dt=nothing, kdot=nothing, gpus=nothing, engine::Symbol=:auto,
    # the reference implementations' execution keywords, for calls written for
    # them: the Array path's are ignored, the CUDA path's get its validation
    # (kernel_operator.jl:223-236, explicit_gpu_operator.jl:313-320) and
    # change nothing (the GB300 engine replaces those execution strategies)
    nBlock::Integer=50, arrayType=CuArray, verbose::Bool=false,
    backend::Symbol=:legacy, block_size::Int=320, phase_backend::Symbol=:kernel, gemm_backend::Symbol=:cublas,
    phase_cache_bytes::Integer=0, forward_threads::Int=256, adjoint_threads::Int=512,
) where {T<:AbstractFloat}
    if backend !== :legacy
        backend in (:direct, :blocked, :cached, :cached_full) || throw(ArgumentError("unknown explicit backend $backend"))
        isnothing(kspha_dt) || throw(ArgumentError("kspha_dt requires backend=:legacy"))
        phase_cache_bytes >= 0 || throw(ArgumentError("phase_cache_bytes must be nonnegative"))
        phase_cache_bytes == 0 || backend === :blocked || throw(ArgumentError(
            "phase_cache_bytes applies to backend=:blocked; cached backends already retain the complete phase matrix"))
        phase_backend in (:kernel, :gemm) || throw(ArgumentError("unknown phase backend $phase_backend"))
        gemm_backend in (:cublas, :auto) || throw(ArgumentError("gemm_backend must be :cublas or :auto"))
        block_size > 0 || throw(ArgumentError("block_size must be positive"))
        forward_threads in (64, 128, 256, 512) || throw(ArgumentError("unsupported forward_threads"))
        adjoint_threads in (64, 128, 256, 512) || throw(ArgumentError("unsupported adjoint_threads"))
    else
        iszero(phase_cache_bytes) || throw(ArgumentError("phase_cache_bytes requires backend=:blocked"))
    end
    if gpus !== nothing
        ids = Int.(collect(gpus))
        length(ids) == 1 || throw(ArgumentError("the :gb300 operator uses exactly one GPU"))
        0 <= only(ids) < length(collect(CUDA.devices())) || throw(ArgumentError("invalid visible GPU ID"))
        CUDA.device!(only(ids))
    end
    engine in (:tc, :fp32, :auto) || throw(ArgumentError("engine must be :tc, :fp32 or :auto"))
    nTerm, nSam = size(kspha)
    nTerm in (9, 16) || throw(ArgumentError("kspha requires 9 or 16 terms"))
    length(times) == nSam || throw(DimensionMismatch("times and kspha"))
    length(mask) == prod(grid.matrixSize) || throw(DimensionMismatch("mask and grid"))
    length(fieldmap) == length(mask) || throw(DimensionMismatch("fieldmap and mask"))
    nCha = size(csm, ndims(csm))
    length(csm) == length(mask) * nCha || throw(DimensionMismatch("csm and grid"))
    indices = findall(vec(mask))
    nVox = length(indices)
    nVox > 0 || throw(ArgumentError("mask must contain voxels"))
    derivative = kspha_dt !== nothing
    derivative && size(kspha_dt) != size(kspha) && throw(ArgumentError("kspha_dt must have same size as kspha"))
    kd = derivative ? kspha_dt : kdot
    kd !== nothing && size(kd) != size(kspha) && throw(ArgumentError("kspha_dt must have same size as kspha"))

    prepared = prep_kspha(kspha, k_nominal, nTerm; recon_terms)
    bf = basisfunc_spha(grid.x[indices], grid.y[indices], grid.z[indices], collect(1:nTerm))
    bf, prepared = prep_concomitant(bf, prepared, grid, vec(mask);
                                    concomitant=derivative ? nothing : concomitant)
    bf64 = Matrix{Float64}(bf)
    k64 = Matrix{Float64}(prepared)
    t64 = Vector{Float64}(times)
    f64 = Vector{Float64}(vec(fieldmap)[indices])
    c128 = Matrix{ComplexF64}(reshape(csm, :, nCha)[indices, :])
    idx32 = Int32.(indices .- 1)
    kd64 = kd === nothing ? nothing : Matrix{Float64}(kd)
    dev = CUDA.device()
    handle = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve bf64 k64 t64 f64 c128 idx32 kd64 begin
        desc = Ref(HoeDesc(HOE_ABI_VERSION, grid.nX, grid.nY, grid.nZ, nSam, nCha, nTerm,
            Int32(size(k64, 1) != nTerm), nVox,
            engine === :tc ? HOE_ENGINE_TC_BF16X3 : engine === :fp32 ? HOE_ENGINE_FP32_SIMT : HOE_ENGINE_AUTO,
            Int32(CUDA.deviceid(dev)), Int32(0), Int32(0), Int32(0),
            pointer(idx32), pointer(bf64), pointer(k64), pointer(t64), pointer(f64),
            Ptr{Float64}(pointer(c128)), kd64 === nothing ? Ptr{Float64}(C_NULL) : pointer(kd64)))
        check(ccall((:hoe_create, libhoe), Cint, (Ref{Ptr{Cvoid}}, Ref{HoeDesc}), handle, desc))
    end
    op = nothing
    prodf = (res, x) -> forward!(op, res, x)
    ctprodf = (res, y) -> adjoint!(op, res, y)
    op = GB300ExplicitOp{Float32,typeof(prodf),typeof(ctprodf)}(
        nSam * nCha, prod(grid.matrixSize), false, false, prodf, nothing, ctprodf, 0, 0, 0,
        CUDA.zeros(ComplexF32, 0), CUDA.zeros(ComplexF32, 0), handle[], dev, nSam, nCha,
        size(k64, 1), derivative, kd !== nothing)
    finalizer(o -> ccall((:hoe_free, libhoe), Cvoid, (Ptr{Cvoid},), o.handle), op)
    return op
end

function Base.adjoint(op::GB300ExplicitOp{T}) where {T}
    return LinearOperator{Complex{T}}(op.ncol, op.nrow, false, false,
        op.ctprod!, nothing, op.prod!; S=CuVector{Complex{T}})
end

# normalOperator(op, D) with the validation of explicit_gpu_operator.jl:399-416:
# D = W^H W (real, non-negative, finite), one entry per sample or per sample and coil.
function LinearOperatorCollection.normalOperator(op::GB300ExplicitOp{T}, weights=nothing; kwargs...) where {T}
    activate(op)
    raw = weights isa LinearOperatorCollection.WeightingOp ? weights.weights : weights
    D = raw === nothing ? ones(T, op.nSam * op.nCha) : vec(Array(raw))
    length(D) == op.nSam && (D = repeat(D, op.nCha))
    length(D) == op.nrow || throw(DimensionMismatch("normal weights"))
    all(isfinite, D) || throw(ArgumentError("normal weights must be finite"))
    maximum(abs, imag.(D)) <= 10eps(T) * max(one(T), maximum(abs, D)) ||
        throw(ArgumentError("normal weights must already be real nonnegative WᴴW"))
    minimum(real.(D)) >= zero(T) || throw(ArgumentError("normal weights must be nonnegative"))
    diagonal = CuArray(Float32.(real.(D)))
    normal = (out, x) -> begin
        h = activate(op)
        check(ccall((:hoe_normal, libhoe), Cint,
                    (Ptr{Cvoid}, CuPtr{Float32}, CuPtr{ComplexF32}, CuPtr{ComplexF32}, CUDA.CUstream),
                    h, diagonal, x, out, stream_handle()), h)
        out
    end
    return LinearOperator{Complex{T}}(op.ncol, op.ncol, false, true, normal, nothing, normal;
                                      S=CuVector{Complex{T}})
end

# W ∘ op from recon_HOOp: normalOperator receives W^H W from LinearOperatorCollection.
HighOrderMRI.explicit_gpu_normal(op::GB300ExplicitOp; weights=nothing) =
    LinearOperatorCollection.normalOperator(op, weights === nothing ? nothing : abs2.(weights))

function Base.close(op::GB300ExplicitOp)
    op.handle == C_NULL && return nothing
    CUDA.device!(op.device)
    ccall((:hoe_close, libhoe), Cint, (Ptr{Cvoid},), op.handle)
    return nothing
end

"""
    explicit_backward(op, x, r; kspha=true, fieldmap=true, t0_b0=true, t0_coef=false)

Gradient of `0.5*norm(op*x - y)^2` given the residual `r = op*x - y`
(`CuVector{ComplexF32}` each): returns `(dkspha::CuMatrix{Float32}
(nTermEff, nSam), dfieldmap::CuVector{Float32} (full grid, zero outside the
mask), dt0::Float64)`.  The same call is the pullback of `x -> op*x` for the
phase parameters when `r` is the output cotangent.  `t0_coef` needs
`kspha_dt` or `kdot` at construction.  With `engine=:tc` (or `:auto` on a GB300) the
gradient is formed on the tensor cores for up to 16 coils with residual widths
up to 24 and up to 32 coils with widths up to 16, else on the FP32 kernel (up to
16 coils).
"""
function explicit_backward(op::GB300ExplicitOp, x, r; kspha=true, fieldmap=true, t0_b0=true, t0_coef=false)
    h = activate(op)
    flags = Int32((kspha ? HOE_GRAD_KSPHA : 0) | (fieldmap ? HOE_GRAD_FIELDMAP : 0) |
                  (t0_b0 ? HOE_GRAD_T0_B0 : 0) | (t0_coef ? HOE_GRAD_T0_COEF : 0))
    dk = CUDA.zeros(Float32, op.nTermEff, op.nSam)
    ddf = CUDA.zeros(Float32, op.ncol)
    dt0 = CUDA.zeros(Float64, 1)
    check(ccall((:hoe_backward, libhoe), Cint,
                (Ptr{Cvoid}, CuPtr{ComplexF32}, CuPtr{ComplexF32}, CuPtr{Float32}, CuPtr{Float32},
                 CuPtr{Float64}, Int32, CUDA.CUstream),
                h, x, r, dk, ddf, dt0, flags, stream_handle()), h)
    return dk, ddf, Array(dt0)[1]
end

"""
    encode(op, kspha, fieldmap, t0, x) = op * x

Differentiable application for phase-model refinement (coefficient and
field-map synchronisation).  `kspha` (nTermEff x nSam: the coefficients the
operator applies, after order selection, with the concomitant rows appended),
`fieldmap` (Hz, the grid's shape) and `t0` (s; 0 for the operator as built)
name the model that `op` was built with.  They are not read again: the
operator holds its own copy, and a changed model needs a new operator or
`hoe_set_kspha`.  They are arguments so that the pullback can return their
cotangents beside the one of `x`.

For a real loss L of `y = op * x`, ChainRulesCore's cotangent of a complex
output is ȳ = ∂L/∂Re(y) + i ∂L/∂Im(y) (for L = ½‖y - d‖² it is y - d).  The
pullback returns, for `op` nothing (`NoTangent`), then
- kspha:    Re Σ conj(ȳ) ∂y/∂kspha   (nTermEff x nSam, Float32)
- fieldmap: Re Σ conj(ȳ) ∂y/∂fieldmap (reshaped to `size(fieldmap)`, zero outside the mask)
- t0:       Re Σ conj(ȳ) ∂y/∂t0 with ∂φ/∂t0 = -fieldmap - Σ_l bf_l kdot_l, the
            coefficient part only when the operator was built with `kdot`
- x:        op' * ȳ
These are the gradients of hoe_backward with ȳ in the place of the residual.
"""
encode(op::GB300ExplicitOp, kspha, fieldmap, t0, x) = op * x

function ChainRulesCore.rrule(::typeof(encode), op::GB300ExplicitOp, kspha, fieldmap, t0, x)
    y = op * x
    function encode_pullback(ȳ)
        ybar = CuArray{ComplexF32}(unthunk(ȳ))
        dk, ddf, dt0 = explicit_backward(op, x, ybar; t0_coef=op.has_kdot)
        return NoTangent(), NoTangent(), dk, reshape(ddf, size(fieldmap)), dt0, op' * ybar
    end
    return y, encode_pullback
end

# ---------------------------------------------------------------------------
# recon_HOOp (src/Recon/recon_HOOp.jl:52-88) on the device: CGNR with an L2
# regularizer runs as one CUDA graph (hoe_recon); any other solver or
# regularizer goes through the generic RegularizedLeastSquares path, which
# only needs prod!/ctprod!/normalOperator.

struct HoeCgParams
    iterations::Int32; use_graph::Int32; rel_tol::Float64; lambda::Float64
end
struct HoeCgStats
    iterations::Int32; status::Int32; residual0::Float64; residual::Float64
end

function HighOrderMRI.recon_HOOp(op::GB300ExplicitOp{T}, Data::CuMatrix{Complex{T}},
                                 weight::CuVector{Complex{T}}, recParams::Dict;
                                 release_backend::Bool=true) where {T}
    params = merge(HighOrderMRI.defaultRecoParams(), recParams)
    reg = params[:reg]
    reg = reg isa AbstractVector && length(reg) == 1 ? only(reg) : reg
    if params[:solver] !== HighOrderMRI.CGNR || !(reg isa HighOrderMRI.L2Regularization)
        return invoke(HighOrderMRI.recon_HOOp, Tuple{HighOrderMRI.HOOp{Complex{T}}, AbstractArray{Complex{T},2},
                      AbstractVector{Complex{T}}, Dict}, op, Data, weight, recParams; release_backend)
    end
    size(Data, 1) == op.nSam && size(Data, 2) == op.nCha || throw(DimensionMismatch("Data and operator"))
    h = activate(op)
    x = CuVector{ComplexF32}(undef, op.ncol)
    p = Ref(HoeCgParams(Int32(params[:iterations]), Int32(1),
                        Float64(get(params, :relTol, eps(real(T)))), Float64(HighOrderMRI.λ(reg))))
    st = Ref(HoeCgStats(0, 0, 0.0, 0.0))
    check(ccall((:hoe_recon, libhoe), Cint,
                (Ptr{Cvoid}, CuPtr{ComplexF32}, CuPtr{ComplexF32}, CuPtr{ComplexF32}, Ref{HoeCgParams},
                 Ref{HoeCgStats}, CUDA.CUstream), h, Data, weight, x, p, st, stream_handle()), h)
    return Array(reshape(x, params[:reconSize]))
end

# ---------------------------------------------------------------------------
# Batches of slices (hoe_batch_*): every direction of all members in one
# persistent launch; members are borrowed (close the batch first).

mutable struct GB300Batch
    handle::Ptr{Cvoid}
    ops::Vector{GB300ExplicitOp}
end

function GB300Batch(ops::Vector{<:GB300ExplicitOp})
    hs = Ptr{Cvoid}[activate(o) for o in ops]
    out = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:hoe_batch_create, libhoe), Cint, (Ref{Ptr{Cvoid}}, Ptr{Ptr{Cvoid}}, Int32),
                out, hs, Int32(length(hs))))
    b = GB300Batch(out[], collect(GB300ExplicitOp, ops))
    finalizer(x -> ccall((:hoe_batch_free, libhoe), Cvoid, (Ptr{Cvoid},), x.handle), b)
    return b
end

_ptrs(v) = Ptr{Cvoid}[reinterpret(Ptr{Cvoid}, pointer(a)) for a in v]

function batch_check(rc::Cint, b::GB300Batch)
    rc == 0 && return nothing
    msg = unsafe_string(ccall((:hoe_batch_last_error, libhoe), Cstring, (Ptr{Cvoid},), b.handle))
    rc == -2 && throw(DimensionMismatch(msg))
    rc in (-1, -6, -7) && throw(ArgumentError(msg))
    rc == -3 && throw(OutOfMemoryError())
    error(msg)
end

function forward(b::GB300Batch, xs::Vector{<:CuVector{ComplexF32}})
    ys = [CuVector{ComplexF32}(undef, o.nrow) for o in b.ops]
    batch_check(ccall((:hoe_batch_forward, libhoe), Cint, (Ptr{Cvoid}, Ptr{Ptr{Cvoid}}, Ptr{Ptr{Cvoid}}, CUDA.CUstream),
                      b.handle, _ptrs(xs), _ptrs(ys), stream_handle()), b)
    return ys
end

function adjoint_apply(b::GB300Batch, ys::Vector{<:CuVector{ComplexF32}})
    xs = [CuVector{ComplexF32}(undef, o.ncol) for o in b.ops]
    batch_check(ccall((:hoe_batch_adjoint, libhoe), Cint, (Ptr{Cvoid}, Ptr{Ptr{Cvoid}}, Ptr{Ptr{Cvoid}}, CUDA.CUstream),
                      b.handle, _ptrs(ys), _ptrs(xs), stream_handle()), b)
    return xs
end

"""
    recon(b::GB300Batch, datas, weights; iterations=10, relTol=eps(Float32), λ=0)

`recon_HOOp`'s weighted CGNR for every member in lockstep (one CUDA graph);
returns the images as device vectors.
"""
function recon(b::GB300Batch, datas::Vector{<:CuMatrix{ComplexF32}}, weights::Vector{<:CuVector{ComplexF32}};
               iterations::Integer=10, relTol::Real=eps(Float32), λ::Real=0)
    xs = [CuVector{ComplexF32}(undef, o.ncol) for o in b.ops]
    p = Ref(HoeCgParams(Int32(iterations), Int32(1), Float64(relTol), Float64(λ)))
    batch_check(ccall((:hoe_batch_recon, libhoe), Cint,
                      (Ptr{Cvoid}, Ptr{Ptr{Cvoid}}, Ptr{Ptr{Cvoid}}, Ptr{Ptr{Cvoid}}, Ref{HoeCgParams},
                       Ptr{HoeCgStats}, CUDA.CUstream),
                      b.handle, _ptrs(datas), _ptrs(weights), _ptrs(xs), p, C_NULL, stream_handle()), b)
    return xs
end

# ---------------------------------------------------------------------------
# Delay synchronisation (src/Synchronization/FindDelay.jl:139-214) and
# InterpTrajTime (InterpTraj.jl:18-40) on the device.

"""
    set_kspha!(op, kspha_dev, kspha_dt_dev=nothing)

Replace the operator's coefficients on the device (hoe_set_kspha):
`kspha_dev::CuMatrix{Float64}` (nTermEff, nSam) prepared as at construction.
"""
function set_kspha!(op::GB300ExplicitOp, k::CuMatrix{Float64}, kdt::Union{Nothing,CuMatrix{Float64}}=nothing)
    h = activate(op)
    check(ccall((:hoe_set_kspha, libhoe), Cint, (Ptr{Cvoid}, CuPtr{Float64}, CuPtr{Float64}, CUDA.CUstream),
                h, k, kdt === nothing ? CU_NULL : kdt, stream_handle()), h)
    return op
end

function HighOrderMRI.InterpTrajTime(traj::CuMatrix{Float64}, dt::Real, delTime::Real,
                                     datatime::CuVector{Float64}; kwargs...)
    out = CuMatrix{Float64}(undef, length(datatime), size(traj, 2))
    check(ccall((:hoe_interp_traj_time, libhoe), Cint,
                (CuPtr{Float64}, Int64, Int32, Float64, Float64, CuPtr{Float64}, Int64, CuPtr{Float64}, Int32,
                 CUDA.CUstream), traj, size(traj, 1), Int32(size(traj, 2)), Float64(dt), Float64(delTime),
                datatime, length(datatime), out, Int32(0), stream_handle()))
    return out
end

# the per-shot overload (InterpTraj.jl:79-99): (nShot, nField, nTerm) series,
# one delay per shot, datatime (nShot, nADC) -> (nShot, nADC, nTerm)
function HighOrderMRI.InterpTrajTime(traj::CuArray{Float64,3}, dt::Real, delTime::AbstractVector{Float64},
                                     datatime::CuMatrix{Float64}; kwargs...)
    @assert size(traj, 1) == length(delTime) "Number of shots in trajectory must match length of delTime vector"
    @assert size(datatime, 1) == length(delTime) "Number of shots in datatime must match length of delTime vector"
    out = CuArray{Float64}(undef, size(traj, 1), size(datatime, 2), size(traj, 3))
    for i in axes(traj, 1)
        out[i, :, :] = HighOrderMRI.InterpTrajTime(traj[i, :, :], dt, delTime[i], datatime[i, :])
    end
    return out
end

struct HoeDelayParams
    start_time::Float64; dt::Float64; dtau_min::Float64; jump_fact::Float64; lambda::Float64
    term_mask::Ptr{Float64}; iter_max::Int32; max_outer::Int32
end
struct HoeDelayResult
    tau::Float64; tau_last::Float64; dtau::Float64; jump::Float64; iterations::Int32; status::Int32
end

"""
    find_delay(op, data, kspha, StartTime, dt; weights=nothing, JumpFact=3, Δτ_min, iter_max=10,
               λ=0, term_mask=nothing, max_outer=50)

FindDelay for an operator built on the ADC times (`op.times == datatime`)
without concomitant terms; `kspha::CuMatrix{Float64}` is the
(nFieldSample, nTerm) coefficient series.  Returns the delay τ.
"""
function find_delay(op::GB300ExplicitOp, data::CuMatrix{ComplexF32}, kspha::CuMatrix{Float64},
                    StartTime::Real, dt::Real; weights::Union{Nothing,CuVector{ComplexF32}}=nothing,
                    JumpFact::Real=3, Δτ_min::Real, iter_max::Integer=10, λ::Real=0,
                    term_mask::Union{Nothing,Vector{Float64}}=nothing, max_outer::Integer=50)
    h = activate(op)
    GC.@preserve term_mask begin
        p = Ref(HoeDelayParams(Float64(StartTime), Float64(dt), Float64(Δτ_min), Float64(JumpFact), Float64(λ),
                               term_mask === nothing ? Ptr{Float64}(C_NULL) : pointer(term_mask),
                               Int32(iter_max), Int32(max_outer)))
        res = Ref(HoeDelayResult(0, 0, 0, 0, 0, 0))
        check(ccall((:hoe_find_delay, libhoe), Cint,
                    (Ptr{Cvoid}, Ref{HoeDelayParams}, CuPtr{ComplexF32}, CuPtr{ComplexF32}, CuPtr{Float64}, Int64,
                     CuPtr{ComplexF32}, Ref{HoeDelayResult}, CUDA.CUstream),
                    h, p, data, weights === nothing ? CU_NULL : weights, kspha, size(kspha, 1), CU_NULL, res,
                    stream_handle()), h)
    end
    return res[].tau
end

"""
    find_delay_multishot(op, data, kspha, StartTime, dt; op_resid=nothing, weights=nothing, JumpFact=3,
                         Δτ_min, iter_max=10, λ=0, term_mask=nothing, max_outer=50)

FindDelay_multishot (FindDelay_multishot.jl:65-158) for an operator built on
all shots' samples, shot-major, with the concatenated ADC times and without
concomitant terms.  `kspha::CuArray{Float64,3}` holds each shot's
(nFieldSample, nTerm) series, shots last; `StartTime` one start per shot.
`op_resid`: the operator for the per-shot residual and derivative products
(`nothing` for `op`); the reference builds them on the concatenated time
vector, i.e. on the first shot's times, which an operator on those times
repeated reproduces.  Returns the delay τ.
"""
function find_delay_multishot(op::GB300ExplicitOp, data::CuMatrix{ComplexF32}, kspha::CuArray{Float64,3},
                              StartTime::AbstractVector{<:Real}, dt::Real;
                              op_resid::Union{Nothing,GB300ExplicitOp}=nothing,
                              weights::Union{Nothing,CuVector{ComplexF32}}=nothing, JumpFact::Real=3,
                              Δτ_min::Real, iter_max::Integer=10, λ::Real=0,
                              term_mask::Union{Nothing,Vector{Float64}}=nothing, max_outer::Integer=50)
    h = activate(op)
    hr = op_resid === nothing ? C_NULL : activate(op_resid)
    starts = Vector{Float64}(StartTime)
    GC.@preserve term_mask starts begin
        p = Ref(HoeDelayParams(0.0, Float64(dt), Float64(Δτ_min), Float64(JumpFact), Float64(λ),
                               term_mask === nothing ? Ptr{Float64}(C_NULL) : pointer(term_mask),
                               Int32(iter_max), Int32(max_outer)))
        res = Ref(HoeDelayResult(0, 0, 0, 0, 0, 0))
        check(ccall((:hoe_find_delay_multishot, libhoe), Cint,
                    (Ptr{Cvoid}, Ptr{Cvoid}, Ref{HoeDelayParams}, Int32, Ptr{Float64}, CuPtr{ComplexF32},
                     CuPtr{ComplexF32}, CuPtr{Float64}, Int64, CuPtr{ComplexF32}, Ref{HoeDelayResult}, CUDA.CUstream),
                    h, hr, p, Int32(size(kspha, 3)), pointer(starts), data,
                    weights === nothing ? CU_NULL : weights, kspha, size(kspha, 1), CU_NULL, res,
                    stream_handle()), h)
    end
    return res[].tau
end

end # module
