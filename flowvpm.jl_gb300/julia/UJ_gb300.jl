#=##############################################################################
# UJ_gb300.jl -- drop-in UJ hooks for FLOWVPM.jl backed by libvpm_gb300.so,
# and ChainRulesCore rules for the pair sums on device arrays.
#
#   include("UJ_gb300.jl")
#   pfield = FLOWVPM.ParticleField(maxp; UJ=UJ_gb300)          # FP64
#   pfield = FLOWVPM.ParticleField(maxp; UJ=UJ_gb300_mixed)    # FP32-comp
#
# UJ_gb300 / UJ_gb300_mixed have the signature and semantics of
# FLOWVPM.UJ_direct(pfield; rbf, sfs, reset, reset_sfs) (src/FLOWVPM_UJ.jl:21-37):
# `rbf` is accepted and ignored, as UJ_direct ignores it.  They pass the
# particle matrix itself (column-major 46 x maxparticles Float64,
# src/FLOWVPM_particlefield.jl:134) to `vpm_uj` of include/vpm_gb300.h, and are
# plain functions, so FLOWVPM's settings writer records them as
# "*userfunction" (src/FLOWVPM_utils.jl:381-389).
#
# Differentiation.  uj_gb300_core(X, Γ, σ; kernel, precision) -> (U, J) and
# estr_gb300_core(X, Γ, σ, J; kernel, precision, transposed) -> SFS evaluate the
# self-induced pair sums of one particle set on CUDA arrays (X, Γ, U: 3 x n;
# σ: n; J: 9 x n; column-major, so each particle's entries are contiguous: the
# per-particle interleaved layout of the C ABI).  Their ChainRulesCore.rrule
# pullbacks call the hand-written adjoint kernels vpm_uj_adjoint_dev and
# vpm_estr_adjoint_dev; they replace the rule of src/FLOWVPM_rrules.jl:179-330,
# which is not included by src/FLOWVPM.jl and stops at "SFS pullback not
# implemented yet!" (src/FLOWVPM_rrules.jl:153-157).  The Python package
# vpm_gb300.autodiff wraps the same calls as torch.autograd.Functions
# (UJFunction, EstrFunction) and is what the test suite exercises.
#
# Needs CUDA.jl and ChainRulesCore.jl in the environment that includes it.  Not
# executed in this repository's test environment (no Julia toolchain); the same
# C calls are exercised through Python's ctypes in tests/.
=###############################################################################
module VPMGB300

import FLOWVPM
import CUDA
import ChainRulesCore
using CUDA: CuArray, CuPtr

const libvpm = get(ENV, "VPM_GB300_LIB", joinpath(@__DIR__, "..", "lib", "libvpm_gb300.so"))

const VPM_RESET = Cint(1)
const VPM_RESET_SFS = Cint(2)
const VPM_SFS = Cint(4)
const VPM_TRANSPOSED = Cint(8)
const VPM_FP64 = Cint(0)
const VPM_FP32COMP = Cint(1)

const _ctx = Ref{Ptr{Cvoid}}(C_NULL)

_lasterror(h) = unsafe_string(ccall((:vpm_last_error, libvpm), Cstring, (Ptr{Cvoid},), h))
_check(rc, h, what) = rc == 0 || error("$what failed ($rc): " * _lasterror(h))

"One libvpm_gb300 context on CUDA device 0, created on first use."
function context()
    if _ctx[] == C_NULL
        h = Ref{Ptr{Cvoid}}(C_NULL)
        rc = ccall((:vpm_ctx_create, libvpm), Cint, (Ptr{Ptr{Cvoid}}, Cint), h, 0)
        rc == 0 || error("vpm_ctx_create failed ($rc): " * _lasterror(C_NULL))
        _ctx[] = h[]
        atexit(() -> (ccall((:vpm_ctx_destroy, libvpm), Cint, (Ptr{Cvoid},), _ctx[]); _ctx[] = C_NULL))
    end
    return _ctx[]
end

"The context runs on CUDA.jl's current stream, so its kernels are ordered after the arrays' producers."
function _on_current_stream(h)
    s = CUDA.stream()
    _check(ccall((:vpm_ctx_set_stream, libvpm), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), h,
                 Base.unsafe_convert(Ptr{Cvoid}, s.handle)), h, "vpm_ctx_set_stream")
    return h
end

"Kernel id of one of FLOWVPM's standard kernels (src/FLOWVPM.jl:129-132)."
function kernel_id(k)
    k === FLOWVPM.kernel_singular && return Cint(0)
    k === FLOWVPM.kernel_gaussian && return Cint(1)
    k === FLOWVPM.kernel_gaussianerf && return Cint(2)
    k === FLOWVPM.kernel_winckelmans && return Cint(3)
    error("UJ_gb300 supports only the standard kernels (singular, gaussian, gaussianerf, winckelmans)")
end
kernel_id(k::Integer) = Cint(k)

# ------------------------------------------------------------- drop-in hooks
function _uj(pfield, precision::Cint; rbf::Bool=false, sfs::Bool=false, reset::Bool=true,
             reset_sfs::Bool=false, optargs...)
    # rbf is accepted and ignored, as UJ_direct does (src/FLOWVPM_UJ.jl:21-37)
    P = pfield.particles
    eltype(P) == Float64 || error("UJ_gb300 needs a Float64 particle field (got $(eltype(P)))")
    flags = (reset ? VPM_RESET : Cint(0)) | (reset_sfs ? VPM_RESET_SFS : Cint(0)) |
            (sfs ? VPM_SFS : Cint(0)) | (pfield.transposed ? VPM_TRANSPOSED : Cint(0))
    h = context()
    rc = ccall((:vpm_uj, libvpm), Cint,
               (Ptr{Cvoid}, Ptr{Float64}, Int64, Int64, Cint, Cint, Cint),
               h, P, size(P, 1), pfield.np, kernel_id(pfield.kernel), precision, flags)
    _check(rc, h, "UJ_gb300")
    return nothing
end

"UJ_direct on the GB300, FP64 (the reference formula)."
UJ_gb300(pfield; optargs...) = _uj(pfield, VPM_FP64; optargs...)

"UJ_direct on the GB300, FP32 pair math with FP64 positions and block reduction."
UJ_gb300_mixed(pfield; optargs...) = _uj(pfield, VPM_FP32COMP; optargs...)

"UJ_direct(source, target) (src/FLOWVPM_UJ.jl:48-50): accumulate, no reset."
function UJ_gb300(source::FLOWVPM.ParticleField, target::FLOWVPM.ParticleField; precision=VPM_FP64)
    h = context()
    rc = ccall((:vpm_uj_cross, libvpm), Cint,
               (Ptr{Cvoid}, Ptr{Float64}, Int64, Int64, Ptr{Float64}, Int64, Int64, Cint, Cint),
               h, source.particles, size(source.particles, 1), source.np,
               target.particles, size(target.particles, 1), target.np, kernel_id(source.kernel), precision)
    _check(rc, h, "UJ_gb300")
    return nothing
end

"zeta_direct(pfield) (src/FLOWVPM_viscous.jl:467-488): rows 16:18 of every particle set to the RBF basis field."
function zeta_gb300(pfield; precision=VPM_FP64)
    h = context()
    P = pfield.particles
    rc = ccall((:vpm_zeta, libvpm), Cint, (Ptr{Cvoid}, Ptr{Float64}, Int64, Int64, Cint, Cint),
               h, P, size(P, 1), pfield.np, kernel_id(pfield.kernel), precision)
    _check(rc, h, "zeta_gb300")
    return nothing
end

# ---------------------------------------------- differentiable device core
"(U, J) = self-induced UJ of the particle set (X 3xn, Γ 3xn, σ n) on the GPU."
function uj_gb300_core(X::CuArray{Float64}, Γ::CuArray{Float64}, σ::CuArray{Float64};
                       kernel, precision=VPM_FP64)
    n = size(X, 2)
    U = CUDA.zeros(Float64, 3, n)
    J = CUDA.zeros(Float64, 9, n)
    h = _on_current_stream(context())
    rc = ccall((:vpm_uj_dev, libvpm), Cint,
               (Ptr{Cvoid}, Int64, CuPtr{Float64}, Int64, CuPtr{Float64}, CuPtr{Float64}, CuPtr{Float64},
                CuPtr{Float64}, CuPtr{Float64}, Cint, Cint),
               h, n, X, n, X, Γ, σ, U, J, kernel_id(kernel), precision)
    _check(rc, h, "vpm_uj_dev")
    return U, J
end

"SFS = self-induced Estr (src/FLOWVPM_subfilterscale_models.jl:16-92) of the particle set, with gradients J (9xn)."
function estr_gb300_core(X::CuArray{Float64}, Γ::CuArray{Float64}, σ::CuArray{Float64}, J::CuArray{Float64};
                         kernel, precision=VPM_FP64, transposed::Bool=true)
    n = size(X, 2)
    SFS = CUDA.zeros(Float64, 3, n)
    h = _on_current_stream(context())
    rc = ccall((:vpm_estr_dev, libvpm), Cint,
               (Ptr{Cvoid}, Int64, CuPtr{Float64}, CuPtr{Float64}, Ptr{UInt8}, Int64, CuPtr{Float64},
                CuPtr{Float64}, CuPtr{Float64}, CuPtr{Float64}, Ptr{UInt8}, CuPtr{Float64}, Cint, Cint, Cint),
               h, n, X, J, C_NULL, n, X, Γ, σ, J, C_NULL, SFS, kernel_id(kernel), precision,
               transposed ? VPM_TRANSPOSED : Cint(0))
    _check(rc, h, "vpm_estr_dev")
    return SFS
end

_dense(t, like) = t isa ChainRulesCore.AbstractZero ? zero(like) : CuArray{Float64}(ChainRulesCore.unthunk(t))

function ChainRulesCore.rrule(::typeof(uj_gb300_core), X, Γ, σ; kernel, precision=VPM_FP64)
    U, J = uj_gb300_core(X, Γ, σ; kernel=kernel, precision=precision)
    function uj_gb300_core_pullback(ȳ)
        Ū, J̄ = _dense(ȳ[1], U), _dense(ȳ[2], J)
        X̄, Γ̄, σ̄ = zero(X), zero(Γ), zero(σ)
        h = _on_current_stream(context())
        rc = ccall((:vpm_uj_adjoint_dev, libvpm), Cint,
                   (Ptr{Cvoid}, Int64, CuPtr{Float64}, CuPtr{Float64}, CuPtr{Float64}, CuPtr{Float64},
                    CuPtr{Float64}, CuPtr{Float64}, CuPtr{Float64}, CuPtr{Float64}, Cint, Cint),
                   h, size(X, 2), X, Γ, σ, Ū, J̄, X̄, Γ̄, σ̄, kernel_id(kernel), precision)
        _check(rc, h, "vpm_uj_adjoint_dev")
        return ChainRulesCore.NoTangent(), X̄, Γ̄, σ̄
    end
    return (U, J), uj_gb300_core_pullback
end

function ChainRulesCore.rrule(::typeof(estr_gb300_core), X, Γ, σ, J; kernel, precision=VPM_FP64,
                              transposed::Bool=true)
    SFS = estr_gb300_core(X, Γ, σ, J; kernel=kernel, precision=precision, transposed=transposed)
    function estr_gb300_core_pullback(S̄)
        S̄d = _dense(S̄, SFS)
        X̄, Γ̄, σ̄, J̄ = zero(X), zero(Γ), zero(σ), zero(J)
        h = _on_current_stream(context())
        rc = ccall((:vpm_estr_adjoint_dev, libvpm), Cint,
                   (Ptr{Cvoid}, Int64, CuPtr{Float64}, CuPtr{Float64}, CuPtr{Float64}, CuPtr{Float64}, Ptr{UInt8},
                    CuPtr{Float64}, CuPtr{Float64}, CuPtr{Float64}, CuPtr{Float64}, CuPtr{Float64}, Cint, Cint, Cint),
                   h, size(X, 2), X, Γ, σ, J, C_NULL, S̄d, X̄, Γ̄, σ̄, J̄, kernel_id(kernel), precision,
                   transposed ? VPM_TRANSPOSED : Cint(0))
        _check(rc, h, "vpm_estr_adjoint_dev")
        return ChainRulesCore.NoTangent(), X̄, Γ̄, σ̄, J̄
    end
    return SFS, estr_gb300_core_pullback
end

export UJ_gb300, UJ_gb300_mixed, zeta_gb300, uj_gb300_core, estr_gb300_core

end # module

using .VPMGB300: UJ_gb300, UJ_gb300_mixed, zeta_gb300, uj_gb300_core, estr_gb300_core
