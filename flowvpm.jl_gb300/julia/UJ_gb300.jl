#=##############################################################################
# UJ_gb300.jl -- drop-in UJ hooks for FLOWVPM.jl backed by libvpm_gb300.so.
#
#   include("UJ_gb300.jl")
#   pfield = FLOWVPM.ParticleField(maxp; UJ=UJ_gb300)          # FP64
#   pfield = FLOWVPM.ParticleField(maxp; UJ=UJ_gb300_mixed)    # FP32-comp
#
# Both functions have the signature and semantics of
# FLOWVPM.UJ_direct(pfield; rbf, sfs, reset, reset_sfs) (src/FLOWVPM_UJ.jl:21-37)
# and pass the particle matrix itself (column-major 46 x maxparticles Float64,
# src/FLOWVPM_particlefield.jl:134) to `vpm_uj` of include/vpm_gb300.h.  They
# are plain functions, so FLOWVPM's settings writer records them as
# "*userfunction" (src/FLOWVPM_utils.jl:381-389).
#
# Not executed in this repository's test environment (no Julia toolchain); the
# same calls are exercised through Python's ctypes in tests/.
=###############################################################################
module VPMGB300

import FLOWVPM

const libvpm = get(ENV, "VPM_GB300_LIB", joinpath(@__DIR__, "..", "lib", "libvpm_gb300.so"))

const VPM_RESET = Cint(1)
const VPM_RESET_SFS = Cint(2)
const VPM_SFS = Cint(4)
const VPM_TRANSPOSED = Cint(8)
const VPM_FP64 = Cint(0)
const VPM_FP32COMP = Cint(1)

const _ctx = Ref{Ptr{Cvoid}}(C_NULL)

_lasterror(h) = unsafe_string(ccall((:vpm_last_error, libvpm), Cstring, (Ptr{Cvoid},), h))

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

"Kernel id of one of FLOWVPM's standard kernels (src/FLOWVPM.jl:129-132)."
function kernel_id(k)
    k === FLOWVPM.kernel_singular && return Cint(0)
    k === FLOWVPM.kernel_gaussian && return Cint(1)
    k === FLOWVPM.kernel_gaussianerf && return Cint(2)
    k === FLOWVPM.kernel_winckelmans && return Cint(3)
    error("UJ_gb300 supports only the standard kernels (singular, gaussian, gaussianerf, winckelmans)")
end

function _uj(pfield, precision::Cint; rbf::Bool=false, sfs::Bool=false, reset::Bool=true,
             reset_sfs::Bool=false, optargs...)
    rbf && error("UJ_gb300: rbf=true (zeta evaluation for the RBF solve) is not supported")
    P = pfield.particles
    eltype(P) == Float64 || error("UJ_gb300 needs a Float64 particle field (got $(eltype(P)))")
    flags = (reset ? VPM_RESET : Cint(0)) | (reset_sfs ? VPM_RESET_SFS : Cint(0)) |
            (sfs ? VPM_SFS : Cint(0)) | (pfield.transposed ? VPM_TRANSPOSED : Cint(0))
    h = context()
    rc = ccall((:vpm_uj, libvpm), Cint,
               (Ptr{Cvoid}, Ptr{Float64}, Int64, Int64, Cint, Cint, Cint),
               h, P, size(P, 1), pfield.np, kernel_id(pfield.kernel), precision, flags)
    rc == 0 || error("UJ_gb300 failed ($rc): " * _lasterror(h))
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
    rc == 0 || error("UJ_gb300 failed ($rc): " * _lasterror(h))
    return nothing
end

export UJ_gb300, UJ_gb300_mixed

end # module

using .VPMGB300: UJ_gb300, UJ_gb300_mixed
