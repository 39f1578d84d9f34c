# Julia glue: plugs libfit_gb300 into FlowInvariantTransfer.jl as a new spectral backend
# (`GB300Spectral`) and execution backend (`GB300Execution`), overriding the positional
# dispatch points of the reference package. Untested in this repository (no Julia toolchain
# here); every ccall below binds a declaration of include/fit_gb300.h one to one.
#
# Usage (inside a Julia environment that has FlowInvariantTransfer.jl):
#   ENV["FIT_GB300_LIB"] = "/path/to/libfit_gb300.so"
#   include("FlowInvariantTransferGB300Ext.jl"); using .FlowInvariantTransferGB300Ext: GB300Spectral, GB300Execution
#   calculate_spectral_flux(û, ks; spectral=GB300Spectral(), binning=LinearBinning(1.0))
#   calculate_shell_to_shell_transfer(û, ks; spectral=GB300Spectral(:fp32), execution=GB300Execution())
module FlowInvariantTransferGB300Ext

using FlowInvariantTransfer: FlowInvariantTransfer as FET
using FlowInvariantTransfer.Types: AbstractSpectralBackend, AbstractExecutionBackend, AbstractDealiasing,
    NoDealiasing, OrszagTwoThirds, PaddedThreeHalves, AbstractInvariant, KineticEnergy, PassiveScalar, Helicity,
    Enstrophy, ShellToShellResult, ShellMagnitude
using FlowInvariantTransfer.ShellBinning: shell_edges, shell_coordinate

export GB300Spectral, GB300Execution

const LIB = get(ENV, "FIT_GB300_LIB", "libfit_gb300")

"""
    GB300Spectral(precision=:fp64)

Spectral backend running the nonlinear term and the shell reductions in libfit_gb300 on the GPU.
`:fp64` is the plain FP64 method; `:fp32` runs transforms and products in FP32 with FP64 shell sums.
"""
struct GB300Spectral <: AbstractSpectralBackend
    precision::Symbol
end
GB300Spectral() = GB300Spectral(:fp64)

"""
    GB300Execution(mode=:batched)

Execution backend for the shell-to-shell mediator loop: `:batched` (mediators batched, fused
kernels, CUDA-graph replay) or `:plain` (one nonlinear term per mediator).
"""
struct GB300Execution <: AbstractExecutionBackend
    mode::Symbol
end
GB300Execution() = GB300Execution(:batched)

_dealias(::NoDealiasing) = Cint(0)
_dealias(::OrszagTwoThirds) = Cint(1)
_dealias(::PaddedThreeHalves) = Cint(2)
_inv(::KineticEnergy) = Cint(0)
_inv(::PassiveScalar) = Cint(1)
_inv(::Helicity) = Cint(2)
_inv(::Enstrophy) = Cint(3)
_prec(b::GB300Spectral) = b.precision === :fp32 ? Cint(32) : Cint(64)

function _check(rc)
    rc == 0 && return nothing
    msg = unsafe_string(ccall((:fit_last_error, LIB), Cstring, ()))
    rc in (-1, -2) ? throw(ArgumentError(msg)) : error("libfit_gb300: " * msg)
end

# Plan bundle owned by the workspace (the `plans` hook of src/Workspaces.jl:46-75); the
# finalizer frees the device buffers and the stream.
mutable struct GB300Plan
    ptr::Ptr{Cvoid}
end

function _plan(f̂, ks, dealiasing, backend::GB300Spectral; advecting=f̂)
    nd = length(ks)
    ns = Int64[size(f̂, d) for d in 1:nd]
    kk = [Vector{Float64}(k) for k in ks]
    kp = [pointer(k) for k in kk]
    io64 = eltype(f̂) <: Complex{Float64} ? Cint(1) : Cint(0)
    out = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve kk begin
        _check(ccall((:fit_plan_create, LIB), Cint,
            (Ptr{Ptr{Cvoid}}, Cint, Ptr{Int64}, Cint, Cint, Cint, Cint, Cint, Ptr{Ptr{Float64}}),
            out, nd, ns, size(f̂, nd + 1), size(advecting, nd + 1), _dealias(dealiasing), _prec(backend), io64, kp))
    end
    p = GB300Plan(out[])
    finalizer(q -> ccall((:fit_plan_destroy, LIB), Cint, (Ptr{Cvoid},), q.ptr), p)
    return p
end

_dims_mask(g::ShellMagnitude, nd) = g.dims === nothing ? UInt32(2^nd - 1) :
    UInt32(sum(1 << (d - 1) for d in g.dims))

# 1. nonlinear term (src/NonlinearTerm.jl:102-116)
function FET.NonlinearTerm._compute_nonlinear_term!(ws, velocity_hat, ks, backend::GB300Spectral,
                                                    dealiasing::AbstractDealiasing; advecting_hat=velocity_hat)
    p = _plan(velocity_hat, ks, dealiasing, backend; advecting=advecting_hat)
    adv = advecting_hat === velocity_hat ? C_NULL : advecting_hat
    _check(ccall((:fit_nonlinear_term, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cint),
                 p.ptr, velocity_hat, adv, ws.N̂, 0))
    return ws.N̂
end

# 2. shell-to-shell (src/ShellToShell/ShellToShellTransfer.jl:152-159)
function FET.ShellToShellTransfer._calculate_shell_to_shell!(result, ws, velocity_hat, ks, ex::GB300Execution,
        spectral::GB300Spectral; dealiasing, verify_antisymmetry, invariant=KineticEnergy(),
        advecting_hat=velocity_hat)
    p = _plan(velocity_hat, ks, dealiasing, spectral; advecting=advecting_hat)
    edges = Vector{Float64}(result.shell_edges)
    nsh = length(edges) - 1
    T = Matrix{Float64}(undef, nsh, nsh)
    net = Vector{Float64}(undef, nsh)
    asym = Ref{Float64}(NaN)
    adv = advecting_hat === velocity_hat ? C_NULL : advecting_hat
    coord32 = eltype(ks[1]) == Float32 ? Cint(1) : Cint(0)
    _check(ccall((:fit_shell_to_shell, LIB), Cint,
        (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Float64}, Cint, UInt32, Cint, Cint, Cint, Cint, Ptr{Float64},
         Ptr{Float64}, Ptr{Float64}, Cint),
        p.ptr, velocity_hat, adv, edges, length(edges), UInt32(2^length(ks) - 1), coord32, _inv(invariant),
        ex.mode === :plain ? Cint(0) : Cint(1), Cint(verify_antisymmetry), T, net, asym, 0))
    result.transfer_matrix .= T
    result.net_transfer .= net
    return verify_antisymmetry ? eltype(result.transfer_matrix)(asym[]) : eltype(result.transfer_matrix)(NaN)
end

# 3. spectral flux with the binning on the device (src/SpectralFlux.jl:66-94)
function FET.SpectralFlux._calculate_spectral_flux_decomposed(û_decomp::AbstractArray{<:Complex}, velocity_hat, ks,
        binning, dealiasing, invariant, spectral::GB300Spectral, advecting_hat, geometry)
    p = _plan(velocity_hat, ks, dealiasing, spectral; advecting=advecting_hat)
    κ = shell_coordinate(geometry, ks)
    edges = Vector{Float64}(shell_edges(binning, maximum(κ)))
    centers = FET.ShellBinning.shell_centers(binning, maximum(κ))
    nsh = length(edges) - 1
    T = Vector{Float64}(undef, nsh); Π = Vector{Float64}(undef, nsh)
    adv = advecting_hat === velocity_hat ? C_NULL : advecting_hat
    car = û_decomp === velocity_hat ? C_NULL : û_decomp
    coord32 = eltype(ks[1]) == Float32 ? Cint(1) : Cint(0)
    _check(ccall((:fit_spectral_flux, LIB), Cint,
        (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Float64}, Cint, UInt32, Cint, Cint, Ptr{Float64},
         Ptr{Float64}, Cint),
        p.ptr, velocity_hat, adv, car, edges, length(edges), _dims_mask(geometry, length(ks)), coord32,
        _inv(invariant), T, Π, 0))
    FT = real(eltype(velocity_hat))
    return FET.Types.SpectralFluxResult(centers, FT.(T), FT.(Π))
end

end # module
