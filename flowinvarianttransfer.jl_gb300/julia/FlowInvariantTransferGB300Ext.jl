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
#   calculate_partial_fluxes(GB300Array(û; spectral=GB300Spectral(:fp32)), ks; binning=DyadicBinning(1.0))
#   calculate_band_to_band_transfer(GB300Array(û), ks; bands=SmoothBands([2.0, 4.0, 8.0]))
module FlowInvariantTransferGB300Ext

using FlowInvariantTransfer: FlowInvariantTransfer as FET
using FlowInvariantTransfer.Types: AbstractSpectralBackend, AbstractExecutionBackend, AbstractDealiasing,
    NoDealiasing, OrszagTwoThirds, PaddedThreeHalves, AbstractInvariant, KineticEnergy, PassiveScalar, Helicity,
    Enstrophy, ShellToShellResult, ShellMagnitude
using FlowInvariantTransfer.ShellBinning: shell_edges, shell_centers, shell_coordinate
using FlowInvariantTransfer.Types: HelicalDecomposition, HelmholtzDecomposition, ToroidalPoloidalDecomposition,
    SmoothBands, IsotropicShells, SpectralFluxResult, ModeToModeTriadResult

export GB300Spectral, GB300Execution, GB300Array

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

# 4. reference functions whose backend is a keyword only (src/SpectralFlux.jl:240-285,
# src/ScaleToScale/ScaleToScaleTransfer.jl:49-91, src/BandTransfer.jl:65-113) dispatch on the
# array: a field wrapped in GB300Array runs them in libfit_gb300.
"""
    GB300Array(û; spectral=GB300Spectral())

A spectral field (column-major `(ns..., comp)`, interleaved complex) marked for the GB300 backend.
`calculate_partial_fluxes`, `calculate_mode_to_mode_transfer` and `calculate_band_to_band_transfer`
called on it run in libfit_gb300 and return the reference's result types.
"""
struct GB300Array{T, N, A <: AbstractArray{T, N}} <: AbstractArray{T, N}
    data::A
    spectral::GB300Spectral
end
GB300Array(A::AbstractArray; spectral=GB300Spectral()) = GB300Array{eltype(A), ndims(A), typeof(A)}(A, spectral)
Base.size(a::GB300Array) = size(a.data)
Base.getindex(a::GB300Array, i...) = getindex(a.data, i...)
Base.unsafe_convert(::Type{Ptr{T}}, a::GB300Array) where {T} = Base.unsafe_convert(Ptr{T}, a.data)
Base.cconvert(::Type{Ptr{Cvoid}}, a::GB300Array) = a.data

_decomp(::HelicalDecomposition) = (Cint(1), (:positive, :negative))
_decomp(::HelmholtzDecomposition) = (Cint(2), (:rotational, :divergent))
_decomp(::ToroidalPoloidalDecomposition) = (Cint(3), (:toroidal, :poloidal))
_coord32(ks) = eltype(ks[1]) == Float32 ? Cint(1) : Cint(0)

function FET.SpectralFlux.calculate_partial_fluxes(velocity_hat::GB300Array, ks;
        decomposition=HelicalDecomposition(), binning=FET.SpectralFlux._default_binning(ks),
        dealiasing=OrszagTwoThirds(), spectral=velocity_hat.spectral, geometry=IsotropicShells())
    û = velocity_hat.data
    p = _plan(û, ks, dealiasing, spectral isa GB300Spectral ? spectral : velocity_hat.spectral)
    code, names = _decomp(decomposition)
    κ = shell_coordinate(geometry, ks)
    edges = Vector{Float64}(shell_edges(binning, maximum(κ)))
    centers = collect(shell_centers(binning, maximum(κ)))
    nsh = length(edges) - 1
    Tc = Vector{Float64}(undef, 8 * nsh)
    _check(ccall((:fit_partial_fluxes, LIB), Cint,
        (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Cint, Ptr{Float64}, Cint, UInt32, Cint, Ptr{Float64}, Cint),
        p.ptr, û, code, Cint(0), edges, length(edges), _dims_mask(geometry, length(ks)), _coord32(ks), Tc, 0))
    FT = real(eltype(û))
    channels = Dict{NTuple{3, Symbol}, SpectralFluxResult}()
    for (ik, sk) in enumerate(names), (ip, sp) in enumerate(names), (iq, sq) in enumerate(names)
        off = ((ik - 1) * 4 + (ip - 1) * 2 + (iq - 1)) * nsh
        T = FT.(Tc[off+1:off+nsh])
        channels[(sk, sp, sq)] = SpectralFluxResult(centers, T, cumsum(T))
    end
    total = SpectralFluxResult(centers, sum(c.transfer_spectrum for c in values(channels)),
                               sum(c.flux for c in values(channels)))
    return (channels = channels, total = total, k_shells = centers)
end

function FET.ScaleToScaleTransfer.calculate_mode_to_mode_transfer(velocity_hat::GB300Array, ks;
        invariant=KineticEnergy(),
        dealiasing=OrszagTwoThirds(), spectral=velocity_hat.spectral, max_modes::Int=1024, force::Bool=false,
        advecting_hat=velocity_hat)
    û = velocity_hat.data
    nd = length(ks)
    ns = size(û)[1:nd]
    nm = prod(ns)
    (force || nm <= max_modes) || throw(ArgumentError(
        "calculate_mode_to_mode_transfer resolves S(k|p) over all $(nm)x$(nm) mode pairs; N_modes=$nm exceeds " *
        "max_modes=$max_modes (pass force=true)."))
    adv = advecting_hat isa GB300Array ? advecting_hat.data : advecting_hat
    p = _plan(û, ks, dealiasing, spectral isa GB300Spectral ? spectral : velocity_hat.spectral; advecting=adv)
    S = Array{Float64}(undef, ns..., ns...)
    net = Array{Float64}(undef, ns...)
    _check(ccall((:fit_mode_to_mode, LIB), Cint,
        (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cint, Cint, Ptr{Float64}, Ptr{Float64}, Cint),
        p.ptr, û, adv === û ? C_NULL : adv, _inv(invariant), Cint(1), S, net, 0))
    FT = real(eltype(û))
    return ModeToModeTriadResult(invariant, ks, FT.(net), FT.(S))
end

function FET.BandTransfer.calculate_band_to_band_transfer(velocity_hat::GB300Array, ks; bands::SmoothBands,
        dealiasing=OrszagTwoThirds(), invariant=KineticEnergy(), spectral=velocity_hat.spectral,
        advecting_hat=velocity_hat, geometry=IsotropicShells())
    û = velocity_hat.data
    adv = advecting_hat isa GB300Array ? advecting_hat.data : advecting_hat
    p = _plan(û, ks, dealiasing, spectral isa GB300Spectral ? spectral : velocity_hat.spectral; advecting=adv)
    centers = Vector{Float64}(bands.centers)
    nb = length(centers)
    T = Matrix{Float64}(undef, nb, nb)
    net = Vector{Float64}(undef, nb)
    asym = Ref{Float64}(NaN)
    _check(ccall((:fit_band_to_band, LIB), Cint,
        (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Float64}, Cint, Cdouble, UInt32, Cint, Cint, Ptr{Float64},
         Ptr{Float64}, Ptr{Float64}, Cint),
        p.ptr, û, adv === û ? C_NULL : adv, centers, nb, Float64(bands.logwidth), _dims_mask(geometry, length(ks)),
        _coord32(ks), _inv(invariant), T, net, asym, 0))
    FT = real(eltype(û))
    return (centers = collect(bands.centers), transfer_matrix = FT.(T), net_transfer = FT.(net),
            max_antisymmetry_error = FT(asym[]))
end

end # module
