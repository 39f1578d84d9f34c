# Julia glue: plugs libfit_gb300 into FlowInvariantTransfer.jl as a new spectral backend
# (`GB300Spectral`) and execution backend (`GB300Execution`), overriding the positional
# dispatch points of the reference package. Untested in this repository (no Julia toolchain
# here); every ccall below binds a declaration of include/fit_gb300.h one to one (the
# repository's CPU tests parse these ccalls and check them against the header).
#
# Usage (inside a Julia environment that has FlowInvariantTransfer.jl):
#   ENV["FIT_GB300_LIB"] = "/path/to/libfit_gb300.so"
#   include("FlowInvariantTransferGB300Ext.jl"); using .FlowInvariantTransferGB300Ext: GB300Spectral, GB300Execution, GB300Array
#   calculate_spectral_flux(û, ks; spectral=GB300Spectral(), binning=LinearBinning(1.0))
#   ua = GB300Array(û)   # owns the device plans: repeated calls on it reuse them (graph replay)
#   calculate_shell_to_shell_transfer(ua, ks; spectral=GB300Spectral(:fp32), execution=GB300Execution())
#   calculate_partial_fluxes(GB300Array(û; spectral=GB300Spectral(:fp32)), ks; binning=DyadicBinning(2.0))
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

# ---- plans and the workspace's plan bundle ------------------------------------------------------
# One libfit_gb300 plan: device buffers, transform tables, one CUDA stream. The finalizer frees them.
# `idx` is the shell-index array last installed with fit_set_shell_index (compared by identity), or
# `nothing` after a call that binned by shell edges (which replaces the plan's shell table).
mutable struct GB300Plan
    ptr::Ptr{Cvoid}
    idx::Any
end

# The plan bundle that `Workspaces._make_fft_plans` returns for a GB300Array (the `plans` hook of
# src/Workspaces.jl:15-22,73, as the FFTW extension's bundle at ext/FlowInvariantTransferFFTWExt.jl:26-49):
# it owns one plan per (grid, components, dealiasing, precision, wavenumbers) configuration, created
# on first use and reused by every later call, so a second call with the same array replays the
# batched shell-to-shell CUDA graph instead of rebuilding tables.
struct GB300PlanBundle
    plans::Dict{Any, GB300Plan}
    lock::ReentrantLock
end
GB300PlanBundle() = GB300PlanBundle(Dict{Any, GB300Plan}(), ReentrantLock())

# plans of plain (unwrapped) arrays, shared by key; bounded so that a long session does not keep
# the device memory of every grid it ever saw
const _SHARED = GB300PlanBundle()
const _SHARED_MAX = 8

"""
    GB300Array(û; spectral=GB300Spectral())

A spectral field (column-major `(ns..., comp)`, interleaved complex) marked for the GB300 backend.
It owns the device plans of the calls made on it (reused across calls), and
`calculate_partial_fluxes`, `calculate_mode_to_mode_transfer` and `calculate_band_to_band_transfer`
called on it run in libfit_gb300 and return the reference's result types.
"""
struct GB300Array{T, N, A <: AbstractArray{T, N}} <: AbstractArray{T, N}
    data::A
    spectral::GB300Spectral
    plans::GB300PlanBundle
end
GB300Array(A::AbstractArray; spectral=GB300Spectral()) =
    GB300Array{eltype(A), ndims(A), typeof(A)}(A, spectral, GB300PlanBundle())
Base.size(a::GB300Array) = size(a.data)
Base.getindex(a::GB300Array, i...) = getindex(a.data, i...)
Base.setindex!(a::GB300Array, v, i...) = setindex!(a.data, v, i...)
Base.similar(a::GB300Array, ::Type{S}, dims::Dims) where {S} = similar(a.data, S, dims)
Base.unsafe_convert(::Type{Ptr{T}}, a::GB300Array) where {T} = Base.unsafe_convert(Ptr{T}, a.data)
Base.cconvert(::Type{Ptr{Cvoid}}, a::GB300Array) = a.data

_raw(a::GB300Array) = a.data
_raw(a) = a

# More specific than both the core fallback and the FFTW extension's method for complex arrays
# (ext/FlowInvariantTransferFFTWExt.jl:37): every workspace built on a GB300Array gets its bundle.
FET.Workspaces._make_fft_plans(a::GB300Array{<:Complex}, ks) = a.plans

_bundle(ws) = hasproperty(ws, :plans) && ws.plans isa GB300PlanBundle ? ws.plans :
    hasproperty(ws, :nonlinear) ? _bundle(ws.nonlinear) : nothing

function _plan(f̂, ks, dealiasing, backend::GB300Spectral; advecting=f̂, bundle=nothing)
    data, adv = _raw(f̂), _raw(advecting)
    nd = length(ks)
    ns = Int64[size(data, d) for d in 1:nd]
    kk = [Vector{Float64}(k) for k in ks]
    io64 = eltype(data) <: Complex{Float64} ? Cint(1) : Cint(0)
    M, D = size(data, nd + 1), size(adv, nd + 1)
    key = (Tuple(ns), M, D, _dealias(dealiasing), _prec(backend), io64, hash(kk))
    b = bundle !== nothing ? bundle : f̂ isa GB300Array ? f̂.plans : _SHARED
    lock(b.lock) do
        p = get(b.plans, key, nothing)
        p === nothing || return p
        if b === _SHARED && length(b.plans) >= _SHARED_MAX
            empty!(b.plans)   # dropped plans are freed by their finalizers once unreferenced
        end
        out = Ref{Ptr{Cvoid}}(C_NULL)
        kp = [pointer(k) for k in kk]
        GC.@preserve kk begin
            _check(ccall((:fit_plan_create, LIB), Cint,
                (Ptr{Ptr{Cvoid}}, Cint, Ptr{Int64}, Cint, Cint, Cint, Cint, Cint, Ptr{Ptr{Float64}}),
                out, nd, ns, M, D, _dealias(dealiasing), _prec(backend), io64, kp))
        end
        p = GB300Plan(out[], nothing)
        finalizer(q -> ccall((:fit_plan_destroy, LIB), Cint, (Ptr{Cvoid},), q.ptr), p)
        b.plans[key] = p
        return p
    end
end

_dims_mask(g::ShellMagnitude, nd) = g.dims === nothing ? UInt32(2^nd - 1) :
    UInt32(sum(1 << (d - 1) for d in g.dims))
_coord32(ks) = eltype(ks[1]) == Float32 ? Cint(1) : Cint(0)
_advptr(advecting_hat, velocity_hat) = advecting_hat === velocity_hat ? C_NULL : _raw(advecting_hat)

# 1. nonlinear term (src/NonlinearTerm.jl:102-116)
function FET.NonlinearTerm._compute_nonlinear_term!(ws, velocity_hat, ks, backend::GB300Spectral,
                                                    dealiasing::AbstractDealiasing; advecting_hat=velocity_hat)
    p = _plan(velocity_hat, ks, dealiasing, backend; advecting=advecting_hat, bundle=_bundle(ws))
    _check(ccall((:fit_nonlinear_term, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cint),
                 p.ptr, velocity_hat, _advptr(advecting_hat, velocity_hat), ws.N̂, 0))
    return ws.N̂
end

# 2. shell-to-shell (src/ShellToShell/ShellToShellTransfer.jl:152-159): binned by the workspace's
# own ws.shell_idx (built for the caller's shell geometry, src/Workspaces.jl:154-169), which is
# installed in the plan once per index array and reused while the same array comes back.
function FET.ShellToShellTransfer._calculate_shell_to_shell!(result, ws, velocity_hat, ks, ex::GB300Execution,
        spectral::GB300Spectral; dealiasing, verify_antisymmetry, invariant=KineticEnergy(),
        advecting_hat=velocity_hat)
    p = _plan(velocity_hat, ks, dealiasing, spectral; advecting=advecting_hat, bundle=_bundle(ws))
    nsh = size(result.transfer_matrix, 1)
    T = Matrix{Float64}(undef, nsh, nsh)
    net = Vector{Float64}(undef, nsh)
    asym = Ref{Float64}(NaN)
    run() = ccall((:fit_shell_to_shell_indexed, LIB), Cint,
        (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cint, Cint, Cint, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Cint),
        p.ptr, velocity_hat, _advptr(advecting_hat, velocity_hat), _inv(invariant),
        ex.mode === :plain ? Cint(0) : Cint(1), Cint(verify_antisymmetry), T, net, asym, 0)
    install() = begin
        idx = ws.shell_idx isa Array{Int64} ? ws.shell_idx : Array{Int64}(ws.shell_idx)
        _check(ccall((:fit_set_shell_index, LIB), Cint, (Ptr{Cvoid}, Ptr{Int64}, Cint, Cint),
                     p.ptr, idx, Cint(nsh), 0))
        p.idx = ws.shell_idx
    end
    p.idx === ws.shell_idx || install()
    rc = run()
    if rc == -5   # FIT_ERR_STATE: another call replaced the plan's shell table; install it again
        install()
        rc = run()
    end
    _check(rc)
    result.transfer_matrix .= T
    result.net_transfer .= net
    return verify_antisymmetry ? eltype(result.transfer_matrix)(asym[]) : eltype(result.transfer_matrix)(NaN)
end

function _flux(p, velocity_hat, ks, edges, geometry, dealiasing, invariant, advecting_hat, carrier)
    nsh = length(edges) - 1
    T = Vector{Float64}(undef, nsh); Π = Vector{Float64}(undef, nsh)
    p.idx = nothing   # binning by edges replaces the plan's shell table
    _check(ccall((:fit_spectral_flux, LIB), Cint,
        (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Float64}, Cint, UInt32, Cint, Cint, Ptr{Float64},
         Ptr{Float64}, Cint),
        p.ptr, velocity_hat, _advptr(advecting_hat, velocity_hat), carrier, edges, length(edges),
        _dims_mask(geometry, length(ks)), _coord32(ks), _inv(invariant), T, Π, 0))
    return T, Π
end

# 3. spectral flux with the binning on the device (src/SpectralFlux.jl:66-94)
function FET.SpectralFlux._calculate_spectral_flux_decomposed(û_decomp::AbstractArray{<:Complex}, velocity_hat, ks,
        binning, dealiasing, invariant, spectral::GB300Spectral, advecting_hat, geometry)
    p = _plan(velocity_hat, ks, dealiasing, spectral; advecting=advecting_hat)
    κ = shell_coordinate(geometry, ks)
    edges = Vector{Float64}(shell_edges(binning, maximum(κ)))
    centers = shell_centers(binning, maximum(κ))
    car = û_decomp === velocity_hat ? C_NULL : _raw(û_decomp)
    T, Π = _flux(p, velocity_hat, ks, edges, geometry, dealiasing, invariant, advecting_hat, car)
    FT = real(eltype(velocity_hat))
    return FET.Types.SpectralFluxResult(centers, FT.(T), FT.(Π))
end

# 3b. the NamedTuple branch (src/SpectralFlux.jl:96-122): one result per decomposed component,
# each the flux of the full nonlinear term carried by that component. The library evaluates the
# nonlinear term once per component call; the values are the same as from one shared N̂.
function FET.SpectralFlux._calculate_spectral_flux_decomposed(decomposed::NamedTuple, velocity_hat, ks,
        binning, dealiasing, invariant, spectral::GB300Spectral, advecting_hat, geometry)
    p = _plan(velocity_hat, ks, dealiasing, spectral; advecting=advecting_hat)
    κ = shell_coordinate(geometry, ks)
    edges = Vector{Float64}(shell_edges(binning, maximum(κ)))
    centers = shell_centers(binning, maximum(κ))
    FT = real(eltype(velocity_hat))
    return map(decomposed) do û_comp
        T, Π = _flux(p, velocity_hat, ks, edges, geometry, dealiasing, invariant, advecting_hat, _raw(û_comp))
        FET.Types.SpectralFluxResult(centers, FT.(T), FT.(Π))
    end
end

# 4. reference functions whose backend is a keyword only (src/SpectralFlux.jl:240-285,
# src/ScaleToScale/ScaleToScaleTransfer.jl:49-91, src/BandTransfer.jl:65-113) dispatch on the
# array: a field wrapped in GB300Array runs them in libfit_gb300.
_decomp(::HelicalDecomposition) = (Cint(1), (:positive, :negative))
_decomp(::HelmholtzDecomposition) = (Cint(2), (:rotational, :divergent))
_decomp(::ToroidalPoloidalDecomposition) = (Cint(3), (:toroidal, :poloidal))

function FET.SpectralFlux.calculate_partial_fluxes(velocity_hat::GB300Array, ks;
        decomposition=HelicalDecomposition(), binning=FET.SpectralFlux._default_binning(ks),
        dealiasing=OrszagTwoThirds(), spectral=velocity_hat.spectral, geometry=IsotropicShells())
    û = velocity_hat.data
    p = _plan(velocity_hat, ks, dealiasing, spectral isa GB300Spectral ? spectral : velocity_hat.spectral)
    code, names = _decomp(decomposition)
    κ = shell_coordinate(geometry, ks)
    edges = Vector{Float64}(shell_edges(binning, maximum(κ)))
    centers = collect(shell_centers(binning, maximum(κ)))
    nsh = length(edges) - 1
    Tc = Vector{Float64}(undef, 8 * nsh)
    p.idx = nothing
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

# S(k|p) products in the backend's precision: FP64 for GB300Spectral(:fp64), FP32 (with FP64 sums)
# for GB300Spectral(:fp32).
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
    sp = spectral isa GB300Spectral ? spectral : velocity_hat.spectral
    p = _plan(velocity_hat, ks, dealiasing, sp; advecting=advecting_hat)
    S = Array{Float64}(undef, ns..., ns...)
    net = Array{Float64}(undef, ns...)
    _check(ccall((:fit_mode_to_mode, LIB), Cint,
        (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cint, Cint, Ptr{Float64}, Ptr{Float64}, Cint),
        p.ptr, û, _advptr(advecting_hat, velocity_hat), _inv(invariant), sp.precision === :fp32 ? Cint(0) : Cint(1),
        S, net, 0))
    FT = real(eltype(û))
    return ModeToModeTriadResult(invariant, ks, FT.(net), FT.(S))
end

function FET.BandTransfer.calculate_band_to_band_transfer(velocity_hat::GB300Array, ks; bands::SmoothBands,
        dealiasing=OrszagTwoThirds(), invariant=KineticEnergy(), spectral=velocity_hat.spectral,
        advecting_hat=velocity_hat, geometry=IsotropicShells())
    û = velocity_hat.data
    p = _plan(velocity_hat, ks, dealiasing, spectral isa GB300Spectral ? spectral : velocity_hat.spectral;
              advecting=advecting_hat)
    centers = Vector{Float64}(bands.centers)
    nb = length(centers)
    T = Matrix{Float64}(undef, nb, nb)
    net = Vector{Float64}(undef, nb)
    asym = Ref{Float64}(NaN)
    p.idx = nothing   # the band form sets its own (single-shell) table
    _check(ccall((:fit_band_to_band, LIB), Cint,
        (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Float64}, Cint, Cdouble, UInt32, Cint, Cint, Ptr{Float64},
         Ptr{Float64}, Ptr{Float64}, Cint),
        p.ptr, û, _advptr(advecting_hat, velocity_hat), centers, nb, Float64(bands.logwidth),
        _dims_mask(geometry, length(ks)), _coord32(ks), _inv(invariant), T, net, asym, 0))
    FT = real(eltype(û))
    return (centers = collect(bands.centers), transfer_matrix = FT.(T), net_transfer = FT.(net),
            max_antisymmetry_error = FT(asym[]))
end

end # module
