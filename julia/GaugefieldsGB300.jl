"""
    GaugefieldsGB300

A Gaugefields.jl backend whose SU(3) gauge-link hot path runs in
`libgfgb300.so` (C-ABI, `include/gaugefields_gb300.h`) on one GB300: the
plaquette, the Wilson-action MD force and the momentum/link updates, the
QPQ/PQP trajectory, stout smearing forward and adjoint, and the RK3 Wilson
flow. The reference's driver code (`md_driver`, `md_trajectory!`, custom
`md_step!` integrators, `CovNeuralnet`, `back_prop`) is kept; the methods
below are found by dispatch on the backend's field types.

Usage:

    using Gaugefields, GaugefieldsGB300
    U = gauge_configuration((32, 32, 32, 32), GB300Backend(); start=:hot, seed=7)
    P = gauge_momenta(U)
    action = GaugeAction(U); push!(action, 3.0, make_loops_fromname("plaquette"))
    driver = md_driver(U, action; steps=20, trajectory_length=1.0)
    gaussian_momenta!(P; seed=1234, sweep=0)
    md_trajectory!(U, P, driver)

`U` is a `Vector` of four `Gaugefields_4D_GB300`, one per direction, as the
reference's configurations are; all four share one device field (the
library's even/odd structure-of-arrays layout), so a call that takes the
whole configuration (`U[1].field`) acts on every direction at once.

Smeared-link HMC goes through an MD action provider (the reference's v1
interface, `src/molecular_dynamics.jl:1-50`): `StoutWilsonAction_GB300`
carries the Wilson coupling, the stout levels and the precision form.

Not run in this repository's environment (no Julia toolchain): the ccall
signatures follow the C header, and a test checks the `gf_md_params` mirror
below against it.
"""
module GaugefieldsGB300

using LinearAlgebra
using Gaugefields
import Gaugefields: md_action_workspace, md_potential, md_force!, md_hamiltonian, update_momenta!,
                    update_gaugefields!, md_trajectory!, md_step!, gauge_configuration, gaussian_momenta!,
                    calculate_Plaquette, substitute_U!, clear_U!, initialize_TA_Gaugefields, back_prop,
                    copy_configuration!, copy_configuration, calculate_Polyakov_loop, save_configuration,
                    load_configuration!
import Gaugefields.AbstractGaugefields_module: Gaugefields_4D, TA_Gaugefields_4D
import Gaugefields.Abstractsmearing_module: CovLayer, apply_layer!, layer_pullback!, parameter_derivatives
import Gaugefields.Gradientflow_module: Gradientflow, flow!

export GB300Backend, Gaugefields_4D_GB300, TA_Gaugefields_4D_GB300, StoutWilsonAction_GB300, host_configuration,
       upload_host!,
       STOUT_Layer_GB300, smear_gb300, GF_FP64, GF_MIXED, GF_DFLOAT

const libgf = get(ENV, "GF_GB300_LIB", joinpath(@__DIR__, "..", "gaugefields.jl_gb300", "libgfgb300.so"))

# field kinds, precision forms, integrators, status codes (include/gaugefields_gb300.h)
const GF_LINK64, GF_LINK32, GF_MOM64, GF_MAT64, GF_MAT32 = 1, 2, 3, 4, 5
const GF_FP64, GF_MIXED, GF_DFLOAT = 0, 1, 2
const GF_QPQ, GF_PQP, GF_OMELYAN = 0, 1, 2
const GF_EINVAL = -1
const GF_MAX_STOUT = 4

"""
    GB300MDParams

Mirror of `gf_md_params`: the same field order and C types (a test compares
it with the header).
"""
struct GB300MDParams
    beta::Cdouble
    tau::Cdouble
    steps::Cint
    integrator::Cint
    precision::Cint
    nstout::Cint
    rho::NTuple{4,Cdouble}
    reunitarize::Cint
    stout_recompute::Cint
    lambda::Cdouble
    c_rect::Cdouble
end

# ---------------------------------------------------------------------------
# context, errors
# ---------------------------------------------------------------------------
struct GB300Backend <: Gaugefields.AbstractGaugeBackend
    device::Int
end
GB300Backend() = GB300Backend(0)

mutable struct Ctx
    h::Ptr{Cvoid}
    L::NTuple{4,Int}
    device::Int
end

last_error(h::Ptr{Cvoid}) = unsafe_string(ccall((:gf_last_error, libgf), Cstring, (Ptr{Cvoid},), h))

# Non-zero status -> the reference's exceptions: ArgumentError for invalid
# arguments (GF_EINVAL, as the reference validates with ArgumentError),
# ErrorException otherwise.
function check(rc::Integer, ctx::Union{Ctx,Nothing}=nothing)
    rc == 0 && return nothing
    msg = last_error(ctx === nothing ? C_NULL : ctx.h)
    rc == GF_EINVAL ? throw(ArgumentError(msg)) : error(msg)
end

function Ctx(L::NTuple{4,Int}, device::Int)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:gf_ctx_create, libgf), Cint, (Ptr{Cint}, Cint, Ref{Ptr{Cvoid}}), Cint[L...], device, h))
    c = Ctx(h[], L, device)
    finalizer(x -> ccall((:gf_ctx_destroy, libgf), Cint, (Ptr{Cvoid},), x.h), c)
    return c
end

# One device field with its owner context (freed by the finalizer).
mutable struct DeviceField
    ctx::Ctx
    h::Ptr{Cvoid}
    kind::Int
end

function DeviceField(ctx::Ctx, kind::Integer)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:gf_field_alloc, libgf), Cint, (Ptr{Cvoid}, Cint, Ref{Ptr{Cvoid}}), ctx.h, kind, h), ctx)
    f = DeviceField(ctx, h[], Int(kind))
    finalizer(x -> ccall((:gf_field_free, libgf), Cint, (Ptr{Cvoid},), x.h), f)
    return f
end

# ---------------------------------------------------------------------------
# field types: one wrapper per direction over a shared four-direction field
# ---------------------------------------------------------------------------
"""
    Gaugefields_4D_GB300 <: Gaugefields_4D{3}

Direction `mu` of a four-direction SU(3) link field on the device. The
reference keeps `U::Vector` of four fields (`src/4D/gaugefields_4D.jl:10`);
here the four wrappers of a configuration share one `GF_LINK64` field.
`similar` gives a wrapper whose storage is allocated on first use (the MD
driver's own temporaries are never touched by the fused kernels).
"""
mutable struct Gaugefields_4D_GB300 <: Gaugefields_4D{3}
    ctx::Ctx
    field::Union{DeviceField,Nothing}
    mu::Int
    NC::Int
    NX::Int
    NY::Int
    NZ::Int
    NT::Int
    NV::Int
end

"""
    TA_Gaugefields_4D_GB300 <: TA_Gaugefields_4D{3}

Direction `mu` of the su(3) momenta (8 fp64 coefficients per link, the
reference's order) over a shared `GF_MOM64` field.
"""
mutable struct TA_Gaugefields_4D_GB300 <: TA_Gaugefields_4D{3}
    ctx::Ctx
    field::DeviceField
    mu::Int
    NC::Int
    NV::Int
end

const GB300Config = AbstractVector{<:Gaugefields_4D_GB300}
const GB300Momenta = AbstractVector{<:TA_Gaugefields_4D_GB300}

function links(ctx::Ctx, field)
    NX, NY, NZ, NT = ctx.L
    return [Gaugefields_4D_GB300(ctx, field, mu, 3, NX, NY, NZ, NT, NX * NY * NZ * NT) for mu in 1:4]
end

function storage(u::Gaugefields_4D_GB300)
    if u.field === nothing
        u.field = DeviceField(u.ctx, GF_LINK64)
    end
    return u.field
end

# the shared device field of a configuration or of momenta
function config_field(U::GB300Config)
    length(U) == 4 || throw(ArgumentError("the gauge configuration has length $(length(U)); expected 4"))
    f = storage(U[1])
    all(u -> u.field === f && u.mu == findfirst(==(u), U), U) ||
        throw(ArgumentError("the four directions must be the views of one GB300 configuration"))
    return f
end
function momenta_field(P::GB300Momenta)
    length(P) == 4 || throw(ArgumentError("the momenta have length $(length(P)); expected 4"))
    f = P[1].field
    all(p -> p.field === f, P) || throw(ArgumentError("the four directions must share one GB300 momentum field"))
    return f
end

# the reference's configuration accessors (src/API.jl:262-295): the size of a
# direction as (NC, NC, NX, NY, NZ, NT), no halo (neighbours come from index
# arithmetic), one process
Base.size(u::Gaugefields_4D_GB300) = (u.NC, u.NC, u.NX, u.NY, u.NZ, u.NT)
Gaugefields.gauge_backend(u::Gaugefields_4D_GB300) = GB300Backend(u.ctx.device)
Gaugefields.gauge_halo_width(::Gaugefields_4D_GB300) = 0
# no halo to refresh (set_wing_U!, src/AbstractGaugefields.jl): a no-op
Gaugefields.set_wing_U!(::Gaugefields_4D_GB300) = nothing
Gaugefields.set_wing_U!(::GB300Config) = nothing

Base.similar(u::Gaugefields_4D_GB300) =
    Gaugefields_4D_GB300(u.ctx, nothing, u.mu, u.NC, u.NX, u.NY, u.NZ, u.NT, u.NV)
Base.similar(U::Vector{<:Gaugefields_4D_GB300}) = links(U[1].ctx, DeviceField(U[1].ctx, GF_LINK64))

function initialize_TA_Gaugefields(U::GB300Config)
    ctx = U[1].ctx
    f = DeviceField(ctx, GF_MOM64)
    check(ccall((:gf_field_zero, libgf), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), ctx.h, f.h), ctx)
    return [TA_Gaugefields_4D_GB300(ctx, f, mu, 3, U[1].NV) for mu in 1:4]
end
initialize_TA_Gaugefields(u::Gaugefields_4D_GB300) = initialize_TA_Gaugefields(links(u.ctx, storage(u)))

function substitute_U!(A::GB300Config, B::GB300Config)
    ctx = A[1].ctx
    check(ccall((:gf_field_copy, libgf), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}), ctx.h, config_field(A).h,
                config_field(B).h), ctx)
    return A
end
# copy_configuration!(destination, source) / copy_configuration(source)
# (src/API.jl:300-328): one device copy of the shared four-direction field
function copy_configuration!(destination::GB300Config, source::GB300Config)
    length(destination) == length(source) ||
        throw(DimensionMismatch("destination and source have different numbers of directions"))
    destination[1].ctx.L == source[1].ctx.L || throw(DimensionMismatch("destination and source lattice sizes differ"))
    if destination[1].ctx === source[1].ctx
        substitute_U!(destination, source)
    else
        upload!(destination, download(source))
    end
    return destination
end
copy_configuration(source::GB300Config) = copy_configuration!(similar(source), source)

function clear_U!(P::GB300Momenta)
    ctx = P[1].ctx
    check(ccall((:gf_field_zero, libgf), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), ctx.h, momenta_field(P).h), ctx)
    return P
end

# ---------------------------------------------------------------------------
# gauge_configuration with the backend as a positional selector
# ---------------------------------------------------------------------------
"""
    gauge_configuration(lattice::NTuple{4,<:Integer}, backend::GB300Backend;
                        colors=3, start=:cold, seed=nothing)

The reference's `gauge_configuration(lattice; backend=...)` (`src/API.jl:
178-251`) chooses between its own backends inside one method, so this
backend adds a method with the backend as a second positional argument
instead of redefining the keyword method. Validation follows the
reference's (`ArgumentError` texts of `_validate_lattice_size` and of the
`start` check); SU(3) only, extents even.
"""
function gauge_configuration(lattice::NTuple{4,<:Integer}, backend::GB300Backend; colors::Integer=3,
                             start::Symbol=:cold, seed=nothing)
    all(>(0), lattice) || throw(ArgumentError("all lattice extents must be positive; got $lattice"))
    colors == 3 || throw(ArgumentError("the GB300 backend implements SU(3); got colors=$colors"))
    start in (:cold, :hot) || throw(ArgumentError("start must be :cold or :hot; got $start"))
    L = ntuple(i -> Int(lattice[i]), 4)
    ctx = Ctx(L, backend.device)
    f = DeviceField(ctx, GF_LINK64)
    if start == :cold
        check(ccall((:gf_cold_start, libgf), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), ctx.h, f.h), ctx)
    else
        s = seed === nothing ? rand(UInt64) : UInt64(seed)
        check(ccall((:gf_hot_start, libgf), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, UInt64), ctx.h, f.h, s), ctx)
    end
    return links(ctx, f)
end

"""
    gaussian_momenta!(P::Vector{<:TA_Gaugefields_4D_GB300}; sigma=1, seed, sweep=0)

`gaussian_momenta!` (`src/API.jl:341-368`): p_a ~ N(0, sigma^2) from the
counter-based generator keyed by (seed, sweep).
"""
function gaussian_momenta!(P::GB300Momenta; sigma=1, seed=nothing, sweep=0, kwargs...)
    ctx = P[1].ctx
    f = momenta_field(P)
    s = seed === nothing ? rand(UInt64) : UInt64(seed)
    check(ccall((:gf_gaussian_momenta, libgf), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, UInt64, UInt64), ctx.h, f.h, s,
                UInt64(sweep)), ctx)
    if sigma != 1
        check(ccall((:gf_mom_scale, libgf), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Cdouble), ctx.h, f.h, sigma), ctx)
    end
    return P
end

# ---------------------------------------------------------------------------
# measurements and host transfer
# ---------------------------------------------------------------------------
"""
    calculate_Plaquette(U::Vector{<:Gaugefields_4D_GB300}, temp, staple)

`calculate_Plaquette` (`src/AbstractGaugefields.jl:2684-2699`): the sum over
sites and planes of Re tr P, deterministic (fixed-order fp64 reduction).
"""
function calculate_Plaquette(U::GB300Config, temp=nothing, staple=nothing)
    ctx = U[1].ctx
    out = Ref{Cdouble}(0)
    check(ccall((:gf_plaquette, libgf), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ref{Cdouble}), ctx.h, config_field(U).h, out),
          ctx)
    return out[]
end

"""
    calculate_Polyakov_loop(U::Vector{<:Gaugefields_4D_GB300}, temp1, temp2)

`calculate_Polyakov_loop` (`src/AbstractGaugefields.jl:2929-2956`): the mean
over the first time slice of tr of the product of the time links (complex);
`measure_polyakov_loop` divides it by 3. Deterministic.
"""
function calculate_Polyakov_loop(U::GB300Config, temp1=nothing, temp2=nothing)
    ctx = U[1].ctx
    out = zeros(Cdouble, 2)
    check(ccall((:gf_polyakov_loop, libgf), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cdouble}), ctx.h, config_field(U).h,
                out), ctx)
    return complex(out[1], out[2])
end

"""
    download(U) -> Array{ComplexF64,6}, upload!(U, A)

The configuration in the reference layout `(3, 3, NX, NY, NZ, NT)` per
direction (stacked along a last dimension of 4); exact round trip.
"""
function download(U::GB300Config)
    ctx = U[1].ctx
    A = Array{ComplexF64}(undef, 3, 3, ctx.L..., 4)
    GC.@preserve A check(ccall((:gf_download_links, libgf), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{ComplexF64}), ctx.h,
                                config_field(U).h, A), ctx)
    return A
end
function upload!(U::GB300Config, A::Array{ComplexF64})
    ctx = U[1].ctx
    size(A) == (3, 3, ctx.L..., 4) || throw(ArgumentError("expected an array of size $((3, 3, ctx.L..., 4))"))
    GC.@preserve A check(ccall((:gf_upload_links, libgf), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{ComplexF64}), ctx.h,
                                config_field(U).h, A), ctx)
    return U
end

# ---------------------------------------------------------------------------
# configuration files through the reference's own readers and writers
# ---------------------------------------------------------------------------
"""
    host_configuration(U::Vector{<:Gaugefields_4D_GB300}) -> host configuration

The configuration as the reference's own host fields (`LegacyBackend`,
`src/API.jl:178-251`), one download: for the reference's configuration
writers and any host-side analysis. `upload_host!(U, H)` copies host fields
back.
"""
function host_configuration(U::GB300Config)
    A = download(U)
    NX, NY, NZ, NT = U[1].ctx.L
    H = gauge_configuration((NX, NY, NZ, NT); backend=Gaugefields.LegacyBackend(), start=:cold)
    for mu in 1:4, it in 1:NT, iz in 1:NZ, iy in 1:NY, ix in 1:NX, b in 1:3, a in 1:3
        H[mu][a, b, ix, iy, iz, it] = A[a, b, ix, iy, iz, it, mu]
    end
    Gaugefields.set_wing_U!(H)
    return H
end

function upload_host!(U::GB300Config, H)
    NX, NY, NZ, NT = U[1].ctx.L
    length(H) == 4 || throw(ArgumentError("the host configuration has length $(length(H)); expected 4"))
    A = Array{ComplexF64}(undef, 3, 3, NX, NY, NZ, NT, 4)
    for mu in 1:4, it in 1:NT, iz in 1:NZ, iy in 1:NY, ix in 1:NX, b in 1:3, a in 1:3
        A[a, b, ix, iy, iz, it, mu] = H[mu][a, b, ix, iy, iz, it]
    end
    return upload!(U, A)
end

"""
    save_configuration(filename, U::Vector{<:Gaugefields_4D_GB300}; format=:jld2, kwargs...)
    load_configuration!(U::Vector{<:Gaugefields_4D_GB300}, filename; format=:jld2)

`save_configuration` / `load_configuration!` (`src/API.jl:711-826`) for
device configurations: the reference's own writers and readers (portable
JLD2, ILDG, Bridge++) run on a host copy (`host_configuration`), so the files
are the reference's byte for byte.
"""
save_configuration(filename, U::GB300Config; kwargs...) = save_configuration(filename, host_configuration(U); kwargs...)

function load_configuration!(U::GB300Config, filename; format::Symbol=:jld2)
    H = host_configuration(U)
    load_configuration!(H, filename; format)
    upload_host!(U, H)
    return U
end

# ---------------------------------------------------------------------------
# MD action providers (src/molecular_dynamics.jl:1-50, 238-276)
# ---------------------------------------------------------------------------
# Plaquette and rectangle coefficients of a GaugeAction: loops of 4 links are
# plaquettes, of 6 links rectangles; the backend takes real coefficients.
function loop_coefficients(action::Gaugefields.GaugeAction)
    cp, cr = 0.0, 0.0
    for d in action.dataset
        isreal(d.β) || throw(ArgumentError("the GB300 backend takes real loop coefficients; got $(d.β)"))
        n = length(d.closedloops[1])
        if n == 4
            cp += real(d.β)
        elseif n == 6
            cr += real(d.β)
        else
            throw(ArgumentError("the GB300 backend supports plaquette and rectangle loops; got loops of $n links"))
        end
    end
    return cp, cr
end

"""
    StoutWilsonAction_GB300(beta, rho; precision=GF_DFLOAT, recompute=false, c_rect=0.0)

An MD action provider: the Wilson action `push!(action, beta/2, plaq ∪ plaq')`
(with `c_rect` ≠ 0 also `push!(action, c_rect, rect ∪ rect')`, e.g. Iwasaki)
evaluated on `length(rho)` plaquette stout levels of the thin links. The
force runs the hand-written stout adjoint on the device. `precision` selects
the plain fp64 form (`GF_FP64`), the double-float form (`GF_DFLOAT`, Delta H
within ~1e-7 of fp64 at 32^4) or the mixed fp32-force form (`GF_MIXED`).
"""
struct StoutWilsonAction_GB300
    beta::Float64
    rho::Vector{Float64}
    precision::Int
    recompute::Bool
    c_rect::Float64
end
function StoutWilsonAction_GB300(beta::Real, rho; precision::Integer=GF_DFLOAT, recompute::Bool=false,
                                 c_rect::Real=0.0)
    r = collect(Float64, rho)
    1 <= length(r) <= GF_MAX_STOUT || throw(ArgumentError("1..$GF_MAX_STOUT stout levels are supported"))
    precision in (GF_FP64, GF_MIXED, GF_DFLOAT) || throw(ArgumentError("precision must be GF_FP64, GF_MIXED or GF_DFLOAT"))
    isfinite(c_rect) || throw(ArgumentError("c_rect must be finite"))
    return StoutWilsonAction_GB300(Float64(beta), r, Int(precision), recompute, Float64(c_rect))
end

# The workspace of every GB300 provider: the gf_md_params of its action and
# zero momenta (the potential is the Hamiltonian at P = 0).
struct GB300Workspace{P}
    params::GB300MDParams
    zero_momenta::P
end

function action_params(action::Gaugefields.GaugeAction; precision=GF_FP64)
    cp, cr = loop_coefficients(action)
    return GB300MDParams(2cp, 1.0, 1, GF_QPQ, precision, 0, (0.0, 0.0, 0.0, 0.0), 1, 0, 0.0, cr)
end
function action_params(action::StoutWilsonAction_GB300)
    rho = ntuple(i -> i <= length(action.rho) ? action.rho[i] : 0.0, 4)
    return GB300MDParams(action.beta, 1.0, 1, GF_QPQ, action.precision, length(action.rho), rho, 1,
                         action.recompute ? 1 : 0, 0.0, action.c_rect)
end

md_action_workspace(action::Gaugefields.GaugeAction, U::GB300Config) =
    GB300Workspace(action_params(action), initialize_TA_Gaugefields(U))
md_action_workspace(action::StoutWilsonAction_GB300, U::GB300Config) =
    GB300Workspace(action_params(action), initialize_TA_Gaugefields(U))

function md_potential(action::Union{Gaugefields.GaugeAction,StoutWilsonAction_GB300}, U::GB300Config,
                      ws::GB300Workspace)
    ctx = U[1].ctx
    out = Ref{Cdouble}(0)
    check(ccall((:gf_hamiltonian, libgf), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ref{GB300MDParams}, Ref{Cdouble}),
                ctx.h, config_field(U).h, momenta_field(ws.zero_momenta).h, Ref(ws.params), out), ctx)
    return out[]
end

"""
    md_force!(F, action, U, ws)

`md_force!` (`src/molecular_dynamics.jl:251-267`): F_mu = -(1/3) TA(U_mu dS/dU_mu)
for a plaquette + rectangle GaugeAction, or through the stout adjoint for a
`StoutWilsonAction_GB300`: the force is F = 0 advanced by one unit step,
one fused device pass.
"""
function md_force!(F::GB300Momenta, action::Union{Gaugefields.GaugeAction,StoutWilsonAction_GB300},
                   U::GB300Config, ws::GB300Workspace)
    length(F) == length(U) || throw(ArgumentError("force and U must have the same number of directions"))
    clear_U!(F)
    ctx = U[1].ctx
    check(ccall((:gf_md_mom_update, libgf), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cdouble, Ref{GB300MDParams}),
                ctx.h, momenta_field(F).h, config_field(U).h, 1.0, Ref(ws.params)), ctx)
    return nothing
end

# ---------------------------------------------------------------------------
# the MD driver's steps (src/molecular_dynamics.jl:494-730), typed on MDDriver
# ---------------------------------------------------------------------------
# The driver's gf_md_params: the action's, with the driver's trajectory.
function driver_params(driver::Gaugefields.MDDriver)
    p = driver.action_workspace isa GB300Workspace ? driver.action_workspace.params :
        throw(ArgumentError("the driver's action has no GB300 provider"))
    integ = driver.integrator isa Gaugefields.PQP ? GF_PQP : GF_QPQ
    return GB300MDParams(p.beta, driver.trajectory_length, driver.steps, integ, p.precision, p.nstout, p.rho,
                         p.reunitarize, p.stout_recompute, p.lambda, p.c_rect)
end

function md_hamiltonian(U::GB300Config, P::GB300Momenta, driver::Gaugefields.MDDriver)
    length(U) == length(P) || throw(ArgumentError("U and p must have the same number of directions"))
    ctx = U[1].ctx
    out = Ref{Cdouble}(0)
    check(ccall((:gf_hamiltonian, libgf), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ref{GB300MDParams}, Ref{Cdouble}),
                ctx.h, config_field(U).h, momenta_field(P).h, Ref(driver_params(driver)), out), ctx)
    return out[]
end

"""
    update_momenta!(P, U, step_size, driver::MDDriver)

`update_momenta!` (`src/molecular_dynamics.jl:539-551`): P += step_size * F(U)
with the driver's action, smearing and precision, fused in one device pass.
"""
function update_momenta!(P::GB300Momenta, U::GB300Config, step_size, driver::Gaugefields.MDDriver)
    length(P) == length(U) || throw(ArgumentError("P and U must have the same number of directions"))
    isfinite(step_size) || throw(ArgumentError("the momentum step size must be finite; got $step_size"))
    ctx = U[1].ctx
    check(ccall((:gf_md_mom_update, libgf), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cdouble, Ref{GB300MDParams}),
                ctx.h, momenta_field(P).h, config_field(U).h, step_size, Ref(driver_params(driver))), ctx)
    return P
end

"""
    update_momenta!(P, U, step_size, driver::MDDriver, group::MDForceGroup)

The elementary kick of `SextonWeingarten` (`src/molecular_dynamics.jl:
553-584`): the selected members of the driver's `MDActionSet` are Wilson
(plaquette + rectangle) actions, whose force is linear in the coefficients,
so the kick is one fused pass with the summed coefficients.
"""
function update_momenta!(P::GB300Momenta, U::GB300Config, step_size, driver::Gaugefields.MDDriver,
                         ::Gaugefields.MDForceGroup{Names}) where {Names}
    length(P) == length(U) || throw(ArgumentError("P and U must have the same number of directions"))
    isfinite(step_size) || throw(ArgumentError("the momentum step size must be finite; got $step_size"))
    cp, cr = 0.0, 0.0
    for name in Names
        a, b = loop_coefficients(getproperty(driver.action.terms, name))
        cp += a
        cr += b
    end
    p = driver_params(driver)
    q = GB300MDParams(2cp, p.tau, p.steps, p.integrator, p.precision, p.nstout, p.rho, p.reunitarize,
                      p.stout_recompute, p.lambda, cr)
    ctx = U[1].ctx
    check(ccall((:gf_md_mom_update, libgf), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cdouble, Ref{GB300MDParams}),
                ctx.h, momenta_field(P).h, config_field(U).h, step_size, Ref(q)), ctx)
    return P
end

# An MDActionSet of GaugeActions: the workspace is the summed action's.
function md_action_workspace(actions::Gaugefields.MDActionSet, U::GB300Config)
    cp, cr = 0.0, 0.0
    for a in values(actions.terms)
        x, y = loop_coefficients(a)
        cp += x
        cr += y
    end
    return GB300Workspace(GB300MDParams(2cp, 1.0, 1, GF_QPQ, GF_FP64, 0, (0.0, 0.0, 0.0, 0.0), 1, 0, 0.0, cr),
                          initialize_TA_Gaugefields(U))
end

"""
    update_gaugefields!(U, P, step_size, driver::MDDriver)

`update_gaugefields!` (`src/molecular_dynamics.jl:513-531`):
U_mu <- exp(step_size P_mu) U_mu (Cayley-Hamilton), re-unitarised.
"""
function update_gaugefields!(U::GB300Config, P::GB300Momenta, step_size, driver::Gaugefields.MDDriver)
    length(U) == length(P) || throw(ArgumentError("U and P must have the same number of directions"))
    isfinite(step_size) || throw(ArgumentError("the gauge-field step size must be finite; got $step_size"))
    ctx = U[1].ctx
    check(ccall((:gf_md_link_update, libgf), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cdouble, Ref{GB300MDParams}),
                ctx.h, config_field(U).h, momenta_field(P).h, step_size, Ref(driver_params(driver))), ctx)
    return U
end

"""
    md_trajectory!(U, P, driver::MDDriver; diagnostics=true)

`md_trajectory!` (`src/molecular_dynamics.jl:712-730`). `QPQ()` and `PQP()`
run as one native call (adjacent half link steps merged, as the reference's
`_md_fast_qpq!`); any other integrator steps through `md_step!`, which
dispatches to the methods above.
"""
function md_trajectory!(U::GB300Config, P::GB300Momenta, driver::Gaugefields.MDDriver; diagnostics::Bool=true)
    length(U) == length(P) || throw(ArgumentError("U and P must have the same number of directions"))
    if !(driver.integrator isa Union{Gaugefields.QPQ,Gaugefields.PQP})
        return invoke(md_trajectory!, Tuple{Any,Any,Gaugefields.MDDriver}, U, P, driver; diagnostics)
    end
    ctx = U[1].ctx
    out = zeros(Cdouble, 3)
    check(ccall((:gf_md_trajectory, libgf), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ref{GB300MDParams}, Ptr{Cdouble}),
                ctx.h, config_field(U).h, momenta_field(P).h, Ref(driver_params(driver)), out), ctx)
    diagnostics || return nothing
    return (initial_hamiltonian=out[1], final_hamiltonian=out[2], delta_hamiltonian=out[3])
end

# ---------------------------------------------------------------------------
# gradient flow (src/smearing/gradientflow.jl:171-238)
# ---------------------------------------------------------------------------
# precision = GF_DFLOAT runs the force and the exponentials in double-float
# arithmetic on the fp32 pipes (the fields stay fp64); GF_FP64 is the
# reference's arithmetic
function flow!(U::GB300Config, g::Gradientflow; precision::Integer=GF_FP64)
    ctx = U[1].ctx
    check(ccall((:gf_flow_precision, libgf), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Cdouble, Cint, Cint), ctx.h,
                config_field(U).h, g.eps, g.Nflow, precision), ctx)
    return U
end

# ---------------------------------------------------------------------------
# stout smearing as a CovLayer (src/smearing/Abstractsmearing.jl:488-509)
# ---------------------------------------------------------------------------
"""
    STOUT_Layer_GB300(U, rho; precision=GF_FP64)

A plaquette stout layer on the device, a `CovLayer{4}`, so `CovNeuralnet`,
`calc_smearedU`, `back_prop` and `get_parameter_derivatives` work unchanged:
`apply_layer!` runs the forward level (`gf_stout_forward`),
`layer_pullback!` the adjoint (`gf_stout_backward`, the hand-written
Lambda-matrix recursion of `backward_dSdUαUβρ_add!`, `src/smearing/
stout_fast.jl:317-408`) and `parameter_derivatives` returns dS/drho
(`gf_stout_param_derivatives`). Derivative fields are `GF_MAT64` views
(`Gaugefields_4D_GB300` wrappers whose shared field holds general 3x3 matrices).
"""
mutable struct STOUT_Layer_GB300 <: CovLayer{4}
    ctx::Ctx
    h::Ptr{Cvoid}
    rho::Vector{Float64}
    dSdrho::Vector{Float64}
end

function STOUT_Layer_GB300(U::GB300Config, rho::Real; precision::Integer=GF_FP64)
    ctx = U[1].ctx
    h = Ref{Ptr{Cvoid}}(C_NULL)
    r = Cdouble[rho]
    check(ccall((:gf_stout_create, libgf), Cint, (Ptr{Cvoid}, Cint, Ptr{Cdouble}, Cint, Cint, Ref{Ptr{Cvoid}}),
                ctx.h, 1, r, precision, 1, h), ctx)
    layer = STOUT_Layer_GB300(ctx, h[], Float64[rho], [0.0])
    finalizer(x -> ccall((:gf_stout_destroy, libgf), Cint, (Ptr{Cvoid},), x.h), layer)
    return layer
end

Gaugefields.Abstractsmearing_module.get_name(::STOUT_Layer_GB300) = "STOUT_GB300"
Gaugefields.Abstractsmearing_module.get_parameters(l::STOUT_Layer_GB300) = copy(l.rho)
Gaugefields.Abstractsmearing_module.get_parameter_derivatives(l::STOUT_Layer_GB300) = copy(l.dSdrho)
Gaugefields.Abstractsmearing_module.zero_grad!(l::STOUT_Layer_GB300) = (l.dSdrho .= 0; l)

function apply_layer!(Uout::GB300Config, layer::STOUT_Layer_GB300, Uin::GB300Config, temps, temps_F)
    check(ccall((:gf_stout_forward, libgf), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}),
                layer.ctx.h, layer.h, config_field(Uin).h, config_field(Uout).h), layer.ctx)
    return Uout
end

# dS/dU of the layer's input from dS/dUbar; the forward state of the layer
# is the one of the last apply_layer! (CovNeuralnet applies, then pulls back
# in reverse order; a layer's state is recomputed when its input changed).
function layer_pullback!(δ_prev::GB300Config, δ_next::GB300Config, layer::STOUT_Layer_GB300, Uprev::GB300Config,
                         temps, tempf)
    ctx = layer.ctx
    check(ccall((:gf_stout_forward, libgf), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}), ctx.h, layer.h,
                config_field(Uprev).h, C_NULL), ctx)
    check(ccall((:gf_stout_backward, libgf), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}), ctx.h, layer.h,
                config_field(δ_next).h, config_field(δ_prev).h), ctx)
    return δ_prev
end

"""
    parameter_derivatives(δ_current, layer::STOUT_Layer_GB300, U_current, temps)

dS/drho of the layer (`parameter_derivatives`, `src/smearing/
Abstractsmearing.jl:505`): 2 Re sum tr(Σ' dUbar/drho) with Σ' = δ_current,
the derivative with respect to the layer's output, on the layer's input
`U_current`. Accumulated into the layer's gradient and returned.
"""
function parameter_derivatives(δ_current::GB300Config, layer::STOUT_Layer_GB300, U_current::GB300Config, temps)
    ctx = layer.ctx
    out = zeros(Cdouble, 1)
    check(ccall((:gf_stout_param_derivatives, libgf), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cdouble}),
                ctx.h, layer.h, config_field(U_current).h, config_field(δ_current).h, out), ctx)
    layer.dSdrho[1] += out[1]
    return out
end

# ---------------------------------------------------------------------------
# automatic differentiation: the hand-written adjoint as the rule of smear
# ---------------------------------------------------------------------------
"""
    smear_gb300(U, rho; precision=GF_FP64) -> Ubar

A stout stack of `length(rho)` levels applied to `U` (a new configuration).
Its differentiation rules (a ChainRulesCore `rrule` and an Enzyme
`augmented_primal`/`reverse` pair, defined when those packages are loaded)
call the device adjoint instead of differentiating the lattice loops: the
pullback of a cotangent dS/dUbar is dS/dU of `gf_stout_backward`, with the
smeared levels either stored by the forward pass or recomputed from the thin
links (`recompute=true`). This replaces Enzyme's sweep over the lattice
kernels (`ext/GaugefieldsEnzymeExt.jl:115-150`).
"""
mutable struct GB300StoutStack
    ctx::Ctx
    h::Ptr{Cvoid}
end

function GB300StoutStack(ctx::Ctx, rho; precision::Integer=GF_FP64, recompute::Bool=false)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    r = collect(Cdouble, rho)
    check(ccall((:gf_stout_create, libgf), Cint, (Ptr{Cvoid}, Cint, Ptr{Cdouble}, Cint, Cint, Ref{Ptr{Cvoid}}),
                ctx.h, length(r), r, precision, recompute ? 0 : 1, h), ctx)
    s = GB300StoutStack(ctx, h[])
    finalizer(x -> ccall((:gf_stout_destroy, libgf), Cint, (Ptr{Cvoid},), x.h), s)
    return s
end

function smear_forward(U::GB300Config, stack::GB300StoutStack)
    Ubar = similar(U)
    check(ccall((:gf_stout_forward, libgf), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}), stack.ctx.h,
                stack.h, config_field(U).h, config_field(Ubar).h), stack.ctx)
    return Ubar
end

function smear_pullback(stack::GB300StoutStack, dUbar::GB300Config)
    ctx = stack.ctx
    dU = links(ctx, DeviceField(ctx, GF_MAT64))
    check(ccall((:gf_stout_backward, libgf), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}), ctx.h, stack.h,
                config_field(dUbar).h, config_field(dU).h), ctx)
    return dU
end

smear_gb300(U::GB300Config, rho; precision::Integer=GF_FP64, recompute::Bool=false) =
    smear_forward(U, GB300StoutStack(U[1].ctx, rho; precision, recompute))

# ChainRulesCore and EnzymeRules are weak dependencies: the rules are defined
# only where the packages are loaded (ChainRulesCore is absent from the
# reference's Project.toml).
function __init__()
    if isdefined(Main, :ChainRulesCore)
        @eval begin
            import ChainRulesCore
            function ChainRulesCore.rrule(::typeof(smear_gb300), U::GB300Config, rho; precision::Integer=GF_FP64,
                                          recompute::Bool=false)
                stack = GB300StoutStack(U[1].ctx, rho; precision, recompute)
                Ubar = smear_forward(U, stack)
                function smear_gb300_pullback(dUbar)
                    dU = smear_pullback(stack, ChainRulesCore.unthunk(dUbar))
                    return (ChainRulesCore.NoTangent(), dU, ChainRulesCore.NoTangent())
                end
                return Ubar, smear_gb300_pullback
            end
        end
    end
    if isdefined(Main, :EnzymeRules) || isdefined(Main, :Enzyme)
        @eval begin
            import Enzyme
            import Enzyme.EnzymeRules
            # augmented primal: run the forward pass and keep the stack (its
            # levels and C matrices) as the tape
            function EnzymeRules.augmented_primal(config, func::Enzyme.Const{typeof(smear_gb300)}, ::Type{RT},
                                                  U::Enzyme.Duplicated, rho::Enzyme.Const) where {RT}
                stack = GB300StoutStack(U.val[1].ctx, rho.val)
                Ubar = smear_forward(U.val, stack)
                dUbar = links(U.val[1].ctx, DeviceField(U.val[1].ctx, GF_MAT64))
                check(ccall((:gf_field_zero, libgf), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), stack.ctx.h,
                            config_field(dUbar).h), stack.ctx)
                primal = EnzymeRules.needs_primal(config) ? Ubar : nothing
                shadow = EnzymeRules.needs_shadow(config) ? dUbar : nothing
                return EnzymeRules.AugmentedReturn(primal, shadow, (stack, dUbar))
            end
            # reverse: dS/dU += the adjoint of the shadow dS/dUbar
            function EnzymeRules.reverse(config, func::Enzyme.Const{typeof(smear_gb300)}, ::Type{RT}, tape,
                                         U::Enzyme.Duplicated, rho::Enzyme.Const) where {RT}
                stack, dUbar = tape
                dU = smear_pullback(stack, dUbar)
                ctx = stack.ctx
                # U.dval (MAT64 shadow) += dU: the library's axpy on matrix fields
                check(ccall((:gf_field_axpy, libgf), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Cdouble, Ptr{Cvoid}), ctx.h,
                            config_field(U.dval).h, 1.0, config_field(dU).h), ctx)
                return (nothing, nothing)
            end
        end
    end
    return nothing
end

end # module
