"""
    OceananigansGB300Ext

Package extension that runs `time_step!(model::NonhydrostaticModel, Δt)` on one
GB300 through the C ABI of `libgb300ocean.so` (declared in `include/gbo.h`).

Usage:

    grid  = RectilinearGrid(GB300(), size=(256, 256, 128), x=(0, 512), y=(0, 512), z=(-256, 0))
    model = NonhydrostaticModel(grid; advection=WENO(), closure=SmagorinskyLilly(),
                                buoyancy=BuoyancyTracer(), tracers=:b, coriolis=FPlane(f=1e-4))
    set!(model, u=u₀, b=b₀)       # fields are uploaded, then projected on the device
    run!(Simulation(model, Δt=2, stop_iteration=200))

The library owns the device state; host `Field`s are refreshed on demand
(`sync_fields!`) for output and diagnostics.
"""
module OceananigansGB300Ext

using Oceananigans
using Oceananigans.Grids: topology, Periodic, Bounded, Flat
using Oceananigans.ImmersedBoundaries: ImmersedBoundaryGrid
using Oceananigans.Fields: interior
using Oceananigans.Models.NonhydrostaticModels: NonhydrostaticModel
using Oceananigans.Simulations: TimeStepWizard
using Oceananigans.Utils: IterationInterval
import Oceananigans.TimeSteppers: time_step!
import Oceananigans.Fields: set!
import Oceananigans: prognostic_state, restore_prognostic_state!
import Oceananigans.Simulations: run!
import Oceananigans.Advection: cell_advection_timescale

# run!(sim) on a GB300 model: the whole loop on the device when its callbacks allow,
# else the reference loop, which calls the time_step! method below once per step
function run!(sim::Simulation{<:NonhydrostaticModel{<:Any, <:Any, <:Any, <:GB300}}; pickup=false, kw...)
    pickup == false && isempty(kw) && device_run!(sim) && return nothing
    return invoke(run!, Tuple{Any}, sim; pickup, kw...)
end

const libgbo = get(ENV, "GB300OCEAN_LIB", "libgb300ocean.so")

# --- mirrors of the C structs in include/gbo.h --------------------------------
struct GridDesc
    size::NTuple{3, Int32}
    topology::NTuple{3, Int32}
    x::NTuple{2, Float64}
    y::NTuple{2, Float64}
    z::NTuple{2, Float64}
    z_faces::Ptr{Float64}
    bottom_height::Ptr{Float64}
    float_type::Int32
end

struct ModelDesc
    advection::Int32
    closure::Int32
    closure_C::Float64
    closure_Cb::Float64
    closure_Pr::Float64
    ntracers::Int32
    buoyancy_tracer::Int32
    has_coriolis::Int32
    coriolis_f::Float64
    tracer_flux_top::NTuple{4, Float64}
    tracer_flux_bottom::NTuple{4, Float64}
    pressure_solver::Int32
    preconditioner::Int32
    cg_reltol::Float64
    cg_abstol::Float64
    cg_maxiter::Int32
    closure_nu::Float64
    closure_kappa::NTuple{4, Float64}
    timestepper::Int32
    ab2_chi::Float64
    closure_min_numerator::Float64   # DynamicSmagorinsky(...).coefficient.minimum_numerator
    closure_averaging::Int32         # 0: averaging=(1, 2); 1: LagrangianAveraging()
end

const handles = IdDict{Any, Ptr{Cvoid}}()

# --- model → descriptor (oceananigans_gb300.api.model_descriptor does the same) --------
using Oceananigans.TurbulenceClosures: ScalarDiffusivity, AnisotropicMinimumDissipation
using Oceananigans.TurbulenceClosures.Smagorinskys: Smagorinsky, LillyCoefficient, DynamicCoefficient,
                                                    LagrangianAveraging
using Oceananigans.BuoyancyFormulations: BuoyancyTracer
using Oceananigans.Coriolis: FPlane
using Oceananigans.BoundaryConditions: BoundaryCondition, Flux
using Oceananigans.Solvers: FFTBasedPoissonSolver, FourierTridiagonalPoissonSolver, ConjugateGradientPoissonSolver
using Oceananigans.TimeSteppers: QuasiAdamsBashforth2TimeStepper, RungeKutta3TimeStepper

# a copy of d with the named fields replaced
function with(d::ModelDesc; kw...)
    vals = ntuple(fieldcount(ModelDesc)) do n
        f = fieldname(ModelDesc, n)
        haskey(kw, f) ? convert(fieldtype(ModelDesc, f), kw[f]) : getfield(d, n)
    end
    return ModelDesc(vals...)
end

one_value(x::Number) = Float64(x)
one_value(x::NamedTuple) = Float64(first(values(x)))   # one Pr / κ for every tracer
padded4(x::Number) = ntuple(_ -> Float64(x), 4)
padded4(x::NamedTuple) = ntuple(n -> n ≤ length(x) ? Float64(values(x)[n]) : 0.0, 4)

# WENO(order=5) is the only advection scheme of the library (the reference's default,
# Centered(), and bounded or lower-order WENO are refused rather than replaced)
advection_desc(a::WENO{3}) = isnothing(a.bounds) ? (; advection = Int32(5)) :
    throw(ArgumentError("bounded WENO advection is not available on GB300"))
advection_desc(a) = throw(ArgumentError("advection $(summary(a)) is not available on GB300: use WENO(order=5)"))

closure_desc(::Nothing) = (; closure = Int32(0))
# a constant coefficient is the Lilly form with Cb = 0 (smagorinsky.jl:47,106)
closure_desc(c::Smagorinsky{<:Any, <:Number}) =
    (; closure = Int32(1), closure_C = Float64(c.coefficient), closure_Cb = 0.0, closure_Pr = one_value(c.Pr))
closure_desc(c::Smagorinsky{<:Any, <:LillyCoefficient}) =
    (; closure = Int32(1), closure_C = Float64(c.coefficient.smagorinsky),
       closure_Cb = Float64(c.coefficient.reduction_factor), closure_Pr = one_value(c.Pr))
function closure_desc(c::Smagorinsky{<:Any, <:DynamicCoefficient})
    a = c.coefficient.averaging
    avg = a isa LagrangianAveraging ? Int32(1) : (a isa Tuple && sort(collect(a)) == [1, 2]) ? Int32(0) : Int32(-1)
    return (; closure = Int32(4), closure_Pr = one_value(c.Pr), closure_averaging = avg,
              closure_min_numerator = Float64(c.coefficient.minimum_numerator))
end
function closure_desc(c::AnisotropicMinimumDissipation)
    isnothing(c.Cb) || throw(ArgumentError("AnisotropicMinimumDissipation with Cb is not available on GB300"))
    Cκ = c.Cκ isa NamedTuple ? collect(values(c.Cκ)) : [c.Cκ]
    all(==(c.Cν), Cκ) || throw(ArgumentError("AnisotropicMinimumDissipation with Cκ ≠ Cν is not available on GB300"))
    return (; closure = Int32(2), closure_C = one_value(c.Cν))
end
closure_desc(c::ScalarDiffusivity) = (; closure = Int32(3), closure_nu = Float64(c.ν), closure_kappa = padded4(c.κ))
closure_desc(c) = throw(ArgumentError("closure $(summary(c)) is not available on GB300"))

flux_value(bc::BoundaryCondition{<:Flux}) = bc.condition isa Number ? Float64(bc.condition) :
    throw(ArgumentError("only constant FluxBoundaryConditions are available on GB300"))
flux_value(bc) = 0.0   # nothing / no-flux

solver_desc(::FFTBasedPoissonSolver) = (; pressure_solver = Int32(0))
solver_desc(::FourierTridiagonalPoissonSolver) = (; pressure_solver = Int32(1))
function solver_desc(s::ConjugateGradientPoissonSolver)
    cg = s.conjugate_gradient_solver
    return (; pressure_solver = Int32(2), preconditioner = Int32(0), cg_reltol = Float64(cg.reltol),
              cg_abstol = Float64(cg.abstol), cg_maxiter = Int32(cg.maxiter))
end

function describe(model, md::ModelDesc)
    tracers = model.tracers
    tops = ntuple(n -> n ≤ length(tracers) ? flux_value(tracers[n].boundary_conditions.top) : 0.0, 4)
    bots = ntuple(n -> n ≤ length(tracers) ? flux_value(tracers[n].boundary_conditions.bottom) : 0.0, 4)
    b = model.buoyancy isa Nothing ? 0 :
        (model.buoyancy.formulation isa BuoyancyTracer && first(keys(tracers)) == :b) ? 1 :
        throw(ArgumentError("only BuoyancyTracer with b as the first tracer is available on GB300"))
    f = model.coriolis isa FPlane ? (; has_coriolis = Int32(1), coriolis_f = Float64(model.coriolis.f)) :
        model.coriolis isa Nothing ? (; has_coriolis = Int32(0)) :
        throw(ArgumentError("only FPlane Coriolis is available on GB300"))
    ts = model.timestepper isa QuasiAdamsBashforth2TimeStepper ?
         (; timestepper = Int32(1), ab2_chi = Float64(model.timestepper.χ)) :
         model.timestepper isa RungeKutta3TimeStepper ? (; timestepper = Int32(0)) :
         throw(ArgumentError("timestepper $(summary(model.timestepper)) is not available on GB300"))
    return with(md; ntracers = Int32(length(tracers)), buoyancy_tracer = Int32(b),
                tracer_flux_top = tops, tracer_flux_bottom = bots,
                advection_desc(model.advection)..., closure_desc(model.closure)..., solver_desc(model.pressure_solver)...,
                f..., ts...)
end

check(rc, h=C_NULL) = rc == 0 ||
    throw(ErrorException(unsafe_string(ccall((:gbo_last_error, libgbo), Cstring, (Ptr{Cvoid},), h))))

topo_code(::Type{Periodic}) = Int32(1)
topo_code(::Type{Bounded})  = Int32(2)
topo_code(::Type{Flat})     = Int32(0)

function handle(model::NonhydrostaticModel)
    get!(handles, model) do
        grid = model.grid
        TX, TY, TZ = topology(grid)
        FT = eltype(grid)
        ug = grid isa ImmersedBoundaryGrid ? grid.underlying_grid : grid
        zf = ug.z.cᵃᵃᶠ isa Number ? Float64[] : Float64.(collect(ug.z.cᵃᵃᶠ[1:grid.Nz+1]))
        # GridFittedBottom heights at cell centres, x fastest (Nx*Ny values)
        bh = grid isa ImmersedBoundaryGrid ?
             Float64.(vec(Array(interior(grid.immersed_boundary.bottom_height))[:, :, 1])) : Float64[]
        gd = GridDesc((grid.Nx, grid.Ny, grid.Nz), (topo_code(TX), topo_code(TY), topo_code(TZ)),
                      (grid.xᶠᵃᵃ[1], grid.xᶠᵃᵃ[1] + grid.Lx), (grid.yᵃᶠᵃ[1], grid.yᵃᶠᵃ[1] + grid.Ly),
                      (-grid.Lz, 0.0), isempty(zf) ? C_NULL : pointer(zf), isempty(bh) ? C_NULL : pointer(bh),
                      FT == Float32 ? Int32(4) : Int32(8))
        md0 = Ref{ModelDesc}()
        ccall((:gbo_model_desc_default, libgbo), Cvoid, (Ref{ModelDesc},), md0)
        md = Ref(describe(model, md0[]))
        h = Ref{Ptr{Cvoid}}(C_NULL)
        GC.@preserve zf bh check(ccall((:gbo_model_create, libgbo), Cint,
                                    (Ref{GridDesc}, Ref{ModelDesc}, Ref{Ptr{Cvoid}}), Ref(gd), md, h))
        finalizer(m -> ccall((:gbo_model_destroy, libgbo), Cvoid, (Ptr{Cvoid},), handles[m]), model)
        h[]
    end
end

function set!(model::NonhydrostaticModel{<:Any, <:Any, <:Any, <:GB300}; enforce_incompressibility=true, kw...)
    h = handle(model)
    for (name, value) in kw
        field = name ∈ (:u, :v, :w) ? getproperty(model.velocities, name) : getproperty(model.tracers, name)
        set!(field, value)                          # evaluate on the host as the reference does
        data = Array{Float64}(interior(field))
        id = name == :u ? 0 : name == :v ? 1 : name == :w ? 2 : 3 + findfirst(==(name), keys(model.tracers)) - 1
        check(ccall((:gbo_set_field, libgbo), Cint, (Ptr{Cvoid}, Int32, Ptr{Float64}, Int32, Int64),
                    h, id, data, 8, length(data)), h)
    end
    check(ccall((:gbo_set_finalize, libgbo), Cint, (Ptr{Cvoid}, Int32), h, enforce_incompressibility), h)
    return nothing
end

function time_step!(model::NonhydrostaticModel{<:Any, <:Any, <:Any, <:GB300}, Δt; callbacks=[])
    isempty(callbacks) || throw(ArgumentError("TendencyCallsite / UpdateStateCallsite callbacks are not supported on GB300"))
    h = handle(model)
    check(ccall((:gbo_time_step, libgbo), Cint, (Ptr{Cvoid}, Float64, Int32), h, Δt, 1), h)
    t = Ref{Float64}(); it = Ref{Int64}()
    ccall((:gbo_clock, libgbo), Cint, (Ptr{Cvoid}, Ref{Float64}, Ref{Int64}), h, t, it)
    model.clock.time = t[]
    model.clock.iteration = it[]
    return nothing
end

# --- checkpointing: the state blob of gbo_get_state / gbo_set_state -------------------
function prognostic_state(model::NonhydrostaticModel{<:Any, <:Any, <:Any, <:GB300})
    h = handle(model)
    buf = Vector{UInt8}(undef, ccall((:gbo_state_bytes, libgbo), Int64, (Ptr{Cvoid},), h))
    check(ccall((:gbo_get_state, libgbo), Cint, (Ptr{Cvoid}, Ptr{UInt8}, Int64), h, buf, length(buf)), h)
    return (; gb300_state = buf)
end

function restore_prognostic_state!(model::NonhydrostaticModel{<:Any, <:Any, <:Any, <:GB300}, from)
    h = handle(model)
    buf = from.gb300_state
    check(ccall((:gbo_set_state, libgbo), Cint, (Ptr{Cvoid}, Ptr{UInt8}, Int64), h, buf, length(buf)), h)
    t = Ref{Float64}(); it = Ref{Int64}()
    ccall((:gbo_clock, libgbo), Cint, (Ptr{Cvoid}, Ref{Float64}, Ref{Int64}), h, t, it)
    model.clock.time, model.clock.iteration = t[], it[]
    return model
end

# --- run!(sim) as one device loop when its callbacks are the ones gbo_run implements ----
struct RunDesc
    dt::Float64
    stop_time::Float64
    stop_iteration::Float64
    wall_time_limit::Float64
    align_time_step::Int32
    minimum_relative_step::Float64
    nan_check_interval::Int32
    nan_erroring::Int32
    wizard_interval::Int32
    cfl::Float64
    diffusive_cfl::Float64
    max_change::Float64
    min_change::Float64
    max_dt::Float64
    min_dt::Float64
    iterations_per_launch::Int32
end

struct RunResult
    dt::Float64
    time::Float64
    iteration::Int64
    steps::Int64
    stop_reason::Int32
    nan_detected::Int32
end

const default_callbacks = (:stop_time_exceeded, :stop_iteration_exceeded, :wall_time_limit_exceeded, :nan_checker)

function device_run!(sim)
    model = sim.model
    extra = [k for k in keys(sim.callbacks) if k ∉ default_callbacks]
    wizard = length(extra) == 1 ? sim.callbacks[extra[1]] : nothing
    device_loop = isempty(sim.output_writers) && isempty(sim.diagnostics) &&
                  (isempty(extra) || (wizard !== nothing && wizard.func isa TimeStepWizard &&
                                      wizard.schedule isa IterationInterval && wizard.schedule.offset == 0))
    device_loop || return false
    nan = get(sim.callbacks, :nan_checker, nothing)
    w = wizard === nothing ? TimeStepWizard() : wizard.func
    d = RunDesc(sim.Δt, sim.stop_time, sim.stop_iteration, sim.wall_time_limit, sim.align_time_step,
                sim.minimum_relative_step, nan === nothing ? 0 : nan.schedule.interval,
                nan === nothing ? 0 : nan.func.erroring, wizard === nothing ? 0 : wizard.schedule.interval,
                w.cfl, w.diffusive_cfl, w.max_change, w.min_change, w.max_Δt, w.min_Δt, 100)
    r = Ref{RunResult}()
    h = handle(model)
    check(ccall((:gbo_run, libgbo), Cint, (Ptr{Cvoid}, Ref{RunDesc}, Ref{RunResult}), h, Ref(d), r), h)
    sim.Δt = r[].dt
    model.clock.time, model.clock.iteration = r[].time, r[].iteration
    r[].nan_detected != 0 && (nan.func.nan_detected = true)
    sim.running = false
    return true
end

function cell_advection_timescale(model::NonhydrostaticModel{<:Any, <:Any, <:Any, <:GB300})
    τ = Ref{Float64}()
    check(ccall((:gbo_cell_advection_timescale, libgbo), Cint, (Ptr{Cvoid}, Ref{Float64}), handle(model), τ))
    return τ[]
end

"Copy the device state into the host `Field`s (for output writers and diagnostics)."
function sync_fields!(model::NonhydrostaticModel)
    h = handle(model)
    for (id, field) in enumerate((model.velocities..., model.tracers...))
        buf = Array{Float64}(undef, size(interior(field)))
        check(ccall((:gbo_get_field, libgbo), Cint, (Ptr{Cvoid}, Int32, Ptr{Float64}, Int32, Int64),
                    h, id - 1, buf, 8, length(buf)), h)
        interior(field) .= buf
    end
    return nothing
end

end # module
