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
import Oceananigans.TimeSteppers: time_step!
import Oceananigans.Fields: set!

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
end

const handles = IdDict{Any, Ptr{Cvoid}}()

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
        md = Ref{ModelDesc}()
        ccall((:gbo_model_desc_default, libgbo), Cvoid, (Ref{ModelDesc},), md)
        # closure / buoyancy / coriolis / boundary conditions are translated here
        # exactly as oceananigans_gb300.api.model_descriptor does for Python.
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
