"""Host-side mirror of the reference's NonhydrostaticModel API over the C ABI.

Names and argument meanings follow Oceananigans.jl:
  RectilinearGrid(size, x, y, z, topology)        src/Grids/rectilinear_grid.jl:266
  ImmersedBoundaryGrid(grid, GridFittedBottom(h)) src/ImmersedBoundaries/immersed_boundary_grid.jl:46
  NonhydrostaticModel(grid; advection, closure, buoyancy, coriolis, tracers,
                      boundary_conditions, pressure_solver)
                                                  src/Models/NonhydrostaticModels/nonhydrostatic_model.jl:124
  set!(model; u=..., b=...)                       set_nonhydrostatic_model.jl:39   -> set_
  time_step!(model, Δt)                           src/TimeSteppers/runge_kutta_3.jl:103 -> time_step_
  Simulation(model; Δt, stop_time), run!(sim)     src/Simulations/simulation.jl:12, run.jl:151 -> run_
  TimeStepWizard, cell_advection_timescale       src/Simulations/time_step_wizard.jl:66, Advection/cell_advection_timescale.jl:15
A trailing underscore stands for Julia's `!`.  Errors mirror the reference:
invalid configurations raise ValueError (ArgumentError there).
"""
import ctypes
import math
import warnings

import numpy as np

from . import _lib as L

Periodic, Bounded, Flat = "Periodic", "Bounded", "Flat"
_TOPO = {Periodic: L.GBO_PERIODIC, Bounded: L.GBO_BOUNDED, Flat: L.GBO_FLAT}


# ---------------------------------------------------------------------------
# Grids
# ---------------------------------------------------------------------------
class RectilinearGrid:
    """RectilinearGrid(size, x, y, z, extent, topology, float_type).

    `z` is an extent tuple (regular spacing) or a callable / array of Nz+1
    increasing face positions (stretched), as in the reference.  `extent = (Lx, Ly, Lz)`
    ((Lx, Ly) with a Flat z) places the domain at 0 ≤ x ≤ Lx, 0 ≤ y ≤ Ly, -Lz ≤ z ≤ 0
    and excludes x, y and z (src/Grids/rectilinear_grid.jl:121-124,
    input_validation.jl:107-117).
    """

    def __init__(self, size, x=None, y=None, z=None, topology=(Periodic, Periodic, Bounded),
                 float_type=np.float64, halo=None, extent=None):
        if extent is not None:
            if x is not None or y is not None or z is not None:
                raise ValueError("Cannot specify both 'extent' and 'x, y, z' keyword arguments.")
            flat = tuple(topology)[2] == Flat
            extent = tuple(float(e) for e in extent)
            if len(extent) != (2 if flat else 3):
                raise ValueError("extent must have %d entries for this topology" % (2 if flat else 3))
            x, y = (0.0, extent[0]), (0.0, extent[1])
            z = None if flat else (-extent[2], 0.0)
        x = (0.0, 1.0) if x is None else x
        y = (0.0, 1.0) if y is None else y
        z = (-1.0, 0.0) if z is None else z
        topology = tuple(topology)
        if topology[0] != Periodic or topology[1] != Periodic:
            raise ValueError("only Periodic x and y topologies are supported")
        if topology[2] not in (Bounded, Flat):
            raise ValueError("z topology must be Bounded or Flat")
        size = tuple(int(s) for s in size)
        if topology[2] == Flat and len(size) == 2:
            size = size + (1,)
        self.Nx, self.Ny, self.Nz = size
        self.topology = topology
        self.x = tuple(float(a) for a in x)
        self.y = tuple(float(a) for a in y)
        self.float_type = np.dtype(float_type).type
        self.z_faces = None
        if topology[2] == Flat:
            self.Nz = 1
            self.z = (0.0, 1.0)
        elif callable(z):
            self.z_faces = np.array([z(k) for k in range(1, self.Nz + 2)], dtype=np.float64)
            self.z = (float(self.z_faces[0]), float(self.z_faces[-1]))
        elif np.ndim(z) == 1 and len(z) == self.Nz + 1:
            self.z_faces = np.asarray(z, dtype=np.float64).copy()
            self.z = (float(self.z_faces[0]), float(self.z_faces[-1]))
        else:
            self.z = tuple(float(a) for a in z)
        if self.z_faces is not None and not np.all(np.diff(self.z_faces) > 0):
            raise ValueError("The elements of z must be increasing!")
        self.bottom_height = None

    @property
    def Lx(self):
        return self.x[1] - self.x[0]

    @property
    def Ly(self):
        return self.y[1] - self.y[0]

    @property
    def Lz(self):
        return self.z[1] - self.z[0]

    def size(self):
        return (self.Nx, self.Ny, self.Nz)

    def nodes(self):
        """Cell-centre coordinates (xᶜ, yᶜ, zᶜ)."""
        xc = self.x[0] + (np.arange(self.Nx) + 0.5) * self.Lx / self.Nx
        yc = self.y[0] + (np.arange(self.Ny) + 0.5) * self.Ly / self.Ny
        if self.z_faces is not None:
            zc = 0.5 * (self.z_faces[1:] + self.z_faces[:-1])
        else:
            zc = self.z[0] + (np.arange(self.Nz) + 0.5) * self.Lz / self.Nz
        return xc, yc, zc

    def descriptor(self):
        d = L.GridDesc()
        d.size[:] = (self.Nx, self.Ny, self.Nz)
        d.topology[:] = tuple(_TOPO[t] for t in self.topology)
        d.x[:] = self.x
        d.y[:] = self.y
        d.z[:] = self.z
        keep = []
        if self.z_faces is not None:
            zf = np.ascontiguousarray(self.z_faces, dtype=np.float64)
            keep.append(zf)
            d.z_faces = zf.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        if self.bottom_height is not None:
            h = np.ascontiguousarray(np.asarray(self.bottom_height, dtype=np.float64).ravel(order="F"))
            keep.append(h)
            d.bottom_height = h.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        d.float_type = L.GBO_FLOAT32 if self.float_type == np.float32 else L.GBO_FLOAT64
        d._keep = keep
        return d


class GridFittedBottom:
    """GridFittedBottom(h) with h an (Nx, Ny) array or a callable h(x, y)."""

    def __init__(self, bottom_height):
        self.bottom_height = bottom_height


class ImmersedBoundaryGrid(RectilinearGrid):
    def __init__(self, grid, boundary):
        self.__dict__.update(grid.__dict__)
        self.underlying_grid = grid
        h = boundary.bottom_height
        if callable(h):
            xc, yc, _ = grid.nodes()
            X, Y = np.meshgrid(xc, yc, indexing="ij")
            h = np.vectorize(h)(X, Y)
        self.bottom_height = np.asarray(h, dtype=np.float64).reshape(grid.Nx, grid.Ny)


# ---------------------------------------------------------------------------
# Physics options
# ---------------------------------------------------------------------------
class WENO:
    def __init__(self, order=5):
        if order != 5:
            raise ValueError("only WENO(order=5) is implemented on GB300")
        self.order = order


class Smagorinsky:
    """Smagorinsky(; coefficient=0.16, Pr=1) with a constant coefficient
    (turbulence_closure_implementations/Smagorinskys/smagorinsky.jl:47,77-83,90-106):
    νₑ = C² Δᶠ² √(2Σ²).  That is the Lilly form with Cb = 0 (ς = 1 wherever Σ² > 0,
    and νₑ = 0 where Σ² = 0 in both), so it runs as SmagorinskyLilly(C, Cb=0)."""

    def __init__(self, coefficient=0.16, Pr=1.0):
        if isinstance(coefficient, bool) or not isinstance(coefficient, (int, float)):
            raise ValueError("Smagorinsky: the coefficient must be a number (use SmagorinskyLilly or "
                             "DynamicSmagorinsky for the other coefficients)")
        self.C, self.Pr = float(coefficient), float(Pr)


class SmagorinskyLilly:
    def __init__(self, C=0.16, Cb=1.0, Pr=1.0):
        self.C, self.Cb, self.Pr = float(C), float(Cb), float(Pr)


class AnisotropicMinimumDissipation:
    """AnisotropicMinimumDissipation(; C=1/3, Cν=C, Cκ=C, Cb=nothing)
    (anisotropic_minimum_dissipation.jl:138-147), with Cν as `Cnu` and Cκ as `Ckappa`.
    The library carries one coefficient for the viscosity and the diffusivities and no
    buoyancy modification: Ckappa ≠ Cnu or a Cb raise ValueError."""

    def __init__(self, C=1.0 / 3.0, Cnu=None, Ckappa=None, Cb=None):
        cnu = float(C if Cnu is None else Cnu)
        ckappa = float(C if Ckappa is None else Ckappa)
        if ckappa != cnu:
            raise ValueError("AnisotropicMinimumDissipation with Cκ ≠ Cν is not available on GB300")
        if Cb is not None:
            raise ValueError("AnisotropicMinimumDissipation with Cb is not available on GB300")
        self.C = cnu


class LagrangianAveraging:
    """LagrangianAveraging() (Smagorinskys/dynamic_coefficient.jl:133-135): the dynamic
    coefficient averaged along fluid trajectories."""


class DynamicSmagorinsky:
    """DynamicSmagorinsky(; averaging=LagrangianAveraging(), Pr=1, schedule=IterationInterval(1),
    minimum_numerator=1e-32) (turbulence_closure_implementations/Smagorinskys/
    dynamic_coefficient.jl:104-117,215-487).  Either averaging: LagrangianAveraging (the
    default; 𝒥ᴸᴹ, 𝒥ᴹᴹ relaxed along trajectories once per time step, model fields "jlm" and
    "jmm") or averaging=(1, 2) (the coefficient averaged over x and y at every state
    update).  Other averagings and schedules raise ValueError here."""

    def __init__(self, averaging=None, Pr=1.0, minimum_numerator=1e-32, schedule=1):
        if averaging is None or isinstance(averaging, LagrangianAveraging):
            self.averaging = LagrangianAveraging()
        else:
            avg = tuple(averaging) if isinstance(averaging, (tuple, list)) else (averaging,)
            if tuple(sorted(avg)) != (1, 2):
                raise ValueError("DynamicSmagorinsky: only averaging=(1, 2) is available on GB300")
            self.averaging = (1, 2)
        if schedule != 1:
            raise ValueError("DynamicSmagorinsky: only schedule=IterationInterval(1) is available on GB300")
        self.Pr = float(Pr)
        self.minimum_numerator = float(minimum_numerator)


class ScalarDiffusivity:
    """ScalarDiffusivity(; ν=0, κ=0) with constant coefficients, isotropic
    (ThreeDimensionalFormulation) and explicit (turbulence_closure_implementations/
    scalar_diffusivity.jl:8-80).  κ is one number for every tracer or a dict by tracer."""

    def __init__(self, nu=0.0, kappa=0.0):
        self.nu = float(nu)
        self.kappa = dict(kappa) if isinstance(kappa, dict) else float(kappa)

    def kappa_of(self, tracer):
        if isinstance(self.kappa, dict):
            if tracer not in self.kappa:
                raise ValueError("ScalarDiffusivity κ has no entry for tracer %s" % tracer)
            return float(self.kappa[tracer])
        return self.kappa


class QuasiAdamsBashforth2TimeStepper:
    """QuasiAdamsBashforth2TimeStepper(; χ = 0.1) (src/TimeSteppers/quasi_adams_bashforth_2.jl:60-65)."""

    def __init__(self, chi=0.1):
        self.chi = float(chi)


class BuoyancyTracer:
    pass


class FPlane:
    """FPlane(; f, rotation_rate=7.292115e-5, latitude) (Coriolis/f_plane.jl:30-50, the
    rotation rate default of src/Oceananigans.jl:171): either f, or a rotation rate and a
    latitude in degrees with f = 2 Ω sin(latitude).  (Julia's `sind` converts degrees in
    extended precision, so f can differ from it in the last bit.)"""

    def __init__(self, f=None, rotation_rate=7.292115e-5, latitude=None):
        if (f is None) == (latitude is None):
            raise ValueError("Either both keywords rotation_rate and latitude must be specified, "
                             "*or* only f must be specified.")
        self.f = float(f) if f is not None else 2 * float(rotation_rate) * math.sin(math.radians(float(latitude)))


class FluxBoundaryCondition:
    def __init__(self, value):
        self.value = float(value)


class FieldBoundaryConditions:
    def __init__(self, top=None, bottom=None):
        self.top = top
        self.bottom = bottom


class FFTBasedPoissonSolver:
    kind = L.GBO_SOLVER_FFT


class FourierTridiagonalPoissonSolver:
    kind = L.GBO_SOLVER_FOURIER_TRIDIAGONAL


class ConjugateGradientPoissonSolver:
    kind = L.GBO_SOLVER_CONJUGATE_GRADIENT

    def __init__(self, reltol=0.0, abstol=0.0, maxiter=0, preconditioner="fft"):
        self.reltol, self.abstol, self.maxiter = reltol, abstol, maxiter
        self.preconditioner = {"fft": L.GBO_PRECOND_FFT, None: L.GBO_PRECOND_NONE,
                               "learned": L.GBO_PRECOND_LEARNED}[preconditioner]


def _grid_is_regular(grid):
    return grid.z_faces is None


def model_descriptor(grid, advection=None, closure=None, buoyancy=None, coriolis=None, tracers=(),
                     boundary_conditions=None, pressure_solver=None, timestepper="RungeKutta3"):
    """Translate NonhydrostaticModel keyword arguments into the C ABI's gbo_model_desc.

    Follows the reference constructor's choices: the pressure solver picked from the grid
    (nonhydrostatic_pressure_solver, src/Models/NonhydrostaticModels/NonhydrostaticModels.jl:
    30-76), and ArgumentError-style failures raised as ValueError.  The reference's default
    advection, Centered() (nonhydrostatic_model.jl:126), is not implemented here, so
    `advection` must be given: WENO() (order 5).
    """
    if isinstance(timestepper, QuasiAdamsBashforth2TimeStepper):
        ab2_chi, timestepper = timestepper.chi, "QuasiAdamsBashforth2"
    else:
        ab2_chi = 0.1
    if timestepper not in ("RungeKutta3", "QuasiAdamsBashforth2"):
        raise ValueError("timestepper = :%s is not supported; use :RungeKutta3 or :QuasiAdamsBashforth2" % timestepper)
    if advection is None:
        raise ValueError("advection: the reference's default Centered() is not implemented; pass advection=WENO()")
    if not isinstance(advection, WENO):
        raise ValueError("advection must be WENO(order=5)")
    if isinstance(tracers, str):
        tracers = (tracers,)
    tracers = tuple(tracers)
    if isinstance(buoyancy, BuoyancyTracer):
        if "b" not in tracers:
            raise ValueError("BuoyancyTracer requires a tracer named b")
        tracers = ("b",) + tuple(t for t in tracers if t != "b")
    d = L.ModelDesc()
    L.load().gbo_model_desc_default(ctypes.byref(d))
    d.advection = L.GBO_ADVECTION_WENO5
    if isinstance(closure, Smagorinsky):
        d.closure = L.GBO_CLOSURE_SMAGORINSKY_LILLY
        d.closure_C, d.closure_Cb, d.closure_Pr = closure.C, 0.0, closure.Pr
    elif isinstance(closure, SmagorinskyLilly):
        d.closure = L.GBO_CLOSURE_SMAGORINSKY_LILLY
        d.closure_C, d.closure_Cb, d.closure_Pr = closure.C, closure.Cb, closure.Pr
    elif isinstance(closure, AnisotropicMinimumDissipation):
        d.closure = L.GBO_CLOSURE_AMD
        d.closure_C = closure.C
    elif isinstance(closure, DynamicSmagorinsky):
        d.closure = L.GBO_CLOSURE_DYNAMIC_SMAGORINSKY
        d.closure_Pr = closure.Pr
        d.closure_min_numerator = closure.minimum_numerator
        d.closure_averaging = (L.GBO_AVERAGING_LAGRANGIAN if isinstance(closure.averaging, LagrangianAveraging)
                               else L.GBO_AVERAGING_XY)
    elif isinstance(closure, ScalarDiffusivity):
        d.closure = L.GBO_CLOSURE_SCALAR_DIFFUSIVITY
        d.closure_nu = closure.nu
        for n, name in enumerate(tracers):
            d.closure_kappa[n] = closure.kappa_of(name)
    elif closure is not None:
        raise ValueError("unsupported closure %r" % (closure,))
    d.ntracers = len(tracers)
    d.buoyancy_tracer = int(isinstance(buoyancy, BuoyancyTracer))
    if isinstance(coriolis, FPlane):
        d.has_coriolis = 1
        d.coriolis_f = coriolis.f
    for name, bcs in (boundary_conditions or {}).items():
        if name not in tracers:
            raise ValueError("boundary conditions are supported on tracers only (got %s)" % name)
        n = tracers.index(name)
        if bcs.top is not None:
            d.tracer_flux_top[n] = bcs.top.value
        if bcs.bottom is not None:
            d.tracer_flux_bottom[n] = bcs.bottom.value
    if pressure_solver is None:
        if grid.bottom_height is not None:
            # nonhydrostatic_pressure_solver(arch, ibg::IBGWithFFT, ...) (NonhydrostaticModels.jl:54-73):
            # the spectral solver of the underlying grid, with a warning
            warnings.warn("The FFT-based pressure_solver for NonhydrostaticModels on ImmersedBoundaryGrid is "
                          "approximate and will probably produce velocity fields that are divergent adjacent to "
                          "the immersed boundary; pass pressure_solver=ConjugateGradientPoissonSolver() for the "
                          "iterative solver.")
        if _grid_is_regular(grid):
            pressure_solver = FFTBasedPoissonSolver()
        else:
            pressure_solver = FourierTridiagonalPoissonSolver()
    d.timestepper = L.GBO_TIMESTEPPER_QAB2 if timestepper == "QuasiAdamsBashforth2" else L.GBO_TIMESTEPPER_RK3
    d.ab2_chi = ab2_chi
    d.pressure_solver = pressure_solver.kind
    if isinstance(pressure_solver, ConjugateGradientPoissonSolver):
        d.preconditioner = pressure_solver.preconditioner
        d.cg_reltol, d.cg_abstol, d.cg_maxiter = pressure_solver.reltol, pressure_solver.abstol, pressure_solver.maxiter
    return d, tracers


# ---------------------------------------------------------------------------
# Model
# ---------------------------------------------------------------------------
class NonhydrostaticModel:
    """NonhydrostaticModel(grid; advection, closure, buoyancy, coriolis, tracers,
    boundary_conditions, pressure_solver) on one GB300.  State lives on the device.
    """

    def __init__(self, grid, advection=None, closure=None, buoyancy=None, coriolis=None, tracers=(),
                 boundary_conditions=None, pressure_solver=None, timestepper="RungeKutta3"):
        d, self.tracers = model_descriptor(grid, advection=advection, closure=closure, buoyancy=buoyancy,
                                           coriolis=coriolis, tracers=tracers,
                                           boundary_conditions=boundary_conditions,
                                           pressure_solver=pressure_solver, timestepper=timestepper)
        self.grid = grid
        self.desc = d
        self._gdesc = grid.descriptor()
        h = ctypes.c_void_p()
        lib = L.load()
        rc = lib.gbo_model_create(ctypes.byref(self._gdesc), ctypes.byref(d), ctypes.byref(h))
        if rc == L.GBO_ERR_INVALID:
            raise ValueError(lib.gbo_last_error(None).decode())
        L.check(rc)
        self._h = h
        self.dtype = grid.float_type

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and getattr(self, "_owner", None) is None:
            L.load().gbo_model_destroy(h)
        self._h = None

    @classmethod
    def _member(cls, owner, grid, desc, tracers, handle):
        """A member handle of an Ensemble (owned and stepped by the ensemble)."""
        self = cls.__new__(cls)
        self.grid, self.desc, self.tracers = grid, desc, tracers
        self._gdesc = grid.descriptor()
        self._h = ctypes.c_void_p(handle)
        self._owner = owner
        self.dtype = grid.float_type
        return self

    # -- field access --------------------------------------------------------
    def _fid(self, name):
        ids = {"u": L.GBO_FIELD_U, "v": L.GBO_FIELD_V, "w": L.GBO_FIELD_W, "p": L.GBO_FIELD_PNHS,
               "pNHS": L.GBO_FIELD_PNHS, "pHY": L.GBO_FIELD_PHY, "pHY′": L.GBO_FIELD_PHY,
               "nu": L.GBO_FIELD_NU, "νₑ": L.GBO_FIELD_NU, "kappa": L.GBO_FIELD_KAPPA,
               "jlm": L.GBO_FIELD_JLM, "𝒥ᴸᴹ": L.GBO_FIELD_JLM, "jmm": L.GBO_FIELD_JMM, "𝒥ᴹᴹ": L.GBO_FIELD_JMM}
        if name in ids:
            return ids[name]
        if name in self.tracers:
            return L.GBO_FIELD_TRACER + self.tracers.index(name)
        raise ValueError("name %s not found in model.velocities or model.tracers." % name)

    def field_shape(self, name):
        g = self.grid
        if name == "w" and g.topology[2] == Bounded:
            return (g.Nx, g.Ny, g.Nz + 1)
        return (g.Nx, g.Ny, g.Nz)

    def set_field(self, name, value):
        shp = self.field_shape(name)
        if callable(value):
            value = self._evaluate(name, value)
        a = np.broadcast_to(np.asarray(value, dtype=np.float64), shp)
        flat = np.ascontiguousarray(np.asfortranarray(a).ravel(order="F"))
        L.check(L.load().gbo_set_field(self._h, self._fid(name), flat.ctypes.data, L.GBO_FLOAT64, flat.size), self._h)

    def _evaluate(self, name, fn):
        g = self.grid
        xc, yc, zc = g.nodes()
        xf = g.x[0] + np.arange(g.Nx) * g.Lx / g.Nx
        yf = g.y[0] + np.arange(g.Ny) * g.Ly / g.Ny
        xs = xf if name == "u" else xc
        ys = yf if name == "v" else yc
        if name == "w" and g.topology[2] == Bounded:
            zs = g.z_faces if g.z_faces is not None else g.z[0] + np.arange(g.Nz + 1) * g.Lz / g.Nz
        else:
            zs = zc
        X, Y, Zz = np.meshgrid(xs, ys, zs, indexing="ij")
        # one call on the coordinate arrays when fn maps them elementwise to an array of
        # the field's shape; otherwise (scalar-only code, or a result that is not per point,
        # such as one random draw) fn is called at every point, as the reference does
        try:
            with np.errstate(all="ignore"):
                out = np.asarray(fn(X, Y, Zz), dtype=np.float64)
            if out.shape == X.shape:
                return out
        except Exception:  # noqa: BLE001  (any failure means fn is not array-safe)
            pass
        return np.vectorize(fn, otypes=[np.float64])(X, Y, Zz)

    def get(self, name, dtype=np.float64):
        shp = self.field_shape(name)
        out = np.zeros(int(np.prod(shp)), dtype=dtype)
        code = L.GBO_FLOAT32 if np.dtype(dtype) == np.float32 else L.GBO_FLOAT64
        L.check(L.load().gbo_get_field(self._h, self._fid(name), out.ctypes.data, code, out.size), self._h)
        return out.reshape(shp, order="F")

    @property
    def clock(self):
        t = ctypes.c_double()
        it = ctypes.c_int64()
        L.load().gbo_clock(self._h, ctypes.byref(t), ctypes.byref(it))
        return t.value, it.value

    def device_pointer(self, name):
        p = ctypes.c_void_p()
        n = ctypes.c_int64()
        L.check(L.load().gbo_field_device_pointer(self._h, self._fid(name), ctypes.byref(p), ctypes.byref(n)), self._h)
        return p.value, n.value

    def reference_profile(self, name):
        """The per-level reference profile a tracer's device array is a departure from
        (zeros where the tracer is stored directly: FP64 models, Flat z)."""
        out = np.zeros(self.grid.Nz, dtype=np.float64)
        L.check(L.load().gbo_field_reference_profile(self._h, self._fid(name),
                                                      out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), out.size),
                self._h)
        return out

    def poisson_solve_device(self, phi_ptr, rhs_ptr):
        L.check(L.load().gbo_poisson_solve_device(self._h, ctypes.c_void_p(phi_ptr), ctypes.c_void_p(rhs_ptr)), self._h)

    def set_learned_preconditioner(self, weights):
        """Load the learned correction of the CG's FFT preconditioner (an FP32 array of
        gbo_learned_weight_count() values, or a path to one saved with numpy.save);
        None restores the plain FFT preconditioner.  No reference counterpart."""
        lib = L.load()
        if weights is None:
            L.check(lib.gbo_learned_preconditioner(self._h, None, 0), self._h)
            return
        if isinstance(weights, str):
            weights = np.load(weights)
        w = np.ascontiguousarray(weights, dtype=np.float32)
        L.check(lib.gbo_learned_preconditioner(self._h, w.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), w.size),
                self._h)

    def poisson_operator_device(self, x_ptr, out_ptr):
        """out = V∇²x (the CG operator) on device buffers of the model's float type."""
        L.check(L.load().gbo_poisson_operator_device(self._h, ctypes.c_void_p(x_ptr), ctypes.c_void_p(out_ptr)), self._h)

    def precondition_device(self, r_ptr, z_ptr):
        """z = M r with the model's CG preconditioner, on device buffers."""
        L.check(L.load().gbo_precondition_device(self._h, ctypes.c_void_p(r_ptr), ctypes.c_void_p(z_ptr)), self._h)

    @property
    def launch_shape(self):
        """The launch shape (dict: dct_columns, x_lines, y_columns, levels); tuning only."""
        sh = L.LaunchShape()
        L.check(L.load().gbo_get_launch_shape(self._h, ctypes.byref(sh)), self._h)
        return {f: int(getattr(sh, f)) for f, _ in L.LaunchShape._fields_}

    def set_launch_shape(self, **shape):
        """Replace some of the launch shape's entries (gbo_set_launch_shape)."""
        cur = self.launch_shape
        cur.update({k: int(v) for k, v in shape.items()})
        sh = L.LaunchShape(**cur)
        rc = L.load().gbo_set_launch_shape(self._h, ctypes.byref(sh))
        if rc == L.GBO_ERR_INVALID:
            raise ValueError(L.load().gbo_last_error(self._h).decode())
        L.check(rc, self._h)

    def prognostic_state(self):
        """prognostic_state(model): the restart state as a numpy byte array."""
        lib = L.load()
        buf = np.empty(int(lib.gbo_state_bytes(self._h)), dtype=np.uint8)
        L.check(lib.gbo_get_state(self._h, buf.ctypes.data, buf.size), self._h)
        return buf

    def restore_prognostic_state_(self, state):
        """restore_prognostic_state!(model, state)."""
        buf = np.ascontiguousarray(state, dtype=np.uint8)
        L.check(L.load().gbo_set_state(self._h, buf.ctypes.data, buf.size), self._h)

    @property
    def solver_iterations(self):
        return L.load().gbo_last_solver_iterations(self._h)


class Ensemble:
    """Independent NonhydrostaticModels advanced together: one CUDA graph launch per
    step runs every member's RK3 step as a parallel branch.  `specs` is a list of
    (grid, keyword arguments of NonhydrostaticModel).  No reference counterpart."""

    def __init__(self, specs):
        n = len(specs)
        grids = (L.GridDesc * n)()
        descs = (L.ModelDesc * n)()
        self._keep, info = [], []
        for i, (grid, kw) in enumerate(specs):
            d, tracers = model_descriptor(grid, **kw)
            g = grid.descriptor()
            self._keep.append(g)
            ctypes.memmove(ctypes.byref(grids, i * ctypes.sizeof(L.GridDesc)), ctypes.byref(g), ctypes.sizeof(L.GridDesc))
            ctypes.memmove(ctypes.byref(descs, i * ctypes.sizeof(L.ModelDesc)), ctypes.byref(d), ctypes.sizeof(L.ModelDesc))
            info.append((grid, d, tracers))
        lib = L.load()
        h = ctypes.c_void_p()
        rc = lib.gbo_ensemble_create(n, grids, descs, ctypes.byref(h))
        if rc == L.GBO_ERR_INVALID:
            raise ValueError(lib.gbo_last_error(None).decode())
        L.check(rc)
        self._h = h
        self.members = [NonhydrostaticModel._member(self, g, d, t, lib.gbo_ensemble_member(h, i))
                        for i, (g, d, t) in enumerate(info)]

    def __len__(self):
        return len(self.members)

    def __getitem__(self, i):
        return self.members[i]

    def time_step(self, dt, nsteps=1):
        L.check(L.load().gbo_ensemble_time_step(self._h, float(dt), int(nsteps)))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            for mm in getattr(self, "members", []):
                mm._h = None
            L.load().gbo_ensemble_destroy(h)
            self._h = None


def set_(model, enforce_incompressibility=True, **fields):
    """set!(model; enforce_incompressibility=true, kwargs...)."""
    for name, value in fields.items():
        model.set_field(name, value)
    L.check(L.load().gbo_set_finalize(model._h, int(bool(enforce_incompressibility))), model._h)


def time_step_(model, dt, nsteps=1):
    """time_step!(model, Δt) (nsteps times; one CUDA-graph launch per step)."""
    L.check(L.load().gbo_time_step(model._h, float(dt), int(nsteps)), model._h)


class TimeStepWizard:
    """TimeStepWizard(; cfl=0.2, diffusive_cfl=Inf, max_change=1.1, min_change=0.5,
    max_Δt=Inf, min_Δt=0) (src/Simulations/time_step_wizard.jl:66-89).  Attached to a
    Simulation as a callback on IterationInterval(interval); evaluated on the device."""

    def __init__(self, cfl=0.2, diffusive_cfl=math.inf, max_change=1.1, min_change=0.5, max_dt=math.inf, min_dt=0.0):
        if min_change >= 1:
            raise ValueError("min_change must be < 1. You provided min_change = %r." % min_change)
        if max_change <= 1:
            raise ValueError("max_change must be > 1. You provided max_change = %r." % max_change)
        self.cfl, self.diffusive_cfl = float(cfl), float(diffusive_cfl)
        self.max_change, self.min_change = float(max_change), float(min_change)
        self.max_dt, self.min_dt = float(max_dt), float(min_dt)


class Simulation:
    """Simulation(model; Δt, stop_time, stop_iteration, wall_time_limit, align_time_step,
    minimum_relative_step) with the default NaNChecker (u every 100 iterations)
    (src/Simulations/simulation.jl:68-119).  `dt` is converted to the model's float
    type as in the reference; `wizard` / `wizard_interval` add a TimeStepWizard callback."""

    def __init__(self, model, dt=None, stop_time=math.inf, stop_iteration=math.inf, wall_time_limit=math.inf,
                 align_time_step=True, minimum_relative_step=0.0, nan_check_interval=100, nan_erroring=False,
                 wizard=None, wizard_interval=10, Δt=None):
        if (dt is None) == (Δt is None):
            raise ValueError("Simulation needs the time step as dt or Δt (one of them)")
        dt = Δt if dt is None else dt
        self.model = model
        ft = np.float32 if model.dtype == np.float32 else np.float64
        self.dt = float(ft(dt))
        self.stop_time = stop_time
        self.stop_iteration = stop_iteration
        self.wall_time_limit = wall_time_limit
        self.align_time_step = bool(align_time_step)
        self.minimum_relative_step = float(minimum_relative_step)
        self.nan_check_interval = int(nan_check_interval)
        self.nan_erroring = bool(nan_erroring)
        self.wizard = wizard
        self.wizard_interval = int(wizard_interval)
        self.running = False
        self.stop_reason = None
        self.nan_detected = False


def conjure_time_step_wizard_(sim, interval=10, **wizard_kw):
    """conjure_time_step_wizard!(simulation, IterationInterval(interval); wizard_kw...)
    (src/Simulations/time_step_wizard.jl:117-126)."""
    sim.wizard = TimeStepWizard(**wizard_kw)
    sim.wizard_interval = int(interval)


STOP_REASONS = {L.GBO_STOP_NONE: None, L.GBO_STOP_TIME: "stop_time", L.GBO_STOP_ITERATION: "stop_iteration",
                L.GBO_STOP_NAN: "nan", L.GBO_STOP_WALL_TIME: "wall_time_limit"}


def run_(sim, iterations_per_launch=100):
    """run!(sim) (src/Simulations/run.jl:151-187): the whole loop -- Δt alignment with
    stop_time, time steps, stop criteria, NaN check, TimeStepWizard -- runs on the device
    as one CUDA-graph launch per `iterations_per_launch` iterations."""
    lib = L.load()
    d = L.RunDesc()
    lib.gbo_run_desc_default(ctypes.byref(d))
    d.dt = sim.dt
    d.stop_time = float(sim.stop_time)
    d.stop_iteration = float(sim.stop_iteration)
    d.wall_time_limit = float(sim.wall_time_limit)
    d.align_time_step = int(sim.align_time_step)
    d.minimum_relative_step = sim.minimum_relative_step
    d.nan_check_interval = sim.nan_check_interval
    d.nan_erroring = int(sim.nan_erroring)
    if sim.wizard is not None:
        w = sim.wizard
        d.wizard_interval = sim.wizard_interval
        d.cfl, d.diffusive_cfl = w.cfl, w.diffusive_cfl
        d.max_change, d.min_change = w.max_change, w.min_change
        d.max_dt, d.min_dt = w.max_dt, w.min_dt
    d.iterations_per_launch = int(iterations_per_launch)
    r = L.RunResult()
    sim.running = True
    try:
        L.check(lib.gbo_run(sim.model._h, ctypes.byref(d), ctypes.byref(r)), sim.model._h)
    finally:
        sim.running = False
    sim.dt = r.dt
    sim.stop_reason = STOP_REASONS.get(r.stop_reason)
    sim.nan_detected = bool(r.nan_detected)
    return r


def cell_advection_timescale(model):
    """cell_advection_timescale(model) (src/Advection/cell_advection_timescale.jl:15-21)."""
    out = ctypes.c_double()
    L.check(L.load().gbo_cell_advection_timescale(model._h, ctypes.byref(out)), model._h)
    return out.value


def cell_diffusion_timescale(model):
    """cell_diffusion_timescale(model) (src/TurbulenceClosures/turbulence_closure_diagnostics.jl:21-63)."""
    out = ctypes.c_double()
    L.check(L.load().gbo_cell_diffusion_timescale(model._h, ctypes.byref(out)), model._h)
    return out.value
