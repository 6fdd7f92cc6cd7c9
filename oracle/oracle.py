"""ctypes harness for the FP64 CPU oracle (ocean_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the product package.  The oracle is a
C++ restatement of Oceananigans.jl's NonhydrostaticModel RK3 step; see the
header of ocean_oracle.cpp for what it follows and how it is pinned.
"""
import ctypes
import math
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SRC = os.path.join(HERE, "ocean_oracle.cpp")

GBO_FLAT, GBO_PERIODIC, GBO_BOUNDED = 0, 1, 2
GBO_FLOAT32, GBO_FLOAT64 = 4, 8
MAX_TRACERS = 4


class GridDesc(ctypes.Structure):
    _fields_ = [("size", ctypes.c_int32 * 3), ("topology", ctypes.c_int32 * 3),
                ("x", ctypes.c_double * 2), ("y", ctypes.c_double * 2), ("z", ctypes.c_double * 2),
                ("z_faces", ctypes.POINTER(ctypes.c_double)),
                ("bottom_height", ctypes.POINTER(ctypes.c_double)),
                ("float_type", ctypes.c_int32)]


class ModelDesc(ctypes.Structure):
    _fields_ = [("advection", ctypes.c_int32), ("closure", ctypes.c_int32),
                ("closure_C", ctypes.c_double), ("closure_Cb", ctypes.c_double), ("closure_Pr", ctypes.c_double),
                ("ntracers", ctypes.c_int32), ("buoyancy_tracer", ctypes.c_int32),
                ("has_coriolis", ctypes.c_int32), ("coriolis_f", ctypes.c_double),
                ("tracer_flux_top", ctypes.c_double * MAX_TRACERS),
                ("tracer_flux_bottom", ctypes.c_double * MAX_TRACERS),
                ("pressure_solver", ctypes.c_int32), ("preconditioner", ctypes.c_int32),
                ("cg_reltol", ctypes.c_double), ("cg_abstol", ctypes.c_double), ("cg_maxiter", ctypes.c_int32),
                ("closure_nu", ctypes.c_double), ("closure_kappa", ctypes.c_double * MAX_TRACERS),
                ("timestepper", ctypes.c_int32), ("ab2_chi", ctypes.c_double),
                ("closure_min_numerator", ctypes.c_double), ("closure_averaging", ctypes.c_int32)]


def build(force=False):
    """Compile the oracle with g++ (OpenMP) into oracle/_build/liboracle.so."""
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-o", LIB + ".tmp", SRC]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        L.orc_create.restype = ctypes.c_void_p
        L.orc_create.argtypes = [ctypes.POINTER(GridDesc), ctypes.POINTER(ModelDesc)]
        L.orc_destroy.argtypes = [ctypes.c_void_p]
        dp = ctypes.POINTER(ctypes.c_double)
        L.orc_set_field.argtypes = [ctypes.c_void_p, ctypes.c_int, dp, ctypes.c_int64]
        L.orc_get_field.argtypes = [ctypes.c_void_p, ctypes.c_int, dp, ctypes.c_int64]
        L.orc_set_finalize.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc_time_step.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_int]
        L.orc_poisson_solve.argtypes = [ctypes.c_void_p, dp, dp]
        L.orc_z_spacings.argtypes = [ctypes.c_void_p, dp, dp, ctypes.c_int]
        L.orc_weno5.restype = ctypes.c_double
        L.orc_weno5.argtypes = [dp, ctypes.c_int]
        L.orc_clock.argtypes = [ctypes.c_void_p, dp, ctypes.POINTER(ctypes.c_int64)]
        L.orc_parent.argtypes = [ctypes.c_void_p, ctypes.c_int, dp, ctypes.c_int64, ctypes.POINTER(ctypes.c_int)]
        L.orc_lagrangian_update.argtypes = [ctypes.c_void_p, ctypes.c_double]
        L.orc_last_cg_iterations.argtypes = [ctypes.c_void_p]
        L.orc_set_threads.argtypes = [ctypes.c_int]
        L.orc_max_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


FIELD_IDS = {"u": 0, "v": 1, "w": 2, "p": 100, "pHY": 101, "nu": 102, "kappa": 103,
             "jlm": 104, "jmm": 105}  # 𝒥ᴸᴹ, 𝒥ᴹᴹ of a Lagrangian-averaged DynamicSmagorinsky


class OracleModel:
    """FP64 oracle of NonhydrostaticModel with the same descriptors as the CUDA library."""

    def __init__(self, grid_desc, model_desc, tracers=()):
        self._keep = grid_desc._keep if hasattr(grid_desc, "_keep") else None
        self.grid = grid_desc
        self.desc = model_desc
        self.tracers = tuple(tracers)
        self.h = lib().orc_create(ctypes.byref(grid_desc), ctypes.byref(model_desc))
        Nx, Ny, Nz = grid_desc.size
        self.flat = grid_desc.topology[2] == GBO_FLAT
        self.shape = (Nx, Ny, 1 if self.flat else Nz)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def _fid(self, name):
        if name in FIELD_IDS:
            return FIELD_IDS[name]
        return 3 + self.tracers.index(name)

    def field_shape(self, name):
        Nx, Ny, Nz = self.shape
        if name == "w" and not self.flat:
            return (Nx, Ny, Nz + 1)
        return (Nx, Ny, Nz)

    def set(self, **fields):
        for name, val in fields.items():
            shp = self.field_shape(name)
            a = np.asfortranarray(np.broadcast_to(np.asarray(val, dtype=np.float64), shp))
            flat = np.ascontiguousarray(a.ravel(order="F"))
            rc = lib().orc_set_field(self.h, self._fid(name), _dptr(flat), flat.size)
            if rc:
                raise ValueError("oracle set failed for %s" % name)

    def finalize_set(self, enforce_incompressibility=True):
        return _checked(lib().orc_set_finalize(self.h, int(enforce_incompressibility)))

    def get(self, name):
        shp = self.field_shape(name)
        out = np.zeros(int(np.prod(shp)), dtype=np.float64)
        rc = lib().orc_get_field(self.h, self._fid(name), _dptr(out), out.size)
        if rc:
            raise ValueError("oracle get failed for %s" % name)
        return out.reshape(shp, order="F")

    def parent(self, name):
        """The field's parent array, halos included, indexed [i, j, k] (1-based interior
        index i at parent index i + H - 1)."""
        dims = (ctypes.c_int * 3)()
        if lib().orc_parent(self.h, self._fid(name), None, 0, dims):
            raise ValueError("oracle has no parent array for %s" % name)
        out = np.zeros(dims[0] * dims[1] * dims[2], dtype=np.float64)
        _checked(lib().orc_parent(self.h, self._fid(name), _dptr(out), out.size, dims))
        return out.reshape((dims[0], dims[1], dims[2]), order="F")

    def lagrangian_update(self, dt):
        """One Lagrangian update of 𝒥ᴸᴹ, 𝒥ᴹᴹ from the current state, the clock advanced by dt."""
        return _checked(lib().orc_lagrangian_update(self.h, float(dt)))

    def time_step(self, dt, nsteps=1):
        return _checked(lib().orc_time_step(self.h, float(dt), int(nsteps)))

    def clock(self):
        t = ctypes.c_double()
        it = ctypes.c_int64()
        lib().orc_clock(self.h, ctypes.byref(t), ctypes.byref(it))
        return t.value, it.value

    def poisson_solve(self, rhs):
        rhs = np.asfortranarray(np.asarray(rhs, dtype=np.float64).reshape(self.shape, order="F"))
        flat = np.ascontiguousarray(rhs.ravel(order="F"))
        out = np.zeros_like(flat)
        _checked(lib().orc_poisson_solve(self.h, _dptr(out), _dptr(flat)))
        return out.reshape(self.shape, order="F")

    def z_spacings(self):
        Nz = self.shape[2]
        H = 0 if self.flat else (4 if self.grid.bottom_height else 3)
        n = Nz + 2 * H + 1
        dzc = np.zeros(n)
        dzf = np.zeros(n)
        lib().orc_z_spacings(self.h, _dptr(dzc), _dptr(dzf), n)
        return dzc, dzf

    def last_cg_iterations(self):
        return lib().orc_last_cg_iterations(self.h)


class OracleNotConverged(RuntimeError):
    pass


# ---------------------------------------------------------------------------
# Configuration.  The oracle's grid and model descriptors are built here from a
# plain description of the physics, and every parameter the description leaves
# out takes the reference's default, restated below from the Oceananigans.jl
# v0.110.19 sources.  Nothing is read from the library under test (its defaults
# are checked against this table by tests/test_oracle_config.py).
# ---------------------------------------------------------------------------
REFERENCE_DEFAULTS = {
    # SmagorinskyLilly(...; C=0.16, Cb=1, Pr=1)  (Smagorinskys/lilly_coefficient.jl:109)
    "SmagorinskyLilly": {"C": 0.16, "Cb": 1.0, "Pr": 1.0},
    # Smagorinsky(; coefficient=0.16, Pr=1.0)  (Smagorinskys/smagorinsky.jl:51-52, 78)
    "Smagorinsky": {"coefficient": 0.16, "Pr": 1.0},
    # AnisotropicMinimumDissipation(; C=1/3, Cν=C, Cκ=C, Cb=nothing)
    # (anisotropic_minimum_dissipation.jl:139-142)
    "AnisotropicMinimumDissipation": {"C": 1.0 / 3.0},
    # DynamicSmagorinsky(; averaging=LagrangianAveraging(), Pr=1, minimum_numerator=1e-32)
    # (Smagorinskys/dynamic_coefficient.jl:107-112)
    "DynamicSmagorinsky": {"averaging": "lagrangian", "Pr": 1.0, "minimum_numerator": 1e-32},
    # ScalarDiffusivity(; ν=0, κ=0)  (scalar_diffusivity.jl:113-116)
    "ScalarDiffusivity": {"nu": 0.0, "kappa": 0.0},
    # QuasiAdamsBashforth2TimeStepper(; χ=0.1)  (TimeSteppers/quasi_adams_bashforth_2.jl:63)
    "QuasiAdamsBashforth2": {"chi": 0.1},
    # ConjugateGradientPoissonSolver(grid; reltol=sqrt(eps(grid)), abstol=sqrt(eps(grid)))
    # (Solvers/conjugate_gradient_poisson_solver.jl:134-137), maxiter=prod(size(template_field))
    # (Solvers/conjugate_gradient_solver.jl:91), the FFT solver of the underlying grid as the
    # preconditioner of an immersed grid (conjugate_gradient_poisson_solver.jl:141-147)
    "ConjugateGradientPoissonSolver": {"reltol": "sqrt(eps(FT))", "abstol": "sqrt(eps(FT))",
                                       "maxiter": "Nx*Ny*Nz", "preconditioner": "fft"},
    # FPlane(; rotation_rate=Oceananigans.defaults.planet_rotation_rate)
    # (Coriolis/f_plane.jl:17; src/Oceananigans.jl:171)
    "FPlane": {"rotation_rate": 7.292115e-5},
}

# descriptor codes (the C layout both libraries accept)
_CLOSURE_CODES = {None: 0, "SmagorinskyLilly": 1, "Smagorinsky": 1, "AnisotropicMinimumDissipation": 2,
                  "ScalarDiffusivity": 3, "DynamicSmagorinsky": 4}
_SOLVER_CODES = {"FFTBasedPoissonSolver": 0, "FourierTridiagonalPoissonSolver": 1,
                 "ConjugateGradientPoissonSolver": 2}
_PRECOND_CODES = {"fft": 0, None: 1, "learned": 2}


def grid_desc(size, x, y, z=(-1.0, 0.0), topology=("Periodic", "Periodic", "Bounded"), float_type=np.float64,
              bottom_height=None):
    """GridDesc of RectilinearGrid(size, x, y, z, topology), optionally wrapped in
    ImmersedBoundaryGrid(GridFittedBottom(h)): `z` is an extent or the Nz+1 increasing
    face positions; `bottom_height` a callable h(x, y) evaluated here at the cell centres
    (rectilinear_grid.jl:266-305), or an (Nx, Ny) array."""
    flat = topology[2] == "Flat"
    size = tuple(int(s) for s in size)
    if flat and len(size) == 2:
        size = size + (1,)
    Nx, Ny, Nz = size
    g = GridDesc()
    g.size[:] = (Nx, Ny, 1 if flat else Nz)
    codes = {"Flat": GBO_FLAT, "Periodic": GBO_PERIODIC, "Bounded": GBO_BOUNDED}
    g.topology[:] = tuple(codes[t] for t in topology)
    g.x[:] = tuple(float(a) for a in x)
    g.y[:] = tuple(float(a) for a in y)
    keep = []
    if flat:
        g.z[:] = (0.0, 1.0)
    elif np.ndim(z) == 1 and len(z) == Nz + 1:
        zf = np.ascontiguousarray(z, dtype=np.float64)
        keep.append(zf)
        g.z_faces = zf.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        g.z[:] = (float(zf[0]), float(zf[-1]))
    else:
        g.z[:] = tuple(float(a) for a in z)
    if bottom_height is not None:
        if callable(bottom_height):
            xc = g.x[0] + (np.arange(Nx) + 0.5) * (g.x[1] - g.x[0]) / Nx
            yc = g.y[0] + (np.arange(Ny) + 0.5) * (g.y[1] - g.y[0]) / Ny
            X, Y = np.meshgrid(xc, yc, indexing="ij")
            h = np.vectorize(bottom_height, otypes=[np.float64])(X, Y)
        else:
            h = np.asarray(bottom_height, dtype=np.float64).reshape(Nx, Ny)
        h = np.ascontiguousarray(h.ravel(order="F"))
        keep.append(h)
        g.bottom_height = h.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    g.float_type = GBO_FLOAT32 if np.dtype(float_type) == np.float32 else GBO_FLOAT64
    g._keep = keep
    return g


def model_desc(grid, closure=None, buoyancy=False, coriolis=None, tracers=(), flux_top=None, flux_bottom=None,
               pressure_solver=None, timestepper="RungeKutta3"):
    """ModelDesc of NonhydrostaticModel(grid; advection=WENO(), closure, buoyancy, coriolis,
    tracers, boundary_conditions, pressure_solver, timestepper).

    closure, pressure_solver, timestepper: None, a name, or (name, {parameters}); a parameter
    left out takes REFERENCE_DEFAULTS.  coriolis: f, or {"latitude": φ[, "rotation_rate": Ω]}.
    buoyancy: True for BuoyancyTracer (tracer b first).  flux_top / flux_bottom: {tracer: flux}.
    The pressure solver defaults as in nonhydrostatic_pressure_solver
    (NonhydrostaticModels.jl:30-76): FFT on a regular grid, Fourier-tridiagonal on a stretched one.
    """
    def named(spec):
        if spec is None:
            return None, {}
        if isinstance(spec, str):
            return spec, {}
        return spec[0], dict(spec[1])

    tracers = tuple(tracers)
    if buoyancy:
        tracers = ("b",) + tuple(t for t in tracers if t != "b")
    Nx, Ny, Nz = grid.size
    ft = np.float32 if grid.float_type == GBO_FLOAT32 else np.float64
    d = ModelDesc()
    d.advection = 5
    name, p = named(closure)
    d.closure = _CLOSURE_CODES[name]
    if name is not None:
        q = dict(REFERENCE_DEFAULTS[name], **p)
        if name == "SmagorinskyLilly":
            d.closure_C, d.closure_Cb, d.closure_Pr = q["C"], q["Cb"], q["Pr"]
        elif name == "Smagorinsky":  # constant coefficient: the Lilly form without the N² reduction
            d.closure_C, d.closure_Cb, d.closure_Pr = q["coefficient"], 0.0, q["Pr"]
        elif name == "AnisotropicMinimumDissipation":
            d.closure_C = q["C"]
        elif name == "DynamicSmagorinsky":
            d.closure_Pr, d.closure_min_numerator = q["Pr"], q["minimum_numerator"]
            d.closure_averaging = 1 if q["averaging"] == "lagrangian" else 0
        elif name == "ScalarDiffusivity":
            d.closure_nu = q["nu"]
            for n, t in enumerate(tracers):
                d.closure_kappa[n] = q["kappa"][t] if isinstance(q["kappa"], dict) else q["kappa"]
    d.ntracers = len(tracers)
    d.buoyancy_tracer = int(bool(buoyancy))
    if coriolis is not None:
        d.has_coriolis = 1
        if isinstance(coriolis, dict):
            omega = coriolis.get("rotation_rate", REFERENCE_DEFAULTS["FPlane"]["rotation_rate"])
            d.coriolis_f = 2 * omega * math.sin(math.radians(coriolis["latitude"]))
        else:
            d.coriolis_f = float(coriolis)
    for src, dst in ((flux_top or {}, d.tracer_flux_top), (flux_bottom or {}, d.tracer_flux_bottom)):
        for t, q in src.items():
            dst[tracers.index(t)] = q
    name, p = named(pressure_solver)
    if name is None:
        name = "FFTBasedPoissonSolver" if not grid.z_faces else "FourierTridiagonalPoissonSolver"
    d.pressure_solver = _SOLVER_CODES[name]
    if name == "ConjugateGradientPoissonSolver":
        q = dict(REFERENCE_DEFAULTS[name], **p)
        tol = math.sqrt(float(np.finfo(ft).eps))
        d.cg_reltol = tol if q["reltol"] == "sqrt(eps(FT))" else q["reltol"]
        d.cg_abstol = tol if q["abstol"] == "sqrt(eps(FT))" else q["abstol"]
        d.cg_maxiter = Nx * Ny * Nz if q["maxiter"] == "Nx*Ny*Nz" else q["maxiter"]
        d.preconditioner = _PRECOND_CODES[q["preconditioner"]]
    name, p = named(timestepper)
    d.timestepper = 1 if name == "QuasiAdamsBashforth2" else 0
    d.ab2_chi = dict(REFERENCE_DEFAULTS["QuasiAdamsBashforth2"], **p)["chi"]
    return d, tracers


def model(grid_kw, **physics):
    """An OracleModel from grid_desc keywords and model_desc keywords."""
    g = grid_desc(**grid_kw)
    d, tracers = model_desc(g, **physics)
    return OracleModel(g, d, tracers=tracers)


def _checked(rc):
    if rc == -4:
        raise OracleNotConverged("oracle conjugate-gradient solve hit maxiter")
    if rc != 0:
        raise RuntimeError("oracle call failed with status %d" % rc)
    return rc


def set_threads(n):
    lib().orc_set_threads(int(n))


def max_threads():
    return lib().orc_max_threads()


def weno5(stencil, left=True):
    s = np.ascontiguousarray(np.asarray(stencil, dtype=np.float64))
    return lib().orc_weno5(_dptr(s), int(bool(left)))


# ---------------------------------------------------------------------------
# run!(simulation) restated over the oracle model (FP64): the checker of the
# device-side simulation loop of the library.
# ---------------------------------------------------------------------------
STOP_TIME, STOP_ITERATION, STOP_NAN = 1, 2, 3


def cell_advection_timescale(ref):
    """min over cells of 1 / (|u|/Δxᶠᶜᶜ + |v|/Δyᶜᶠᶜ + |w|/Δzᶜᶜᶠ)
    (src/Advection/cell_advection_timescale.jl:15-36); w at the bottom face of each cell."""
    g = ref.grid
    Nx, Ny, Nz = ref.shape
    rdx, rdy = 1 / ((g.x[1] - g.x[0]) / Nx), 1 / ((g.y[1] - g.y[0]) / Ny)
    inv = np.abs(ref.get("u")) * rdx + np.abs(ref.get("v")) * rdy
    if not ref.flat:
        H = 4 if g.bottom_height else 3
        _, dzf = ref.z_spacings()
        inv = inv + np.abs(ref.get("w")[:, :, :Nz]) * (1 / dzf[H:H + Nz])[None, None, :]
    with np.errstate(divide="ignore"):
        return float(np.min(1 / inv))


def cell_diffusion_timescale(ref):
    """Diffusion timescale of the closure (TurbulenceClosures/turbulence_closure_diagnostics.jl:8-13,
    48-63): Δ² / (max νₑ max(1, 1/Pr)) for Smagorinsky (Lilly or dynamic), min(Δ²/max νₑ, Δ²/max κₑ) for AMD
    (max κₑ = Inf without tracers), Inf without a closure; Δ = min(Δx, Δy, min Δzᶜ)."""
    g, d = ref.grid, ref.desc
    if d.closure == 0:
        return math.inf
    Nx, Ny, Nz = ref.shape
    D = min((g.x[1] - g.x[0]) / Nx, (g.y[1] - g.y[0]) / Ny)
    if not ref.flat:
        H = 4 if g.bottom_height else 3
        dzc, _ = ref.z_spacings()
        D = min(D, float(np.min(dzc[H:H + Nz])))
    d2 = np.float64(D * D)
    numax = np.max(ref.get("nu"))
    with np.errstate(divide="ignore"):  # Δ²/0 = Inf as in Julia
        if d.closure in (1, 4):  # every Smagorinsky, the dynamic one included
            pr = d.closure_Pr if d.ntracers > 0 else 1.0
            return float(d2 / (numax * max(1.0, 1 / pr)))
        kmax = np.max(ref.get("kappa")) if d.ntracers > 0 else np.inf
        return float(min(d2 / numax, d2 / kmax))


def new_time_step(old_dt, tau_adv, tau_dif, cfl=0.2, diffusive_cfl=math.inf, max_change=1.1, min_change=0.5,
                  max_dt=math.inf, min_dt=0.0):
    """new_time_step(old_Δt, wizard, model) (src/Simulations/time_step_wizard.jl:97-112)."""
    adv = cfl * tau_adv
    dif = math.inf if math.isinf(diffusive_cfl) else diffusive_cfl * tau_dif
    dt = min(adv, dif)
    dt = min(max_change * old_dt, dt)
    dt = max(min_change * old_dt, dt)
    return min(max(dt, min_dt), max_dt)


def run(ref, dt, stop_time=math.inf, stop_iteration=math.inf, align_time_step=True, nan_check_interval=100,
        wizard=None, wizard_interval=10, float_type=np.float64):
    """run!(Simulation(model; Δt, stop_time, stop_iteration, align_time_step)) with the default
    NaNChecker and an optional TimeStepWizard (keyword dict) on IterationInterval(wizard_interval)
    (src/Simulations/run.jl:151-262, simulation.jl:68-119,243-269, run.jl:319-347).  Δt and
    stop_time are rounded to the model's float type as Simulation does.  Returns the final
    simulation Δt, the steps taken, the first stop reason and whether a NaN was found."""
    ft = float_type
    sim_dt = float(ft(dt))
    stop_time = float(ft(stop_time))
    st = {"running": True, "reason": 0, "nan": False, "dt": sim_dt}

    def callbacks(every):
        t, it = ref.clock()
        if t >= stop_time:
            st["running"] = False
            st["reason"] = st["reason"] or STOP_TIME
        if it >= stop_iteration:
            st["running"] = False
            st["reason"] = st["reason"] or STOP_ITERATION
        if nan_check_interval > 0 and (every or it % nan_check_interval == 0) and np.isnan(ref.get("u")).any():
            st["running"] = False
            st["nan"] = True
            st["reason"] = st["reason"] or STOP_NAN
        if wizard is not None and wizard_interval > 0 and (every or it % wizard_interval == 0):
            new = new_time_step(st["dt"], cell_advection_timescale(ref), cell_diffusion_timescale(ref), **wizard)
            st["dt"] = float(ft(new))

    if ref.clock()[1] == 0:  # initialize!(sim) of a fresh simulation
        callbacks(True)
    steps = 0
    while True:
        step_dt = st["dt"]
        if align_time_step:
            a = min(step_dt, stop_time - ref.clock()[0])
            step_dt = step_dt if a <= 0 else a
        ref.time_step(step_dt, 1)
        steps += 1
        callbacks(False)
        if not st["running"]:
            break
    return {"dt": st["dt"], "steps": steps, "reason": st["reason"], "nan": st["nan"]}
