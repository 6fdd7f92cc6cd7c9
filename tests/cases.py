"""Seeded synthetic cases shared by the GPU parity tests and the oracle.

The inputs follow the workload descriptions of the path's benchmark cases
(2-D turbulence, 3-D free convection, stretched-grid convection, seamount),
scaled down so the FP64 CPU oracle finishes in seconds.  The same numpy
arrays are fed to both sides.

Each case describes its configuration twice from the same plain numbers: as
the library's NonhydrostaticModel keyword objects (GPU side) and as the
oracle's own grid / model description (oracle side), whose unspecified
parameters take the reference defaults restated in the oracle.  The oracle's
configuration therefore never passes through the library under test.
"""
import numpy as np

import oceananigans_gb300 as og
import oracle


class Case:
    """A grid, the NonhydrostaticModel keyword arguments, seeded initial fields, and the
    oracle's description of the same configuration (`ogrid`: oracle.grid_desc keywords,
    `ophysics`: oracle.model_desc keywords)."""

    def __init__(self, grid, init, ogrid, ophysics, **physics):
        self.grid, self.init, self.physics = grid, init, physics
        self.ogrid, self.ophysics = ogrid, ophysics

    def gpu_model(self):
        return og.NonhydrostaticModel(self.grid, **self.physics)

    def oracle_model(self):
        """An FP64 oracle model configured by the oracle's own descriptors."""
        return oracle.model(self.ogrid, **self.ophysics)

    def start_oracle(self):
        ref = self.oracle_model()
        ref.set(**self.init)
        ref.finalize_set(True)
        return ref

    def start_gpu(self):
        m = self.gpu_model()
        og.set_(m, **self.init)
        return m

    def with_physics(self, ophysics, **physics):
        """The same grid and initial fields with other physics."""
        return Case(self.grid, self.init, self.ogrid, ophysics, **physics)


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def turbulence_2d(N=64, float_type=np.float64, seed=0):
    """2-D WENO5 turbulence on (Periodic, Periodic, Flat), u, v ~ U[-1, 1]."""
    gkw = dict(size=(N, N), x=(0, 2 * np.pi), y=(0, 2 * np.pi), topology=("Periodic", "Periodic", "Flat"),
               float_type=float_type)
    grid = og.RectilinearGrid(**gkw)
    rng = np.random.default_rng(seed)
    init = {"u": rng.uniform(-1, 1, (N, N, 1)), "v": rng.uniform(-1, 1, (N, N, 1))}
    return Case(grid, init, gkw, {}, advection=og.WENO())


# closures by name: (the library's object, the oracle's description with the reference defaults)
def _closure(name):
    return {None: (None, None),
            "smagorinsky": (og.SmagorinskyLilly, "SmagorinskyLilly"),
            "amd": (og.AnisotropicMinimumDissipation, "AnisotropicMinimumDissipation"),
            "scalar": (lambda: og.ScalarDiffusivity(nu=0.5, kappa=0.2), ("ScalarDiffusivity", {"nu": 0.5, "kappa": 0.2})),
            "dynamic": (lambda: og.DynamicSmagorinsky(averaging=(1, 2)), ("DynamicSmagorinsky", {"averaging": (1, 2)})),
            "lagrangian": (og.DynamicSmagorinsky, "DynamicSmagorinsky")}[name]


def convection_3d(N=(32, 32, 16), float_type=np.float64, seed=0, L=(512.0, 512.0, 256.0),
                  closure="smagorinsky", stretched=False, N2=1e-5, flux=1e-8, f=1e-4, U0=1e-3,
                  timestepper="RungeKutta3"):
    """3-D free convection: BuoyancyTracer b = N² z + 1e-8 noise, velocities 1e-3 U[-1,1]."""
    Nx, Ny, Nz = N
    if stretched:
        Lz = L[2]
        zf = np.array([-Lz * (1 - np.tanh(2 * (k / Nz)) / np.tanh(2)) for k in range(Nz + 1)])
        z = zf
    else:
        z = (-L[2], 0.0)
    gkw = dict(size=N, x=(0, L[0]), y=(0, L[1]), z=z, topology=("Periodic", "Periodic", "Bounded"),
               float_type=float_type)
    grid = og.RectilinearGrid(**gkw)
    cl, ocl = _closure(closure)
    cl = cl() if cl else None
    bcs = {"b": og.FieldBoundaryConditions(top=og.FluxBoundaryCondition(flux))}
    rng = np.random.default_rng(seed)
    _, _, zc = grid.nodes()
    b = N2 * zc[None, None, :] + 1e-8 * rng.standard_normal((Nx, Ny, Nz))
    init = {"u": U0 * rng.uniform(-1, 1, (Nx, Ny, Nz)),
            "v": U0 * rng.uniform(-1, 1, (Nx, Ny, Nz)),
            "w": U0 * rng.uniform(-1, 1, (Nx, Ny, Nz + 1)),
            "b": b}
    ophys = dict(closure=ocl, buoyancy=True, coriolis=f if f else None, tracers=("b",), flux_top={"b": flux},
                 timestepper=timestepper)
    return Case(grid, init, gkw, ophys, advection=og.WENO(), closure=cl, buoyancy=og.BuoyancyTracer(),
                coriolis=og.FPlane(f) if f else None, tracers=("b",), boundary_conditions=bcs,
                timestepper=timestepper)


def diffusion_cosine(fieldname, timestepper="RungeKutta3", N=128, m=2):
    """test_dynamics.jl:63-85 on a Periodic x, y grid: one of u, v, c = cos(m z) on
    z in (0, π/2), ScalarDiffusivity(ν=1, κ=1), no buoyancy, everything else zero."""
    gkw = dict(size=(8, 8, N), x=(0, 1), y=(0, 1), z=(0, np.pi / 2), topology=("Periodic", "Periodic", "Bounded"))
    grid = og.RectilinearGrid(**gkw)
    _, _, zc = grid.nodes()
    init = {name: np.zeros((8, 8, N)) for name in ("u", "v", "c")}
    init[fieldname] = np.broadcast_to(np.cos(m * zc)[None, None, :], (8, 8, N)).copy()
    ophys = dict(closure=("ScalarDiffusivity", {"nu": 1.0, "kappa": 1.0}), tracers=("c",), timestepper=timestepper)
    return Case(grid, init, gkw, ophys, advection=og.WENO(), closure=og.ScalarDiffusivity(nu=1.0, kappa=1.0),
                tracers=("c",), timestepper=timestepper)


def seamount(N=(32, 32, 16), float_type=np.float64, seed=0, solver="cg", reltol=0.0, abstol=0.0,
             height=1200.0, width=800.0, N2=1e-6, U=0.1, noise=1e-3, stretched=False, closure=None,
             timestepper="RungeKutta3"):
    """Seamount on an ImmersedBoundaryGrid(GridFittedBottom): x, y in [-5, 5] km, z in [-2, 0] km,
    h = -2000 + height exp(-(x² + y²) / (2 width²)), b = N² z, u = U + noise, v, w = noise.
    reltol = 0 / abstol = 0 leave the CG tolerances at their defaults."""
    Nx, Ny, Nz = N
    if stretched:
        zf = np.array([-2000.0 * (1 - np.tanh(1.5 * (k / Nz)) / np.tanh(1.5)) for k in range(Nz + 1)])
        z = zf
    else:
        z = (-2000.0, 0.0)

    def bottom(x, y):
        return -2000.0 + height * np.exp(-(x * x + y * y) / (2 * width * width))

    gkw = dict(size=N, x=(-5000.0, 5000.0), y=(-5000.0, 5000.0), z=z, topology=("Periodic", "Periodic", "Bounded"),
               float_type=float_type)
    under = og.RectilinearGrid(**gkw)
    grid = og.ImmersedBoundaryGrid(under, og.GridFittedBottom(bottom))
    tols = dict(([("reltol", reltol)] if reltol else []) + ([("abstol", abstol)] if abstol else []))
    if solver == "cg":
        ps = og.ConjugateGradientPoissonSolver(reltol=reltol, abstol=abstol)
        ops = ("ConjugateGradientPoissonSolver", tols)
    elif solver == "cg-none":
        ps = og.ConjugateGradientPoissonSolver(reltol=reltol, abstol=abstol, preconditioner=None)
        ops = ("ConjugateGradientPoissonSolver", dict(tols, preconditioner=None))
    elif solver == "fft":
        ps = og.FourierTridiagonalPoissonSolver() if stretched else og.FFTBasedPoissonSolver()
        ops = "FourierTridiagonalPoissonSolver" if stretched else "FFTBasedPoissonSolver"
    else:
        raise ValueError(solver)
    rng = np.random.default_rng(seed)
    _, _, zc = under.nodes()
    init = {"u": U + noise * rng.uniform(-1, 1, (Nx, Ny, Nz)),
            "v": noise * rng.uniform(-1, 1, (Nx, Ny, Nz)),
            "w": noise * rng.uniform(-1, 1, (Nx, Ny, Nz + 1)),
            "b": N2 * zc[None, None, :] + 1e-9 * rng.standard_normal((Nx, Ny, Nz))}
    cl, ocl = _closure(closure)
    ophys = dict(closure=ocl, buoyancy=True, tracers=("b",), pressure_solver=ops, timestepper=timestepper)
    return Case(grid, init, dict(gkw, bottom_height=bottom), ophys, advection=og.WENO(), buoyancy=og.BuoyancyTracer(),
                tracers=("b",), pressure_solver=ps, closure=cl() if cl else None, timestepper=timestepper)


def immersed_mask(grid):
    """Boolean (Nx, Ny, Nz) array: cell centre at or below the bottom height."""
    _, _, zc = grid.nodes()
    return zc[None, None, :] <= grid.bottom_height[:, :, None]


def conditional_laplacian(grid, x, dzc, dzf):
    """V∇²x with differences zeroed across faces that touch an immersed cell or a wall,
    restated in numpy (ImmersedBoundaries/conditional_differences.jl:15-43).  dzc: the Nz
    cell thicknesses Δzᶜ; dzf: the Nz+1 centre-to-centre spacings Δzᶠ at the faces."""
    Nx, Ny, Nz = x.shape
    imm = immersed_mask(grid)
    dx, dy = grid.Lx / Nx, grid.Ly / Ny
    Ax = dy * dzc[None, None, :]
    Ay = dx * dzc[None, None, :]
    Az = dx * dy
    fx = np.where(imm | np.roll(imm, 1, 0), 0.0, Ax * (x - np.roll(x, 1, 0)) / dx)  # west faces
    fy = np.where(imm | np.roll(imm, 1, 1), 0.0, Ay * (x - np.roll(x, 1, 1)) / dy)
    fz = np.zeros((Nx, Ny, Nz + 1))
    both = imm[:, :, 1:] | imm[:, :, :-1]
    fz[:, :, 1:-1] = np.where(both, 0.0, Az * (x[:, :, 1:] - x[:, :, :-1]) / dzf[None, None, 1:-1])
    return (np.roll(fx, -1, 0) - fx) + (np.roll(fy, -1, 1) - fy) + (fz[:, :, 1:] - fz[:, :, :-1])


def interior_spacings(ref, Nz, H=4):
    """Δzᶜ of cells 1..Nz and Δzᶠ of faces 1..Nz+1 from an oracle model (halo H)."""
    dzc, dzf = ref.z_spacings()
    return dzc[H:H + Nz], dzf[H:H + Nz + 1]
