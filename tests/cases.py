"""Seeded synthetic cases shared by the GPU parity tests and the oracle.

The inputs follow the workload descriptions of the path's benchmark cases
(2-D turbulence, 3-D free convection, stretched-grid convection, seamount),
scaled down so the FP64 CPU oracle finishes in seconds.  The same numpy
arrays are fed to both sides.
"""
import numpy as np

import oceananigans_gb300 as og
import oracle
from oceananigans_gb300.api import model_descriptor


class Case:
    """A grid, the NonhydrostaticModel keyword arguments and seeded initial fields."""

    def __init__(self, grid, init, **physics):
        self.grid, self.init, self.physics = grid, init, physics

    def gpu_model(self):
        return og.NonhydrostaticModel(self.grid, **self.physics)

    def oracle_model(self):
        """An FP64 oracle model with exactly the same grid and physics descriptors."""
        d = self.grid.descriptor()
        g = oracle.GridDesc()
        for f, _ in oracle.GridDesc._fields_:
            setattr(g, f, getattr(d, f))
        g._keep = d._keep
        mdesc, tracers = model_descriptor(self.grid, **self.physics)
        md = oracle.ModelDesc()
        for f, _ in oracle.ModelDesc._fields_:
            setattr(md, f, getattr(mdesc, f))
        return oracle.OracleModel(g, md, tracers=tracers)

    def start_oracle(self):
        ref = self.oracle_model()
        ref.set(**self.init)
        ref.finalize_set(True)
        return ref

    def start_gpu(self):
        m = self.gpu_model()
        og.set_(m, **self.init)
        return m


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def turbulence_2d(N=64, float_type=np.float64, seed=0):
    """2-D WENO5 turbulence on (Periodic, Periodic, Flat), u, v ~ U[-1, 1]."""
    grid = og.RectilinearGrid(size=(N, N), x=(0, 2 * np.pi), y=(0, 2 * np.pi),
                              topology=("Periodic", "Periodic", "Flat"), float_type=float_type)
    rng = np.random.default_rng(seed)
    init = {"u": rng.uniform(-1, 1, (N, N, 1)), "v": rng.uniform(-1, 1, (N, N, 1))}
    return Case(grid, init, advection=og.WENO())


def convection_3d(N=(32, 32, 16), float_type=np.float64, seed=0, L=(512.0, 512.0, 256.0),
                  closure="smagorinsky", stretched=False, N2=1e-5, flux=1e-8, f=1e-4, U0=1e-3):
    """3-D free convection: BuoyancyTracer b = N² z + 1e-8 noise, velocities 1e-3 U[-1,1]."""
    Nx, Ny, Nz = N
    if stretched:
        Lz = L[2]
        zf = np.array([-Lz * (1 - np.tanh(2 * (k / Nz)) / np.tanh(2)) for k in range(Nz + 1)])
        z = zf
    else:
        z = (-L[2], 0.0)
    grid = og.RectilinearGrid(size=N, x=(0, L[0]), y=(0, L[1]), z=z, topology=("Periodic", "Periodic", "Bounded"),
                              float_type=float_type)
    cl = og.SmagorinskyLilly() if closure == "smagorinsky" else (og.AnisotropicMinimumDissipation() if closure == "amd" else None)
    bcs = {"b": og.FieldBoundaryConditions(top=og.FluxBoundaryCondition(flux))}
    rng = np.random.default_rng(seed)
    _, _, zc = grid.nodes()
    b = N2 * zc[None, None, :] + 1e-8 * rng.standard_normal((Nx, Ny, Nz))
    init = {"u": U0 * rng.uniform(-1, 1, (Nx, Ny, Nz)),
            "v": U0 * rng.uniform(-1, 1, (Nx, Ny, Nz)),
            "w": U0 * rng.uniform(-1, 1, (Nx, Ny, Nz + 1)),
            "b": b}
    return Case(grid, init, advection=og.WENO(), closure=cl, buoyancy=og.BuoyancyTracer(),
                coriolis=og.FPlane(f) if f else None, tracers=("b",), boundary_conditions=bcs)
