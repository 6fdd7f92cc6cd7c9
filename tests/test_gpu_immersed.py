"""GPU parity on an ImmersedBoundaryGrid (GridFittedBottom seamount) against the
FP64 oracle, through the C ABI: the naive spectral projection, the
conjugate-gradient projection with the FFT / Fourier-tridiagonal
preconditioner and without one, and the CG Poisson solve itself.

Tolerances: the spectral paths are deterministic and match within 1e-12
relative L2 after one step, 1e-8 after ten.  The CG paths run to a relative
residual of 1e-13 on both sides, so the two solutions agree to about that
level; fields are compared within 1e-10 after one step and 1e-8 after five,
and the iteration counts within one.
"""
import numpy as np
import pytest

import cases
import oceananigans_gb300 as og
from test_gpu_parity import compare

pytestmark = pytest.mark.gpu

FIELDS = ("u", "v", "w", "b", "p", "pHY")


@pytest.mark.parametrize("stretched", [False, True])
def test_seamount_spectral_projection_fp64(stretched):
    c = cases.seamount((32, 32, 16), solver="fft", stretched=stretched)
    m, r = c.start_gpu(), c.start_oracle()
    compare(m, r, FIELDS, 1e-12)
    og.time_step_(m, 50.0)
    r.time_step(50.0)
    compare(m, r, FIELDS, 1e-12)
    og.time_step_(m, 50.0, 9)
    r.time_step(50.0, 9)
    compare(m, r, FIELDS, 1e-8)


@pytest.mark.parametrize("solver,stretched", [("cg", False), ("cg", True), ("cg-none", False)])
def test_seamount_cg_projection_fp64(solver, stretched):
    c = cases.seamount((32, 32, 16), solver=solver, reltol=1e-13, abstol=1e-300, stretched=stretched)
    m, r = c.start_gpu(), c.start_oracle()
    compare(m, r, FIELDS, 1e-10)
    assert abs(m.solver_iterations - r.last_cg_iterations()) <= 1
    og.time_step_(m, 50.0)
    r.time_step(50.0)
    compare(m, r, FIELDS, 1e-10)
    assert abs(m.solver_iterations - r.last_cg_iterations()) <= 1
    og.time_step_(m, 50.0, 4)
    r.time_step(50.0, 4)
    compare(m, r, FIELDS, 1e-8)
    imm = cases.immersed_mask(c.grid)
    assert np.all(m.get("b")[imm] == 0.0)
    assert np.all(m.get("u")[imm | np.roll(imm, 1, 0)] == 0.0)


@pytest.mark.parametrize("reltol,tol", [(1e-5, 2e-3), (0.0, 5e-2)])
def test_seamount_fp32_cg(reltol, tol):
    # FP32 state and CG vectors (dot products accumulate in FP64) against the converged FP64
    # oracle; reltol 0 selects the defaults reltol = abstol = sqrt(eps(Float32)), where the
    # absolute tolerance (in s⁻¹) stops the iteration early and bounds the agreement
    c32 = cases.seamount((32, 32, 16), float_type=np.float32, solver="cg", reltol=reltol,
                         abstol=1e-300 if reltol else 0.0)
    c64 = cases.seamount((32, 32, 16), solver="cg", reltol=1e-13, abstol=1e-300)
    m, r = c32.start_gpu(), c64.start_oracle()
    og.time_step_(m, 50.0, 3)
    r.time_step(50.0, 3)
    errs = compare(m, r, ("u", "v", "w", "b"), tol)
    print("fp32 CG (reltol %g) vs fp64 oracle after 3 steps:" % reltol, errs, "iterations", m.solver_iterations)
    imm = cases.immersed_mask(c32.grid)
    assert np.all(m.get("b")[imm] == 0.0)


def test_cg_poisson_solve_against_oracle():
    torch = pytest.importorskip("torch")
    for solver in ("cg", "cg-none"):
        c = cases.seamount((32, 32, 16), solver=solver, reltol=1e-13, abstol=1e-300)
        m, r = c.gpu_model(), c.oracle_model()
        imm = cases.immersed_mask(c.grid)
        rng = np.random.default_rng(5)
        b = rng.standard_normal(imm.shape)
        b[imm] = 0.0
        b[~imm] -= b[~imm].mean()
        rhs = torch.tensor(b.ravel(order="F"), dtype=torch.float64, device="cuda")
        phi = torch.zeros_like(rhs)
        m.poisson_solve_device(phi.data_ptr(), rhs.data_ptr())
        got = phi.cpu().numpy().reshape(b.shape, order="F")
        want = r.poisson_solve(b)
        assert cases.rel_l2(got, want) < 1e-11
        assert abs(m.solver_iterations - r.last_cg_iterations()) <= 1


def test_fft_preconditioned_cg_one_iteration_without_immersed_cells():
    torch = pytest.importorskip("torch")
    c = cases.seamount((32, 32, 16), solver="cg", reltol=1e-12, abstol=1e-300, height=-500.0)
    m = c.gpu_model()
    rng = np.random.default_rng(6)
    b = rng.standard_normal((32, 32, 16))
    b -= b.mean()
    rhs = torch.tensor(b.ravel(order="F"), dtype=torch.float64, device="cuda")
    phi = torch.zeros_like(rhs)
    m.poisson_solve_device(phi.data_ptr(), rhs.data_ptr())
    assert m.solver_iterations == 1


@pytest.mark.parametrize("closure", ["smagorinsky", "amd"])
def test_seamount_closure_fp64(closure):
    # turbulence closures on the immersed grid: conditional strain rates and diffusive
    # fluxes zeroed on the immersed periphery (immersed_diffusive_fluxes.jl:25-44)
    c = cases.seamount((32, 32, 16), solver="cg", reltol=1e-13, abstol=1e-300, closure=closure, U=0.02, noise=2e-2)
    m, r = c.start_gpu(), c.start_oracle()
    names = FIELDS + ("nu",) + (("kappa",) if closure == "amd" else ())
    compare(m, r, names, 1e-10)
    og.time_step_(m, 20.0)
    r.time_step(20.0)
    compare(m, r, names, 1e-10)
    og.time_step_(m, 20.0, 4)
    r.time_step(20.0, 4)
    compare(m, r, names, 1e-8)
