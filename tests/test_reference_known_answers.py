"""Known-answer tests of the reference's own suite (test/test_dynamics.jl), run on the FP64
oracle with the reference's tolerances.  They anchor the oracle, which the GPU parity
tests compare the library against, to the reference's own expectations at the level of
whole time steps.  Differences from the reference's setups: WENO(order=5) advection in
place of the default Centered() (the only scheme of this path), Periodic x and y with
a Bounded z (the path's topology), and no SeawaterBuoyancy (not in the path: the
advected tracer is passive)."""
import math

import numpy as np
import pytest

import cases
import oceananigans_gb300 as og

TIMESTEPPERS = ("RungeKutta3", "QuasiAdamsBashforth2")


def _case(size, extent, init, ophys, **physics):
    gkw = dict(size=size, x=(0, extent[0]), y=(0, extent[1]), z=(-extent[2], 0),
               topology=("Periodic", "Periodic", "Bounded"))
    return cases.Case(og.RectilinearGrid(**gkw), init, gkw, ophys, advection=og.WENO(), **physics)


def _diffusive(size, init, timestepper, nu=1.0, kappa=1.0):
    ophys = dict(closure=("ScalarDiffusivity", {"nu": nu, "kappa": kappa}), tracers=("c",), timestepper=timestepper)
    return _case(size, (1, 1, 1), init, ophys, closure=og.ScalarDiffusivity(nu=nu, kappa=kappa), tracers=("c",),
                 timestepper=timestepper)


@pytest.mark.parametrize("timestepper", TIMESTEPPERS)
@pytest.mark.parametrize("fieldname", ["u", "v", "c"])
def test_diffusion_simple(fieldname, timestepper):
    # test_diffusion_simple (test_dynamics.jl:15-30): a constant field under
    # ScalarDiffusivity(ν=1, κ=1) stays that constant through 10 steps of Δt = 1
    size = (8, 8, 16)
    c = _diffusive(size, {fieldname: np.full(size, math.pi)}, timestepper)
    r = c.start_oracle()
    r.time_step(1.0, 10)
    assert np.allclose(r.get(fieldname), math.pi, rtol=1e-15, atol=0)


@pytest.mark.parametrize("timestepper", TIMESTEPPERS)
@pytest.mark.parametrize("fieldname", ["u", "v", "c"])
def test_scalar_diffusivity_budget(fieldname, timestepper):
    # test_diffusion_budget / test_ScalarDiffusivity_budget (test_dynamics.jl:32-54): the
    # mean of a random field is conserved by 10 steps of Δt = 1e-4 Δz² / κ
    # (isapprox's default relative tolerance, √eps)
    size = (8, 8, 8)
    rng = np.random.default_rng(7)
    c = _diffusive(size, {fieldname: rng.uniform(0, 1, size)}, timestepper)
    r = c.start_oracle()
    before = r.get(fieldname).mean()
    dz = 1.0 / size[2]
    r.time_step(1e-4 * dz ** 2 / 1.0, 10)
    assert r.get(fieldname).mean() == pytest.approx(before, rel=math.sqrt(np.finfo(float).eps))


@pytest.mark.parametrize("timestepper", TIMESTEPPERS)
def test_passive_tracer_advection(timestepper):
    # passive_tracer_advection_test (test_dynamics.jl:175-207): a Gaussian advected by a
    # uniform (U, V) for 100 steps of Δt = 0.05 Δx / |U|, ν = κ = 1e-12;
    # mean((T - T_exact)²) / mean(T_exact²) < 1e-4
    N, L, U, V = 128, 1.0, 0.5, 0.8
    delta, x0, y0 = L / 15, L / 2, L / 2
    dt = 0.05 * L / N / math.sqrt(U ** 2 + V ** 2)
    xc = (np.arange(N) + 0.5) * L / N

    def exact(t):
        X, Y = np.meshgrid(xc, xc, indexing="ij")
        T = np.exp(-((X - U * t - x0) ** 2 + (Y - V * t - y0) ** 2) / (2 * delta ** 2))
        return np.broadcast_to(T[:, :, None], (N, N, 2)).copy()

    size = (N, N, 2)
    init = {"u": np.full(size, U), "v": np.full(size, V), "T": exact(0.0)}
    ophys = dict(closure=("ScalarDiffusivity", {"nu": 1e-12, "kappa": 1e-12}), tracers=("T",), timestepper=timestepper)
    c = _case(size, (L, L, L), init, ophys, closure=og.ScalarDiffusivity(nu=1e-12, kappa=1e-12), tracers=("T",),
              timestepper=timestepper)
    r = c.start_oracle()
    r.time_step(dt, 100)
    t, _ = r.clock()
    num, ex = r.get("T"), exact(t)
    assert np.mean((num - ex) ** 2) / np.mean(ex ** 2) < 1e-4


def test_immersed_diffusion():
    # test_immersed_diffusion (test_dynamics.jl:87-114, 601-615): a Gaussian c = exp(-z² / 0.02)
    # diffused (κ = 1, Δt = 0.1 Δz² / κ, 100 steps) above a GridFittedBottom at z = 0 equals
    # the upper half of the same Gaussian diffused on the full z in (-0.5, 0.5), whose
    # symmetry makes the flux through z = 0 vanish.  The reference's column is Flat in x and
    # y; here 8 x 8 Periodic columns with a flat bottom carry the same one-dimensional
    # problem.  Velocities are zero and there is no buoyancy.
    Nx, Nz = 8, 128
    gkw = dict(size=(Nx, Nx, Nz), x=(0, 1), y=(0, 1), z=(-0.5, 0.5), topology=("Periodic", "Periodic", "Bounded"))
    zc = -0.5 + (np.arange(Nz) + 0.5) / Nz
    init = {"c": np.broadcast_to(np.exp(-zc ** 2 / 0.02)[None, None, :], (Nx, Nx, Nz)).copy()}
    ophys = dict(closure=("ScalarDiffusivity", {"nu": 0.0, "kappa": 1.0}), tracers=("c",))
    under = og.RectilinearGrid(**gkw)
    full = cases.Case(under, init, gkw, ophys, advection=og.WENO(), closure=og.ScalarDiffusivity(nu=0.0, kappa=1.0),
                      tracers=("c",))

    def bottom(x, y):
        return np.zeros_like(np.asarray(x, dtype=float) + np.asarray(y, dtype=float))

    imm = cases.Case(og.ImmersedBoundaryGrid(under, og.GridFittedBottom(bottom)), init, dict(gkw, bottom_height=bottom),
                     dict(ophys, pressure_solver="FFTBasedPoissonSolver"), advection=og.WENO(),
                     closure=og.ScalarDiffusivity(nu=0.0, kappa=1.0), tracers=("c",),
                     pressure_solver=og.FFTBasedPoissonSolver())
    dt = 0.1 * (1.0 / Nz) ** 2 / 1.0
    a, b = full.start_oracle(), imm.start_oracle()
    a.time_step(dt, 100)
    b.time_step(dt, 100)
    half = Nz // 2  # 0-based: the levels above z = 0
    ca, cb = a.get("c")[:, :, half:], b.get("c")[:, :, half:]
    assert np.allclose(cb, ca, rtol=math.sqrt(np.finfo(float).eps), atol=0)
    # the profile has diffused: the check compares evolved values
    assert np.max(np.abs(ca - init["c"][:, :, half:])) > 1e-2


@pytest.mark.parametrize("side", ["top", "bottom"])
def test_tracer_flux_budget(side):
    # test_nonhydrostatic_flux_budget (test_boundary_conditions_integration.jl:32-56,
    # 671-722): a tracer starting at zero under a Flux boundary condition of magnitude π
    # into the domain (−π on the top, +π on the bottom: the flux is positive upward), no
    # closure, one step of Δt = 1: the domain mean is flux t / Lz.  The reference's
    # 2 x 2 x 2 box of (0, 0.3) x (0, 0.4) x (0, 0.5) becomes 8 x 8 x 8 cells of the same box
    # (the budget does not depend on the resolution) with Periodic x and y.
    size, Lz = (8, 8, 8), 0.5
    flux = math.pi * (-1 if side == "top" else 1)
    gkw = dict(size=size, x=(0, 0.3), y=(0, 0.4), z=(0, Lz), topology=("Periodic", "Periodic", "Bounded"))
    ophys = dict(tracers=("c",), **{"flux_" + side: {"c": flux}})
    bc = og.FieldBoundaryConditions(**{side: og.FluxBoundaryCondition(flux)})
    c = cases.Case(og.RectilinearGrid(**gkw), {"c": np.zeros(size)}, gkw, ophys, advection=og.WENO(), tracers=("c",),
                   boundary_conditions={"c": bc})
    r = c.start_oracle()
    r.time_step(1.0, 1)
    t, _ = r.clock()
    assert r.get("c").mean() == pytest.approx(math.pi * t / Lz, rel=math.sqrt(np.finfo(float).eps))


def _analytic_poisson_l1(N, mode):
    # analytical_poisson_solver_test (dependencies_for_poisson_solvers.jl:139-165) on
    # (Periodic, Periodic, Bounded) over (0, 2π)³: Ψ = cos(n x) cos(n y) cos(n z / 2),
    # ∇²Ψ = -(n² + n² + n²/4) Ψ; the L¹ error of the FFT solve against Ψ at the centres
    L = 2 * math.pi
    gkw = dict(size=(N, N, N), x=(0, L), y=(0, L), z=(0, L), topology=("Periodic", "Periodic", "Bounded"))
    r = cases.Case(og.RectilinearGrid(**gkw), {}, gkw, dict(pressure_solver="FFTBasedPoissonSolver")).oracle_model()
    c = (np.arange(N) + 0.5) * L / N
    X, Y, Z = np.meshgrid(c, c, c, indexing="ij")
    psi = np.cos(mode * X) * np.cos(mode * Y) * np.cos(mode * Z / 2)
    f = -(mode ** 2 + mode ** 2 + (mode / 2) ** 2) * psi
    return np.mean(np.abs(r.poisson_solve(f) - psi))


@pytest.mark.parametrize("sizes,mode", [((64, 128), 1), ((67, 131), 2)])
def test_fft_poisson_solver_second_order_convergence(sizes, mode):
    # poisson_solver_convergence (dependencies_for_poisson_solvers.jl:167-178, run by
    # test_poisson_solvers.jl:110-117): the L¹ error falls at rate 2 between two
    # resolutions, isapprox(rate, 2, rtol=5e-3); the reference's two pairs (the second of
    # prime sizes, which the oracle's transforms take and the GPU passes do not)
    n1, n2 = sizes
    e1, e2 = _analytic_poisson_l1(n1, mode), _analytic_poisson_l1(n2, mode)
    rate = math.log(e1 / e2) / math.log(n2 / n1)
    assert rate == pytest.approx(2, rel=5e-3), rate


def test_inertial_oscillation():
    # inertial_oscillations_work_with_rotation_in_different_axis (test_dynamics.jl:354-396),
    # its FPlane half: a uniform u = 1 under FPlane(f = 1), no buoyancy, tracers or closure,
    # RungeKutta3 with Δt = 1e-3 to t = π (half an inertial period, the last step shortened
    # to land on it, as run! with a stop_time does): w stays exactly 0 and the speed stays
    # 1 (isapprox, √eps); the velocity has turned to (u, v) = (cos t, -sin t) = (-1, 0)
    # within the RK3 error.  The reference's grid has no points (Flat x, y, z); here a
    # uniform flow on 8 x 8 x 8 Periodic, Periodic, Bounded cells.
    size = (8, 8, 8)
    gkw = dict(size=size, x=(0, 1), y=(0, 1), z=(-1, 0), topology=("Periodic", "Periodic", "Bounded"))
    c = cases.Case(og.RectilinearGrid(**gkw), {"u": np.ones(size)}, gkw, dict(coriolis=1.0),
                   advection=og.WENO(), coriolis=og.FPlane(1.0))
    r = c.start_oracle()
    dt, stop = 1e-3, math.pi
    n = int(stop / dt)
    r.time_step(dt, n)
    r.time_step(stop - n * dt)
    t, _ = r.clock()
    assert t == pytest.approx(stop, rel=1e-15)
    u, v, w = r.get("u"), r.get("v"), r.get("w")
    assert np.all(w == 0.0)
    assert np.allclose(np.hypot(u, v), 1.0, rtol=math.sqrt(np.finfo(float).eps), atol=0)
    assert np.allclose(u, math.cos(t), atol=1e-7) and np.allclose(v, -math.sin(t), atol=1e-7)


def test_stratified_fluid_remains_at_rest():
    # stratified_fluid_remains_at_rest_with_tilted_gravity_buoyancy_tracer
    # (test_dynamics.jl:261-304) at θ = 0, one of the reference's angles (:722-729):
    # b = N² z with N² = 1e-5 in a 2000 m box, no closure, 6 steps of 10 minutes; the
    # fluid stays at rest and ∂z b = N² everywhere (isapprox), ∂y b = 0.  The reference's
    # Gradient(N²) condition on b at the walls is the path's default no-flux condition here,
    # so the walls' own faces are left out of the ∂z b check; the reference's 1 x 32 x 32
    # (Periodic, Bounded, Bounded) box is 8 x 32 x 32 Periodic, Periodic, Bounded cells.
    size, L, N2 = (8, 32, 32), 2000.0, 1e-5
    gkw = dict(size=size, x=(0, L), y=(0, L), z=(-L, 0), topology=("Periodic", "Periodic", "Bounded"))
    zc = -L + (np.arange(size[2]) + 0.5) * L / size[2]
    b0 = np.broadcast_to(N2 * zc[None, None, :], size).copy()
    c = cases.Case(og.RectilinearGrid(**gkw), {"b": b0}, gkw, dict(buoyancy=True, tracers=("b",)),
                   advection=og.WENO(), buoyancy=og.BuoyancyTracer(), tracers=("b",))
    r = c.start_oracle()
    r.time_step(600.0, 6)
    for name in ("u", "v", "w"):
        assert np.all(r.get(name) == 0.0), name
    b = r.get("b")
    dzb = np.diff(b, axis=2) / (L / size[2])
    assert np.allclose(dzb, N2, rtol=math.sqrt(np.finfo(float).eps), atol=0)
    assert np.all(np.diff(b, axis=1) == 0.0)
