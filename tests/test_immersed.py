"""CPU tests of the oracle on an ImmersedBoundaryGrid: the conjugate-gradient
Poisson solver (test/test_conjugate_gradient_poisson_solver.jl) and the
immersed-boundary time step (test/test_immersed_advection.jl,
test/test_immersed_boundary_grid.jl), checked against independent numpy
restatements and against exact properties."""
import numpy as np
import pytest

import cases
import oceananigans_gb300 as og


def _random_active_source(case, seed=3):
    """Random right-hand side in the active cells with zero sum (a compatible Neumann problem)."""
    imm = cases.immersed_mask(case.grid)
    rng = np.random.default_rng(seed)
    b = rng.standard_normal(imm.shape)
    b[imm] = 0.0
    b[~imm] -= b[~imm].mean()
    return b, imm


@pytest.mark.parametrize("stretched", [False, True])
@pytest.mark.parametrize("solver", ["cg", "cg-none"])
def test_cg_solution_satisfies_conditional_poisson(solver, stretched):
    # test_conjugate_gradient_poisson_solver.jl:40-83: V∇²ϕ recovers the source on a random bottom
    c = cases.seamount((16, 16, 12), solver=solver, reltol=1e-13, abstol=1e-300, stretched=stretched)
    ref = c.oracle_model()
    b, imm = _random_active_source(c)
    x = ref.poisson_solve(b)
    dzc, dzf = cases.interior_spacings(ref, 12)
    lap = cases.conditional_laplacian(c.grid, x, dzc, dzf)
    assert np.abs(lap - b).max() < 1e-9 * np.abs(b).max()
    assert np.all(x[imm] == 0.0)                    # immersed cells are masked by the gauge
    assert abs(x[~imm].mean()) < 1e-12 * np.abs(x).max()  # zero-mean gauge over active cells
    it = ref.last_cg_iterations()
    assert 0 < it < 300
    if solver == "cg":
        # the FFT preconditioner is far better than none
        plain = cases.seamount((16, 16, 12), solver="cg-none", reltol=1e-13, abstol=1e-300,
                               stretched=stretched).oracle_model()
        plain.poisson_solve(b)
        assert it < plain.last_cg_iterations()


def test_fft_preconditioned_cg_is_exact_without_immersed_cells():
    # with no immersed cells the FFT preconditioner is the exact inverse: one iteration
    c = cases.seamount((16, 16, 12), solver="cg", reltol=1e-12, abstol=1e-300, height=-500.0)
    assert not cases.immersed_mask(c.grid).any()
    ref = c.oracle_model()
    b, _ = _random_active_source(c)
    x = ref.poisson_solve(b)
    assert ref.last_cg_iterations() == 1
    direct = cases.seamount((16, 16, 12), solver="fft", height=-500.0).oracle_model()
    dzc, _ = cases.interior_spacings(ref, 12)
    V = (c.grid.Lx / 16) * (c.grid.Ly / 16) * dzc[None, None, :]
    phi = direct.poisson_solve(b / V)  # the FFT solver takes ∇²ϕ = b / V
    phi -= phi.mean()
    assert np.abs(x - phi).max() < 1e-10 * np.abs(phi).max()


def test_immersed_grid_without_immersed_cells_matches_rectilinear():
    # an ImmersedBoundaryGrid whose bottom lies below the domain reproduces the
    # RectilinearGrid step: out-of-domain cells are inactive, so the immersed
    # reconstruction rule reduces to the Bounded-wall buffer rule
    flat = cases.seamount((16, 16, 12), solver="fft", height=-500.0)
    ref_ibg = flat.start_oracle()
    plain_grid = flat.grid.underlying_grid
    plain_ogrid = {k: v for k, v in flat.ogrid.items() if k != "bottom_height"}
    plain = cases.Case(plain_grid, flat.init, plain_ogrid,
                       dict(buoyancy=True, tracers=("b",), pressure_solver="FFTBasedPoissonSolver"),
                       advection=og.WENO(), buoyancy=og.BuoyancyTracer(), tracers=("b",),
                       pressure_solver=og.FFTBasedPoissonSolver())
    ref_plain = plain.start_oracle()
    for r in (ref_ibg, ref_plain):
        r.time_step(50.0, 2)
    for name in ("u", "v", "w", "b", "p"):
        a, b = ref_ibg.get(name), ref_plain.get(name)
        assert np.abs(a - b).max() <= 1e-13 * max(np.abs(b).max(), 1e-30), name


def test_seamount_step_masks_and_incompressibility():
    # masks: u, v, w and b vanish on the immersed periphery (mask_immersed_field.jl:65-77);
    # the CG projection makes u divergence-free in the active cells
    c = cases.seamount((16, 16, 12), solver="cg", reltol=1e-12, abstol=1e-300)
    ref = c.start_oracle()
    ref.time_step(50.0, 2)
    imm = cases.immersed_mask(c.grid)
    u, v, w, b = ref.get("u"), ref.get("v"), ref.get("w"), ref.get("b")
    assert np.all(b[imm] == 0.0)
    # u at face i is on the periphery when cell i-1 or i is immersed
    assert np.all(u[imm | np.roll(imm, 1, 0)] == 0.0)
    assert np.all(v[imm | np.roll(imm, 1, 1)] == 0.0)
    wi = w[:, :, 1:-1]
    assert np.all(wi[imm[:, :, 1:] | imm[:, :, :-1]] == 0.0)
    dzc, _ = cases.interior_spacings(ref, 12)
    dx, dy = c.grid.Lx / 16, c.grid.Ly / 16
    div = (np.roll(u, -1, 0) - u) / dx + (np.roll(v, -1, 1) - v) / dy + (w[:, :, 1:] - w[:, :, :-1]) / dzc
    assert np.abs(div[~imm]).max() < 1e-9 * 0.1 / dx
    assert 0 < ref.last_cg_iterations() < 100


@pytest.mark.parametrize("closure", ["smagorinsky", "amd"])
def test_immersed_closure_without_immersed_cells_matches_rectilinear(closure):
    # conditional strain rates and diffusive-flux masks reduce to the RectilinearGrid
    # closure when no cell is immersed
    flat = cases.seamount((16, 16, 12), solver="fft", height=-500.0, closure=closure, U=0.02, noise=2e-2)
    ref_ibg = flat.start_oracle()
    plain_ogrid = {k: v for k, v in flat.ogrid.items() if k != "bottom_height"}
    plain = cases.Case(flat.grid.underlying_grid, flat.init, plain_ogrid,
                       dict(flat.ophysics, pressure_solver="FFTBasedPoissonSolver"),
                       **dict(flat.physics, pressure_solver=og.FFTBasedPoissonSolver()))
    ref_plain = plain.start_oracle()
    for r in (ref_ibg, ref_plain):
        r.time_step(20.0, 2)
    for name in ("u", "v", "w", "b", "p", "nu"):
        a, b = ref_ibg.get(name), ref_plain.get(name)
        assert np.abs(a - b).max() <= 1e-13 * max(np.abs(b).max(), 1e-30), name


@pytest.mark.parametrize("closure", ["smagorinsky", "amd"])
def test_immersed_closure_masks_fluxes(closure):
    # with a closure the masks still hold and the active cells stay divergence-free
    c = cases.seamount((16, 16, 12), solver="cg", reltol=1e-12, abstol=1e-300, closure=closure, U=0.02, noise=2e-2)
    ref = c.start_oracle()
    ref.time_step(20.0, 2)
    imm = cases.immersed_mask(c.grid)
    u, v, w, b = ref.get("u"), ref.get("v"), ref.get("w"), ref.get("b")
    assert np.all(b[imm] == 0.0)
    assert np.all(u[imm | np.roll(imm, 1, 0)] == 0.0)
    dzc, _ = cases.interior_spacings(ref, 12)
    dx, dy = c.grid.Lx / 16, c.grid.Ly / 16
    div = (np.roll(u, -1, 0) - u) / dx + (np.roll(v, -1, 1) - v) / dy + (w[:, :, 1:] - w[:, :, :-1]) / dzc
    assert np.abs(div[~imm]).max() < 1e-9 * 0.1 / dx
    assert np.isfinite(ref.get("nu")).all()
