"""CPU tests of the FP64 oracle: analytic and property checks that pin it to
the reference's own tests (the Julia reference cannot run here)."""
import numpy as np
import pytest

import cases
import oracle


def test_projection_is_divergence_free_2d():
    # set! projects the initial velocities (set_nonhydrostatic_model.jl:65-70)
    c = cases.turbulence_2d(32)
    r = c.start_oracle()
    u, v = r.get("u"), r.get("v")
    dx = 2 * np.pi / 32
    div = (np.roll(u, -1, 0) - u) / dx + (np.roll(v, -1, 1) - v) / dx
    assert abs(div).max() < 1e-12


def _divergence_3d(r, case):
    g = case.grid
    u, v, w = r.get("u"), r.get("v"), r.get("w")
    dx, dy = g.Lx / g.Nx, g.Ly / g.Ny
    dzc, _ = r.z_spacings()
    dz = dzc[3:3 + g.Nz]
    return (np.roll(u, -1, 0) - u) / dx + (np.roll(v, -1, 1) - v) / dy + (w[:, :, 1:] - w[:, :, :-1]) / dz


@pytest.mark.parametrize("stretched", [False, True])
def test_incompressibility_after_steps(stretched):
    # test/test_time_stepping.jl:138-171: max |div u| small after 1 and 10 steps
    c = cases.convection_3d((16, 16, 12), closure="amd" if stretched else "smagorinsky", stretched=stretched,
                            N2=1e-7, U0=2e-2)
    r = c.start_oracle()
    for n in (1, 9):
        r.time_step(1.0, n)
        assert abs(_divergence_3d(r, c)).max() < 5e-8
    w = r.get("w")
    assert np.all(w[:, :, 0] == 0) and np.all(w[:, :, -1] == 0)


def test_poisson_analytic_mode():
    # dependencies_for_poisson_solvers.jl:139-165: a single eigenmode is solved exactly
    c = cases.convection_3d((16, 12, 10))
    r = c.oracle_model()
    g = c.grid
    xc, yc, zc = g.nodes()
    X, Y, Z = np.meshgrid(xc, yc, zc, indexing="ij")
    kx, ky, kz = 2 * np.pi * 2 / g.Lx, 2 * np.pi * 1 / g.Ly, np.pi * 3 / g.Lz
    phi = np.cos(kx * X) * np.cos(ky * Y) * np.cos(kz * (Z - g.z[0]))
    dx, dy, dz = g.Lx / g.Nx, g.Ly / g.Ny, g.Lz / g.Nz
    lam = (2 * np.sin(kx * dx / 2) / dx) ** 2 + (2 * np.sin(ky * dy / 2) / dy) ** 2 + (2 * np.sin(kz * dz / 2) / dz) ** 2
    got = r.poisson_solve(-lam * phi)
    assert np.abs(got - phi).max() < 1e-12


def test_fourier_tridiagonal_matches_dense_solve():
    # test_batched_tridiagonal_solver.jl / test_poisson_solvers_stretched_grids.jl: ∇²ϕ = R on a stretched grid
    c = cases.convection_3d((8, 6, 10), stretched=True)
    r = c.oracle_model()
    g = c.grid
    rng = np.random.default_rng(5)
    dzc_all, dzf_all = r.z_spacings()
    H = 3
    dzc = lambda k: dzc_all[k - (1 - H)]
    dzf = lambda k: dzf_all[k - (1 - H)]
    b = rng.standard_normal((8, 6, 10))
    w = np.array([dzc(k) for k in range(1, 11)])
    b -= (b * w).sum() / (w.sum() * 48)
    phi = r.poisson_solve(b)
    dx, dy = g.Lx / 8, g.Ly / 6
    lap = (np.roll(phi, -1, 0) - 2 * phi + np.roll(phi, 1, 0)) / dx ** 2 + (np.roll(phi, -1, 1) - 2 * phi + np.roll(phi, 1, 1)) / dy ** 2
    for k in range(1, 11):
        up = (phi[:, :, k] - phi[:, :, k - 1]) / dzf(k + 1) if k < 10 else 0
        dn = (phi[:, :, k - 1] - phi[:, :, k - 2]) / dzf(k) if k > 1 else 0
        lap[:, :, k - 1] += (up - dn) / dzc(k)
    assert np.abs(lap - b).max() < 1e-10
    assert abs(phi.mean()) < 1e-15 * np.abs(phi).max()


def test_weno5_reproduces_polynomials_and_is_symmetric():
    # Smooth quadratic data: WENO5 is exact for the cell-averaged reconstruction of smooth
    # low-order polynomials up to the ε-weighting; bias mirror symmetry must hold exactly.
    x = np.arange(-3, 3, dtype=float)
    s = 1.0 + 0.5 * x
    assert abs(oracle.weno5(s, True) - 0.75) < 1e-12  # linear: face value at x=-1/2
    a = np.array([1.0, 4.0, -2.0, 0.5, 3.0, 2.0])
    # right-biased reconstruction = left-biased reconstruction of the mirrored stencil
    # (the right stencils of weno_interpolants.jl:543-545 are the mirrored left ones)
    assert oracle.weno5(a, False) == oracle.weno5(a[::-1].copy(), True)


def test_stretched_grid_halo_spacings_wrap():
    # generate_coordinate (grid_generation.jl:16-19) extends spacings periodically into the halos
    c = cases.convection_3d((8, 8, 10), stretched=True)
    r = c.oracle_model()
    dzc, dzf = r.z_spacings()
    zf = c.grid.z_faces
    H = 3
    assert dzc[H] == pytest.approx(zf[1] - zf[0])           # Δzᶜ(1)
    assert dzc[H - 1] == pytest.approx(zf[-1] - zf[-2])     # Δzᶜ(0) wraps from the top
    assert dzf[H + 10] == pytest.approx(0.5 * (zf[-1] - zf[-2]) + 0.5 * (zf[1] - zf[0]))  # Δzᶠ(Nz+1)


@pytest.mark.parametrize("closure", ["scalar", "smagorinsky", "amd", "dynamic"])
def test_tracer_mean_conserved(closure):
    # test_time_stepping.jl:179-213 (tracer_conserved_in_channel) within this path:
    # Periodic x, y and Bounded z without boundary fluxes, each closure, a
    # buoyancy tracer of mean ~10 with a vertical gradient and noise; the mean after
    # 10 steps equals the initial one within Nx·Ny·Nz·eps, the reference's tolerance
    c = cases.convection_3d((16, 16, 16), closure=closure, flux=0.0, N2=5e-3, U0=2e-2, seed=7)
    c.init["b"] = c.init["b"] + 10.0
    r = c.start_oracle()
    b0 = r.get("b").mean()
    r.time_step(2.0, 10)
    b1 = r.get("b").mean()
    assert abs(b1 - b0) <= 16 ** 3 * np.finfo(np.float64).eps
    assert not np.allclose(r.get("b"), c.init["b"])  # the flow did move the tracer
