"""The reference's internal-wave known-answer test (test/test_internal_wave_dynamics.jl:1-86,
run by test/test_dynamics.jl:625-690 for NonhydrostaticModel): a packet of the linear
inertia-gravity wave solution of the Boussinesq equations (ScalarDiffusivity ν = κ = 1e-9,
BuoyancyTracer, FPlane f = 0.2, N = 1, m = 16, k = 1) on a 128 x 128 (x, z) grid of
(0, 2π) x (-2π, 0), advanced 10 steps of Δt = 0.01 / σ; the reference asserts
mean((u - u_exact)²) / mean(u_exact²) < 1e-4.

The reference runs it with its default Centered() advection; this library and its oracle
implement WENO(order=5), which the test uses instead (the wave's amplitude, 1e-3, makes the
momentum advection a small term, and WENO5 reproduces the linear background b = N² z
exactly).  The grid is Periodic in y with 8 points (the solution does not depend on y)
instead of the reference's Ny = 1 or Flat y.  The FP64 oracle (CPU) and the library (GPU)
must each pass the reference's tolerance, on u as the reference checks and on v (w is not
compared: the exact w is not discretely divergence-free, and set! projects it)."""
import math

import numpy as np
import pytest

import cases
import oceananigans_gb300 as og

NX, NY, NZ = 128, 8, 128
L = 2 * math.pi

# internal_wave_solution (test_internal_wave_dynamics.jl:4-60), background_stratification=false
NU = KAPPA = 1e-9
Z0, DELTA, A0, M, K, F, N = -L / 3, L / 20, 1e-3, 16, 1, 0.2, 1.0
SIGMA = math.sqrt((N ** 2 * K ** 2 + F ** 2 * M ** 2) / (K ** 2 + M ** 2))
DT = 0.01 / SIGMA
CG = M * SIGMA / (K ** 2 + M ** 2) * (F ** 2 / SIGMA ** 2 - 1)
U = A0 * K * SIGMA / (SIGMA ** 2 - F ** 2)
V = A0 * K * F / (SIGMA ** 2 - F ** 2)
W = A0 * M * SIGMA / (SIGMA ** 2 - N ** 2)
B = A0 * M * N ** 2 / (SIGMA ** 2 - N ** 2)


def _a(x, z, t):
    return np.exp(-(z - CG * t - Z0) ** 2 / (2 * DELTA) ** 2)


def solution(x, z, t):
    ph = K * x + M * z - SIGMA * t
    a = _a(x, z, t)
    return {"u": a * U * np.cos(ph), "v": a * V * np.sin(ph), "w": a * W * np.cos(ph),
            "b": a * B * np.sin(ph) + N ** 2 * z}


def nodes():
    dx, dz = L / NX, L / NZ
    xc, xf = (np.arange(NX) + 0.5) * dx, np.arange(NX) * dx
    zc, zf = -L + (np.arange(NZ) + 0.5) * dz, -L + np.arange(NZ + 1) * dz
    return xc, xf, zc, zf


def field(name, t):
    """The exact field at its location (u at x faces, w at z faces), broadcast over y."""
    xc, xf, zc, zf = nodes()
    x = xf if name == "u" else xc
    z = zf if name == "w" else zc
    X, Z = np.meshgrid(x, z, indexing="ij")
    return np.broadcast_to(solution(X, Z, t)[name][:, None, :], (NX, NY, len(z))).copy()


def relative_error(num, exact):
    # relative_error (test_dynamics.jl:8-13): mean squared error over the mean square
    return np.mean((num - exact) ** 2) / np.mean(exact ** 2)


def case():
    gkw = dict(size=(NX, NY, NZ), x=(0, L), y=(0, L), z=(-L, 0), topology=("Periodic", "Periodic", "Bounded"))
    init = {n: field(n, 0.0) for n in ("u", "v", "w", "b")}
    ophys = dict(closure=("ScalarDiffusivity", {"nu": NU, "kappa": KAPPA}), buoyancy=True, coriolis=F, tracers=("b",))
    return cases.Case(og.RectilinearGrid(**gkw), init, gkw, ophys, advection=og.WENO(),
                      closure=og.ScalarDiffusivity(nu=NU, kappa=KAPPA), buoyancy=og.BuoyancyTracer(),
                      coriolis=og.FPlane(F), tracers=("b",))


def test_oracle_internal_wave_against_the_exact_solution():
    r = case().start_oracle()
    r.time_step(DT, 10)
    t, it = r.clock()
    assert it == 10 and t == pytest.approx(10 * DT, rel=1e-14)
    for name in ("u", "v"):
        err = relative_error(r.get(name), field(name, t))
        assert err < 1e-4, (name, err)


@pytest.mark.gpu
def test_gpu_internal_wave_against_the_exact_solution():
    m = case().start_gpu()
    og.time_step_(m, DT, 10)
    for name in ("u", "v"):
        err = relative_error(m.get(name), field(name, 10 * DT))
        assert err < 1e-4, (name, err)
