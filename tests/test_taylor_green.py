"""The reference's Taylor-Green vortex known-answer test (test/test_dynamics.jl:214-259,
run there with QuasiAdamsBashforth2): u = -sin(2πy) e^(-4π²νt), v = sin(2πx) e^(-4π²νt)
on a 64 x 64 x Nz grid of extent (1, 1, 1), ScalarDiffusivity ν = 1, 10 steps of
Δt = Δx² / (10πν); the reference asserts max |u - u_exact| / |u_exact| < 5e-6, and the
same for v.

The reference builds the model with its default Centered() advection; this library and
its oracle implement WENO(order=5), which the test uses instead (the advection of this
flow is balanced by the pressure gradient, and its 64-points-per-wavelength sinusoids
are resolved far below the bar either way), and 8 levels in z instead of 2 (the library
needs at least 6 on a Bounded z; the flow does not depend on z).  Both the FP64 oracle
(CPU) and the library (GPU) must pass the reference's bar."""
import math

import numpy as np
import pytest

import cases
import oceananigans_gb300 as og

N, NZ, NT, NU = 64, 8, 10, 1.0
DX = 1.0 / N
DT = (1 / (10 * math.pi)) * DX ** 2 / NU


def u_exact(x, y, t):
    return -np.sin(2 * np.pi * y) * np.exp(-4 * np.pi ** 2 * NU * t)


def v_exact(x, y, t):
    return np.sin(2 * np.pi * x) * np.exp(-4 * np.pi ** 2 * NU * t)


def fields(t):
    """u at (xᶠ, yᶜ), v at (xᶜ, yᶠ), broadcast over z."""
    xc, xf = (np.arange(N) + 0.5) * DX, np.arange(N) * DX
    yc, yf = xc, xf
    u = u_exact(xf[:, None], yc[None, :], t)
    v = v_exact(xc[:, None], yf[None, :], t)
    return (np.broadcast_to(u[:, :, None], (N, N, NZ)).copy(), np.broadcast_to(v[:, :, None], (N, N, NZ)).copy())


def case():
    # extent = (1, 1, 1): x, y in (0, 1), z in (-1, 0), Periodic x, y, Bounded z (the defaults)
    gkw = dict(size=(N, N, NZ), x=(0, 1), y=(0, 1), z=(-1, 0), topology=("Periodic", "Periodic", "Bounded"))
    u0, v0 = fields(0.0)
    return cases.Case(og.RectilinearGrid(**gkw), {"u": u0, "v": v0}, gkw,
                      dict(closure=("ScalarDiffusivity", {"nu": NU, "kappa": 0.0}), timestepper="QuasiAdamsBashforth2"),
                      advection=og.WENO(), closure=og.ScalarDiffusivity(nu=NU, kappa=0.0),
                      timestepper="QuasiAdamsBashforth2")


def max_rel_errors(u, v, t):
    ue, ve = fields(t)
    return np.max(np.abs((u - ue) / ue)), np.max(np.abs((v - ve) / ve))


def test_oracle_taylor_green_against_the_exact_solution():
    r = case().start_oracle()
    r.time_step(DT, NT)
    t, it = r.clock()
    assert it == NT
    eu, ev = max_rel_errors(r.get("u"), r.get("v"), t)
    assert eu < 5e-6 and ev < 5e-6, (eu, ev)


@pytest.mark.gpu
def test_gpu_taylor_green_against_the_exact_solution():
    m = case().start_gpu()
    og.time_step_(m, DT, NT)
    eu, ev = max_rel_errors(m.get("u"), m.get("v"), NT * DT)
    assert eu < 5e-6 and ev < 5e-6, (eu, ev)
