"""CPU tests of the oracle's ScalarDiffusivity closure and QuasiAdamsBashforth2 time
stepper: the diffusing cosine of test/test_dynamics.jl:63-85 (with its tolerance),
and the exact modal amplification of each scheme.  cos(m z) on a cell-centred grid
with no-flux walls is an eigenvector of the discrete Laplacian with eigenvalue
λ = (2 cos(mΔz) - 2)/Δz², so one step multiplies it by the scheme's polynomial in λΔt."""
import numpy as np
import pytest

import cases
import oceananigans_gb300 as og

N, M = 128, 2
DZ = (np.pi / 2) / N
LAM = (2 * np.cos(M * DZ) - 2) / DZ**2  # κ = 1


def julia_isapprox(a, b, atol, rtol):
    return np.linalg.norm(a - b) <= max(atol, rtol * max(np.linalg.norm(a), np.linalg.norm(b)))


@pytest.mark.parametrize("timestepper", ["RungeKutta3", "QuasiAdamsBashforth2"])
@pytest.mark.parametrize("fieldname", ["u", "v", "c"])
def test_diffusion_cosine(fieldname, timestepper):
    c = cases.diffusion_cosine(fieldname, timestepper)
    ref = c.start_oracle()
    dt = 1e-6 * (np.pi / 2) ** 2
    ref.time_step(dt, 5)
    t = ref.clock()[0]
    _, _, zc = c.grid.nodes()
    exact = np.exp(-M**2 * t) * np.cos(M * zc)[None, None, :] * np.ones((8, 8, 1))
    assert julia_isapprox(ref.get(fieldname), exact, atol=1e-6, rtol=1e-6)


def _amplitude(ref, fieldname, c0):
    f = ref.get(fieldname)[0, 0, :]
    return float(np.dot(f, c0) / np.dot(c0, c0))


def test_modal_amplification_rk3_and_qab2():
    _, _, zc = cases.diffusion_cosine("c").grid.nodes()
    c0 = np.cos(M * zc)
    dt = 2e-5
    z = LAM * dt
    # RK3: any three-stage third-order Runge-Kutta step multiplies by 1 + z + z²/2 + z³/6
    ref = cases.diffusion_cosine("c").start_oracle()
    ref.time_step(dt, 1)
    assert _amplitude(ref, "c", c0) == pytest.approx(1 + z + z * z / 2 + z**3 / 6, rel=1e-12)
    # QAB2: the first step is Euler; then A(n+1) = A(n) + z((3/2 + χ)A(n) - (1/2 + χ)A(n-1))
    chi = 0.1
    ref = cases.diffusion_cosine("c", "QuasiAdamsBashforth2").start_oracle()
    amps = [1.0]
    for n in range(4):
        ref.time_step(dt, 1)
        amps.append(_amplitude(ref, "c", c0))
    assert amps[1] == pytest.approx(1 + z, rel=1e-12)
    for n in range(1, 4):
        expect = amps[n] + z * ((1.5 + chi) * amps[n] - (0.5 + chi) * amps[n - 1])
        assert amps[n + 1] == pytest.approx(expect, rel=1e-12)
    # a change of Δt makes the next step an Euler step again (quasi_adams_bashforth_2.jl:101)
    ref.time_step(dt / 2, 1)
    assert _amplitude(ref, "c", c0) == pytest.approx(amps[-1] * (1 + z / 2), rel=1e-12)


def test_scalar_diffusivity_descriptor():
    c = cases.diffusion_cosine("c")
    m_desc = c.oracle_model().desc
    assert m_desc.closure == 3 and m_desc.closure_nu == 1.0 and m_desc.closure_kappa[0] == 1.0
    with pytest.raises(ValueError, match="tracer"):
        og.api.model_descriptor(c.grid, advection=og.WENO(), closure=og.ScalarDiffusivity(nu=1, kappa={"d": 1.0}), tracers=("c",))
    with pytest.raises(ValueError, match="timestepper"):
        og.api.model_descriptor(c.grid, advection=og.WENO(), timestepper="SplitRungeKutta3")
