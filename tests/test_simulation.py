"""CPU tests of the run!(simulation) restatement in the oracle (src/Simulations/run.jl,
simulation.jl, time_step_wizard.jl) and of the host-side argument checks of the
Python Simulation / TimeStepWizard mirror."""
import math

import numpy as np
import pytest

import cases
import oceananigans_gb300 as og
import oracle


def test_stop_time_alignment_ends_exactly_on_stop_time():
    # aligned_time_step (run.jl:37-53): the last step is shortened to land on stop_time
    ref = cases.turbulence_2d(16).start_oracle()
    out = oracle.run(ref, 0.3, stop_time=1.0)
    t, it = ref.clock()
    assert out["reason"] == oracle.STOP_TIME
    assert it == 4 and out["steps"] == 4
    assert t == 0.3 + 0.3 + 0.3 + (1.0 - 0.8999999999999999)


def test_at_least_one_step_and_iteration_stop():
    # time_step!(sim) steps once even when initialize! already stopped the run
    ref = cases.turbulence_2d(16).start_oracle()
    out = oracle.run(ref, 0.01, stop_iteration=0)
    assert out["steps"] == 1 and ref.clock()[1] == 1
    assert out["reason"] == oracle.STOP_ITERATION
    out = oracle.run(ref, 0.01, stop_iteration=5)
    assert ref.clock()[1] == 5 and out["steps"] == 4


def test_wizard_change_limits_and_clamp():
    # new_time_step: growth limited to max_change, then clamped to max_Δt (time_step_wizard.jl:97-112)
    assert oracle.new_time_step(1.0, 100.0, math.inf, cfl=1.0) == 1.1
    assert oracle.new_time_step(1.0, 1e-3, math.inf, cfl=1.0) == 0.5
    assert oracle.new_time_step(1.0, 100.0, math.inf, cfl=1.0, max_dt=1.05) == 1.05
    assert oracle.new_time_step(1.0, 0.8, 0.5, cfl=1.0, diffusive_cfl=1.0) == 0.5
    # diffusive_cfl = Inf ignores the diffusion timescale
    assert oracle.new_time_step(1.0, 0.8, 1e-9, cfl=1.0) == 0.8


def test_wizard_run_follows_the_advective_cfl():
    ref = cases.turbulence_2d(16).start_oracle()
    tau0 = oracle.cell_advection_timescale(ref)
    out = oracle.run(ref, 1e-4, stop_iteration=30, wizard={"cfl": 0.5, "max_change": 2.0}, wizard_interval=1)
    tau = oracle.cell_advection_timescale(ref)
    # after enough doublings the step sits at cfl × the advective timescale
    assert out["dt"] == pytest.approx(0.5 * tau, rel=1e-12)
    assert 0.1 * tau0 < out["dt"] < 10 * tau0


def test_advection_timescale_restatement():
    ref = cases.convection_3d((8, 8, 6), U0=0.05, N2=1e-8).start_oracle()
    u, v, w = ref.get("u"), ref.get("v"), ref.get("w")
    dzc, dzf = cases.interior_spacings(ref, 6, H=3)
    inv = np.abs(u) / 64.0 + np.abs(v) / 64.0 + np.abs(w[:, :, :6]) / dzf[None, None, :6]
    assert oracle.cell_advection_timescale(ref) == pytest.approx(1 / inv.max(), rel=1e-14)
    # Smagorinsky: Δ = min(Δx, Δy, Δz) with Pr = 1
    nu = ref.get("nu")
    assert nu.max() > 0
    assert oracle.cell_diffusion_timescale(ref) == pytest.approx(min(64.0, dzc.min()) ** 2 / nu.max(), rel=1e-14)


def test_wizard_argument_checks():
    # TimeStepWizard throws ArgumentError for min_change ≥ 1 or max_change ≤ 1 (time_step_wizard.jl:75-77)
    with pytest.raises(ValueError, match="min_change"):
        og.TimeStepWizard(min_change=1.0)
    with pytest.raises(ValueError, match="max_change"):
        og.TimeStepWizard(max_change=1.0)


def test_simulation_time_step_keyword():
    # Simulation(model; Δt, ...) (simulation.jl:68-119); dt is the ASCII spelling, and Δt is
    # converted to the model's float type
    from types import SimpleNamespace
    import oceananigans_gb300 as og
    m = SimpleNamespace(dtype=np.float32)
    assert og.Simulation(m, Δt=0.1).dt == float(np.float32(0.1))
    assert og.Simulation(m, dt=2.0, stop_iteration=3).dt == 2.0
    with pytest.raises(ValueError, match="dt or Δt"):
        og.Simulation(m)
    with pytest.raises(ValueError, match="dt or Δt"):
        og.Simulation(m, dt=1.0, Δt=1.0)
