"""The device-side simulation loop (gbo_run: run!(simulation) with stop criteria,
stop_time alignment, NaNChecker and TimeStepWizard as nodes of one CUDA graph) and the
CFL reductions, against the oracle's restatement of run.jl / time_step_wizard.jl and
against gbo_time_step.  FP64 tolerances are the parity bar of the time step; FP32 is
compared with the FP32 bar (1e-4 relative L2) after a few steps."""
import math

import numpy as np
import pytest

import cases
import oceananigans_gb300 as og
import oracle

pytestmark = pytest.mark.gpu


def _case(kind, float_type=np.float64):
    if kind == "smagorinsky":
        return cases.convection_3d((32, 32, 16), float_type=float_type, U0=0.05, N2=1e-8)
    if kind == "amd":
        return cases.convection_3d((32, 24, 16), float_type=float_type, closure="amd", U0=0.05, N2=1e-8)
    if kind == "seamount":
        return cases.seamount((32, 32, 16), float_type=float_type, solver="cg", reltol=1e-12, abstol=1e-300)
    return cases.turbulence_2d(64, float_type=float_type)


@pytest.mark.parametrize("float_type", [np.float64, np.float32])
@pytest.mark.parametrize("kind", ["smagorinsky", "amd", "seamount", "turbulence2d"])
def test_timescales_match_oracle(kind, float_type):
    c = _case(kind, float_type)
    m, ref = c.start_gpu(), c.start_oracle()
    tol = 1e-12 if float_type == np.float64 else 1e-5
    assert og.cell_advection_timescale(m) == pytest.approx(oracle.cell_advection_timescale(ref), rel=tol)
    expect = oracle.cell_diffusion_timescale(ref)
    got = og.cell_diffusion_timescale(m)
    if math.isinf(expect):
        assert math.isinf(got)
    else:
        assert got == pytest.approx(expect, rel=tol)


def test_run_with_fixed_dt_equals_time_steps():
    c = _case("smagorinsky", np.float32)
    a, b = c.start_gpu(), c.start_gpu()
    sim = og.Simulation(a, dt=2.0, stop_iteration=7)
    r = og.run_(sim)
    og.time_step_(b, 2.0, 7)
    assert r.steps == 7 and sim.stop_reason == "stop_iteration"
    assert a.clock == b.clock
    for name in ("u", "v", "w", "b", "p"):
        assert np.array_equal(a.get(name), b.get(name)), name


def test_run_aligns_the_last_step_with_stop_time():
    c = _case("turbulence2d")
    m, ref = c.start_gpu(), c.start_oracle()
    r = og.run_(og.Simulation(m, dt=0.03, stop_time=0.1))
    out = oracle.run(ref, 0.03, stop_time=0.1)
    assert m.clock == ref.clock()  # identical FP64 clock arithmetic
    assert r.steps == out["steps"] == 4 and r.stop_reason == oracle.STOP_TIME
    for name in ("u", "v"):
        assert cases.rel_l2(m.get(name), ref.get(name)) <= 1e-12, name


@pytest.mark.parametrize("kind", ["smagorinsky", "turbulence2d"])
def test_wizard_run_matches_oracle(kind):
    c = _case(kind)
    m, ref = c.start_gpu(), c.start_oracle()
    wiz = {"cfl": 0.4, "max_change": 1.5, "diffusive_cfl": 0.5}
    dt0 = 0.01 if kind == "turbulence2d" else 1.0
    sim = og.Simulation(m, dt=dt0, stop_iteration=12, wizard=og.TimeStepWizard(**wiz), wizard_interval=2)
    r = og.run_(sim)
    out = oracle.run(ref, dt0, stop_iteration=12, wizard=wiz, wizard_interval=2)
    assert r.steps == out["steps"] == 12
    assert sim.dt == pytest.approx(out["dt"], rel=1e-11)
    assert sim.dt != dt0
    t, it = m.clock
    assert it == 12 and t == pytest.approx(ref.clock()[0], rel=1e-11)
    for name in ("u", "v"):
        assert cases.rel_l2(m.get(name), ref.get(name)) <= 1e-10, name


def test_wizard_run_fp32_against_fp64_oracle():
    c = _case("smagorinsky", np.float32)
    m, ref = c.start_gpu(), c.start_oracle()
    wiz = {"cfl": 0.4, "max_change": 1.5}
    sim = og.Simulation(m, dt=1.0, stop_iteration=6, wizard=og.TimeStepWizard(**wiz), wizard_interval=1)
    og.run_(sim)
    out = oracle.run(ref, 1.0, stop_iteration=6, wizard=wiz, wizard_interval=1, float_type=np.float32)
    assert sim.dt == pytest.approx(out["dt"], rel=1e-5)
    for name in ("u", "v", "w", "b"):
        assert cases.rel_l2(m.get(name), ref.get(name)) <= 1e-4, name


def test_launch_chunking_does_not_change_the_run():
    c = _case("smagorinsky", np.float32)
    a, b = c.start_gpu(), c.start_gpu()
    kw = dict(dt=1.0, stop_iteration=10, wizard=og.TimeStepWizard(cfl=0.3), wizard_interval=3)
    ra = og.run_(og.Simulation(a, **kw), iterations_per_launch=3)
    rb = og.run_(og.Simulation(b, **kw), iterations_per_launch=100)
    assert ra.steps == rb.steps == 10 and ra.dt == rb.dt
    for name in ("u", "v", "w", "b"):
        assert np.array_equal(a.get(name), b.get(name)), name


def test_run_on_immersed_grid_with_cg():
    # the CG solve's conditional loop nested in the simulation loop
    c = _case("seamount")
    a, b = c.start_gpu(), c.start_gpu()
    r = og.run_(og.Simulation(a, dt=50.0, stop_iteration=3))
    og.time_step_(b, 50.0, 3)
    assert r.steps == 3 and a.clock == b.clock
    for name in ("u", "v", "w", "b", "p"):
        assert cases.rel_l2(a.get(name), b.get(name)) <= 1e-10, name


def test_nan_checker_stops_the_run():
    c = _case("turbulence2d")
    m = c.gpu_model()
    u = c.init["u"].copy()
    u[3, 5, 0] = np.nan
    og.set_(m, u=u, v=c.init["v"], enforce_incompressibility=False)
    sim = og.Simulation(m, dt=0.01, stop_iteration=50)
    r = og.run_(sim)
    # initialize!(sim) finds the NaN at iteration 0; the first time step is still taken
    assert r.steps == 1 and sim.nan_detected and sim.stop_reason == "nan"
    m2 = c.gpu_model()
    og.set_(m2, u=u, v=c.init["v"], enforce_incompressibility=False)
    with pytest.raises(og.NaNError, match="NaN found in field u"):
        og.run_(og.Simulation(m2, dt=0.01, stop_iteration=50, nan_erroring=True))


def test_wall_time_limit_and_argument_checks():
    c = _case("turbulence2d")
    m = c.start_gpu()
    r = og.run_(og.Simulation(m, dt=0.01, stop_iteration=1000, wall_time_limit=0.0), iterations_per_launch=4)
    assert r.stop_reason == og.api.L.GBO_STOP_WALL_TIME and r.steps == 4
    with pytest.raises(og.GboError, match="minimum_relative_step"):
        og.run_(og.Simulation(m, dt=0.01, stop_iteration=5, minimum_relative_step=0.1))
