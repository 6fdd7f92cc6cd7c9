"""GPU parity of ScalarDiffusivity and the QuasiAdamsBashforth2 time stepper against
the FP64 oracle, with the bars of the time-step parity tests (1e-12 relative L2 after
one step, 1e-8 after twenty; FP32 1e-4 against the FP64 oracle), the diffusing
cosine of test/test_dynamics.jl:63-85, and QAB2 through the simulation loop, the
checkpoint and the ensemble checks."""
import numpy as np
import pytest

import cases
import oceananigans_gb300 as og
import oracle

pytestmark = pytest.mark.gpu


def compare(model, ref, names, tol, p_tol=None):
    """Relative L2 per field.  pNHS may be held to p_tol: it solves a Poisson problem whose
    source div u* is a small difference of O(|u|) face values, so its roundoff floor is
    |u| / (|div u*| L) times that of the velocities."""
    errs = {n: cases.rel_l2(model.get(n), ref.get(n)) for n in names}
    bad = {n: e for n, e in errs.items() if not e <= (p_tol if (n == "p" and p_tol) else tol)}
    assert not bad, "relative L2 above %.1e: %s (all: %s)" % (tol, bad, errs)


@pytest.mark.parametrize("timestepper", ["RungeKutta3", "QuasiAdamsBashforth2"])
@pytest.mark.parametrize("fieldname", ["u", "v", "c"])
def test_diffusion_cosine(fieldname, timestepper):
    c = cases.diffusion_cosine(fieldname, timestepper)
    m, ref = c.start_gpu(), c.start_oracle()
    dt = 1e-6 * (np.pi / 2) ** 2
    og.time_step_(m, dt, 5)
    ref.time_step(dt, 5)
    t = m.clock[0]
    _, _, zc = c.grid.nodes()
    exact = np.exp(-4 * t) * np.cos(2 * zc)[None, None, :] * np.ones((8, 8, 1))
    got = m.get(fieldname)
    assert np.linalg.norm(got - exact) <= max(1e-6, 1e-6 * max(np.linalg.norm(got), np.linalg.norm(exact)))
    compare(m, ref, (fieldname,), 1e-12)
    # the other fields stay at roundoff of the pressure solve (about 1e-30 on both sides)
    for other in {"u", "v", "c"} - {fieldname}:
        assert np.linalg.norm(m.get(other) - ref.get(other)) <= 1e-20 * np.linalg.norm(got), other


@pytest.mark.parametrize("closure,timestepper", [("scalar", "RungeKutta3"), ("scalar", "QuasiAdamsBashforth2"),
                                                 ("smagorinsky", "QuasiAdamsBashforth2"),
                                                 (None, "QuasiAdamsBashforth2")])
def test_convection_fp64(closure, timestepper):
    c = cases.convection_3d((32, 24, 16), closure=closure, N2=1e-7, U0=2e-2, timestepper=timestepper)
    m, r = c.start_gpu(), c.start_oracle()
    names = ("u", "v", "w", "b", "p", "pHY") + (("nu",) if closure else ())
    og.time_step_(m, 2.0)
    r.time_step(2.0)
    compare(m, r, names, 1e-12, p_tol=1e-11)
    og.time_step_(m, 2.0, 19)
    r.time_step(2.0, 19)
    compare(m, r, names, 1e-8)


def test_qab2_fp32_against_fp64_oracle():
    c = cases.convection_3d((32, 32, 16), float_type=np.float32, closure="scalar", N2=1e-6, U0=2e-2,
                            timestepper="QuasiAdamsBashforth2")
    m, r = c.start_gpu(), c.start_oracle()
    og.time_step_(m, 2.0, 5)
    r.time_step(2.0, 5)
    compare(m, r, ("u", "v", "w", "b"), 1e-4)


def test_qab2_euler_step_on_every_change_of_dt():
    c = cases.convection_3d((32, 24, 16), closure="scalar", N2=1e-7, U0=2e-2, timestepper="QuasiAdamsBashforth2")
    m, r = c.start_gpu(), c.start_oracle()
    for dt, n in ((2.0, 3), (1.5, 2), (2.0, 1), (2.0, 2)):
        og.time_step_(m, dt, n)
        r.time_step(dt, n)
    assert m.clock == r.clock()
    compare(m, r, ("u", "v", "w", "b", "p"), 1e-10)


def test_immersed_scalar_diffusivity_qab2_cg():
    c = cases.seamount((32, 32, 16), solver="cg", reltol=1e-12, abstol=1e-300, closure="scalar",
                       timestepper="QuasiAdamsBashforth2")
    m, r = c.start_gpu(), c.start_oracle()
    og.time_step_(m, 20.0, 3)
    r.time_step(20.0, 3)
    compare(m, r, ("u", "v", "w", "b", "p"), 1e-9)


def test_qab2_simulation_loop_with_wizard():
    # the wizard changes Δt at every call, so each of those steps is an Euler step
    c = cases.convection_3d((32, 24, 16), closure="scalar", N2=1e-7, U0=5e-2, timestepper="QuasiAdamsBashforth2")
    m, r = c.start_gpu(), c.start_oracle()
    wiz = {"cfl": 0.3, "max_change": 1.3}
    sim = og.Simulation(m, dt=1.0, stop_iteration=9, wizard=og.TimeStepWizard(**wiz), wizard_interval=3)
    og.run_(sim, iterations_per_launch=4)
    out = oracle.run(r, 1.0, stop_iteration=9, wizard=wiz, wizard_interval=3)
    assert sim.dt == pytest.approx(out["dt"], rel=1e-11)
    assert m.clock[1] == 9 and m.clock[0] == pytest.approx(r.clock()[0], rel=1e-11)
    compare(m, r, ("u", "v", "w", "b"), 1e-10)


def test_qab2_checkpoint_restart_is_exact():
    c = cases.convection_3d((32, 32, 16), float_type=np.float32, closure="scalar", N2=1e-6, U0=2e-2,
                            timestepper="QuasiAdamsBashforth2")
    a = c.start_gpu()
    og.time_step_(a, 2.0, 3)
    state = a.prognostic_state()
    og.time_step_(a, 2.0, 4)
    b = c.gpu_model()
    b.restore_prognostic_state_(state)
    og.time_step_(b, 2.0, 4)  # G⁻ and last Δt restored: AB2 steps, no Euler restart
    assert a.clock == b.clock
    for name in ("u", "v", "w", "b", "p"):
        assert np.array_equal(a.get(name), b.get(name)), name
    rk3 = cases.convection_3d((32, 32, 16), float_type=np.float32, closure="scalar").gpu_model()
    with pytest.raises(og.GboError, match="size|timestepper"):
        rk3.restore_prognostic_state_(state)


def test_ensemble_rejects_qab2():
    c = cases.convection_3d((32, 32, 16), timestepper="QuasiAdamsBashforth2")
    with pytest.raises(ValueError, match="RungeKutta3"):
        og.Ensemble([(c.grid, c.physics)])
