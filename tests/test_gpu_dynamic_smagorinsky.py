"""DynamicSmagorinsky on the GPU against the FP64 oracle, through the C ABI: averaging=(1, 2)
and the reference's default LagrangianAveraging (dynamic_coefficient.jl:364-487).

Tolerances.  The prognostic fields keep the path's bar (1e-12 relative L2 after a step,
1e-8 after 20).  νₑ is held to 1e-10: its coefficient is the x-y mean of LᵢⱼMᵢⱼ, whose
terms cancel (Σ|LM| / |ΣLM| reaches ~900 on these levels), so the mean's roundoff, and
with it νₑ's, is that ratio times the per-cell roundoff; the GPU sums tiles in FP64 in
another order than the oracle.  On the stretched grid p keeps the 1e-11 of the other
Fourier-tridiagonal parity tests.

LagrangianAveraging: 𝒥ᴸᴹ, 𝒥ᴹᴹ start at set! as domain means of LM and MM (the same
cancellation, over the whole domain) and then relax pointwise; they and νₑ are held to
1e-10 after set! and after one step, 1e-8 after 100 steps with the prognostic fields."""
import numpy as np
import pytest

import cases
import oceananigans_gb300 as og

pytestmark = pytest.mark.gpu


def compare(model, ref, names, tol):
    errs = {n: cases.rel_l2(model.get(n), ref.get(n)) for n in names}
    bad = {n: e for n, e in errs.items() if not e <= tol}
    assert not bad, "relative L2 above %.1e: %s (all: %s)" % (tol, bad, errs)
    return errs


def test_dynamic_convection_fp64():
    c = cases.convection_3d((32, 24, 16), closure="dynamic", N2=1e-7, U0=2e-2)
    m, r = c.start_gpu(), c.start_oracle()
    compare(m, r, ("u", "v", "w", "b", "p"), 1e-12)
    compare(m, r, ("nu",), 1e-10)
    assert np.any(m.get("nu") > 0)
    og.time_step_(m, 2.0)
    r.time_step(2.0)
    compare(m, r, ("u", "v", "w", "b", "p", "pHY"), 1e-12)
    compare(m, r, ("nu",), 1e-10)
    og.time_step_(m, 2.0, 19)
    r.time_step(2.0, 19)
    compare(m, r, ("u", "v", "w", "b", "p", "nu"), 1e-8)


def test_dynamic_stretched_fourier_tridiagonal_fp64():
    c = cases.convection_3d((32, 32, 24), closure="dynamic", stretched=True, N2=1e-7, U0=2e-2)
    m, r = c.start_gpu(), c.start_oracle()
    og.time_step_(m, 1.0)
    r.time_step(1.0)
    compare(m, r, ("u", "v", "w", "b"), 1e-12)
    compare(m, r, ("p",), 1e-11)
    compare(m, r, ("nu",), 1e-10)


def test_dynamic_fp32_against_fp64_oracle():
    c64 = cases.convection_3d((32, 32, 16), closure="dynamic", N2=1e-7, U0=2e-2)
    c32 = cases.convection_3d((32, 32, 16), closure="dynamic", N2=1e-7, U0=2e-2, float_type=np.float32)
    m, r = c32.start_gpu(), c64.start_oracle()
    og.time_step_(m, 2.0, 10)
    r.time_step(2.0, 10)
    # the FP32 state against the FP64 oracle after 10 steps (the FP32 bar of the other closures)
    compare(m, r, ("u", "v", "w", "b"), 1e-4)


# ---- LagrangianAveraging ----

def test_lagrangian_convection_fp64():
    c = cases.convection_3d((32, 24, 16), closure="lagrangian", N2=1e-7, U0=2e-2)
    m, r = c.start_gpu(), c.start_oracle()
    # after set!: 𝒥 = the domain means of LM, MM from the projected velocities with the
    # halos of the values set (initialize_closure_fields! after the projection)
    assert np.ptp(m.get("jlm")) == 0 and np.ptp(m.get("jmm")) == 0
    compare(m, r, ("u", "v", "w", "b", "p"), 1e-12)
    compare(m, r, ("jlm", "jmm", "nu"), 1e-10)
    og.time_step_(m, 2.0)
    r.time_step(2.0)
    compare(m, r, ("u", "v", "w", "b", "p", "pHY"), 1e-12)
    print("after 1 step", compare(m, r, ("jlm", "jmm", "nu"), 1e-10))
    assert np.ptp(m.get("jmm")) > 0  # pointwise after the first update
    og.time_step_(m, 2.0, 99)
    r.time_step(2.0, 99)
    print("after 100 steps", compare(m, r, ("u", "v", "w", "b", "p", "jlm", "jmm", "nu"), 1e-8))


def test_lagrangian_strong_flow_clamps_the_departure_point():
    # |u| Δt above a cell width: the displacement is clamped to ±Δ (dynamic_coefficient.jl:387-389)
    c = cases.convection_3d((16, 16, 8), closure="lagrangian", N2=1e-8, U0=0.5, seed=4)
    m, r = c.start_gpu(), c.start_oracle()
    og.time_step_(m, 20.0, 2)
    r.time_step(20.0, 2)
    compare(m, r, ("u", "v", "w", "b"), 1e-11)
    compare(m, r, ("jlm", "jmm", "nu"), 1e-9)


def test_lagrangian_stretched_and_qab2_fp64():
    c = cases.convection_3d((32, 32, 24), closure="lagrangian", stretched=True, N2=1e-7, U0=2e-2)
    m, r = c.start_gpu(), c.start_oracle()
    og.time_step_(m, 1.0, 3)
    r.time_step(1.0, 3)
    compare(m, r, ("u", "v", "w", "b"), 1e-12)
    compare(m, r, ("p",), 1e-11)
    compare(m, r, ("jlm", "jmm", "nu"), 1e-10)
    c = cases.convection_3d((32, 24, 16), closure="lagrangian", N2=1e-7, U0=2e-2, timestepper="QuasiAdamsBashforth2")
    m, r = c.start_gpu(), c.start_oracle()
    og.time_step_(m, 2.0, 3)
    r.time_step(2.0, 3)
    compare(m, r, ("u", "v", "w", "b", "p"), 1e-12)
    compare(m, r, ("jlm", "jmm", "nu"), 1e-10)


def test_lagrangian_run_loop_and_restart():
    c = cases.convection_3d((32, 24, 16), closure="lagrangian", N2=1e-7, U0=2e-2)
    a, b, r = c.start_gpu(), c.start_gpu(), c.start_oracle()
    # the device-side run! loop takes Δt from its own FP64 slot: the same updates as time_step!
    og.run_(og.Simulation(a, dt=2.0, stop_iteration=4))
    og.time_step_(b, 2.0, 4)
    r.time_step(2.0, 4)
    for name in ("u", "v", "w", "b", "jlm", "jmm", "nu"):
        assert np.array_equal(a.get(name), b.get(name)), name
    compare(a, r, ("u", "v", "w", "b", "p"), 1e-12)
    compare(a, r, ("jlm", "jmm", "nu"), 1e-10)
    # 𝒥ᴸᴹ, 𝒥ᴹᴹ and previous_compute_time are prognostic (dynamic_coefficient.jl:524-539)
    state = a.prognostic_state()
    d = c.start_gpu()
    d.restore_prognostic_state_(state)
    og.time_step_(a, 2.0, 3)
    og.time_step_(d, 2.0, 3)
    for name in ("u", "v", "w", "b", "jlm", "jmm", "nu"):
        assert np.array_equal(a.get(name), d.get(name)), name


def test_lagrangian_fp32_against_fp64_oracle():
    c64 = cases.convection_3d((32, 32, 16), closure="lagrangian", N2=1e-7, U0=2e-2)
    c32 = cases.convection_3d((32, 32, 16), closure="lagrangian", N2=1e-7, U0=2e-2, float_type=np.float32)
    m, r = c32.start_gpu(), c64.start_oracle()
    og.time_step_(m, 2.0, 10)
    r.time_step(2.0, 10)
    compare(m, r, ("u", "v", "w", "b"), 1e-4)
