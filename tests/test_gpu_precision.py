"""Single-precision models: tracer departures and the FP32 accuracy bar.

Tracers of FP32 models on a Bounded z are stored as departures from a per-level
reference profile (the horizontal mean of the values they were set to).  The
stratification of the convection benchmark, b = N² z + b′ with |N² z| up to
2.6e-3 and |b′| about 1e-6, loses b′ to the FP32 ulp of N² z (2.3e-10) at
every stage when b itself is stored: FP64 runs whose b is rounded to FP32 once
per step drift by 3.8e-5 (u) and 1.3e-4 (w) in 100 steps, and the FP32 model
that stored b drifted by 1.2e-4 / 4.1e-4, while an FP64 run whose u, v, w and
departures b - N² z are rounded each step stays within 2.2e-7.  These tests
check the storage (the field reads back as profile + departure, masks give
zero, the profile is the horizontal mean) and the bar: FP32 within 1e-5
relative L2 of FP64 per field after 100 steps at 256²×128.
"""
import numpy as np
import pytest

import cases
import oceananigans_gb300 as og

pytestmark = pytest.mark.gpu


def test_tracer_is_stored_as_departures_from_its_level_mean():
    c = cases.convection_3d((32, 24, 16), float_type=np.float32, seed=4)
    m = c.start_gpu()
    want = c.init["b"]
    prof = m.reference_profile("b")
    # the profile is the horizontal mean rounded to FP32, the departures are FP32 values
    assert np.allclose(prof, want.mean(axis=(0, 1)), rtol=1.2e-7, atol=0)
    assert np.array_equal(prof, prof.astype(np.float32).astype(np.float64))
    dep = (want - prof[None, None, :]).astype(np.float32).astype(np.float64)
    assert np.array_equal(m.get("b"), prof[None, None, :] + dep)
    assert np.array_equal(m.get("b", np.float32), (prof[None, None, :] + dep).astype(np.float32))
    # b' keeps its own precision: the stored field is exact to the ulp of the departures
    assert np.abs(m.get("b") - want).max() <= 1e-7 * np.abs(want - prof[None, None, :]).max()
    # FP64 models store tracers as they are
    m64 = cases.convection_3d((32, 24, 16), seed=4).start_gpu()
    assert np.all(m64.reference_profile("b") == 0.0)
    assert np.array_equal(m64.get("b"), want)


def test_departures_survive_restart_and_masks():
    c = cases.seamount((32, 32, 16), float_type=np.float32, solver="cg", reltol=1e-6, abstol=1e-30)
    m = c.start_gpu()
    og.time_step_(m, 50.0, 2)
    imm = cases.immersed_mask(c.grid)
    b = m.get("b")
    assert np.all(b[imm] == 0.0) and np.any(b[~imm] != 0.0)
    state = m.prognostic_state()
    other = c.gpu_model()
    other.restore_prognostic_state_(state)
    assert np.array_equal(other.reference_profile("b"), m.reference_profile("b"))
    assert np.array_equal(other.get("b"), b)


def test_convection_fp32_pressure_anomaly_against_fp64():
    # pHY′ of the departures plus that of the profile equals the FP64 model's pHY′
    c32 = cases.convection_3d((64, 64, 32), float_type=np.float32, seed=6)
    c64 = cases.convection_3d((64, 64, 32), seed=6)
    m32, m64 = c32.start_gpu(), c64.start_gpu()
    og.time_step_(m32, 2.0, 5)
    og.time_step_(m64, 2.0, 5)
    for name in ("b", "pHY"):
        assert cases.rel_l2(m32.get(name), m64.get(name)) <= 1e-6, name
