"""Checkpoint / restart (prognostic_state / restore_prognostic_state!,
nonhydrostatic_model.jl:354-377): a model restored from the state of another
continues exactly as the original, bit for bit (the CG solve sums its block partials
in a fixed order, so it is deterministic too)."""
import numpy as np
import pytest

import cases
import oceananigans_gb300 as og
from oceananigans_gb300 import _lib as L

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind", ["convection_fp32", "seamount_cg"])
def test_restored_model_continues_identically(kind):
    if kind == "convection_fp32":
        c, dt, exact = cases.convection_3d((32, 32, 16), float_type=np.float32, N2=1e-6, U0=2e-2), 2.0, True
    else:
        c, dt, exact = cases.seamount((32, 32, 16), solver="cg", reltol=1e-12, abstol=1e-300), 50.0, True
    a = c.start_gpu()
    og.time_step_(a, dt, 3)
    state = a.prognostic_state()
    assert state.size == L.load().gbo_state_bytes(a._h)
    og.time_step_(a, dt, 4)
    b = c.gpu_model()
    b.restore_prognostic_state_(state)
    assert b.clock[1] == 3
    og.time_step_(b, dt, 4)
    assert a.clock == b.clock
    for name in ("u", "v", "w", "b", "p"):
        x, y = a.get(name), b.get(name)
        if exact:
            assert np.array_equal(x, y), name
        else:
            assert cases.rel_l2(y, x) <= 1e-10, name


def test_restore_rejects_a_state_of_another_model():
    a = cases.convection_3d((32, 32, 16), float_type=np.float32).start_gpu()
    state = a.prognostic_state()
    other = cases.convection_3d((32, 32, 24), float_type=np.float32).gpu_model()
    with pytest.raises(og.GboError, match="size|match"):
        other.restore_prognostic_state_(state)
    bad = state.copy()
    bad[:8] = 0
    with pytest.raises(og.GboError, match="not a state"):
        a.restore_prognostic_state_(bad)
