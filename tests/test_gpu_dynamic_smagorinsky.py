"""DynamicSmagorinsky(averaging=(1, 2)) on the GPU against the FP64 oracle, through the C ABI.

Tolerances.  The prognostic fields keep the path's bar (1e-12 relative L2 after a step,
1e-8 after 20).  νₑ is held to 1e-10: its coefficient is the x-y mean of LᵢⱼMᵢⱼ, whose
terms cancel (Σ|LM| / |ΣLM| reaches ~900 on these levels), so the mean's roundoff, and
with it νₑ's, is that ratio times the per-cell roundoff; the GPU sums tiles in FP64 in
another order than the oracle.  On the stretched grid p keeps the 1e-11 of the other
Fourier-tridiagonal parity tests."""
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
