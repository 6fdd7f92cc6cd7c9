"""Tile copies of the stencil kernels on grids whose x size is not a multiple of a
16-byte chunk, against the FP64 CPU oracle, through the C ABI.

The fused tendency kernel, the tiled Smagorinsky and AMD closures and the
DynamicSmagorinsky tiles copy their shared-memory tiles in 16-byte chunks when Nx is a
multiple of the chunk width (4 values in FP32, 2 in FP64) and the fields are aligned,
and one value per copy otherwise.  Nx = 30 sends FP32 models down the one-value path
(every other FP32 parity test runs the chunked one) and gives FP64 models a domain
narrower than one 32-column tile, whose chunks wrap around the periodic seam more than
once.  Ny = 20 leaves a partial tile in y.  Tolerances: the FP32 bar of the other FP32
parity tests (1e-4 relative L2 after 10 steps) and the FP64 bar (1e-12 after a step;
νₑ of the dynamic closures 1e-10, see test_gpu_dynamic_smagorinsky.py).
"""
import numpy as np
import pytest

import cases
import oceananigans_gb300 as og

pytestmark = pytest.mark.gpu

SIZE = (30, 20, 16)


def compare(model, ref, names, tol):
    errs = {n: cases.rel_l2(model.get(n), ref.get(n)) for n in names}
    bad = {n: e for n, e in errs.items() if not e <= tol}
    assert not bad, "relative L2 above %.1e: %s (all: %s)" % (tol, bad, errs)
    return errs


@pytest.mark.parametrize("closure", ["smagorinsky", "amd", "dynamic", "lagrangian"])
def test_fp32_one_value_copies(closure):
    c64 = cases.convection_3d(SIZE, closure=closure, N2=1e-7, U0=2e-2)
    c32 = cases.convection_3d(SIZE, closure=closure, N2=1e-7, U0=2e-2, float_type=np.float32)
    m, r = c32.start_gpu(), c64.start_oracle()
    og.time_step_(m, 2.0, 10)
    r.time_step(2.0, 10)
    compare(m, r, ("u", "v", "w", "b"), 1e-4)


@pytest.mark.parametrize("closure", ["smagorinsky", "amd", "dynamic", "lagrangian"])
def test_fp64_domain_narrower_than_a_tile(closure):
    c = cases.convection_3d(SIZE, closure=closure, N2=1e-7, U0=2e-2)
    m, r = c.start_gpu(), c.start_oracle()
    og.time_step_(m, 2.0)
    r.time_step(2.0)
    compare(m, r, ("u", "v", "w", "b"), 1e-12)
    compare(m, r, ("nu",), 1e-12 if closure in ("smagorinsky", "amd") else 1e-10)
