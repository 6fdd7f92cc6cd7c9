"""Size-independent properties at the benchmark sizes (where the FP64 oracle is too
slow to compare against): incompressibility after the projection, conservation of
tracer and horizontal momentum in a periodic, wall-bounded box without fluxes or
Coriolis (flux-form advection and closure fluxes telescope, the walls carry no flux,
pressure gradients sum to zero), and divergence-free active cells on the immersed
grid.  Tolerances are FP32 roundoff bounds, stated per test."""
import numpy as np
import pytest

import cases
import oceananigans_gb300 as og

pytestmark = pytest.mark.gpu


def _divergence(m, dzc):
    g = m.grid
    u, v, w = (m.get(n).astype(np.float64) for n in ("u", "v", "w"))
    dx, dy = g.Lx / g.Nx, g.Ly / g.Ny
    return (np.roll(u, -1, 0) - u) / dx + (np.roll(v, -1, 1) - v) / dy + (w[:, :, 1:] - w[:, :, :-1]) / dzc[None, None, :], \
        max(np.abs(u).max() / dx, np.abs(v).max() / dy)


@pytest.mark.parametrize("closure", ["smagorinsky", "amd"])
def test_convection_256x256x128_incompressible_and_conservative(closure):
    c = cases.convection_3d((256, 256, 128), float_type=np.float32, closure=closure, flux=0.0, f=0.0, U0=2e-2, N2=1e-6)
    m = c.start_gpu()
    b0 = m.get("b").astype(np.float64).sum()
    u0 = m.get("u").astype(np.float64).sum()
    og.time_step_(m, 2.0, 10)
    div, scale = _divergence(m, np.full(128, 256.0 / 128))
    # FP32 projection: the residual divergence is roundoff of the FFT solve
    assert np.abs(div).max() <= 1e-4 * scale
    b1 = m.get("b").astype(np.float64)
    assert abs(b1.sum() - b0) <= 1e-6 * np.abs(b1).sum()
    u1 = m.get("u").astype(np.float64)
    assert abs(u1.sum() - u0) <= 1e-5 * np.abs(u1).sum()


def test_stretched_amd_512x512x256_incompressible():
    c = cases.convection_3d((512, 512, 256), float_type=np.float32, closure="amd", stretched=True, flux=0.0, f=0.0,
                            U0=2e-2, N2=1e-6)
    m = c.start_gpu()
    og.time_step_(m, 1.0, 2)
    zf = np.array([-256.0 * (1 - np.tanh(2 * (k / 256)) / np.tanh(2)) for k in range(257)])
    div, scale = _divergence(m, np.diff(zf))
    assert np.abs(div).max() <= 1e-4 * scale


def test_seamount_256x256x128_active_cells_divergence_free():
    c = cases.seamount((256, 256, 128), float_type=np.float32, solver="cg", reltol=1e-7, abstol=1e-30)
    m = c.start_gpu()
    og.time_step_(m, 20.0, 3)
    div, scale = _divergence(m, np.full(128, 2000.0 / 128))
    imm = cases.immersed_mask(c.grid)
    # the CG stops at a 1e-7 relative residual in the V-weighted norm
    assert np.abs(div[~imm]).max() <= 1e-3 * scale
    assert np.all(m.get("b")[imm] == 0.0)
