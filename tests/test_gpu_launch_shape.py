"""Launch shapes (gbo_get_launch_shape / gbo_set_launch_shape).

The tiles of the spectral Poisson passes change speed only: every column and line is
transformed by the same arithmetic whatever the tile, so the same steps give bitwise
equal fields.  The levels each block of the fused tendency kernel marches change where
a block starts its march; the first level of a block forms the fluxes through its
bottom face itself (in the loop they are carried from the level below, in FP32 through
the paired reconstructions), which can round differently.  Those results agree to
rounding: 1e-13 relative L2 in FP64, 1e-6 in FP32 after three steps.

The conjugate-gradient solver of an immersed grid adds its dot products' block sums in a
fixed order, so its runs are bitwise reproducible too: two runs of one seamount model, and
runs under other pass tiles, give equal fields."""
import numpy as np
import pytest

import cases
import oceananigans_gb300 as og

pytestmark = pytest.mark.gpu

TILES = dict(dct_columns=8, x_lines=2, y_columns=4)


def _case(kind):
    if kind == "convection_fp64":
        return cases.convection_3d((64, 48, 32), N2=1e-7, U0=2e-2), 2.0
    if kind == "convection_fp32":
        return cases.convection_3d((64, 64, 32), float_type=np.float32, N2=1e-7, U0=2e-2), 2.0
    if kind == "stretched_amd":
        return cases.convection_3d((32, 32, 24), closure="amd", stretched=True, N2=1e-7, U0=2e-2), 1.0
    return cases.seamount((32, 32, 16), solver="cg", reltol=1e-12, abstol=1e-300), 20.0


@pytest.mark.parametrize("kind", ["convection_fp64", "convection_fp32", "stretched_amd"])
def test_pass_tiles_give_identical_results(kind):
    c, dt = _case(kind)
    a, b = c.start_gpu(), c.start_gpu()
    b.set_launch_shape(**TILES)
    assert {k: b.launch_shape[k] for k in TILES} == TILES
    og.time_step_(a, dt, 3)
    og.time_step_(b, dt, 3)
    for name in ("u", "v", "w", "b", "p"):
        assert np.array_equal(a.get(name), b.get(name)), name


def test_pass_tiles_on_the_cg_preconditioner():
    torch = pytest.importorskip("torch")
    c, dt = _case("seamount")
    a, b = c.start_gpu(), c.start_gpu()
    b.set_launch_shape(**TILES)
    Nx, Ny, Nz = c.grid.Nx, c.grid.Ny, c.grid.Nz
    r = torch.from_numpy(np.random.default_rng(1).standard_normal((Nz, Ny, Nx))).cuda()
    za, zb = torch.zeros_like(r), torch.zeros_like(r)
    a.precondition_device(r.data_ptr(), za.data_ptr())
    b.precondition_device(r.data_ptr(), zb.data_ptr())
    assert torch.equal(za, zb)
    og.time_step_(a, dt, 3)
    og.time_step_(b, dt, 3)
    for name in ("u", "v", "w", "b", "p"):
        assert np.array_equal(a.get(name), b.get(name)), name


@pytest.mark.parametrize("float_type", [np.float64, np.float32])
def test_cg_runs_are_bitwise_reproducible(float_type):
    c = cases.seamount((32, 32, 16), float_type=float_type, solver="cg", reltol=1e-10, abstol=1e-300)
    a, b = c.start_gpu(), c.start_gpu()
    og.time_step_(a, 20.0, 4)
    og.time_step_(b, 20.0, 4)
    for name in ("u", "v", "w", "b", "p"):
        assert np.array_equal(a.get(name), b.get(name)), name
    assert a.solver_iterations == b.solver_iterations


@pytest.mark.parametrize("kind", ["convection_fp64", "convection_fp32", "seamount"])
def test_levels_per_block_agree_to_rounding(kind):
    c, dt = _case(kind)
    a, b = c.start_gpu(), c.start_gpu()
    b.set_launch_shape(levels=4)
    og.time_step_(a, dt, 3)
    og.time_step_(b, dt, 3)
    tol = 1e-6 if kind == "convection_fp32" else 1e-13
    for name in ("u", "v", "w", "b"):
        assert cases.rel_l2(b.get(name), a.get(name)) <= tol, name
    # p is the most rounding-sensitive field: the divergence it balances is a small
    # residual of large terms (FP32), and CG stops at a 1e-12 relative residual (seamount)
    ptol = 1e-3 if kind == "convection_fp32" else (1e-11 if kind == "seamount" else 1e-13)
    assert cases.rel_l2(b.get("p"), a.get("p")) <= ptol


def test_shape_change_between_steps_keeps_the_run():
    c, dt = _case("convection_fp64")
    a, b = c.start_gpu(), c.start_gpu()
    og.time_step_(a, dt, 4)
    og.time_step_(b, dt, 2)
    b.set_launch_shape(**TILES)  # drops the captured graphs; the next step recaptures
    og.time_step_(b, dt, 2)
    for name in ("u", "v", "w", "b", "p"):
        assert np.array_equal(a.get(name), b.get(name)), name


@pytest.mark.parametrize("bad", [dict(dct_columns=3), dict(dct_columns=12), dict(dct_columns=0), dict(x_lines=0),
                                 dict(y_columns=65), dict(y_columns=6), dict(levels=0), dict(levels=33)])
def test_invalid_shapes_are_rejected(bad):
    c, _ = _case("convection_fp64")
    m = c.start_gpu()
    before = m.launch_shape
    with pytest.raises(ValueError):
        m.set_launch_shape(**bad)
    assert m.launch_shape == before
