"""gbo_poisson_solve_fft_static, the allocation-free FFT Poisson solve, against
the model's gbo_poisson_solve_device on the same right-hand side, through the
C ABI.  Both run the same pass kernels; they differ only in where the twiddle
and eigenvalue tables are evaluated (device vs host, FP64 either way), so the
solutions agree within 1e-12 relative L2 in FP64 and 1e-5 in FP32.

The file is named so that it is collected last: the static scratch keeps the
contents of earlier calls and the pass kernels' shared-memory limits are set by
every model created before, so the test must pass after the rest of the suite
as well as alone."""
import ctypes

import numpy as np
import pytest

import cases
import oceananigans_gb300 as og
from oceananigans_gb300 import _lib as L

pytestmark = pytest.mark.gpu

CASES = [
    ("bounded", (32, 24, 20), np.float64, 1e-12),
    ("bounded", (64, 48, 32), np.float32, 1e-5),
    ("flat", (64, 64, 1), np.float64, 1e-12),
    ("flat", (96, 80, 1), np.float32, 1e-5),
]


def _case(kind, shape, float_type):
    if kind == "flat":
        gkw = dict(size=shape[:2], x=(0, 2 * np.pi), y=(0, 3.0), topology=("Periodic", "Periodic", "Flat"),
                   float_type=float_type)
        return cases.Case(og.RectilinearGrid(**gkw), {}, gkw, {}, advection=og.WENO())
    return cases.convection_3d(shape, float_type=float_type)


def _static_solve(grid, phi, rhs, torch):
    desc = grid.descriptor()
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.load().gbo_poisson_solve_fft_static(ctypes.byref(desc), ctypes.c_void_p(phi.data_ptr()),
                                               ctypes.c_void_p(rhs.data_ptr()), ctypes.c_void_p(stream))
    L.check(rc)
    torch.cuda.synchronize()


@pytest.mark.parametrize("kind,shape,float_type,tol", CASES)
def test_static_solve_matches_model_solve(kind, shape, float_type, tol):
    torch = pytest.importorskip("torch")
    tdtype = torch.float32 if float_type == np.float32 else torch.float64
    c = _case(kind, shape, float_type)
    m = c.gpu_model()
    rng = np.random.default_rng(11)
    b = rng.standard_normal(shape)
    b -= b.mean()
    rhs = torch.tensor(b.ravel(order="F"), dtype=tdtype, device="cuda")
    rhs_before = rhs.clone()
    want_t = torch.empty_like(rhs)
    m.poisson_solve_device(want_t.data_ptr(), rhs.data_ptr())
    want = want_t.cpu().numpy().astype(np.float64)
    # two calls in a row into fresh buffers poisoned with NaN: every value is written
    for _ in range(2):
        phi = torch.full_like(rhs, float("nan"))
        _static_solve(c.grid, phi, rhs, torch)
        got = phi.cpu().numpy().astype(np.float64)
        assert np.isfinite(got).all()
        assert cases.rel_l2(got, want) <= tol
    assert torch.equal(rhs, rhs_before)
    # in place: ϕ and rhs the same buffer
    inplace = rhs.clone()
    _static_solve(c.grid, inplace, inplace, torch)
    assert cases.rel_l2(inplace.cpu().numpy().astype(np.float64), want) <= tol
    if float_type == np.float64:
        # and against the FP64 oracle's own FFT solve, which shares no code with either
        # GPU path (its transforms, tables and eigenvalues are its own)
        oracle_phi = c.oracle_model().poisson_solve(b).ravel(order="F")
        assert cases.rel_l2(got, oracle_phi) <= 1e-12


def test_static_solve_rejects_grids_beyond_the_scratch():
    torch = pytest.importorskip("torch")
    grid = og.RectilinearGrid(size=(256, 256, 128), x=(0, 1), y=(0, 1), z=(-1, 0),
                              topology=("Periodic", "Periodic", "Bounded"), float_type=np.float64)
    buf = torch.zeros(8, dtype=torch.float64, device="cuda")  # never touched: the size check comes first
    desc = grid.descriptor()
    rc = L.load().gbo_poisson_solve_fft_static(ctypes.byref(desc), ctypes.c_void_p(buf.data_ptr()),
                                               ctypes.c_void_p(buf.data_ptr()), None)
    assert rc == L.GBO_ERR_INVALID
    msg = L.load().gbo_last_error(None).decode()
    assert "bytes of scratch" in msg and str(32 * 1024 * 1024) in msg
    # a stretched grid is not an FFT grid
    zf = -(1 - np.linspace(0, 1, 17)) ** 2
    sgrid = og.RectilinearGrid(size=(16, 16, 16), x=(0, 1), y=(0, 1), z=zf,
                               topology=("Periodic", "Periodic", "Bounded"), float_type=np.float64)
    sdesc = sgrid.descriptor()
    rc = L.load().gbo_poisson_solve_fft_static(ctypes.byref(sdesc), ctypes.c_void_p(buf.data_ptr()),
                                               ctypes.c_void_p(buf.data_ptr()), None)
    assert rc == L.GBO_ERR_INVALID
    assert "regular grid" in L.load().gbo_last_error(None).decode()
