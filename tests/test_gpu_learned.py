"""GPU tests of the learned preconditioner correction: the BF16 tensor-core inference
kernels against the numpy network (bf16 rounding at the same points; FP32 versus FP64
accumulation flips rare last-bit roundings, hence 2e-2 relative L2 on the correction),
the flexible CG with the correction loaded, and a time step against FFT-PCG."""
import numpy as np
import pytest

import cases
import learned_ref as R
import oceananigans_gb300 as og
from oceananigans_gb300 import _lib as L

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _weights(seed=0, gain=0.5, out_gain=1.0):
    """Random network; out_gain scales the last layer.  An untrained correction is noise
    that slows the CG (at out_gain 1e-2 on the 32²×16 seamount the flexible CG breaks
    down), so the CG tests keep it at 1e-4."""
    rng = np.random.default_rng(seed)
    parts = []
    for name, ci, co in R.LAYERS:
        g = gain * (out_gain if name == "out" else 1.0)
        parts.append(rng.standard_normal(co * ci * 27) * g / np.sqrt(27 * ci))
        parts.append(0.01 * g * rng.standard_normal(co))
    return np.concatenate(parts).astype(np.float32)


def _zyx(a):  # model (x, y, z) array -> (z, y, x), the device layout
    return np.ascontiguousarray(np.asarray(a).transpose(2, 1, 0))


def _precondition(m, r_zyx, dtype):
    r = torch.from_numpy(np.ascontiguousarray(r_zyx, dtype=dtype)).cuda()
    z = torch.empty_like(r)
    m.precondition_device(r.data_ptr(), z.data_ptr())
    torch.cuda.synchronize()
    return z.cpu().numpy().astype(np.float64)


@pytest.mark.parametrize("float_type", [np.float32, np.float64])
def test_inference_matches_numpy_network(float_type):
    c = cases.seamount((32, 32, 16), float_type=float_type, solver="cg", reltol=1e-8)
    m = c.gpu_model()
    active = _zyx(~cases.immersed_mask(c.grid))
    rng = np.random.default_rng(5)
    r = rng.standard_normal(active.shape) * active
    z_fft = _precondition(m, r, float_type)
    w = _weights()
    m.set_learned_preconditioner(w)
    z = _precondition(m, r, float_type)
    got = z - z_fft
    want = R.correction(R.unpack(w), r.astype(float_type), z_fft.astype(float_type), active)
    err = np.linalg.norm(got - want) / np.linalg.norm(want)
    assert np.linalg.norm(want) > 1e-3 * np.linalg.norm(z_fft)
    assert err <= 2e-2, err
    m.set_learned_preconditioner(None)  # back to the FFT preconditioner
    assert np.array_equal(_precondition(m, r, float_type), z_fft)


def test_flexible_cg_with_learned_correction_solves_the_poisson_problem():
    c = cases.seamount((32, 32, 16), solver="cg", reltol=1e-12, abstol=1e-300)
    m = c.gpu_model()
    m.set_learned_preconditioner(_weights(out_gain=1e-4))
    imm = cases.immersed_mask(c.grid)
    rng = np.random.default_rng(3)
    b = rng.standard_normal(imm.shape)
    b[imm] = 0.0
    b[~imm] -= b[~imm].mean()
    rhs = torch.from_numpy(_zyx(b)).cuda()
    phi = torch.zeros_like(rhs)
    m.poisson_solve_device(phi.data_ptr(), rhs.data_ptr())
    torch.cuda.synchronize()
    x = phi.cpu().numpy().transpose(2, 1, 0)
    ref = c.oracle_model()
    dzc, dzf = cases.interior_spacings(ref, 16)
    lap = cases.conditional_laplacian(c.grid, x, dzc, dzf)
    assert np.abs(lap - b).max() < 1e-8 * np.abs(b).max()
    assert 0 < m.solver_iterations < 200


def test_time_step_with_learned_preconditioner_matches_fft_pcg():
    c = cases.seamount((32, 32, 16), solver="cg", reltol=1e-12, abstol=1e-300)
    a, b = c.start_gpu(), c.start_gpu()
    b.set_learned_preconditioner(_weights(out_gain=1e-4))
    og.time_step_(a, 50.0, 2)
    og.time_step_(b, 50.0, 2)
    for name in ("u", "v", "w", "b", "p"):
        assert cases.rel_l2(b.get(name), a.get(name)) <= 1e-8, name


def test_learned_preconditioner_argument_checks():
    c = cases.convection_3d((32, 32, 16))
    m = c.gpu_model()
    with pytest.raises(og.GboError, match="ConjugateGradient"):
        m.set_learned_preconditioner(_weights())
    s = cases.seamount((32, 32, 16), solver="cg").gpu_model()
    with pytest.raises(og.GboError, match="expected"):
        s.set_learned_preconditioner(_weights()[:-1])
    assert L.load().gbo_learned_weight_count() == R.weight_count()
