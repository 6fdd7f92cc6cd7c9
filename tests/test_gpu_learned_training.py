"""Training the learned correction on the GPU with the library's own kernels
(gbo_learned_trainer_*), checked against the FP64 numpy restatement of the network
and of its training loss (oracle/learned_ref.py: loss_and_grads, itself pinned to
torch autograd and to central differences by tests/test_learned.py).

The GPU path keeps activations and gradients in BF16 with FP32 accumulation; the
checker is FP64 throughout, so loss and gradients agree to the precision of BF16
storage (the bounds below), not to rounding."""
import numpy as np
import pytest

import learned_ref
from oceananigans_gb300 import learned

pytestmark = pytest.mark.gpu

N = (32, 32, 16)


def _sample(seed=0):
    rng = np.random.default_rng(seed)
    nx, ny, nz = N
    r = rng.standard_normal((nz, ny, nx)).astype(np.float32)
    z = (0.5 * r + 0.1 * rng.standard_normal((nz, ny, nx))).astype(np.float32)
    e = (z + 0.3 * rng.standard_normal((nz, ny, nx))).astype(np.float32)
    kk, jj, ii = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    active = (kk >= 4 * np.exp(-((ii - 16) ** 2 + (jj - 16) ** 2) / 40.0)).astype(np.float32)
    return r, z, e, active


def _oracle(w, r, z, e, active):
    sr, sz = learned_ref.rms(r), learned_ref.rms(z)
    feat = np.stack([r * (np.float32(1) / sr), z * (np.float32(1) / sz), active], axis=-1)
    target = (e.astype(np.float64) - z) / np.float64(sz)
    return learned_ref.loss_and_grads(learned_ref.unpack(w), feat, target, active)


def _cuda(*arrays):
    torch = pytest.importorskip("torch")
    return [torch.tensor(a, device="cuda").contiguous() for a in arrays]


def test_gpu_loss_and_gradients_match_the_fp64_restatement():
    w = learned.initial_weights(seed=3, out_scale=1.0)
    r, z, e, active = _sample(1)
    tr = learned.GpuTrainer(N, w)
    loss, g = tr.gradients(*_cuda(r, z, e, active))
    want_loss, want = _oracle(w, r, z, e, active)
    want_flat = np.concatenate([np.concatenate([gw.ravel(), gb.ravel()]) for gw, gb in want])
    assert abs(loss - want_loss) <= 2e-2 * want_loss, (loss, want_loss)
    cos = float(g @ want_flat / (np.linalg.norm(g) * np.linalg.norm(want_flat)))
    at = 0
    errs = []
    for (name, ci, co), (gw, gb) in zip(learned_ref.LAYERS, want):
        n = gw.size + gb.size
        got = g[at:at + n]
        ref = np.concatenate([gw.ravel(), gb.ravel()])
        errs.append((name, float(np.linalg.norm(got - ref) / np.linalg.norm(ref))))
        at += n
    print("loss", loss, want_loss, "cosine", cos, "per-layer relative L2", errs)
    assert cos >= 0.995, cos
    assert all(err <= 0.1 for _, err in errs), errs


def test_gpu_training_lowers_the_loss():
    r, z, e, active = _cuda(*_sample(2))
    tr = learned.GpuTrainer(N, learned.initial_weights(seed=4))
    first = tr.step(r, z, e, active, 2e-3)
    for _ in range(100):
        last = tr.step(r, z, e, active, 2e-3)
    w = tr.weights()
    assert np.all(np.isfinite(w)) and w.size == learned_ref.weight_count()
    print("loss", first, "->", last)
    assert last < 0.6 * first
