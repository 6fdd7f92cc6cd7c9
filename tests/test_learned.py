"""CPU tests of the learned preconditioner correction's restatements: the numpy
network (the checker of the CUDA inference kernels) against torch.nn.functional.conv3d
and the training module's PyTorch network, and the weight-file size against the
library.  The network has no counterpart in the reference."""
import numpy as np
import pytest

import learned_ref as R
from oceananigans_gb300 import _lib as L


def test_weight_count_matches_library():
    assert R.weight_count() == L.load().gbo_learned_weight_count()


def test_numpy_convolution_matches_torch_layout():
    torch = pytest.importorskip("torch")
    F = torch.nn.functional
    rng = np.random.default_rng(0)
    x = rng.standard_normal((6, 5, 7, 3))
    w = rng.standard_normal((4, 3, 3, 3, 3))
    b = rng.standard_normal(4)
    ref = R.conv(x, w, b, relu=False, round_out=False)
    t = torch.from_numpy(x).permute(3, 0, 1, 2)[None]  # (N, C, z, y, x)
    t = F.pad(F.pad(t, (1, 1, 1, 1, 0, 0), mode="circular"), (0, 0, 0, 0, 1, 1))
    out = F.conv3d(t, torch.from_numpy(w), torch.from_numpy(b))[0].permute(1, 2, 3, 0).numpy()
    assert np.abs(out - ref).max() < 1e-12 * np.abs(ref).max()


def test_training_network_matches_numpy_network():
    torch = pytest.importorskip("torch")
    from oceananigans_gb300 import learned
    net = learned.make_net(seed=3).double()
    flat = learned.export_weights(net.float())
    layers = R.unpack(flat)
    net = net.double()
    learned.load_weights(net, flat)
    rng = np.random.default_rng(1)
    feat = rng.standard_normal((16, 16, 24, 3)).astype(np.float32)
    want = R.forward(layers, feat.astype(np.float64), bf16_path=False)
    with torch.no_grad():
        got = net.double()(torch.from_numpy(feat.astype(np.float64)).permute(3, 0, 1, 2)[None])[0, 0].numpy()
    assert np.abs(got - want).max() < 1e-10 * max(np.abs(want).max(), 1e-30)


def test_bf16_rounding_is_round_to_nearest_even():
    x = np.array([1.0, 1.0 + 2**-8, 1.0 + 3 * 2**-8, -2.5, 3.0e-3], dtype=np.float32)
    y = R.bf16(x)
    assert y[0] == 1.0 and y[1] == 1.0 and y[2] == 1.0 + 2**-6 and y[3] == -2.5
    assert abs(y[4] - 3.0e-3) <= 3.0e-3 * 2**-8
