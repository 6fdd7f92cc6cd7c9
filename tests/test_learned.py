"""CPU tests of the learned preconditioner correction's restatements: the numpy
network (the checker of the CUDA inference kernels) against torch.nn.functional.conv3d
and a torch.nn restatement of the same network, and the weight-file size against the
library.  The network has no counterpart in the reference."""
import numpy as np
import pytest

import learned_ref as R
from oceananigans_gb300 import _lib as L


# The network of the numpy restatement written with torch.nn (a second, independent
# restatement used to pin the numpy one): 3³ convolutions with periodic x / y and zero z
# padding, average pooling, nearest up-sampling with additive skips.
def make_net(seed=0):
    torch = pytest.importorskip("torch")
    F = torch.nn.functional

    class UNet(torch.nn.Module):
        def __init__(self):
            super().__init__()
            torch.manual_seed(seed)
            self.convs = torch.nn.ModuleList([torch.nn.Conv3d(ci, co, 3, padding=0) for _, ci, co in R.LAYERS])
            with torch.no_grad():
                self.convs[-1].weight.mul_(0.01)
                self.convs[-1].bias.zero_()

        @staticmethod
        def pad(x):
            x = F.pad(x, (1, 1, 1, 1, 0, 0), mode="circular")
            return F.pad(x, (0, 0, 0, 0, 1, 1))

        def conv(self, i, x, relu=True):
            y = self.convs[i](self.pad(x))
            return F.relu(y) if relu else y

        def forward(self, f):
            up = lambda t: t.repeat_interleave(2, 2).repeat_interleave(2, 3).repeat_interleave(2, 4)  # noqa: E731
            e0 = self.conv(0, f)
            e1 = self.conv(1, F.avg_pool3d(e0, 2))
            e2 = self.conv(2, F.avg_pool3d(e1, 2))
            e3 = self.conv(3, F.avg_pool3d(e2, 2))
            d3 = self.conv(4, e3)
            d2 = self.conv(5, up(d3) + e2)
            d1 = self.conv(6, up(d2) + e1)
            return self.conv(7, up(d1) + e0, relu=False)

    return UNet()


def export_weights(net):
    parts = []
    for c in net.convs:
        parts.append(c.weight.detach().float().cpu().numpy().ravel())
        parts.append(c.bias.detach().float().cpu().numpy().ravel())
    return np.concatenate(parts).astype(np.float32)


def load_weights(net, flat):
    torch = pytest.importorskip("torch")
    at = 0
    with torch.no_grad():
        for c in net.convs:
            for p in (c.weight, c.bias):
                n = p.numel()
                p.copy_(torch.from_numpy(np.asarray(flat[at:at + n], dtype=np.float32)).view_as(p))
                at += n


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
    net = make_net(seed=3).double()
    flat = export_weights(net.float())
    layers = R.unpack(flat)
    net = net.double()
    load_weights(net, flat)
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


def test_numpy_gradients_match_torch_autograd():
    # the gradient checker for training kernels: the numpy backward pass of the oracle
    # network against autograd of the training module's network, on the training loss
    torch = pytest.importorskip("torch")
    net = make_net(seed=5)
    with torch.no_grad():  # a last layer of ordinary size, so every gradient is O(1)
        net.convs[-1].weight.mul_(100.0)
        net.convs[-1].bias.fill_(0.1)
    flat = export_weights(net)
    layers = R.unpack(flat)
    net = net.double()
    load_weights(net, flat)
    rng = np.random.default_rng(2)
    nz, ny, nx = 8, 16, 16
    feat = rng.standard_normal((nz, ny, nx, 3))
    active = (rng.uniform(size=(nz, ny, nx)) > 0.2).astype(np.float64)
    target = rng.standard_normal((nz, ny, nx))
    loss, grads = R.loss_and_grads(layers, feat, target, active)
    y = net(torch.from_numpy(feat).permute(3, 0, 1, 2)[None])[0, 0]
    a, t = torch.from_numpy(active), torch.from_numpy(target)
    na = a.sum()
    d = (y - t) * a
    d = d - (d.sum() / na) * a
    tc = (t - (t * a).sum() / na) * a
    lt = (d * d).sum() / (tc * tc).sum()
    lt.backward()
    assert abs(float(lt.detach()) - loss) <= 1e-12 * loss
    for n, ((gw, gb), conv) in enumerate(zip(grads, net.convs)):
        tw, tb = conv.weight.grad.numpy(), conv.bias.grad.numpy()
        assert np.linalg.norm(tw - gw) <= 1e-10 * np.linalg.norm(tw), n
        # the output bias shifts every cell equally, which the mean-free loss ignores: its
        # gradient is zero up to roundoff, so it is measured against the weight gradient
        assert np.linalg.norm(tb - gb) <= 1e-10 * max(np.linalg.norm(tb), np.linalg.norm(tw)), n


def test_numpy_gradient_matches_finite_difference():
    # an independent check of the backward pass that needs no torch: central differences
    # of the loss along random weight directions of three layers
    rng = np.random.default_rng(4)
    layers = []
    for _, ci, co in R.LAYERS:
        layers.append((rng.standard_normal((co, ci, 3, 3, 3)) * np.sqrt(2.0 / (27 * ci)), 0.05 * rng.standard_normal(co)))
    nz, ny, nx = 8, 8, 8
    feat = rng.standard_normal((nz, ny, nx, 3))
    active = np.ones((nz, ny, nx))
    target = rng.standard_normal((nz, ny, nx))
    _, grads = R.loss_and_grads(layers, feat, target, active)
    for li in (0, 3, 7):
        dw = rng.standard_normal(layers[li][0].shape)
        h = 1e-6

        def loss_at(s):
            L = list(layers)
            L[li] = (layers[li][0] + s * dw, layers[li][1])
            return R.loss_and_grads(L, feat, target, active)[0]

        fd = (loss_at(h) - loss_at(-h)) / (2 * h)
        an = float((grads[li][0] * dw).sum())
        assert abs(fd - an) <= 1e-5 * max(abs(an), 1e-12), (li, fd, an)
