"""numpy restatement of the learned preconditioner correction (csrc/gbo_learned.cuh).

TEST INFRASTRUCTURE ONLY: the checker of the CUDA inference kernels, of the
training module's network and (forward_backward, loss_and_grads) of gradients of
the training loss.  The network has no counterpart in the reference, so
it is pinned against torch.nn.functional.conv3d (tests/test_learned.py) rather
than against Oceananigans.jl.

Arrays are (nz, ny, nx, channels); x and y are periodic, z is zero padded.  With
bf16=True the weights, the inputs and every stored activation are rounded to
BF16 (round to nearest even) and sums are accumulated in FP64, as the kernels do
with FP32 accumulation.
"""
import numpy as np

CHANNELS = (16, 32, 48, 64)
# (name, cin, cout) in the weight-file order
LAYERS = (("enc0", 3, 16), ("enc1", 16, 32), ("enc2", 32, 48), ("enc3", 48, 64),
          ("dec3", 64, 48), ("dec2", 48, 32), ("dec1", 32, 16), ("out", 16, 1))


def weight_count():
    return sum(co * ci * 27 + co for _, ci, co in LAYERS)


def unpack(flat):
    """Weight file (FP32) -> list of (W[cout][cin][3][3][3], b[cout])."""
    flat = np.asarray(flat, dtype=np.float32)
    assert flat.size == weight_count()
    out, at = [], 0
    for _, ci, co in LAYERS:
        w = flat[at:at + co * ci * 27].reshape(co, ci, 3, 3, 3)
        at += co * ci * 27
        b = flat[at:at + co]
        at += co
        out.append((w, b))
    return out


def bf16(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).reshape(a.shape)


def conv(x, w, b, relu, round_out):
    """3³ convolution: out[z,y,x,o] = Σ w[o,c,dz+1,dy+1,dx+1] x[z+dz, y+dy, x+dx, c] + b[o]."""
    nz = x.shape[0]
    xp = np.zeros((nz + 2,) + x.shape[1:], dtype=np.float64)
    xp[1:-1] = x
    out = np.zeros(x.shape[:3] + (w.shape[0],), dtype=np.float64)
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                sh = np.roll(xp[1 + dz:1 + dz + nz], shift=(-dy, -dx), axis=(1, 2))
                out += np.einsum("zyxc,oc->zyxo", sh, w[:, :, dz + 1, dy + 1, dx + 1].astype(np.float64))
    out += b.astype(np.float64)
    if relu:
        out = np.maximum(out, 0.0)
    return bf16(out) if round_out else out


def pool(x, rnd):
    nz, ny, nx, c = x.shape
    y = x.reshape(nz // 2, 2, ny // 2, 2, nx // 2, 2, c).astype(np.float64).mean(axis=(1, 3, 5))
    return bf16(y) if rnd else y


def upadd(coarse, skip, rnd):
    up = np.repeat(np.repeat(np.repeat(coarse, 2, axis=0), 2, axis=1), 2, axis=2)
    y = up.astype(np.float64) + skip
    return bf16(y) if rnd else y


def forward(layers, feat, bf16_path=True):
    """The U-Net on features (nz, ny, nx, 3); returns the (nz, ny, nx) output channel."""
    r = bf16_path
    L = [(bf16(w) if r else w, b) for w, b in layers]
    f = bf16(feat) if r else feat
    e0 = conv(f, *L[0], True, r)
    e1 = conv(pool(e0, r), *L[1], True, r)
    e2 = conv(pool(e1, r), *L[2], True, r)
    e3 = conv(pool(e2, r), *L[3], True, r)
    d3 = conv(e3, *L[4], True, r)
    d2 = conv(upadd(d3, e2, r), *L[5], True, r)
    d1 = conv(upadd(d2, e1, r), *L[6], True, r)
    out = conv(upadd(d1, e0, r), *L[7], False, False)
    return out[..., 0]


def rms(a):
    s = np.float32(np.sqrt(np.mean(np.asarray(a, dtype=np.float64) ** 2)))
    return s if s > 0 else np.float32(1)


def correction(layers, r, z, active, bf16_path=True):
    """s_z · net(r/s_r, z/s_z, active) with s_r, s_z the RMS of r and z over all cells
    (fields (nz, ny, nx))."""
    sr, sz = rms(r), rms(z)
    feat = np.stack([np.float32(r) * (np.float32(1) / sr), np.float32(z) * (np.float32(1) / sz),
                     active.astype(np.float32)], axis=-1)
    return np.float64(sz) * forward(layers, feat, bf16_path)


# ---------------------------------------------------------------------------
# Backward pass (FP64, no BF16 rounding): the checker of gradients of the training
# loss.  Each function returns the gradients of its forward counterpart above.
# ---------------------------------------------------------------------------
def conv_backward(x, w, gy):
    """Gradients (gx, gw, gb) of out = Σ w x_shift + b (conv with relu=False) for the
    output gradient gy (nz, ny, nx, cout)."""
    nz = x.shape[0]
    xp = np.zeros((nz + 2,) + x.shape[1:], dtype=np.float64)
    xp[1:-1] = x
    gxp = np.zeros_like(xp)
    gw = np.zeros(w.shape, dtype=np.float64)
    gy = np.asarray(gy, dtype=np.float64)
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                sh = np.roll(xp[1 + dz:1 + dz + nz], shift=(-dy, -dx), axis=(1, 2))
                gw[:, :, dz + 1, dy + 1, dx + 1] = np.einsum("zyxo,zyxc->oc", gy, sh)
                contrib = np.einsum("zyxo,oc->zyxc", gy, w[:, :, dz + 1, dy + 1, dx + 1].astype(np.float64))
                gxp[1 + dz:1 + dz + nz] += np.roll(contrib, shift=(dy, dx), axis=(1, 2))
    return gxp[1:-1], gw, gy.sum(axis=(0, 1, 2))


def pool_backward(gy):
    return np.repeat(np.repeat(np.repeat(gy, 2, axis=0), 2, axis=1), 2, axis=2) / 8.0


def upadd_backward(gy):
    """(g_coarse, g_skip) of upadd(coarse, skip)."""
    nz, ny, nx, c = gy.shape
    return gy.reshape(nz // 2, 2, ny // 2, 2, nx // 2, 2, c).sum(axis=(1, 3, 5)), gy


def forward_backward(layers, feat, gout):
    """The FP64 network output (nz, ny, nx) and the gradients [(gW, gb)] of Σ gout·output
    with respect to every layer's weights and bias."""
    L = [(np.asarray(w, dtype=np.float64), np.asarray(b, dtype=np.float64)) for w, b in layers]
    f = np.asarray(feat, dtype=np.float64)
    e0 = conv(f, *L[0], True, False)
    p0 = pool(e0, False)
    e1 = conv(p0, *L[1], True, False)
    p1 = pool(e1, False)
    e2 = conv(p1, *L[2], True, False)
    p2 = pool(e2, False)
    e3 = conv(p2, *L[3], True, False)
    d3 = conv(e3, *L[4], True, False)
    u2 = upadd(d3, e2, False)
    d2 = conv(u2, *L[5], True, False)
    u1 = upadd(d2, e1, False)
    d1 = conv(u1, *L[6], True, False)
    u0 = upadd(d1, e0, False)
    out = conv(u0, *L[7], False, False)
    grads = [None] * len(L)
    g = np.asarray(gout, dtype=np.float64)[..., None]
    g, grads[7] = _conv_grads(u0, L[7], g)
    g_d1, g_e0 = upadd_backward(g)
    g, grads[6] = _conv_grads(u1, L[6], g_d1 * (d1 > 0))
    g_d2, g_e1 = upadd_backward(g)
    g, grads[5] = _conv_grads(u2, L[5], g_d2 * (d2 > 0))
    g_d3, g_e2 = upadd_backward(g)
    g, grads[4] = _conv_grads(e3, L[4], g_d3 * (d3 > 0))
    g, grads[3] = _conv_grads(p2, L[3], g * (e3 > 0))
    g, grads[2] = _conv_grads(p1, L[2], (pool_backward(g) + g_e2) * (e2 > 0))
    g, grads[1] = _conv_grads(p0, L[1], (pool_backward(g) + g_e1) * (e1 > 0))
    _, grads[0] = _conv_grads(f, L[0], (pool_backward(g) + g_e0) * (e0 > 0))
    return out[..., 0], grads


def _conv_grads(x, layer, gy):
    gx, gw, gb = conv_backward(x, layer[0], gy)
    return gx, (gw, gb)


def loss_and_grads(layers, feat, target, active):
    """The training loss of oceananigans_gb300.learned.train — Σ d² / Σ t_c² with
    d = (y − t)·active less its active-cell mean, t_c = t less its active-cell mean —
    and its gradients.  The mean removal is a projection, so ∂loss/∂y = 2 d / Σ t_c²."""
    a = np.asarray(active, dtype=np.float64)
    t = np.asarray(target, dtype=np.float64)
    na = a.sum()
    y, _ = forward_backward(layers, feat, np.zeros(a.shape))
    d = (y - t) * a
    d = d - (d.sum() / na) * a
    tc = (t - (t * a).sum() / na) * a
    den = max((tc * tc).sum(), 1e-30)
    _, grads = forward_backward(layers, feat, 2.0 * d / den)
    return (d * d).sum() / den, grads
