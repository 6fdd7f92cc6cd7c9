"""numpy restatement of the learned preconditioner correction (csrc/gbo_learned.cuh).

TEST INFRASTRUCTURE ONLY: the checker of the CUDA inference kernels and of the
training module's network.  The network has no counterpart in the reference, so
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
