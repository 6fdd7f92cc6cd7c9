"""Training of the learned correction of the conjugate-gradient preconditioner.

The correction is applied inside the CG loop by libgb300ocean.so (csrc/gbo_learned.cu,
BF16 tensor-core convolutions); this module only produces its weights, offline, with
PyTorch: it runs a model with the CG solver, records pairs (b = V∇²x, x) from the
pressure of every step (exact pairs of the model's own operator), applies the model's
FFT preconditioner to each b, and fits the U-Net to the part of A⁻¹b the FFT solve
misses.  The network and the weight-file layout are those of gbo_learned.cuh:

    z = z_fft + s_z · net(r / s_r, z_fft / s_z, active),   s_r = RMS(r), s_z = RMS(z_fft)

    enc0 3→16, pool, enc1 16→32, pool, enc2 32→48, pool, enc3 48→64, dec3 64→48,
    up + enc2, dec2 48→32, up + enc1, dec1 32→16, up + enc0, out 16→1
    (3³ kernels, ReLU after every layer but the last, x / y periodic, z zero padded)

PyTorch is needed only here; importing the package does not import it.
"""
import ctypes

import numpy as np

from . import _lib as L

LAYERS = (("enc0", 3, 16), ("enc1", 16, 32), ("enc2", 32, 48), ("enc3", 48, 64),
          ("dec3", 64, 48), ("dec2", 48, 32), ("dec1", 32, 16), ("out", 16, 1))


def _torch():
    import torch  # noqa: PLC0415  (optional dependency of the training step only)
    return torch


def make_net(seed=0):
    torch = _torch()
    F = torch.nn.functional

    class UNet(torch.nn.Module):
        def __init__(self):
            super().__init__()
            torch.manual_seed(seed)
            self.convs = torch.nn.ModuleList([torch.nn.Conv3d(ci, co, 3, padding=0) for _, ci, co in LAYERS])
            with torch.no_grad():  # start as a small correction
                self.convs[-1].weight.mul_(0.01)
                self.convs[-1].bias.zero_()

        @staticmethod
        def pad(x):  # (N, C, z, y, x): periodic in x and y, zeros in z
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
    """The weight file: per layer W[cout][cin][3][3][3] then bias, FP32."""
    parts = []
    for c in net.convs:
        parts.append(c.weight.detach().float().cpu().numpy().ravel())
        parts.append(c.bias.detach().float().cpu().numpy().ravel())
    flat = np.concatenate(parts).astype(np.float32)
    assert flat.size == L.load().gbo_learned_weight_count()
    return flat


def load_weights(net, flat):
    torch = _torch()
    at = 0
    with torch.no_grad():
        for c in net.convs:
            for t in (c.weight, c.bias):
                n = t.numel()
                t.copy_(torch.from_numpy(np.asarray(flat[at:at + n], dtype=np.float32)).view_as(t))
                at += n


def _rms(a):
    torch = _torch()
    s = torch.sqrt(torch.mean(a.double() ** 2)).float()
    return torch.where(s > 0, s, torch.ones_like(s))


def features(r, z, active):
    """(1, 3, z, y, x) network input for a residual r and its FFT-preconditioned z
    (fields (z, y, x)), and the output scale s_z."""
    torch = _torch()
    sr, sz = _rms(r), _rms(z)
    return torch.stack([r / sr, z / sz, active], dim=0)[None], sz


def _active_mean_free(a, active):
    return (a - (a * active).sum() / active.sum()) * active


def collect_pairs(model, dt, steps, every=1, cg_iterations=0):
    """Step `model` (CG solver) and record training triples (r, z_fft, e) on the device:
    x = pNHS with its active-cell mean removed, b = V∇²x (mean-free over active cells:
    a compatible right-hand side); with cg_iterations = K also the residuals r_k of K
    FFT-preconditioned CG iterations on b (the inputs the preconditioner meets inside
    the solve), each with its error e_k = x - x_k = A⁻¹r_k and z_fft = M_fft r_k.
    Returns FP32 tensors (n, z, y, x) r, z_fft, e and the active mask."""
    torch = _torch()
    from .api import time_step_  # noqa: PLC0415
    g = model.grid
    Nx, Ny, Nz = g.Nx, g.Ny, g.Nz
    dt_t = torch.float32 if model.dtype == np.float32 else torch.float64
    active = torch.ones((Nz, Ny, Nx), device="cuda", dtype=torch.float32)
    if g.bottom_height is not None:
        _, _, zc = g.nodes()
        imm = zc[None, None, :] <= g.bottom_height[:, :, None]  # (x, y, z)
        active = torch.from_numpy((~imm).transpose(2, 1, 0).astype(np.float32)).cuda()
    act = active.to(dt_t)

    def A(v):
        out = torch.empty_like(v)
        model.poisson_operator_device(v.data_ptr(), out.data_ptr())
        return out

    def M(v):
        out = torch.empty_like(v)
        model.precondition_device(v.data_ptr(), out.data_ptr())
        return out

    rs, zs, es = [], [], []
    for s in range(steps):
        time_step_(model, dt)
        if s % every:
            continue
        p = torch.from_numpy(model.get("p").transpose(2, 1, 0).copy()).cuda().to(dt_t)
        x = _active_mean_free(p, act).contiguous()
        b = _active_mean_free(A(x), act).contiguous()
        # FFT-preconditioned CG from x₀ = 0 (conjugate_gradient_solver.jl:202-235)
        xk = torch.zeros_like(x)
        r = b.clone()
        zk = M(r)
        d = zk.clone()
        rho = (zk * r).sum()
        for k in range(cg_iterations + 1):
            rs.append(r.float())
            zs.append(zk.float())
            es.append(_active_mean_free(x - xk, act).float())
            if k == cg_iterations:
                break
            q = A(d)
            alpha = rho / (d * q).sum()
            xk = xk + alpha * d
            r = _active_mean_free(r - alpha * q, act).contiguous()
            zk = M(r)
            rho_new = (zk * r).sum()
            d = zk + (rho_new / rho) * d
            rho = rho_new
    return torch.stack(rs), torch.stack(zs), torch.stack(es), active


def train(b, z, x, active, epochs=20, lr=1e-3, seed=0, log=None):
    """Fit net(r/s_r, z/s_z, active) to (e - z)/s_z over active cells, up to a constant
    (the Neumann problem's null space), for triples (r = b, z, e = x) as collect_pairs
    returns them.  Returns the network."""
    torch = _torch()
    net = make_net(seed).cuda()
    opt = torch.optim.Adam(net.parameters(), lr=lr)
    n = b.shape[0]
    na = active.sum()
    gen = torch.Generator().manual_seed(seed)
    for ep in range(epochs):
        total = 0.0
        for i in torch.randperm(n, generator=gen).tolist():
            f, s = features(b[i], z[i], active)
            t = (x[i] - z[i]) / s
            y = net(f)[0, 0]
            d = (y - t) * active
            d = d - (d.sum() / na) * active  # constant offsets are free
            tc = (t - (t * active).sum() / na) * active
            loss = (d * d).sum() / (tc * tc).sum().clamp_min(1e-30)
            opt.zero_grad()
            loss.backward()
            opt.step()
            total += float(loss.detach())
        if log:
            log("epoch %d: mean relative loss %.4e" % (ep, total / n))
    return net
