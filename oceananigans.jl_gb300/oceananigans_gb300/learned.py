"""Training of the learned correction of the conjugate-gradient preconditioner.

The correction is applied inside the CG loop by libgb300ocean.so (csrc/gbo_learned.cu,
BF16 tensor-core convolutions); this module only produces its weights, offline, with
PyTorch: it runs a model with the CG solver, records pairs (b = V∇²x, x) from the
pressure of every step (exact pairs of the model's own operator), applies the model's
FFT preconditioner to each b, and fits the U-Net to the part of A⁻¹b the FFT solve
misses -- on the GPU, with the library's own training kernels (GpuTrainer).  The network and the weight-file layout are those of gbo_learned.cuh:

    z = z_fft + s_z · net(r / s_r, z_fft / s_z, active),   s_r = RMS(r), s_z = RMS(z_fft)

    enc0 3→16, pool, enc1 16→32, pool, enc2 32→48, pool, enc3 48→64, dec3 64→48,
    up + enc2, dec2 48→32, up + enc1, dec1 32→16, up + enc0, out 16→1
    (3³ kernels, ReLU after every layer but the last, x / y periodic, z zero padded)

PyTorch (device arrays and the CG iterations that generate the samples) is needed only
here; importing the package does not import it.
"""
import ctypes

import numpy as np

from . import _lib as L

LAYERS = (("enc0", 3, 16), ("enc1", 16, 32), ("enc2", 32, 48), ("enc3", 48, 64),
          ("dec3", 64, 48), ("dec2", 48, 32), ("dec1", 32, 16), ("out", 16, 1))


def _torch():
    import torch  # noqa: PLC0415  (optional dependency of the training step only)
    return torch


def initial_weights(seed=0, out_scale=0.01):
    """A weight file of fresh weights: W, b ~ U[-1/√fan_in, 1/√fan_in] per layer (fan_in =
    27 cin, the default of a 3-D convolution), the output layer's weights scaled by
    `out_scale` and its bias zero so that training starts from a small correction."""
    rng = np.random.default_rng(seed)
    parts = []
    for i, (_, ci, co) in enumerate(LAYERS):
        bound = 1.0 / np.sqrt(27 * ci)
        w = rng.uniform(-bound, bound, co * ci * 27)
        b = rng.uniform(-bound, bound, co)
        if i == len(LAYERS) - 1:
            w, b = w * out_scale, np.zeros(co)
        parts += [w, b]
    return np.concatenate(parts).astype(np.float32)


class GpuTrainer:
    """The network trained on the GPU by the library's own kernels (gbo_learned_trainer_*):
    tcgen05 convolutions forward and for data gradients, tensor-core weight gradients,
    Adam on FP32 master weights.  Samples are CUDA FP32 tensors (nz, ny, nx): residual r,
    FFT-preconditioned z, error e = A⁻¹ r and the active mask."""

    def __init__(self, size, weights=None, seed=0):
        nx, ny, nz = (int(a) for a in size)
        w = initial_weights(seed) if weights is None else np.ascontiguousarray(weights, dtype=np.float32)
        lib = L.load()
        h = ctypes.c_void_p()
        L.check(lib.gbo_learned_trainer_create(nx, ny, nz, w.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), w.size,
                                               ctypes.byref(h)))
        self._h, self.count = h, w.size

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            L.load().gbo_learned_trainer_destroy(h)
            self._h = None

    @staticmethod
    def _ptrs(*ts):
        for t in ts:
            if not (t.is_cuda and t.is_contiguous() and str(t.dtype) == "torch.float32"):
                raise ValueError("trainer samples are contiguous CUDA float32 tensors")
        return [ctypes.c_void_p(t.data_ptr()) for t in ts]

    def stream(self):
        sp = ctypes.c_void_p()
        L.check(L.load().gbo_learned_trainer_stream(self._h, ctypes.byref(sp)))
        return sp.value

    def gradients(self, r, z, e, active):
        """(loss, gradient in the weight-file layout) of one sample; no update."""
        g = np.zeros(self.count, dtype=np.float32)
        loss = ctypes.c_double()
        L.check(L.load().gbo_learned_trainer_gradients(self._h, *self._ptrs(r, z, e, active), ctypes.byref(loss),
                                                       g.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        return loss.value, g

    def step(self, r, z, e, active, lr):
        """One Adam step on one sample; returns the sample's loss before the step."""
        loss = ctypes.c_double()
        L.check(L.load().gbo_learned_trainer_step(self._h, *self._ptrs(r, z, e, active), float(lr), ctypes.byref(loss)))
        return loss.value

    def weights(self):
        w = np.zeros(self.count, dtype=np.float32)
        L.check(L.load().gbo_learned_trainer_weights(self._h, w.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        return w


def _rms(a):
    torch = _torch()
    s = torch.sqrt(torch.mean(a.double() ** 2)).float()
    return torch.where(s > 0, s, torch.ones_like(s))


def _active_mean_free(a, active):
    """a minus its mean over the active cells, zero elsewhere (whatever a holds there)."""
    torch = _torch()
    on = active > 0
    a = torch.where(on, a, torch.zeros_like(a))
    return torch.where(on, a - a.sum() / active.sum(), a)


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
        out = torch.zeros_like(v)
        model.poisson_operator_device(v.data_ptr(), out.data_ptr())
        return out

    def M(v):
        out = torch.zeros_like(v)
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


def train(r, z, e, active, epochs=20, lr=1e-3, seed=0, log=None, weights=None, on_epoch=None):
    """Fit net(r/s_r, z/s_z, active) to (e - z)/s_z over active cells, up to a constant
    (the Neumann problem's null space), for samples (r, z_fft, e) as collect_pairs returns
    them, on the GPU with the library's own kernels (GpuTrainer: tcgen05 convolutions,
    tensor-core weight gradients, Adam).  Starts from `weights` (a weight file) or from
    initial_weights(seed).  on_epoch(epoch, mean loss, weight file) is called after each
    epoch.  Returns the trained weight file (FP32)."""
    torch = _torch()
    n, nz, ny, nx = r.shape
    tr = GpuTrainer((nx, ny, nz), weights, seed)
    act = active.float().contiguous()
    gen = torch.Generator().manual_seed(seed)
    for ep in range(epochs):
        total = 0.0
        for i in torch.randperm(n, generator=gen).tolist():
            total += tr.step(r[i].contiguous(), z[i].contiguous(), e[i].contiguous(), act, lr)
        if log:
            log("epoch %d: mean relative loss %.4e" % (ep, total / n))
        if on_epoch:
            on_epoch(ep, total / n, tr.weights())
    return tr.weights()
