"""What the learned correction gains, trained on the GPU by the library's own kernels.

A seamount model (64×64×32 ImmersedBoundaryGrid, FP32, FFT-preconditioned CG) runs a
few steps; the residuals of FFT-preconditioned CG iterations on its pressure systems,
with their errors e = A⁻¹ r, are the samples (learned.collect_pairs).  The network is
trained on the GPU (learned.train -> GpuTrainer) and evaluated on samples of later
steps it never saw:

* the relative preconditioner error, the training loss Σ d² / Σ t_c²: 1 for the FFT
  preconditioner alone (a zero correction), below 1 where the correction helps;
* CG iterations to a 1e-8 relative residual of the held-out pressure systems with the
  FFT preconditioner and with the learned flexible PCG (printed: both must converge).
"""
import numpy as np
import pytest

import cases
import oceananigans_gb300 as og
from oceananigans_gb300 import learned

pytestmark = [pytest.mark.gpu, pytest.mark.slow]


def test_trained_correction_lowers_the_preconditioner_error():
    torch = pytest.importorskip("torch")
    c = cases.seamount((64, 64, 32), float_type=np.float32, solver="cg", reltol=1e-8, abstol=1e-30)
    m = c.start_gpu()
    og.time_step_(m, 20.0, 2)
    r, z, e, active = learned.collect_pairs(m, 20.0, 10, cg_iterations=3)
    hr, hz, he, _ = learned.collect_pairs(m, 20.0, 4, cg_iterations=3)
    w = learned.train(r, z, e, active, epochs=4, lr=1e-3, seed=1)
    tr = learned.GpuTrainer((64, 64, 32), w)
    act = active.float().contiguous()
    held = [tr.gradients(hr[i].contiguous(), hz[i].contiguous(), he[i].contiguous(), act)[0] for i in range(hr.shape[0])]
    # iterations on the held-out pressure systems (the first residual of each trajectory is b)
    rhs = [hr[i].contiguous() for i in range(0, hr.shape[0], 4)]
    its = {}
    for name, weights in (("fft", None), ("learned", w)):
        m.set_learned_preconditioner(weights)
        n = []
        for b in rhs:
            x = torch.zeros_like(b)
            m.poisson_solve_device(x.data_ptr(), b.data_ptr())
            n.append(m.solver_iterations)
        its[name] = float(np.mean(n))
    m.set_learned_preconditioner(None)
    print("held-out relative preconditioner error with the trained correction: %.3f (FFT alone: 1)" % np.mean(held),
          "CG iterations to 1e-8:", its)
    assert np.mean(held) < 1.0
    assert its["learned"] > 0 and its["fft"] > 0
