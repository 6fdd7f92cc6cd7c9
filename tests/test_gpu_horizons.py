"""Parity over the benchmark horizons, with the benchmark configurations' own parameters.

* FP64 convection with the headline case's physics (N² = 1e-5, velocities 1e-3,
  surface buoyancy flux 1e-8, f = 1e-4, SmagorinskyLilly, Δt = 2 s) at 64×64×32:
  1e-12 after one step (the pressure 1e-11: its source ∇·u* is weak) and 1e-8 after
  100 against the FP64 oracle.
* FP64 seamount with the conjugate-gradient projection (FFT preconditioner, solved
  to 1e-13 on both sides) at 64×64×32, Δt = 20 s: 1e-10 after one step, 1e-8 after
  100, iteration counts within one.
* FP32 stretched-grid AMD with the Fourier-tridiagonal solver (the stretched
  benchmark's physics, Δt = 1 s) at 128×128×64 against the FP64 oracle after 100
  steps, within the FP32 bar of 1e-5 (measured 5.6e-7 against the FP64 GPU path).
* The 64 members of the ensemble benchmark (every size class of Nx = Ny ∈ {64, 96,
  128} × Nz ∈ {32, 48, 64} that the seeded draw produced), FP32 in one ensemble,
  each against its own FP64 run (an FP64 ensemble of the same members) after 100
  steps of Δt = 1 s, within 1e-5 (measured worst member 5.9e-7).
"""
import os
import sys

import numpy as np
import pytest

import cases
import oceananigans_gb300 as og
from test_gpu_parity import compare

pytestmark = [pytest.mark.gpu, pytest.mark.slow]


def test_convection_benchmark_physics_100_steps_fp64():
    c = cases.convection_3d((64, 64, 32))
    m, r = c.start_gpu(), c.start_oracle()
    og.time_step_(m, 2.0)
    r.time_step(2.0)
    names = ("u", "v", "w", "b", "p", "pHY", "nu")
    compare(m, r, ("u", "v", "w", "b", "pHY", "nu"), 1e-12)
    # the projected initial velocities leave a weak source ∇·u* (velocities 1e-3), so the
    # pressure's roundoff floor is higher than the fields' (measured 3.9e-12 after one step)
    compare(m, r, ("p",), 1e-11)
    og.time_step_(m, 2.0, 99)
    r.time_step(2.0, 99)
    compare(m, r, names, 1e-8)
    assert m.clock[1] == 100


def test_seamount_cg_100_steps_fp64():
    c = cases.seamount((64, 64, 32), solver="cg", reltol=1e-13, abstol=1e-300)
    m, r = c.start_gpu(), c.start_oracle()
    og.time_step_(m, 20.0)
    r.time_step(20.0)
    names = ("u", "v", "w", "b", "p", "pHY")
    compare(m, r, names, 1e-10)
    assert abs(m.solver_iterations - r.last_cg_iterations()) <= 1
    og.time_step_(m, 20.0, 99)
    r.time_step(20.0, 99)
    compare(m, r, names, 1e-8)
    assert abs(m.solver_iterations - r.last_cg_iterations()) <= 1


def test_stretched_amd_fp32_100_steps_against_oracle():
    c32 = cases.convection_3d((128, 128, 64), closure="amd", stretched=True, float_type=np.float32)
    c64 = cases.convection_3d((128, 128, 64), closure="amd", stretched=True)
    m, r = c32.start_gpu(), c64.start_oracle()
    og.time_step_(m, 1.0, 100)
    r.time_step(1.0, 100)
    errs = compare(m, r, ("u", "v", "w", "b"), 1e-5)
    print("stretched AMD fp32 vs fp64 oracle at 128x128x64 after 100 steps:", errs)


def test_ensemble_members_fp32_against_their_fp64_runs():
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench  # the ensemble benchmark's members (seeded sizes and physics)
    s32 = bench.ensemble_specs(64, np.float32)
    s64 = bench.ensemble_specs(64, np.float64)
    classes = {tuple(g.size()) for g, _, _ in s32}
    e32 = og.Ensemble([(g, p) for g, p, _ in s32])
    e64 = og.Ensemble([(g, p) for g, p, _ in s64])
    for e, specs in ((e32, s32), (e64, s64)):
        for m, (_, _, init) in zip(e.members, specs):
            og.set_(m, **init)
    e32.time_step(1.0, 100)
    e64.time_step(1.0, 100)
    worst = 0.0
    for i, (a, b) in enumerate(zip(e32.members, e64.members)):
        for name in ("u", "v", "w", "b"):
            err = cases.rel_l2(a.get(name), b.get(name))
            assert err <= 1e-5, (i, s32[i][0].size(), name, err)
            worst = max(worst, err)
    print("ensemble: %d members in %d size classes, worst fp32 vs fp64 after 100 steps %.2e"
          % (len(s32), len(classes), worst))
