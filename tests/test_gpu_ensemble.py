"""Ensembles: members of different sizes and physics advanced by one graph launch
per step must match the same models stepped one by one (bit for bit for the spectral
members; the CG member, solved to a 1e-12 relative residual, within 1e-10), and each
FP32 member must match its own FP64 oracle run within the FP32 bar of the parity tests
(1e-4 relative L2): two mixed members, and one member of every size class of the
64-member benchmark ensemble (Nx = Ny in {64, 96, 128}, Nz in {32, 48, 64})."""
import numpy as np
import pytest

import cases
import oceananigans_gb300 as og

pytestmark = pytest.mark.gpu


def _members():
    return [
        cases.convection_3d((32, 32, 16), float_type=np.float32, seed=1, N2=1e-6, flux=5e-8),
        cases.convection_3d((48, 48, 24), float_type=np.float32, seed=2, N2=1e-5, flux=1e-8),
        cases.convection_3d((32, 24, 16), closure="amd", seed=3, N2=1e-7, U0=2e-2),
        cases.seamount((32, 32, 16), solver="cg", reltol=1e-12, abstol=1e-300),
    ]


def test_ensemble_matches_models_stepped_one_by_one():
    specs = _members()
    ens = og.Ensemble([(c.grid, c.physics) for c in specs])
    assert len(ens) == len(specs)
    for m, c in zip(ens.members, specs):
        og.set_(m, **c.init)
    singles = [c.start_gpu() for c in specs]
    for _ in range(3):
        ens.time_step(2.0)
        for s in singles:
            og.time_step_(s, 2.0)
    for idx, (m, s) in enumerate(zip(ens.members, singles)):
        assert m.clock == s.clock
        for name in ("u", "v", "w", "b", "p"):
            a, b = m.get(name), s.get(name)
            if idx == 3:
                assert cases.rel_l2(a, b) <= 1e-10, (idx, name)
            else:
                assert np.array_equal(a, b), (idx, name)


def test_ensemble_fp32_members_against_fp64_oracle():
    specs = _members()[:2]
    ens = og.Ensemble([(c.grid, c.physics) for c in specs])
    for m, c in zip(ens.members, specs):
        og.set_(m, **c.init)
    ens.time_step(2.0, 5)
    for m, c in zip(ens.members, specs):
        r = c.start_oracle()  # the same descriptors and initial arrays, computed in FP64
        r.time_step(2.0, 5)
        for name in ("u", "v", "w", "b"):
            assert cases.rel_l2(m.get(name), r.get(name)) <= 1e-4, name


def test_ensemble_every_size_class_against_fp64_oracle():
    sizes = [(n, n, nz) for n in (64, 96, 128) for nz in (32, 48, 64)]
    specs = [cases.convection_3d(sz, float_type=np.float32, seed=10 + q) for q, sz in enumerate(sizes)]
    ens = og.Ensemble([(c.grid, c.physics) for c in specs])
    for m, c in zip(ens.members, specs):
        og.set_(m, **c.init)
    ens.time_step(2.0, 5)
    for q, (m, c) in enumerate(zip(ens.members, specs)):
        r = cases.convection_3d(sizes[q], seed=10 + q).start_oracle()
        r.time_step(2.0, 5)
        for name in ("u", "v", "w", "b"):
            assert cases.rel_l2(m.get(name), r.get(name)) <= 1e-4, (sizes[q], name)
