"""The C ABI library loads and exports every entry point declared in include/gbo.h;
argument validation runs without a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

import oceananigans_gb300 as og
from oceananigans_gb300 import _lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "gbo.h")).read()
    return sorted(set(re.findall(r"\b(gbo_[a-z_0-9]+)\s*\(", src)))


def test_header_symbols_exported_and_bound():
    lib = L.load()
    syms = declared_symbols()
    assert syms, "no declarations found"
    for s in syms:
        assert hasattr(lib, s), s
    assert sorted(L.SIGNATURES) == syms


def test_struct_layout_matches_header(tmp_path):
    # compile a probe against include/gbo.h and compare sizes/offsets with the ctypes mirror
    src = tmp_path / "probe.c"
    src.write_text('''#include <stdio.h>
#include <stddef.h>
#include "gbo.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu %zu\\n", sizeof(gbo_grid_desc), offsetof(gbo_grid_desc, z_faces),
         offsetof(gbo_grid_desc, float_type), sizeof(gbo_model_desc), offsetof(gbo_model_desc, pressure_solver),
         offsetof(gbo_model_desc, cg_maxiter), offsetof(gbo_model_desc, closure_min_numerator),
         offsetof(gbo_model_desc, closure_averaging));
  return 0; }
''')
    exe = tmp_path / "probe"
    import subprocess
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    got = [int(v) for v in subprocess.check_output([str(exe)]).split()]
    want = [ctypes.sizeof(L.GridDesc), L.GridDesc.z_faces.offset, L.GridDesc.float_type.offset,
            ctypes.sizeof(L.ModelDesc), L.ModelDesc.pressure_solver.offset, L.ModelDesc.cg_maxiter.offset,
            L.ModelDesc.closure_min_numerator.offset, L.ModelDesc.closure_averaging.offset]
    assert got == want


def test_version_and_defaults():
    lib = L.load()
    assert b"sm_103a" in lib.gbo_version()
    d = L.ModelDesc()
    lib.gbo_model_desc_default(ctypes.byref(d))
    assert d.advection == L.GBO_ADVECTION_WENO5 and d.closure_C == 0.16 and d.pressure_solver == L.GBO_SOLVER_FFT


def test_invalid_extent_rejected_before_device():
    with pytest.raises(ValueError, match="increasing"):
        _create(og.RectilinearGrid(size=(16, 16, 8), x=(1, 0), z=(-1, 0)))


def _create(grid, **kw):
    kw.setdefault("advection", og.WENO())
    d, _ = og.api.model_descriptor(grid, **kw)
    g = grid.descriptor()
    h = ctypes.c_void_p()
    rc = L.load().gbo_model_create(ctypes.byref(g), ctypes.byref(d), ctypes.byref(h))
    if rc == L.GBO_ERR_INVALID:
        raise ValueError(L.load().gbo_last_error(None).decode())
    return rc


def test_validation_messages():
    grid = og.RectilinearGrid(size=(16, 16, 8), z=(-1, 0))
    with pytest.raises(ValueError, match="WENO"):
        og.WENO(order=7)
    with pytest.raises(ValueError, match="Periodic"):
        og.RectilinearGrid(size=(16, 16, 8), topology=("Bounded", "Periodic", "Bounded"))
    with pytest.raises(ValueError, match="BuoyancyTracer"):
        og.api.model_descriptor(grid, advection=og.WENO(), buoyancy=og.BuoyancyTracer(), tracers=("c",))
    stretched = og.RectilinearGrid(size=(16, 16, 8), z=np.linspace(-1, 0, 9) ** 3)
    with pytest.raises(ValueError, match="regular"):
        _create(stretched, pressure_solver=og.FFTBasedPoissonSolver())
    with pytest.raises(ValueError, match="factor"):
        pass_through = og.RectilinearGrid(size=(14, 16, 8), z=(-1, 0))
        rc = _create(pass_through)
        if rc == L.GBO_ERR_NO_DEVICE:
            raise ValueError("factor check needs a device")


def test_no_device_is_reported_cleanly():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    grid = og.RectilinearGrid(size=(16, 16, 8), z=(-1, 0))
    assert _create(grid) == L.GBO_ERR_NO_DEVICE


def test_ensemble_arguments_rejected_before_device():
    # gbo_ensemble_create validates every member before any device work
    import cases
    c = cases.convection_3d((16, 16, 8))
    qab2 = dict(c.physics, timestepper="QuasiAdamsBashforth2")
    with pytest.raises(ValueError, match="member 1: ensembles step RungeKutta3 models only"):
        og.Ensemble([(c.grid, c.physics), (c.grid, qab2)])
    flat = og.RectilinearGrid(size=(16, 16), x=(0, 1), y=(0, 1), topology=("Periodic", "Periodic", "Flat"))
    with pytest.raises(ValueError, match="member 0: DynamicSmagorinsky requires"):
        og.Ensemble([(flat, dict(advection=og.WENO(), closure=og.DynamicSmagorinsky(averaging=(1, 2))))])
    with pytest.raises(ValueError, match="invalid ensemble arguments"):
        og.Ensemble([])


def test_amd_coefficients_mirror_the_reference_keywords():
    # AnisotropicMinimumDissipation(; C, Cν = C, Cκ = C, Cb) (anisotropic_minimum_dissipation.jl:138-147)
    assert og.AnisotropicMinimumDissipation().C == 1.0 / 3.0
    assert og.AnisotropicMinimumDissipation(C=0.2).C == 0.2
    assert og.AnisotropicMinimumDissipation(Cnu=0.25, Ckappa=0.25).C == 0.25
    with pytest.raises(ValueError, match="Cκ ≠ Cν"):
        og.AnisotropicMinimumDissipation(Cnu=0.3, Ckappa=0.2)
    with pytest.raises(ValueError, match="Cb"):
        og.AnisotropicMinimumDissipation(Cb=1.0)


def test_grid_extent_keyword():
    # extent = (Lx, Ly, Lz): 0 ≤ x ≤ Lx, 0 ≤ y ≤ Ly, -Lz ≤ z ≤ 0 (rectilinear_grid.jl:121-124)
    g = og.RectilinearGrid(size=(8, 8, 4), extent=(1, 2, 3))
    assert g.x == (0.0, 1.0) and g.y == (0.0, 2.0) and g.z == (-3.0, 0.0)
    f = og.RectilinearGrid(size=(8, 8), extent=(2 * np.pi, 4 * np.pi), topology=("Periodic", "Periodic", "Flat"))
    assert f.x == (0.0, 2 * np.pi) and f.y == (0.0, 4 * np.pi)
    with pytest.raises(ValueError, match="Cannot specify both"):
        og.RectilinearGrid(size=(8, 8, 4), extent=(1, 1, 1), x=(0, 1))


def test_callable_initial_conditions_evaluate_per_point():
    # set!(model, u = f) evaluates f(x, y, z) at every node of the field's location
    import math
    from types import SimpleNamespace
    g = og.RectilinearGrid(size=(8, 6, 4), extent=(1, 2, 3))
    fake = SimpleNamespace(grid=g)
    ev = lambda name, fn: og.NonhydrostaticModel._evaluate(fake, name, fn)  # noqa: E731
    xc, yc, zc = g.nodes()
    a = ev("b", lambda x, y, z: np.sin(x) * y + z)            # array-safe: one call
    b = ev("b", lambda x, y, z: math.sin(x) * y + z)          # scalar-only: per point
    assert a.shape == (8, 6, 4) and np.allclose(a, b, rtol=0, atol=1e-15)
    assert np.allclose(a, np.sin(xc)[:, None, None] * yc[None, :, None] + zc[None, None, :])
    rng = np.random.default_rng(0)
    r = ev("u", lambda x, y, z: rng.standard_normal())        # one draw per point, not one in all
    assert np.unique(r).size == r.size
    w = ev("w", lambda x, y, z: z)                            # w at the Nz + 1 faces
    assert w.shape == (8, 6, 5) and w[0, 0, 0] == -3.0 and w[0, 0, -1] == 0.0


def test_fplane_keywords():
    # FPlane(; f) or FPlane(; rotation_rate, latitude) with f = 2Ω sind(latitude) (f_plane.jl:30-50)
    assert og.FPlane(1e-4).f == 1e-4 and og.FPlane(f=2e-4).f == 2e-4
    # within a few ulps of the closed form (degree conversion and sin round differently)
    assert abs(og.FPlane(latitude=45).f - 2 * 7.292115e-5 * np.sqrt(0.5)) <= 1e-15 * 1.04e-4
    assert abs(og.FPlane(rotation_rate=1e-4, latitude=90).f - 2e-4) <= 1e-15 * 2e-4
    for bad in (dict(), dict(f=1e-4, latitude=10.0)):
        with pytest.raises(ValueError, match="Either both keywords"):
            og.FPlane(**bad)


def test_launch_table_entries_are_valid():
    # the tuned shapes compiled into the library (written by oceananigans_gb300/autotune.py)
    import re
    path = os.path.join(os.path.dirname(__file__), "..", "oceananigans.jl_gb300", "csrc", "gbo_launch_table.h")
    with open(path) as f:
        text = f.read()
    body = text[text.index("// BEGIN TABLE"):text.index("// END TABLE")]
    rows = [tuple(int(v) for v in m.group(1).split(",")) for m in re.finditer(r"\{([-\d, ]+)\}", body)]
    assert rows and rows[-1] == (0,) * 9  # terminated
    seen = set()
    for nx, ny, nz, fp64, ibg, zt, xl, yt, lev in rows[:-1]:
        assert nx > 0 and ny > 0 and nz > 0 and fp64 in (0, 1) and ibg in (0, 1)
        assert 2 <= zt <= 64 and zt & (zt - 1) == 0 and 1 <= xl <= 32 and 1 <= yt <= 64 and yt & (yt - 1) == 0
        assert 1 <= lev <= nz
        assert (nx, ny, nz, fp64, ibg) not in seen
        seen.add((nx, ny, nz, fp64, ibg))


def test_autotune_selection_and_table_writer(tmp_path):
    # the tuner keeps the default unless a candidate is faster by more than its margin,
    # and writes entries the library's table parser (tuned_shape) reads
    from oceananigans_gb300 import autotune
    entry = {"size": [64, 64, 32], "fp64": False, "ibg": False, "kind": "rect",
             "default": {"dct_columns": 32, "x_lines": 8, "y_columns": 16, "levels": 16},
             "us_per_launch": {"dct_columns": {"16": 9.9, "32": 10.0},         # within the margin: keep 32
                               "x_lines": {"4": 6.0, "8": 7.0},                # faster by 14%: take 4
                               "y_columns": {"4": 8.0, "16": 8.5},             # faster by 6%: take 4
                               "levels": {"2": 40.0, "16": 110.0}}}
    assert autotune.choose(entry) == {"dct_columns": 32, "x_lines": 4, "y_columns": 4, "levels": 2}
    entry["tuned"] = autotune.choose(entry)
    template = os.path.join(os.path.dirname(__file__), "..", "oceananigans.jl_gb300", "csrc", "gbo_launch_table.h")
    out = tmp_path / "table.h"
    autotune.write_table([entry], str(out), template)
    text = out.read_text()
    assert "{64, 64, 32, 0, 0, 32, 4, 4, 2},  // rect" in text
    assert text.count("// BEGIN TABLE") == 1 and "tuned_shape" in text
