"""The library's defaults against the reference defaults restated in the oracle.

The oracle is configured by its own descriptors (oracle.grid_desc / model_desc),
whose unspecified parameters take the reference's defaults written out in
oracle.REFERENCE_DEFAULTS with their source lines.  These CPU tests check that
the library reaches the same numbers for the same keyword arguments: the
Python mirror's constructor defaults, the C library's gbo_model_desc_default,
and the conjugate-gradient defaults the library fills in (gbo_cg_parameters).
A wrong default in the library would therefore fail here rather than pass every
parity test unseen.
"""
import ctypes
import math

import numpy as np
import pytest

import cases
import oceananigans_gb300 as og
import oracle
from oceananigans_gb300 import _lib as L

R = oracle.REFERENCE_DEFAULTS


def test_python_constructor_defaults_are_the_reference_defaults():
    s = og.SmagorinskyLilly()
    assert (s.C, s.Cb, s.Pr) == (R["SmagorinskyLilly"]["C"], R["SmagorinskyLilly"]["Cb"], R["SmagorinskyLilly"]["Pr"])
    c = og.Smagorinsky()
    assert (c.C, c.Pr) == (R["Smagorinsky"]["coefficient"], R["Smagorinsky"]["Pr"])
    assert og.AnisotropicMinimumDissipation().C == R["AnisotropicMinimumDissipation"]["C"]
    d = og.DynamicSmagorinsky()
    assert isinstance(d.averaging, og.LagrangianAveraging) and R["DynamicSmagorinsky"]["averaging"] == "lagrangian"
    assert (d.Pr, d.minimum_numerator) == (R["DynamicSmagorinsky"]["Pr"], R["DynamicSmagorinsky"]["minimum_numerator"])
    k = og.ScalarDiffusivity()
    assert (k.nu, k.kappa) == (R["ScalarDiffusivity"]["nu"], R["ScalarDiffusivity"]["kappa"])
    assert og.QuasiAdamsBashforth2TimeStepper().chi == R["QuasiAdamsBashforth2"]["chi"]
    f = og.FPlane(latitude=45.0).f
    assert f == pytest.approx(2 * R["FPlane"]["rotation_rate"] * math.sin(math.radians(45.0)), rel=1e-15)


def test_c_library_desc_defaults_are_the_reference_defaults():
    d = L.ModelDesc()
    L.load().gbo_model_desc_default(ctypes.byref(d))
    assert d.advection == L.GBO_ADVECTION_WENO5 and d.closure == L.GBO_CLOSURE_NONE
    assert (d.closure_C, d.closure_Cb, d.closure_Pr) == tuple(R["SmagorinskyLilly"][k] for k in ("C", "Cb", "Pr"))
    assert d.ab2_chi == R["QuasiAdamsBashforth2"]["chi"]
    assert d.closure_min_numerator == R["DynamicSmagorinsky"]["minimum_numerator"]
    assert d.closure_averaging == L.GBO_AVERAGING_LAGRANGIAN
    assert d.timestepper == L.GBO_TIMESTEPPER_RK3 and d.pressure_solver == L.GBO_SOLVER_FFT
    assert d.preconditioner == L.GBO_PRECOND_FFT


@pytest.mark.parametrize("float_type", [np.float32, np.float64])
def test_cg_defaults_are_the_reference_defaults(float_type):
    c = cases.seamount((16, 12, 8), float_type=float_type, solver="cg")
    mdesc, _ = og.api.model_descriptor(c.grid, **c.physics)
    got = [ctypes.c_double() for _ in range(3)]
    L.check(L.load().gbo_cg_parameters(ctypes.byref(c.grid.descriptor()), ctypes.byref(mdesc),
                                       *[ctypes.byref(g) for g in got]))
    odesc = c.oracle_model().desc
    want = (odesc.cg_reltol, odesc.cg_abstol, float(odesc.cg_maxiter))
    assert tuple(g.value for g in got) == want
    assert want == (math.sqrt(np.finfo(float_type).eps),) * 2 + (16 * 12 * 8.0,)
    # explicit values pass through unchanged on both sides
    c = cases.seamount((16, 12, 8), float_type=float_type, solver="cg", reltol=1e-9, abstol=1e-20)
    mdesc, _ = og.api.model_descriptor(c.grid, **c.physics)
    L.load().gbo_cg_parameters(ctypes.byref(c.grid.descriptor()), ctypes.byref(mdesc), *[ctypes.byref(g) for g in got])
    assert (got[0].value, got[1].value) == (1e-9, 1e-20) == (c.oracle_model().desc.cg_reltol, c.oracle_model().desc.cg_abstol)


# fields of the descriptor that each closure kind reads
_CLOSURE_FIELDS = {0: (), 1: ("closure_C", "closure_Cb", "closure_Pr"), 2: ("closure_C",),
                   3: ("closure_nu", "closure_kappa"), 4: ("closure_Pr", "closure_min_numerator", "closure_averaging")}
_COMMON = ("advection", "closure", "ntracers", "buoyancy_tracer", "has_coriolis", "coriolis_f", "tracer_flux_top",
           "tracer_flux_bottom", "pressure_solver", "timestepper", "ab2_chi")


@pytest.mark.parametrize("case", [
    lambda: cases.turbulence_2d(16),
    lambda: cases.convection_3d((16, 16, 8)),
    lambda: cases.convection_3d((16, 16, 8), closure="amd", stretched=True),
    lambda: cases.convection_3d((16, 16, 8), closure="dynamic"),
    lambda: cases.convection_3d((16, 16, 8), closure="lagrangian", timestepper="QuasiAdamsBashforth2"),
    lambda: cases.convection_3d((16, 16, 8), closure="scalar", f=0.0),
    lambda: cases.diffusion_cosine("c"),
    lambda: cases.seamount((16, 16, 8), solver="cg-none", closure="smagorinsky"),
    lambda: cases.seamount((16, 16, 8), solver="fft", stretched=True),
])
def test_library_and_oracle_descriptors_agree(case):
    c = case()
    mdesc, tracers = og.api.model_descriptor(c.grid, **c.physics)
    ref = c.oracle_model()
    odesc = ref.desc
    assert tuple(tracers) == ref.tracers
    for f in _COMMON + _CLOSURE_FIELDS[mdesc.closure]:
        a, b = getattr(mdesc, f), getattr(odesc, f)
        if isinstance(a, ctypes.Array):
            a, b = list(a), list(b)
        assert a == b, f
    if mdesc.pressure_solver == L.GBO_SOLVER_CONJUGATE_GRADIENT:
        assert mdesc.preconditioner == odesc.preconditioner
    # the grids: same sizes, topology, extents, faces and bottom heights
    g, og_ = c.grid.descriptor(), ref.grid
    assert list(g.size) == list(og_.size) and list(g.topology) == list(og_.topology)
    assert list(g.x) == list(og_.x) and list(g.y) == list(og_.y) and list(g.z) == list(og_.z)
    assert g.float_type == og_.float_type
    assert bool(g.z_faces) == bool(og_.z_faces) and bool(g.bottom_height) == bool(og_.bottom_height)
    nz = g.size[2] + 1
    if g.z_faces:
        assert g.z_faces[:nz] == og_.z_faces[:nz]
    if g.bottom_height:
        n = g.size[0] * g.size[1]
        assert g.bottom_height[:n] == og_.bottom_height[:n]
