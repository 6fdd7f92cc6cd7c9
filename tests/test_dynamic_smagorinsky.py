"""DynamicSmagorinsky(averaging=(1, 2)) in the oracle, pinned against an independent
numpy restatement of the reference's operators (Smagorinskys/dynamic_coefficient.jl:
215-300, scale_invariant_operators.jl:8-13,94-188, smagorinsky.jl:90-104), plus the
properties the reference's own tests check (test_turbulence_closures.jl:421-465: the
closure builds and yields a non-zero eddy viscosity from random velocities) and the
host-side validation of the C ABI.  The reference has no golden values for this closure.

The numpy version stores every field with 3 halo levels in z (one mirrored layer beyond
each wall for Center fields, zeros beyond it, w zero on and beyond the walls) and wraps
x and y periodically, as the reference's fields are filled."""
import numpy as np
import pytest

import cases
import oceananigans_gb300 as og

H = 3  # z halo levels of the padded arrays


def _X(a, d):
    return np.roll(a, -d, axis=0)


def _Y(a, d):
    return np.roll(a, -d, axis=1)


def _Z(a, d):
    out = np.zeros_like(a)
    if d > 0:
        out[:, :, :-d] = a[:, :, d:]
    else:
        out[:, :, -d:] = a[:, :, :d]
    return out


def _pad_center(c):
    Nx, Ny, Nz = c.shape
    p = np.zeros((Nx, Ny, Nz + 2 * H + 1))
    p[:, :, H:H + Nz] = c
    p[:, :, H - 1] = c[:, :, 0]
    p[:, :, H + Nz] = c[:, :, -1]
    return p


def _pad_face(w):
    Nx, Ny, Nf = w.shape
    p = np.zeros((Nx, Ny, Nf + 2 * H))
    p[:, :, H + 1:H + Nf - 1] = w[:, :, 1:-1]  # walls (faces 0 and Nz) stay zero
    return p


def _filt(a):
    return (6 * a + _X(a, 1) + _X(a, -1) + _Y(a, 1) + _Y(a, -1) + _Z(a, 1) + _Z(a, -1)) / 12


def _strain(U, V, W, dx, dy, dz):
    s11 = (_X(U, 1) - U) / dx
    s22 = (_Y(V, 1) - V) / dy
    s33 = (_Z(W, 1) - W) / dz
    s12 = 0.5 * ((U - _Y(U, -1)) / dy + (V - _X(V, -1)) / dx)
    s13 = 0.5 * ((U - _Z(U, -1)) / dz + (W - _X(W, -1)) / dx)
    s23 = 0.5 * ((V - _Z(V, -1)) / dz + (W - _Y(W, -1)) / dy)
    return s11, s22, s33, s12, s13, s23


def _ixy(q):
    return 0.5 * (0.5 * (q + _X(q, 1)) + 0.5 * (_Y(q, 1) + _X(_Y(q, 1), 1)))


def _ixz(q):
    return 0.5 * (0.5 * (q + _X(q, 1)) + 0.5 * (_Z(q, 1) + _X(_Z(q, 1), 1)))


def _iyz(q):
    return 0.5 * (0.5 * (q + _Y(q, 1)) + 0.5 * (_Z(q, 1) + _Y(_Z(q, 1), 1)))


def _sig2(s):
    s11, s22, s33, s12, s13, s23 = s
    return s11 ** 2 + s22 ** 2 + s33 ** 2 + 2 * _ixy(s12 ** 2) + 2 * _ixz(s13 ** 2) + 2 * _iyz(s23 ** 2)


def numpy_lm_mm(u, v, w, L):
    """Per-cell LᵢⱼMᵢⱼ, MᵢⱼMᵢⱼ, Σ² and Δᶠ on a regular Periodic-Periodic-Bounded grid."""
    Nx, Ny, Nz = u.shape
    dx, dy, dz = L[0] / Nx, L[1] / Ny, L[2] / Nz
    U, V, W = _pad_center(u), _pad_center(v), _pad_face(w)
    interior = slice(H, H + Nz)
    S = _strain(U, V, W, dx, dy, dz)
    FU, FV, FW = _filt(U), _filt(V), _filt(W)
    SB = _strain(FU, FV, FW, dx, dy, dz)
    sig2 = _sig2(S)
    SG = _pad_center(np.sqrt(sig2[:, :, interior]))
    SBB = _pad_center(np.sqrt(_sig2(SB)[:, :, interior]))
    # Leonard stresses from cell-centre products
    ixu, iyv, izw = 0.5 * (U + _X(U, 1)), 0.5 * (V + _Y(V, 1)), 0.5 * (W + _Z(W, 1))
    ixfu, iyfv, izfw = 0.5 * (FU + _X(FU, 1)), 0.5 * (FV + _Y(FV, 1)), 0.5 * (FW + _Z(FW, 1))
    Ls = [_filt(0.5 * (U ** 2 + _X(U, 1) ** 2)) - 0.5 * (FU ** 2 + _X(FU, 1) ** 2),
          _filt(0.5 * (V ** 2 + _Y(V, 1) ** 2)) - 0.5 * (FV ** 2 + _Y(FV, 1) ** 2),
          _filt(0.5 * (W ** 2 + _Z(W, 1) ** 2)) - 0.5 * (FW ** 2 + _Z(FW, 1) ** 2),
          _filt(ixu * iyv) - ixfu * iyfv,
          _filt(ixu * izw) - ixfu * izfw,
          _filt(iyv * izw) - iyfv * izfw]
    s11, s22, s33, s12, s13, s23 = S
    b11, b22, b33, b12, b13, b23 = SB
    ss = [SG * s11, SG * s22, SG * s33, SG * _ixy(s12), SG * _ixz(s13), SG * _iyz(s23)]
    bb = [SBB * b11, SBB * b22, SBB * b33, SBB * _ixy(b12), SBB * _ixz(b13), SBB * _iyz(b23)]
    Df = np.cbrt(dx * dy * dz)
    Ms = [2 * Df ** 2 * (_filt(a) - 4 * b) for a, b in zip(ss, bb)]
    wts = [1, 1, 1, 2, 2, 2]
    LM = sum(c * l * m for c, l, m in zip(wts, Ls, Ms))[:, :, interior]
    MM = sum(c * m * m for c, m in zip(wts, Ms))[:, :, interior]
    return LM, MM, sig2[:, :, interior], Df


def numpy_dynamic_nu(u, v, w, L, min_numerator=1e-32):
    """νₑ of DynamicSmagorinsky(averaging=(1, 2)) on a regular Periodic-Periodic-Bounded grid."""
    LM, MM, sig2, Df = numpy_lm_mm(u, v, w, L)
    jlm, jmm = LM.mean(axis=(0, 1)), MM.mean(axis=(0, 1))
    num = np.maximum(jlm, min_numerator)
    cs2 = np.where(jmm > 0, num / np.where(jmm > 0, jmm, 1.0), 0.0)
    return cs2[None, None, :] * Df ** 2 * np.sqrt(2 * sig2)


def _random_case(N=(12, 10, 8), seed=3, U0=0.3, closure="dynamic", **kw):
    c = cases.convection_3d(N, closure=closure, f=0.0, flux=0.0, U0=U0, seed=seed, **kw)
    w = c.init["w"].copy()
    w[:, :, 0] = 0.0
    w[:, :, -1] = 0.0
    c.init["w"] = w
    return c


def test_oracle_matches_numpy_restatement():
    c = _random_case()
    ref = c.oracle_model()
    ref.set(**c.init)
    ref.finalize_set(False)
    nu = numpy_dynamic_nu(c.init["u"], c.init["v"], c.init["w"], (512.0, 512.0, 256.0))
    got = ref.get("nu")
    assert np.any(nu > 0)
    assert cases.rel_l2(got, nu) <= 1e-13


def test_dynamic_viscosity_nonnegative_and_nonzero_from_random_velocities():
    # test_turbulence_closures.jl:457-465 checks a non-zero νₑ after random velocities
    c = _random_case(N=(16, 16, 8), seed=11)
    ref = c.oracle_model()
    ref.set(**c.init)
    ref.finalize_set(True)
    nu = ref.get("nu")
    assert np.all(nu >= 0) and np.any(nu > 0)


def test_zero_flow_has_zero_viscosity():
    c = _random_case(U0=0.0)
    ref = c.oracle_model()
    ref.set(**c.init)
    ref.finalize_set(False)
    assert np.all(ref.get("nu") == 0.0)


def test_unsupported_averaging_and_grids_rejected():
    with pytest.raises(ValueError, match="averaging"):
        og.DynamicSmagorinsky(averaging=(2, 3))
    with pytest.raises(ValueError, match="schedule"):
        og.DynamicSmagorinsky(schedule=5)
    flat = og.RectilinearGrid(size=(16, 16), x=(0, 1), y=(0, 1), topology=("Periodic", "Periodic", "Flat"))
    # invalid configurations are rejected on the host, before any device work
    with pytest.raises(ValueError, match="Bounded z"):
        og.NonhydrostaticModel(flat, advection=og.WENO(), closure=og.DynamicSmagorinsky())
    c = cases.seamount((16, 16, 8), solver="cg")
    with pytest.raises(ValueError, match="ImmersedBoundaryGrid"):
        og.NonhydrostaticModel(c.grid, advection=og.WENO(), closure=og.DynamicSmagorinsky(),
                               pressure_solver=og.ConjugateGradientPoissonSolver())


# ---- LagrangianAveraging (dynamic_coefficient.jl:322-487): the oracle's restatement ----

def test_lagrangian_initialization_matches_numpy():
    # initialize_closure_fields!: 𝒥ᴸᴹ = max(mean LM, min), 𝒥ᴹᴹ = mean MM over the whole
    # domain, so νₑ = c² Δᶠ² √(2Σ²) with one c² everywhere
    c = _random_case(closure="lagrangian")
    ref = c.oracle_model()
    ref.set(**c.init)
    ref.finalize_set(False)
    LM, MM, sig2, Df = numpy_lm_mm(c.init["u"], c.init["v"], c.init["w"], (512.0, 512.0, 256.0))
    jlm, jmm = max(LM.mean(), 1e-32), MM.mean()
    assert cases.rel_l2(ref.get("jlm"), np.full(LM.shape, jlm)) <= 1e-12
    assert cases.rel_l2(ref.get("jmm"), np.full(LM.shape, jmm)) <= 1e-13
    assert cases.rel_l2(ref.get("nu"), jlm / jmm * Df ** 2 * np.sqrt(2 * sig2)) <= 1e-12


@pytest.mark.parametrize("timestepper", ["RungeKutta3", "QuasiAdamsBashforth2"])
def test_lagrangian_step_bounds(timestepper):
    c = _random_case(N=(16, 16, 8), seed=5, U0=0.05, closure="lagrangian", timestepper=timestepper)
    ref = c.oracle_model()
    ref.set(**c.init)
    ref.finalize_set(True)
    jlm0 = ref.get("jlm")
    ref.time_step(2.0, 3)
    jlm, jmm, nu = ref.get("jlm"), ref.get("jmm"), ref.get("nu")
    assert np.all(np.isfinite(jlm)) and np.all(np.isfinite(jmm))
    assert np.all(jlm >= 1e-32) and np.all(jmm >= 0) and np.all(nu >= 0)
    assert np.ptp(jlm) > 0 and np.ptp(jlm0) == 0  # constant after set!, pointwise after the steps


def test_lagrangian_relaxation_vanishes_with_the_step():
    # ϵ = τ / (1 + τ) with τ = Δt / T: a short step barely moves 𝒥 away from its
    # initial constant, a longer one moves it further
    moves = []
    for dt in (1e-4, 1e-1):
        c = _random_case(N=(16, 16, 8), seed=5, U0=0.05, closure="lagrangian")
        ref = c.oracle_model()
        ref.set(**c.init)
        ref.finalize_set(True)
        j0 = ref.get("jmm").mean()
        ref.time_step(dt)
        moves.append(np.abs(ref.get("jmm") - j0).max() / j0)
    assert moves[0] < 1e-2 and moves[1] > 10 * moves[0]


def test_lagrangian_rejected_in_an_ensemble():
    # an ensemble steps its members together; the Lagrangian clock is per model.  The
    # check runs on the host before any member is built.
    c = _random_case(closure="lagrangian")
    with pytest.raises(ValueError, match="Lagrangian-averaged DynamicSmagorinsky cannot join an ensemble"):
        og.Ensemble([(c.grid, c.physics)])


# ---- the Lagrangian update restated on the oracle's own arrays (halos as they are) ----

def _shift(a, d, axis):
    """out[i] = a[i + d] along axis, zero beyond the array."""
    out = np.zeros_like(a)
    n = a.shape[axis]
    dst, src = [slice(None)] * 3, [slice(None)] * 3
    if d > 0:
        dst[axis], src[axis] = slice(0, n - d), slice(d, n)
    else:
        dst[axis], src[axis] = slice(-d, n), slice(0, n + d)
    out[tuple(dst)] = a[tuple(src)]
    return out


def _lm_mm_parents(U, V, W, dx, dy, dz):
    """LM, MM, Σ², Δᶠ at the interior from parent arrays with 3 halo points on every side
    (all shifts by slicing, so the arrays' own halo values are used)."""
    global _X, _Y, _Z
    saved = (_X, _Y, _Z)
    _X, _Y, _Z = (lambda a, d: _shift(a, d, 0)), (lambda a, d: _shift(a, d, 1)), (lambda a, d: _shift(a, d, 2))
    try:
        Nx, Ny = U.shape[0] - 2 * H, U.shape[1] - 2 * H
        Nz = W.shape[2] - 2 * H - 1
        Uc = np.zeros_like(W)
        Uc[:, :, :-1] = U
        Vc = np.zeros_like(W)
        Vc[:, :, :-1] = V
        I = (slice(H, H + Nx), slice(H, H + Ny), slice(H, H + Nz))

        def fill(c):  # Σ, Σ̄ halos: one mirrored z layer, zeros beyond, periodic x and y
            p = _pad_center(c)
            return np.pad(p, ((H, H), (H, H), (0, 0)), mode="wrap")

        S = _strain(Uc, Vc, W, dx, dy, dz)
        FU, FV, FW = _filt(Uc), _filt(Vc), _filt(W)
        SB = _strain(FU, FV, FW, dx, dy, dz)
        sig2 = _sig2(S)
        SG, SBB = fill(np.sqrt(sig2[I])), fill(np.sqrt(_sig2(SB)[I]))
        ixu, iyv, izw = 0.5 * (Uc + _X(Uc, 1)), 0.5 * (Vc + _Y(Vc, 1)), 0.5 * (W + _Z(W, 1))
        ixfu, iyfv, izfw = 0.5 * (FU + _X(FU, 1)), 0.5 * (FV + _Y(FV, 1)), 0.5 * (FW + _Z(FW, 1))
        Ls = [_filt(0.5 * (Uc ** 2 + _X(Uc, 1) ** 2)) - 0.5 * (FU ** 2 + _X(FU, 1) ** 2),
              _filt(0.5 * (Vc ** 2 + _Y(Vc, 1) ** 2)) - 0.5 * (FV ** 2 + _Y(FV, 1) ** 2),
              _filt(0.5 * (W ** 2 + _Z(W, 1) ** 2)) - 0.5 * (FW ** 2 + _Z(FW, 1) ** 2),
              _filt(ixu * iyv) - ixfu * iyfv, _filt(ixu * izw) - ixfu * izfw, _filt(iyv * izw) - iyfv * izfw]
        s11, s22, s33, s12, s13, s23 = S
        b11, b22, b33, b12, b13, b23 = SB
        ss = [SG * s11, SG * s22, SG * s33, SG * _ixy(s12), SG * _ixz(s13), SG * _iyz(s23)]
        bb = [SBB * b11, SBB * b22, SBB * b33, SBB * _ixy(b12), SBB * _ixz(b13), SBB * _iyz(b23)]
        Df = np.cbrt(dx * dy * dz)
        Ms = [2 * Df ** 2 * (_filt(a) - 4 * b) for a, b in zip(ss, bb)]
        wts = [1, 1, 1, 2, 2, 2]
        LM = sum(c * l * m for c, l, m in zip(wts, Ls, Ms))[I]
        MM = sum(c * m * m for c, m in zip(wts, Ms))[I]
        return LM, MM, I, Df
    finally:
        _X, _Y, _Z = saved


def numpy_lagrangian_update(ref, dt, L, z0, lmin=1e-32):
    """𝒥ᴸᴹ, 𝒥ᴹᴹ after one update from the oracle's current parent arrays
    (_lagrangian_average_LM_MM!, dynamic_coefficient.jl:342-405)."""
    U, V, W = ref.parent("u"), ref.parent("v"), ref.parent("w")
    JL, JM = ref.parent("jlm"), ref.parent("jmm")
    Nx, Ny, Nz = ref.shape
    dx, dy, dz = L[0] / Nx, L[1] / Ny, L[2] / Nz
    LM, MM, I, Df = _lm_mm_parents(U, V, W, dx, dy, dz)
    lmp, mmp = np.maximum(JL[I], lmin), JM[I]
    with np.errstate(divide="ignore"):
        T = 1.5 * Df / np.sqrt(np.sqrt(np.sqrt(lmp * mmp)))
    tau = dt / T
    eps = tau / (1 + tau)
    i, j, k = np.meshgrid(np.arange(1, Nx + 1), np.arange(1, Ny + 1), np.arange(1, Nz + 1), indexing="ij")
    x, y, z = (i - 0.5) * dx, (j - 0.5) * dy, z0 + (k - 0.5) * dz
    ddx = np.clip(U[I] * dt, -dx, dx)
    ddy = np.clip(V[I] * dt, -dy, dy)
    ddz = np.clip(W[I] * dt, -dz, dz)
    fi, fj, fk = (x - ddx - 0.5 * dx) / dx + 1, (y - ddy - 0.5 * dy) / dy + 1, (z - ddz - (z0 + 0.5 * dz)) / dz + 1

    def itp(F):
        i0, j0, k0 = (np.trunc(f).astype(int) for f in (fi, fj, fk))
        a, b, c = np.mod(fi, 1.0), np.mod(fj, 1.0), np.mod(fk, 1.0)
        g = lambda p, q, r: F[p + H - 1, q + H - 1, r + H - 1]  # noqa: E731  (1-based index -> parent)
        return ((1 - a) * (1 - b) * (1 - c) * g(i0, j0, k0) + (1 - a) * (1 - b) * c * g(i0, j0, k0 + 1) +
                (1 - a) * b * (1 - c) * g(i0, j0 + 1, k0) + (1 - a) * b * c * g(i0, j0 + 1, k0 + 1) +
                a * (1 - b) * (1 - c) * g(i0 + 1, j0, k0) + a * (1 - b) * c * g(i0 + 1, j0, k0 + 1) +
                a * b * (1 - c) * g(i0 + 1, j0 + 1, k0) + a * b * c * g(i0 + 1, j0 + 1, k0 + 1))

    jmm = eps * MM + (1 - eps) * itp(JM)
    jlm = np.maximum(eps * LM + (1 - eps) * np.maximum(itp(JL), lmin), lmin)
    return jlm, jmm


@pytest.mark.parametrize("dt", [2.0, 2000.0])
def test_lagrangian_update_matches_numpy(dt):
    # after a step 𝒥 varies in space; one more update from those arrays, in the oracle and
    # in numpy (dt = 2000 s clamps most displacements at one cell)
    c = _random_case(N=(16, 12, 8), seed=9, U0=0.05, closure="lagrangian")
    ref = c.oracle_model()
    ref.set(**c.init)
    ref.finalize_set(True)
    ref.time_step(2.0)
    t = ref.clock()[0]
    if dt > 100:
        assert np.mean(np.abs(ref.get("u")) * dt > 512.0 / 16) > 0.5
    want_lm, want_mm = numpy_lagrangian_update(ref, (t + dt) - t, (512.0, 512.0, 256.0), -256.0)
    ref.lagrangian_update(dt)
    assert cases.rel_l2(ref.get("jmm"), want_mm) <= 1e-12
    assert cases.rel_l2(ref.get("jlm"), want_lm) <= 1e-12


def test_closure_defaults_and_descriptor():
    # DynamicSmagorinsky() defaults to LagrangianAveraging, Pr = 1, minimum_numerator = 1e-32
    # (dynamic_coefficient.jl:104-117); the descriptor carries each choice
    from oceananigans_gb300 import _lib as L
    from oceananigans_gb300.api import model_descriptor
    c = _random_case()
    d0 = og.DynamicSmagorinsky()
    assert isinstance(d0.averaging, og.LagrangianAveraging) and d0.Pr == 1.0 and d0.minimum_numerator == 1e-32
    assert og.DynamicSmagorinsky(averaging=[2, 1]).averaging == (1, 2)
    for closure, avg in ((d0, L.GBO_AVERAGING_LAGRANGIAN),
                         (og.DynamicSmagorinsky(averaging=(1, 2), Pr=0.5, minimum_numerator=1e-20), L.GBO_AVERAGING_XY)):
        d, _ = model_descriptor(c.grid, advection=og.WENO(), closure=closure, tracers=("b",), buoyancy=og.BuoyancyTracer())
        assert d.closure == L.GBO_CLOSURE_DYNAMIC_SMAGORINSKY and d.closure_averaging == avg
        assert d.closure_Pr == closure.Pr and d.closure_min_numerator == closure.minimum_numerator


def test_constant_smagorinsky_is_lilly_without_buoyancy_reduction():
    # Smagorinsky(coefficient=C): νₑ = C² Δᶠ² √(2Σ²) (smagorinsky.jl:90-106), here from the
    # oracle through the Lilly path with Cb = 0, against the numpy strain
    c = _random_case(closure=None)
    c = c.with_physics(dict(c.ophysics, closure=("Smagorinsky", {"coefficient": 0.2})),
                       **dict(c.physics, closure=og.Smagorinsky(coefficient=0.2)))
    ref = c.oracle_model()
    ref.set(**c.init)
    ref.finalize_set(False)
    _, _, sig2, Df = numpy_lm_mm(c.init["u"], c.init["v"], c.init["w"], (512.0, 512.0, 256.0))
    assert cases.rel_l2(ref.get("nu"), 0.2 ** 2 * Df ** 2 * np.sqrt(2 * sig2)) <= 1e-13
    with pytest.raises(ValueError, match="number"):
        og.Smagorinsky(coefficient="dynamic")
