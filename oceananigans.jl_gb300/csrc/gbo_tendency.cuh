// gbo_tendency.cuh -- per-point tendency terms of the NonhydrostaticModel on device.
//
// Each function restates one term of
//   u_velocity_tendency / v_velocity_tendency / w_velocity_tendency / tracer_tendency
//   (src/Models/NonhydrostaticModels/nonhydrostatic_tendency_kernel_functions.jl:71-302)
// in flux form (src/Advection/momentum_advection_operators.jl:47-84,
// tracer_advection_operators.jl:31-35, upwind_biased_advective_fluxes.jl:23-121),
// with the closure divergences of src/TurbulenceClosures/closure_kernel_operators.jl:20-46
// and abstract_scalar_diffusivity_closure.jl:214-262.  Indices are 0-based; the
// reference's 1-based vertical level is kr = k + 1 wherever the Bounded-z buffer
// schemes depend on the absolute level.
#pragma once
#include "gbo_weno.cuh"

template <typename FT>
struct Fields {
    CFld<FT> u, v, nu, phy;
    WFld<FT> w;
};

template <typename FT>
struct Met {
    const GridP<FT>& g;
    GBO_D explicit Met(const GridP<FT>& gg) : g(gg) {}
    GBO_D FT dzc(int k) const { return g.flatz ? FT(1) : g.dzc[k + 1 + g.zoff]; }
    GBO_D FT dzf(int k) const { return g.flatz ? FT(1) : g.dzf[k + 1 + g.zoff]; }
    GBO_D FT rdzc(int k) const { return g.flatz ? FT(1) : g.rdzc[k + 1 + g.zoff]; }
    GBO_D FT rdzf(int k) const { return g.flatz ? FT(1) : g.rdzf[k + 1 + g.zoff]; }
    GBO_D FT Ax(int k) const { return g.dy * dzc(k); }   // Axᶠᶜᶜ
    GBO_D FT Axf(int k) const { return g.dy * dzf(k); }  // Axᶠᶜᶠ
    GBO_D FT Ay(int k) const { return g.dx * dzc(k); }   // Ayᶜᶠᶜ
    GBO_D FT Ayf(int k) const { return g.dx * dzf(k); }  // Ayᶜᶠᶠ
    GBO_D FT Az() const { return g.dx * g.dy; }          // Azᶜᶜᵃ
    GBO_D FT rVc(int k) const { return g.flatz ? FT(1) / Az() : g.rvc[k + 1 + g.zoff]; }
    GBO_D FT rVf(int k) const { return FT(1) / (Az() * dzf(k)); }
};

// ---------------------------------------------------------------------------
// Immersed boundary (GridFittedBottom): a cell is immersed when its centre is at or
// below the bottom (grid_fitted_bottom.jl:150-158); kbot[i + Nx j] is the number of
// immersed cells of the column.  Predicates follow src/Grids/inactive_node.jl and
// src/ImmersedBoundaries/immersed_boundary_interface.jl.
// ---------------------------------------------------------------------------
template <typename FT>
GBO_D bool imm_cell(const GridP<FT>& g, int i, int j, int k) {
    if (!g.kbot || k < 0 || k >= g.Nz) return false;
    return k < __ldg(g.kbot + wrapi(i, g.Nx) + (size_t)g.Nx * wrapi(j, g.Ny));
}
template <typename FT>
GBO_D bool inactive_cell(const GridP<FT>& g, int i, int j, int k) {
    return (!g.flatz && (k < 0 || k >= g.Nz)) || imm_cell(g, i, j, k);
}
// immersed_peripheral_node at a location with Face flags (fx, fy, fz)
template <typename FT>
GBO_D bool imm_periph(const GridP<FT>& g, int i, int j, int k, bool fx, bool fy, bool fz) {
    if (!g.kbot) return false;
    bool any_imm = false, any_out = false;
    for (int a = 0; a <= (fx ? 1 : 0); ++a)
        for (int b = 0; b <= (fy ? 1 : 0); ++b)
            for (int c = 0; c <= (fz ? 1 : 0); ++c) {
                int kk = k - c;
                bool out = !g.flatz && (kk < 0 || kk >= g.Nz);
                any_out |= out;
                any_imm |= (!out) && imm_cell(g, i - a, j - b, kk);
            }
    return any_imm && !any_out;
}
// Reconstruction level near immersed nodes (immersed_advective_fluxes.jl:114-214): 3 (WENO5 /
// Centered 4), 2 (WENO3) or 1 (Centered 2); d = direction, loc_face = Face location of the
// interpolation index.  Out-of-domain cells count as inactive, which reproduces the wall
// buffer rules exactly.
template <typename FT>
GBO_D int ibg_level(const GridP<FT>& g, int d, int i, int j, int k, bool loc_face) {
    for (int B = 3; B >= 2; --B) {
        int lo = loc_face ? -B : -B + 1, hi = loc_face ? B - 1 : B;
        bool near = false;
        for (int o = lo; o <= hi; ++o) {
            int ii = i + (d == 0 ? o : 0), jj = j + (d == 1 ? o : 0), kk = k + (d == 2 ? o : 0);
            bool inact = inactive_cell(g, ii, jj, kk);
            if (!loc_face) inact = inact && inactive_cell(g, ii - (d == 0), jj - (d == 1), kk - (d == 2));
            near |= inact;
        }
        if (!near) return B;
    }
    return 1;
}
// immersed_inactive_node at (i, j, k) of a location with Face flags (fx, fy, fz):
// inactive on the immersed grid (every adjacent cell inactive, inactive_node.jl:127-137)
// but active on the underlying grid (immersed_boundary_interface.jl:59-60)
template <typename FT>
GBO_D bool imm_inactive_node(const GridP<FT>& g, int i, int j, int k, bool fx, bool fy, bool fz) {
    if (!g.kbot) return false;
    bool all = true, all_out = true;
    for (int a = 0; a <= (fx ? 1 : 0); ++a)
        for (int b = 0; b <= (fy ? 1 : 0); ++b)
            for (int c = 0; c <= (fz ? 1 : 0); ++c) {
                const int kk = k - c;
                const bool out = !g.flatz && (kk < 0 || kk >= g.Nz);
                all_out = all_out && out;
                all = all && (out || imm_cell(g, i - a, j - b, kk));
            }
    return all && !all_out;
}
// immersed-aware ∂ mask: a difference across a face is zero when either cell is immersed
template <typename FT>
GBO_D bool cond_zero(const GridP<FT>& g, int i0, int j0, int k0, int i1, int j1, int k1) {
    return g.kbot && (imm_cell(g, i0, j0, k0) || imm_cell(g, i1, j1, k1));
}

GBO_D bool bias_left(float u) { return u > 0.f; }
GBO_D bool bias_left(double u) { return u > 0.0; }

// ---------------------------------------------------------------------------
// Momentum advective fluxes (advection of B by A in advective_momentum_flux_AB)
// ---------------------------------------------------------------------------
template <typename FT>
struct MomentumFluxes {
    const GridP<FT>& g;
    const Fields<FT>& F;
    Met<FT> M;
    GBO_D MomentumFluxes(const GridP<FT>& gg, const Fields<FT>& ff) : g(gg), F(ff), M(gg) {}

    // Uu at (c,c,c)
    // levels of horizontal reconstructions (always WENO5 / C4 away from immersed nodes)
    GBO_D int hl(int d, int i, int j, int k, bool face) const { return g.kbot ? ibg_level(g, d, i, j, k, face) : 3; }
    GBO_D int hs(int d, int i, int j, int k, bool face) const { return hl(d, i, j, k, face) == 3 ? 3 : 1; }
    GBO_D int zb(int i, int j, int k, bool face) const {
        return g.kbot ? ibg_level(g, 2, i, j, k, face) : (face ? zlev_biased_face(k + 1, g.Nz) : zlev_biased_center(k + 1, g.Nz));
    }
    GBO_D int zs(int i, int j, int k, bool face) const {
        return g.kbot ? (ibg_level(g, 2, i, j, k, face) == 3 ? 3 : 1) : (face ? zlev_symm_face(k + 1, g.Nz) : zlev_symm_center(k + 1, g.Nz));
    }
    GBO_D bool zero(int i, int j, int k, bool fx, bool fy, bool fz) const { return imm_periph(g, i, j, k, fx, fy, fz); }

    GBO_D FT Uu(int i, int j, int k) const {
        if (g.kbot && zero(i, j, k, false, false, false)) return FT(0);
        FT Ax = M.Ax(k);
        auto qs = [&](int o) { return Ax * F.u(i + 1 + o, j, k); };
        FT ut = symm<FT>(qs, hs(0, i, j, k, false));
        auto qb = [&](int o) { return F.u(i + 1 + o, j, k); };
        return ut * biased<FT>(qb, bias_left(ut), hl(0, i, j, k, false));
    }
    // Vu at (f,f,c)
    GBO_D FT Vu(int i, int j, int k) const {
        if (g.kbot && zero(i, j, k, true, true, false)) return FT(0);
        FT Ay = M.Ay(k);
        auto qs = [&](int o) { return Ay * F.v(i + o, j, k); };
        FT vt = symm<FT>(qs, hs(0, i, j, k, true));
        auto qb = [&](int o) { return F.u(i, j + o, k); };
        return vt * biased<FT>(qb, bias_left(vt), hl(1, i, j, k, true));
    }
    // Wu at (f,c,f)
    GBO_D FT Wu(int i, int j, int k) const {
        if (g.kbot && zero(i, j, k, true, false, true)) return FT(0);
        FT Az = M.Az();
        auto qs = [&](int o) { return Az * F.w(i + o, j, k); };
        FT wt = symm<FT>(qs, hs(0, i, j, k, true));
        auto q = [&](int o) { return F.u(i, j, k + o); };
        return wt * biased<FT>(q, bias_left(wt), zb(i, j, k, true));
    }
    // Uv at (f,f,c)
    GBO_D FT Uv(int i, int j, int k) const {
        if (g.kbot && zero(i, j, k, true, true, false)) return FT(0);
        FT Ax = M.Ax(k);
        auto qs = [&](int o) { return Ax * F.u(i, j + o, k); };
        FT ut = symm<FT>(qs, hs(1, i, j, k, true));
        auto qb = [&](int o) { return F.v(i + o, j, k); };
        return ut * biased<FT>(qb, bias_left(ut), hl(0, i, j, k, true));
    }
    // Vv at (c,c,c)
    GBO_D FT Vv(int i, int j, int k) const {
        if (g.kbot && zero(i, j, k, false, false, false)) return FT(0);
        FT Ay = M.Ay(k);
        auto qs = [&](int o) { return Ay * F.v(i, j + 1 + o, k); };
        FT vt = symm<FT>(qs, hs(1, i, j, k, false));
        auto qb = [&](int o) { return F.v(i, j + 1 + o, k); };
        return vt * biased<FT>(qb, bias_left(vt), hl(1, i, j, k, false));
    }
    // Wv at (c,f,f)
    GBO_D FT Wv(int i, int j, int k) const {
        if (g.kbot && zero(i, j, k, false, true, true)) return FT(0);
        FT Az = M.Az();
        auto qs = [&](int o) { return Az * F.w(i, j + o, k); };
        FT wt = symm<FT>(qs, hs(1, i, j, k, true));
        auto q = [&](int o) { return F.v(i, j, k + o); };
        return wt * biased<FT>(q, bias_left(wt), zb(i, j, k, true));
    }
    // Uw at (f,c,f)
    GBO_D FT Uw(int i, int j, int k) const {
        if (g.kbot && zero(i, j, k, true, false, true)) return FT(0);
        auto qs = [&](int o) { return M.Ax(k + o) * F.u(i, j, k + o); };
        FT ut = symm<FT>(qs, zs(i, j, k, true));
        auto qb = [&](int o) { return F.w(i + o, j, k); };
        return ut * biased<FT>(qb, bias_left(ut), hl(0, i, j, k, true));
    }
    // Vw at (c,f,f)
    GBO_D FT Vw(int i, int j, int k) const {
        if (g.kbot && zero(i, j, k, false, true, true)) return FT(0);
        auto qs = [&](int o) { return M.Ay(k + o) * F.v(i, j, k + o); };
        FT vt = symm<FT>(qs, zs(i, j, k, true));
        auto qb = [&](int o) { return F.w(i, j + o, k); };
        return vt * biased<FT>(qb, bias_left(vt), hl(1, i, j, k, true));
    }
    // Ww at (c,c,c) level k: reconstructions at face k+1 with centre conditions
    GBO_D FT Ww(int i, int j, int k) const {
        if (g.kbot && zero(i, j, k, false, false, false)) return FT(0);
        FT Az = M.Az();
        auto qs = [&](int o) { return Az * F.w(i, j, k + 1 + o); };
        FT wt = symm<FT>(qs, zs(i, j, k, false));
        auto qb = [&](int o) { return F.w(i, j, k + 1 + o); };
        return wt * biased<FT>(qb, bias_left(wt), zb(i, j, k, false));
    }
};

// ---------------------------------------------------------------------------
// Closure: strain components and eddy-viscosity interpolations
// (velocity_tracer_gradients.jl:1-60; abstract_scalar_diffusivity_closure.jl:330-366)
// ---------------------------------------------------------------------------
// FL supplies u, v, w, nu accessors taking global indices: the global-memory Fields
// (halos synthesised at load) or a shared-memory tile.
template <typename FT, class FL = Fields<FT>>
struct StrainT {
    const GridP<FT>& g;
    const FL& F;
    Met<FT> M;
    GBO_D StrainT(const GridP<FT>& gg, const FL& ff) : g(gg), F(ff), M(gg) {}
    // On an immersed grid every location-specific ∂ is conditional: zero when either
    // differenced node is an immersed-inactive node of the field's location
    // (conditional_differences.jl:15-43).  u at (f,c,c), v at (c,f,c), w at (c,c,f).
    GBO_D bool cu(int i0, int j0, int k0, int i1, int j1, int k1) const {
        return g.kbot && (imm_inactive_node(g, i0, j0, k0, true, false, false) || imm_inactive_node(g, i1, j1, k1, true, false, false));
    }
    GBO_D bool cv(int i0, int j0, int k0, int i1, int j1, int k1) const {
        return g.kbot && (imm_inactive_node(g, i0, j0, k0, false, true, false) || imm_inactive_node(g, i1, j1, k1, false, true, false));
    }
    GBO_D bool cw(int i0, int j0, int k0, int i1, int j1, int k1) const {
        return g.kbot && (imm_inactive_node(g, i0, j0, k0, false, false, true) || imm_inactive_node(g, i1, j1, k1, false, false, true));
    }
    GBO_D FT S11(int i, int j, int k) const { return cu(i, j, k, i + 1, j, k) ? FT(0) : (F.u(i + 1, j, k) - F.u(i, j, k)) * g.rdx; }
    GBO_D FT S22(int i, int j, int k) const { return cv(i, j, k, i, j + 1, k) ? FT(0) : (F.v(i, j + 1, k) - F.v(i, j, k)) * g.rdy; }
    GBO_D FT S33(int i, int j, int k) const {
        return (g.flatz || cw(i, j, k, i, j, k + 1)) ? FT(0) : (F.w(i, j, k + 1) - F.w(i, j, k)) * M.rdzc(k);
    }
    GBO_D FT dyu(int i, int j, int k) const { return cu(i, j - 1, k, i, j, k) ? FT(0) : (F.u(i, j, k) - F.u(i, j - 1, k)) * g.rdy; }
    GBO_D FT dxv(int i, int j, int k) const { return cv(i - 1, j, k, i, j, k) ? FT(0) : (F.v(i, j, k) - F.v(i - 1, j, k)) * g.rdx; }
    GBO_D FT dzu(int i, int j, int k) const {
        return (g.flatz || cu(i, j, k - 1, i, j, k)) ? FT(0) : (F.u(i, j, k) - F.u(i, j, k - 1)) * M.rdzf(k);
    }
    GBO_D FT dxw(int i, int j, int k) const {
        return (g.flatz || cw(i - 1, j, k, i, j, k)) ? FT(0) : (F.w(i, j, k) - F.w(i - 1, j, k)) * g.rdx;
    }
    GBO_D FT dzv(int i, int j, int k) const {
        return (g.flatz || cv(i, j, k - 1, i, j, k)) ? FT(0) : (F.v(i, j, k) - F.v(i, j, k - 1)) * M.rdzf(k);
    }
    GBO_D FT dyw(int i, int j, int k) const {
        return (g.flatz || cw(i, j - 1, k, i, j, k)) ? FT(0) : (F.w(i, j, k) - F.w(i, j - 1, k)) * g.rdy;
    }
    GBO_D FT S12(int i, int j, int k) const { return FT(0.5) * (dyu(i, j, k) + dxv(i, j, k)); }
    GBO_D FT S13(int i, int j, int k) const { return FT(0.5) * (dzu(i, j, k) + dxw(i, j, k)); }
    GBO_D FT S23(int i, int j, int k) const { return FT(0.5) * (dzv(i, j, k) + dyw(i, j, k)); }
    GBO_D FT nu_ffc(int i, int j, int k) const {
        return FT(0.5) * (FT(0.5) * (F.nu(i - 1, j - 1, k) + F.nu(i, j - 1, k)) + FT(0.5) * (F.nu(i - 1, j, k) + F.nu(i, j, k)));
    }
    GBO_D FT nu_fcf(int i, int j, int k) const {
        if (g.flatz) return FT(0.5) * (F.nu(i - 1, j, k) + F.nu(i, j, k));
        return FT(0.5) * (FT(0.5) * (F.nu(i - 1, j, k - 1) + F.nu(i, j, k - 1)) + FT(0.5) * (F.nu(i - 1, j, k) + F.nu(i, j, k)));
    }
    GBO_D FT nu_cff(int i, int j, int k) const {
        if (g.flatz) return FT(0.5) * (F.nu(i, j - 1, k) + F.nu(i, j, k));
        return FT(0.5) * (FT(0.5) * (F.nu(i, j - 1, k - 1) + F.nu(i, j, k - 1)) + FT(0.5) * (F.nu(i, j - 1, k) + F.nu(i, j, k)));
    }
    // viscous fluxes -2 ν Σ (isotropic ScalarDiffusivity form)
    // On an immersed grid each viscous flux is zero on the immersed periphery of its
    // location (conditional_flux, immersed_diffusive_fluxes.jl:25-40); the default
    // immersed boundary condition adds no flux.
    GBO_D bool zp(int i, int j, int k, bool fx, bool fy, bool fz) const { return g.kbot && imm_periph(g, i, j, k, fx, fy, fz); }
    GBO_D FT tau_ux(int i, int j, int k) const { return zp(i, j, k, false, false, false) ? FT(0) : FT(-2) * (F.nu(i, j, k) * S11(i, j, k)); }
    GBO_D FT tau_uy(int i, int j, int k) const { return zp(i, j, k, true, true, false) ? FT(0) : FT(-2) * (nu_ffc(i, j, k) * S12(i, j, k)); }
    GBO_D FT tau_uz(int i, int j, int k) const { return zp(i, j, k, true, false, true) ? FT(0) : FT(-2) * (nu_fcf(i, j, k) * S13(i, j, k)); }
    GBO_D FT tau_vx(int i, int j, int k) const { return zp(i, j, k, true, true, false) ? FT(0) : FT(-2) * (nu_ffc(i, j, k) * S12(i, j, k)); }
    GBO_D FT tau_vy(int i, int j, int k) const { return zp(i, j, k, false, false, false) ? FT(0) : FT(-2) * (F.nu(i, j, k) * S22(i, j, k)); }
    GBO_D FT tau_vz(int i, int j, int k) const { return zp(i, j, k, false, true, true) ? FT(0) : FT(-2) * (nu_cff(i, j, k) * S23(i, j, k)); }
    GBO_D FT tau_wx(int i, int j, int k) const { return zp(i, j, k, true, false, true) ? FT(0) : FT(-2) * (nu_fcf(i, j, k) * S13(i, j, k)); }
    GBO_D FT tau_wy(int i, int j, int k) const { return zp(i, j, k, false, true, true) ? FT(0) : FT(-2) * (nu_cff(i, j, k) * S23(i, j, k)); }
    GBO_D FT tau_wz(int i, int j, int k) const { return zp(i, j, k, false, false, false) ? FT(0) : FT(-2) * (F.nu(i, j, k) * S33(i, j, k)); }
};
template <typename FT>
using Strain = StrainT<FT>;
