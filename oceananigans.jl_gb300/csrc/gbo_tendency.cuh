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
    GBO_D FT rVc(int k) const { return FT(1) / (Az() * dzc(k)); }
    GBO_D FT rVf(int k) const { return FT(1) / (Az() * dzf(k)); }
};

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
    GBO_D FT Uu(int i, int j, int k) const {
        FT Ax = M.Ax(k);
        FT ut = cen4<FT>(Ax * F.u(i - 1, j, k), Ax * F.u(i, j, k), Ax * F.u(i + 1, j, k), Ax * F.u(i + 2, j, k));
        FT S[6];
#pragma unroll
        for (int o = 0; o < 6; ++o) S[o] = F.u(i - 2 + o, j, k);
        return ut * weno5<FT>(S, bias_left(ut));
    }
    // Vu at (f,f,c)
    GBO_D FT Vu(int i, int j, int k) const {
        FT Ay = M.Ay(k);
        FT vt = cen4<FT>(Ay * F.v(i - 2, j, k), Ay * F.v(i - 1, j, k), Ay * F.v(i, j, k), Ay * F.v(i + 1, j, k));
        FT S[6];
#pragma unroll
        for (int o = 0; o < 6; ++o) S[o] = F.u(i, j - 3 + o, k);
        return vt * weno5<FT>(S, bias_left(vt));
    }
    // Wu at (f,c,f)
    GBO_D FT Wu(int i, int j, int k) const {
        FT Az = M.Az();
        FT wt = cen4<FT>(Az * F.w(i - 2, j, k), Az * F.w(i - 1, j, k), Az * F.w(i, j, k), Az * F.w(i + 1, j, k));
        auto q = [&](int o) { return F.u(i, j, k + o); };
        return wt * biased<FT>(q, bias_left(wt), zlev_biased_face(k + 1, g.Nz));
    }
    // Uv at (f,f,c)
    GBO_D FT Uv(int i, int j, int k) const {
        FT Ax = M.Ax(k);
        FT ut = cen4<FT>(Ax * F.u(i, j - 2, k), Ax * F.u(i, j - 1, k), Ax * F.u(i, j, k), Ax * F.u(i, j + 1, k));
        FT S[6];
#pragma unroll
        for (int o = 0; o < 6; ++o) S[o] = F.v(i - 3 + o, j, k);
        return ut * weno5<FT>(S, bias_left(ut));
    }
    // Vv at (c,c,c)
    GBO_D FT Vv(int i, int j, int k) const {
        FT Ay = M.Ay(k);
        FT vt = cen4<FT>(Ay * F.v(i, j - 1, k), Ay * F.v(i, j, k), Ay * F.v(i, j + 1, k), Ay * F.v(i, j + 2, k));
        FT S[6];
#pragma unroll
        for (int o = 0; o < 6; ++o) S[o] = F.v(i, j - 2 + o, k);
        return vt * weno5<FT>(S, bias_left(vt));
    }
    // Wv at (c,f,f)
    GBO_D FT Wv(int i, int j, int k) const {
        FT Az = M.Az();
        FT wt = cen4<FT>(Az * F.w(i, j - 2, k), Az * F.w(i, j - 1, k), Az * F.w(i, j, k), Az * F.w(i, j + 1, k));
        auto q = [&](int o) { return F.v(i, j, k + o); };
        return wt * biased<FT>(q, bias_left(wt), zlev_biased_face(k + 1, g.Nz));
    }
    // Uw at (f,c,f)
    GBO_D FT Uw(int i, int j, int k) const {
        auto qs = [&](int o) { return M.Ax(k + o) * F.u(i, j, k + o); };
        FT ut = symm<FT>(qs, zlev_symm_face(k + 1, g.Nz));
        FT S[6];
#pragma unroll
        for (int o = 0; o < 6; ++o) S[o] = F.w(i - 3 + o, j, k);
        return ut * weno5<FT>(S, bias_left(ut));
    }
    // Vw at (c,f,f)
    GBO_D FT Vw(int i, int j, int k) const {
        auto qs = [&](int o) { return M.Ay(k + o) * F.v(i, j, k + o); };
        FT vt = symm<FT>(qs, zlev_symm_face(k + 1, g.Nz));
        FT S[6];
#pragma unroll
        for (int o = 0; o < 6; ++o) S[o] = F.w(i, j - 3 + o, k);
        return vt * weno5<FT>(S, bias_left(vt));
    }
    // Ww at (c,c,c) level k: reconstructions at face k+1 with centre conditions
    GBO_D FT Ww(int i, int j, int k) const {
        FT Az = M.Az();
        auto qs = [&](int o) { return Az * F.w(i, j, k + 1 + o); };
        FT wt = symm<FT>(qs, zlev_symm_center(k + 1, g.Nz));
        auto qb = [&](int o) { return F.w(i, j, k + 1 + o); };
        return wt * biased<FT>(qb, bias_left(wt), zlev_biased_center(k + 1, g.Nz));
    }
};

// ---------------------------------------------------------------------------
// Closure: strain components and eddy-viscosity interpolations
// (velocity_tracer_gradients.jl:1-60; abstract_scalar_diffusivity_closure.jl:330-366)
// ---------------------------------------------------------------------------
template <typename FT>
struct Strain {
    const GridP<FT>& g;
    const Fields<FT>& F;
    Met<FT> M;
    GBO_D Strain(const GridP<FT>& gg, const Fields<FT>& ff) : g(gg), F(ff), M(gg) {}
    GBO_D FT S11(int i, int j, int k) const { return (F.u(i + 1, j, k) - F.u(i, j, k)) * g.rdx; }
    GBO_D FT S22(int i, int j, int k) const { return (F.v(i, j + 1, k) - F.v(i, j, k)) * g.rdy; }
    GBO_D FT S33(int i, int j, int k) const { return g.flatz ? FT(0) : (F.w(i, j, k + 1) - F.w(i, j, k)) * M.rdzc(k); }
    GBO_D FT dyu(int i, int j, int k) const { return (F.u(i, j, k) - F.u(i, j - 1, k)) * g.rdy; }
    GBO_D FT dxv(int i, int j, int k) const { return (F.v(i, j, k) - F.v(i - 1, j, k)) * g.rdx; }
    GBO_D FT dzu(int i, int j, int k) const { return g.flatz ? FT(0) : (F.u(i, j, k) - F.u(i, j, k - 1)) * M.rdzf(k); }
    GBO_D FT dxw(int i, int j, int k) const { return g.flatz ? FT(0) : (F.w(i, j, k) - F.w(i - 1, j, k)) * g.rdx; }
    GBO_D FT dzv(int i, int j, int k) const { return g.flatz ? FT(0) : (F.v(i, j, k) - F.v(i, j, k - 1)) * M.rdzf(k); }
    GBO_D FT dyw(int i, int j, int k) const { return g.flatz ? FT(0) : (F.w(i, j, k) - F.w(i, j - 1, k)) * g.rdy; }
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
    GBO_D FT tau_ux(int i, int j, int k) const { return FT(-2) * (F.nu(i, j, k) * S11(i, j, k)); }
    GBO_D FT tau_uy(int i, int j, int k) const { return FT(-2) * (nu_ffc(i, j, k) * S12(i, j, k)); }
    GBO_D FT tau_uz(int i, int j, int k) const { return FT(-2) * (nu_fcf(i, j, k) * S13(i, j, k)); }
    GBO_D FT tau_vy(int i, int j, int k) const { return FT(-2) * (F.nu(i, j, k) * S22(i, j, k)); }
    GBO_D FT tau_vz(int i, int j, int k) const { return FT(-2) * (nu_cff(i, j, k) * S23(i, j, k)); }
    GBO_D FT tau_wz(int i, int j, int k) const { return FT(-2) * (F.nu(i, j, k) * S33(i, j, k)); }
};
