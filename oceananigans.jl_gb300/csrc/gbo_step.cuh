// gbo_step.cuh -- fused "tendency + RK3 predictor" kernels.
//
// In the reference a stage is update_state! (halo fills, closure, pHY′,
// compute_tendencies!) followed by the next stage's rk3_substep!
// (compute_flux_bc_tendencies!, _rk3_substep_field!) -- roughly ten launches
// per field.  Here one kernel computes Gⁿ at a point from the corrected state
// (halos synthesised in the loads), adds the flux boundary condition
// (compute_flux_bcs.jl:113-162), stores Gⁿ (it is G⁻ of the next stage) and
// writes the predictor U* = U + Δt(γ Gⁿ + ζ G⁻) (runge_kutta_3.jl:196-204).
#pragma once
#include "gbo_kernels.cuh"

// Δt of this stage: read from device memory when the step graph is Δt-independent
template <typename FT>
GBO_D FT stage_dt(const StepP<FT>& P) {
    return P.dtf ? __ldg(P.dtf + DTF_DT) : P.dt;
}

template <typename FT>
GBO_D FT rk3_update(FT U, FT G, FT Gm, const StepP<FT>& P, FT dt) {
    if (P.first) return U + (dt * P.gamma) * G;
    return U + dt * (P.gamma * G + P.zeta * Gm);
}

// Momentum: Gu, Gv, Gw at one (i, j, k) with the predictor update.
template <typename FT>
__global__ void __launch_bounds__(256) k_momentum(StepP<FT> P) {
    const GridP<FT>& g = P.g;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y * blockDim.y + threadIdx.y;
    int k = blockIdx.z;
    if (i >= g.Nx || j >= g.Ny) return;
    Fields<FT> F{cfld(P.u, g), cfld(P.v, g), cfld(P.nu, g), cfld(P.phy, g), wfld(P.w, g)};
    MomentumFluxes<FT> MF(g, F);
    Strain<FT> S(g, F);
    Met<FT> M(g);
    const size_t idx = i + (size_t)g.Nx * (j + (size_t)g.Ny * k);
    const bool closure = P.closure != CL_NONE;

    // ---------------- u ----------------
    {
        FT dx_ = MF.Uu(i, j, k) - MF.Uu(i - 1, j, k);
        FT dy_ = MF.Vu(i, j + 1, k) - MF.Vu(i, j, k);
        FT dz_ = g.flatz ? FT(0) : (MF.Wu(i, j, k + 1) - MF.Wu(i, j, k));
        FT G = -(M.rVc(k) * (dx_ + dy_ + dz_));
        if (P.has_cor) {
            FT Ay = M.Ay(k);
            // masked_Ay_qᶜᶠᶜ: zero on the immersed periphery (coriolis_schemes.jl:55-58)
            auto AyV = [&](int ii, int jj) { return imm_periph(g, ii, jj, k, false, true, false) ? FT(0) : Ay * F.v(ii, jj, k); };
            FT ixy = FT(0.5) * (FT(0.5) * (AyV(i - 1, j) + AyV(i, j)) + FT(0.5) * (AyV(i - 1, j + 1) + AyV(i, j + 1)));
            FT xfu = -P.f * ixy * (FT(1) / Ay);
            G = G - xfu;
        }
        if (P.has_phy) G = G - (cond_zero(g, i - 1, j, k, i, j, k) ? FT(0) : (F.phy(i, j, k) - F.phy(i - 1, j, k))) * g.rdx;
        if (closure) {
            FT Ax = M.Ax(k), Ay = M.Ay(k), Az = M.Az();
            FT cdx = Ax * S.tau_ux(i, j, k) - Ax * S.tau_ux(i - 1, j, k);
            FT cdy = Ay * S.tau_uy(i, j + 1, k) - Ay * S.tau_uy(i, j, k);
            FT cdz = g.flatz ? FT(0) : (Az * S.tau_uz(i, j, k + 1) - Az * S.tau_uz(i, j, k));
            G = G - M.rVc(k) * (cdx + cdy + cdz);
        }
        FT Gm = P.first ? FT(0) : P.Gu[idx];
        P.Gu[idx] = G;
        P.uo[idx] = rk3_update(P.u[idx], G, Gm, P, stage_dt(P));
    }
    // ---------------- v ----------------
    {
        FT dx_ = MF.Uv(i + 1, j, k) - MF.Uv(i, j, k);
        FT dy_ = MF.Vv(i, j, k) - MF.Vv(i, j - 1, k);
        FT dz_ = g.flatz ? FT(0) : (MF.Wv(i, j, k + 1) - MF.Wv(i, j, k));
        FT G = -(M.rVc(k) * (dx_ + dy_ + dz_));
        if (P.has_cor) {
            FT Ax = M.Ax(k);
            auto AxU = [&](int ii, int jj) { return imm_periph(g, ii, jj, k, true, false, false) ? FT(0) : Ax * F.u(ii, jj, k); };
            FT ixy = FT(0.5) * (FT(0.5) * (AxU(i, j - 1) + AxU(i + 1, j - 1)) + FT(0.5) * (AxU(i, j) + AxU(i + 1, j)));
            FT yfu = P.f * ixy * (FT(1) / Ax);
            G = G - yfu;
        }
        if (P.has_phy) G = G - (cond_zero(g, i, j - 1, k, i, j, k) ? FT(0) : (F.phy(i, j, k) - F.phy(i, j - 1, k))) * g.rdy;
        if (closure) {
            FT Ax = M.Ax(k), Ay = M.Ay(k), Az = M.Az();
            FT cdx = Ax * S.tau_vx(i + 1, j, k) - Ax * S.tau_vx(i, j, k);
            FT cdy = Ay * S.tau_vy(i, j, k) - Ay * S.tau_vy(i, j - 1, k);
            FT cdz = g.flatz ? FT(0) : (Az * S.tau_vz(i, j, k + 1) - Az * S.tau_vz(i, j, k));
            G = G - M.rVc(k) * (cdx + cdy + cdz);
        }
        FT Gm = P.first ? FT(0) : P.Gv[idx];
        P.Gv[idx] = G;
        P.vo[idx] = rk3_update(P.v[idx], G, Gm, P, stage_dt(P));
    }
    // ---------------- w (interior faces only; k = 0 is the wall) ----------------
    if (!g.flatz) {
        if (k == 0) {
            P.wo[idx] = FT(0);
            return;
        }
        FT dx_ = MF.Uw(i + 1, j, k) - MF.Uw(i, j, k);
        FT dy_ = MF.Vw(i, j + 1, k) - MF.Vw(i, j, k);
        FT dz_ = MF.Ww(i, j, k) - MF.Ww(i, j, k - 1);
        FT G = -(M.rVf(k) * (dx_ + dy_ + dz_));
        if (closure) {
            FT Axf = M.Axf(k), Ayf = M.Ayf(k), Az = M.Az();
            FT cdx = Axf * S.tau_wx(i + 1, j, k) - Axf * S.tau_wx(i, j, k);
            FT cdy = Ayf * S.tau_wy(i, j + 1, k) - Ayf * S.tau_wy(i, j, k);
            FT cdz = Az * S.tau_wz(i, j, k) - Az * S.tau_wz(i, j, k - 1);
            G = G - M.rVf(k) * (cdx + cdy + cdz);
        }
        FT Gm = P.first ? FT(0) : P.Gw[idx];
        P.Gw[idx] = G;
        P.wo[idx] = rk3_update(P.w[idx], G, Gm, P, stage_dt(P));
    }
}

// One tracer: advection, diffusion (ν/Pr for Smagorinsky, κₑ for AMD), flux BCs.
template <typename FT>
__global__ void __launch_bounds__(256) k_tracer(StepP<FT> P) {
    const GridP<FT>& g = P.g;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y * blockDim.y + threadIdx.y;
    int k = blockIdx.z;
    if (i >= g.Nx || j >= g.Ny) return;
    CFld<FT> u = cfld(P.u, g), v = cfld(P.v, g), c = cfld(P.c, g, P.cref);
    WFld<FT> w = wfld(P.w, g);
    Met<FT> M(g);
    const size_t idx = i + (size_t)g.Nx * (j + (size_t)g.Ny * k);

    // reconstruction levels: WENO5 away from immersed nodes (and the Bounded-z buffers)
    auto lev = [&](int d, int ii, int jj, int kk) {
        if (g.kbot) return ibg_level(g, d, ii, jj, kk, true);
        return d == 2 ? zlev_biased_face(kk + 1, g.Nz) : 3;
    };
    auto Fx = [&](int ii) {
        FT ut = u(ii, j, k);
        auto q = [&](int o) { return c(ii + o, j, k); };
        return M.Ax(k) * ut * biased<FT>(q, bias_left(ut), lev(0, ii, j, k));
    };
    auto Fy = [&](int jj) {
        FT vt = v(i, jj, k);
        auto q = [&](int o) { return c(i, jj + o, k); };
        return M.Ay(k) * vt * biased<FT>(q, bias_left(vt), lev(1, i, jj, k));
    };
    auto Fz = [&](int kk) {
        FT wt = w(i, j, kk);
        auto q = [&](int o) { return c(i, j, kk + o); };
        return M.Az() * wt * biased<FT>(q, bias_left(wt), lev(2, i, j, kk));
    };
    FT dx_ = Fx(i + 1) - Fx(i);
    FT dy_ = Fy(j + 1) - Fy(j);
    FT dz_ = g.flatz ? FT(0) : (Fz(k + 1) - Fz(k));
    FT G = -(M.rVc(k) * (dx_ + dy_ + dz_));
    if (P.closure != CL_NONE) {
        CFld<FT> K = cfld(P.closure == CL_AMD ? P.kap : P.nu, g);
        const FT rPr = P.closure == CL_AMD ? FT(1) : P.Pr;
        auto kx = [&](int ii) { return P.closure == CL_AMD ? FT(0.5) * (K(ii - 1, j, k) + K(ii, j, k)) : FT(0.5) * (K(ii - 1, j, k) + K(ii, j, k)) / rPr; };
        auto ky = [&](int jj) { return P.closure == CL_AMD ? FT(0.5) * (K(i, jj - 1, k) + K(i, jj, k)) : FT(0.5) * (K(i, jj - 1, k) + K(i, jj, k)) / rPr; };
        auto kz = [&](int kk) { return P.closure == CL_AMD ? FT(0.5) * (K(i, j, kk - 1) + K(i, j, kk)) : FT(0.5) * (K(i, j, kk - 1) + K(i, j, kk)) / rPr; };
        // on an immersed grid: conditional ∂ (conditional_differences.jl:15-43) and zero flux
        // on the immersed periphery of the flux location (immersed_diffusive_fluxes.jl:42-44)
        auto dc = [&](int i0, int j0, int k0, int i1, int j1, int k1, FT d) { return cond_zero(g, i0, j0, k0, i1, j1, k1) ? FT(0) : d; };
        auto zq = [&](int ii, int jj, int kk, bool fx, bool fy, bool fz) { return g.kbot && imm_periph(g, ii, jj, kk, fx, fy, fz); };
        auto qx = [&](int ii) {
            return zq(ii, j, k, true, false, false) ? FT(0) : -kx(ii) * dc(ii - 1, j, k, ii, j, k, (c(ii, j, k) - c(ii - 1, j, k)) * g.rdx);
        };
        auto qy = [&](int jj) {
            return zq(i, jj, k, false, true, false) ? FT(0) : -ky(jj) * dc(i, jj - 1, k, i, jj, k, (c(i, jj, k) - c(i, jj - 1, k)) * g.rdy);
        };
        auto qz = [&](int kk) {
            return zq(i, j, kk, false, false, true) ? FT(0) : -kz(kk) * dc(i, j, kk - 1, i, j, kk, (c(i, j, kk) - c(i, j, kk - 1)) * M.rdzf(kk));
        };
        FT Ax = M.Ax(k), Ay = M.Ay(k), Az = M.Az();
        FT cdx = Ax * qx(i + 1) - Ax * qx(i);
        FT cdy = Ay * qy(j + 1) - Ay * qy(j);
        FT cdz = g.flatz ? FT(0) : (Az * qz(k + 1) - Az * qz(k));
        G = G - M.rVc(k) * (cdx + cdy + cdz);
    }
    if (!g.flatz) {
        if (k == g.Nz - 1 && P.flux_top != FT(0)) G -= P.flux_top * M.Az() / (M.Az() * M.dzc(k));
        if (k == 0 && P.flux_bot != FT(0)) G += P.flux_bot * M.Az() / (M.Az() * M.dzc(k));
    }
    FT Gm = P.first ? FT(0) : P.Gc[idx];
    P.Gc[idx] = G;
    // the update of a departure field acts on the stored departure (the profile is fixed)
    P.co[idx] = rk3_update(P.c[idx], G, Gm, P, stage_dt(P));
}
