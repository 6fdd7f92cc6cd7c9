// gbo_kernels.cuh -- closure, hydrostatic-pressure and fused tendency + RK3 kernels.
#pragma once
#include "gbo_tendency.cuh"

enum { CL_NONE = 0, CL_SMAG = 1, CL_AMD = 2 };

template <typename FT>
struct StepP {
    GridP<FT> g;
    const FT* u; const FT* v; const FT* w;  // corrected state (input)
    const FT* c;                            // tracer (tracer kernel)
    const FT* nu; const FT* kap; const FT* phy;
    const FT* b;                            // buoyancy tracer (closures)
    const FT* cref;                         // reference profile of c (departure storage), or null
    const FT* bref;                         // reference profile of b, or null
    FT* uo; FT* vo; FT* wo; FT* co;         // predictor outputs U*
    FT* Gu; FT* Gv; FT* Gw; FT* Gc;         // tendency buffers (G⁻ in, Gⁿ out)
    FT f;
    int has_cor, has_phy, closure, buoyancy;
    FT Pr;
    FT flux_top, flux_bot;
    FT C, Cb;
    FT dt, gamma, zeta;
    const FT* dtf;                          // stage factors in device memory (Δt overrides dt)
    int first;
    const FT* cs2;                          // DynamicSmagorinsky: c² per level (else null)
    const FT* jlm; const FT* jmm;           // Lagrangian-averaged DynamicSmagorinsky: 𝒥ᴸᴹ, 𝒥ᴹᴹ per cell (else null)
    FT lm_min;                              // its minimum_numerator
};

// ---------------------------------------------------------------------------
// Smagorinsky-Lilly eddy viscosity (Smagorinskys/smagorinsky.jl:90-104,
// lilly_coefficient.jl:122-142, scale_invariant_operators.jl:10-13)
// ---------------------------------------------------------------------------
template <typename FT>
__global__ void k_smagorinsky(StepP<FT> P, FT* __restrict__ nu_out) {
    const GridP<FT>& g = P.g;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y * blockDim.y + threadIdx.y;
    int k = blockIdx.z;
    if (i >= g.Nx || j >= g.Ny) return;
    Fields<FT> F{cfld(P.u, g), cfld(P.v, g), cfld(P.nu, g), cfld(P.phy, g), wfld(P.w, g)};
    Strain<FT> S(g, F);
    Met<FT> M(g);
    auto sq = [](FT x) { return x * x; };
    FT s11 = S.S11(i, j, k), s22 = S.S22(i, j, k), s33 = S.S33(i, j, k);
    FT tr = s11 * s11 + s22 * s22 + s33 * s33;
    FT ixy = FT(0.5) * (FT(0.5) * (sq(S.S12(i, j, k)) + sq(S.S12(i + 1, j, k))) +
                        FT(0.5) * (sq(S.S12(i, j + 1, k)) + sq(S.S12(i + 1, j + 1, k))));
    FT ixz, iyz;
    if (g.flatz) {
        ixz = FT(0.5) * (sq(S.S13(i, j, k)) + sq(S.S13(i + 1, j, k)));
        iyz = FT(0.5) * (sq(S.S23(i, j, k)) + sq(S.S23(i, j + 1, k)));
    } else {
        ixz = FT(0.5) * (FT(0.5) * (sq(S.S13(i, j, k)) + sq(S.S13(i + 1, j, k))) +
                         FT(0.5) * (sq(S.S13(i, j, k + 1)) + sq(S.S13(i + 1, j, k + 1))));
        iyz = FT(0.5) * (FT(0.5) * (sq(S.S23(i, j, k)) + sq(S.S23(i, j + 1, k))) +
                         FT(0.5) * (sq(S.S23(i, j, k + 1)) + sq(S.S23(i, j + 1, k + 1))));
    }
    FT Sig2 = tr + FT(2) * ixy + FT(2) * ixz + FT(2) * iyz;
    FT D3 = g.dx * g.dy * M.dzc(k);
    FT Df = cbrt(D3);
    FT cs2;
    if (P.jlm) {
        // Lagrangian-averaged DynamicSmagorinsky: the cell's coefficient
        // max(𝒥ᴸᴹ, minimum_numerator) / 𝒥ᴹᴹ, a strong zero where 𝒥ᴹᴹ ≤ 0 (dynamic_coefficient.jl:236-248)
        const size_t q = i + (size_t)g.Nx * (j + (size_t)g.Ny * k);
        FT lm = P.jlm[q];
        lm = isnan(lm) ? lm : (lm > P.lm_min ? lm : P.lm_min);
        const FT mm = P.jmm[q];
        cs2 = mm > FT(0) ? lm / mm : FT(0);
    } else if (P.cs2) {
        // DynamicSmagorinsky: the level's averaged coefficient (k_dyn_coef)
        cs2 = P.cs2[k];
    } else {
        FT N2 = FT(0);
        if (P.buoyancy && !g.flatz) {
            CFld<FT> b = cfld(P.b, g, P.bref);
            // N² = ℑz(∂z b), conditional ∂ on an immersed grid
            FT b1 = cond_zero(g, i, j, k - 1, i, j, k) ? FT(0) : (b(i, j, k) - b(i, j, k - 1)) * M.rdzf(k);
            FT b2 = cond_zero(g, i, j, k, i, j, k + 1) ? FT(0) : (b(i, j, k + 1) - b(i, j, k)) * M.rdzf(k + 1);
            N2 = FT(0.5) * (b1 + b2);
        }
        FT N2p = fmax(FT(0), N2);
        FT r = P.Cb * N2p / Sig2;
        FT mn = isnan(r) ? r : fmin(FT(1), r);
        FT vs2 = FT(1) - mn;
        FT vs = (Sig2 == FT(0)) ? FT(0) : sqrt(vs2);
        cs2 = vs * (P.C * P.C);
    }
    nu_out[i + (size_t)g.Nx * (j + (size_t)g.Ny * k)] = cs2 * (Df * Df) * sqrt(FT(2) * Sig2);
}

// ---------------------------------------------------------------------------
// Anisotropic minimum dissipation (anisotropic_minimum_dissipation.jl:161-204,243-358;
// normalised gradients velocity_tracer_gradients.jl:120-250).  Filter widths are
// twice the cell-centre spacings at the evaluation index, as the reference uses.
// ---------------------------------------------------------------------------
template <typename FT, class ST = Strain<FT>>
struct AMD {
    const GridP<FT>& g;
    const ST& S;
    Met<FT> M;
    GBO_D AMD(const GridP<FT>& gg, const ST& s) : g(gg), S(s), M(gg) {}
    GBO_D FT Dfx() const { return FT(2) * g.dx; }
    GBO_D FT Dfy() const { return FT(2) * g.dy; }
    GBO_D FT Dfz(int k) const { return FT(2) * M.dzc(k); }
    GBO_D FT n_dxv(int i, int j, int k) const { return Dfx() / Dfy() * S.dxv(i, j, k); }
    GBO_D FT n_dyu(int i, int j, int k) const { return Dfy() / Dfx() * S.dyu(i, j, k); }
    GBO_D FT n_dxw(int i, int j, int k) const { return Dfx() / Dfz(k) * S.dxw(i, j, k); }
    GBO_D FT n_dzu(int i, int j, int k) const { return Dfz(k) / Dfx() * S.dzu(i, j, k); }
    GBO_D FT n_dyw(int i, int j, int k) const { return Dfy() / Dfz(k) * S.dyw(i, j, k); }
    GBO_D FT n_dzv(int i, int j, int k) const { return Dfz(k) / Dfy() * S.dzv(i, j, k); }
    GBO_D FT n_S12(int i, int j, int k) const { return FT(0.5) * (n_dyu(i, j, k) + n_dxv(i, j, k)); }
    GBO_D FT n_S13(int i, int j, int k) const { return FT(0.5) * (n_dzu(i, j, k) + n_dxw(i, j, k)); }
    GBO_D FT n_S23(int i, int j, int k) const { return FT(0.5) * (n_dzv(i, j, k) + n_dyw(i, j, k)); }
};

#define GBO_IXY(f) (FT(0.5) * (FT(0.5) * ((f)(i, j, k) + (f)(i + 1, j, k)) + FT(0.5) * ((f)(i, j + 1, k) + (f)(i + 1, j + 1, k))))
#define GBO_IXZ(f) (FT(0.5) * (FT(0.5) * ((f)(i, j, k) + (f)(i + 1, j, k)) + FT(0.5) * ((f)(i, j, k + 1) + (f)(i + 1, j, k + 1))))
#define GBO_IYZ(f) (FT(0.5) * (FT(0.5) * ((f)(i, j, k) + (f)(i, j + 1, k)) + FT(0.5) * ((f)(i, j, k + 1) + (f)(i, j + 1, k + 1))))
#define GBO_IX(f) (FT(0.5) * ((f)(i, j, k) + (f)(i + 1, j, k)))
#define GBO_IY(f) (FT(0.5) * ((f)(i, j, k) + (f)(i, j + 1, k)))
#define GBO_IZ(f) (FT(0.5) * ((f)(i, j, k) + (f)(i, j, k + 1)))

// νₑ and (with a tracer accessor c) κₑ at one cell from strain S and tracer c.
template <typename FT, class ST, class CF>
GBO_D void amd_point(const StepP<FT>& P, const GridP<FT>& g, const ST& S, const CF& c, bool has_c, int i, int j, int k,
                     size_t idx, FT* __restrict__ nu_out, FT* __restrict__ kap_out) {
    AMD<FT, ST> A(g, S);
    Met<FT> M(g);
    auto sq = [](FT x) { return x * x; };
    auto dxv2 = [&](int a, int b, int c) { return sq(A.n_dxv(a, b, c)); };
    auto dyu2 = [&](int a, int b, int c) { return sq(A.n_dyu(a, b, c)); };
    auto dxw2 = [&](int a, int b, int c) { return sq(A.n_dxw(a, b, c)); };
    auto dzu2 = [&](int a, int b, int c) { return sq(A.n_dzu(a, b, c)); };
    auto dyw2 = [&](int a, int b, int c) { return sq(A.n_dyw(a, b, c)); };
    auto dzv2 = [&](int a, int b, int c) { return sq(A.n_dzv(a, b, c)); };
    FT S11 = S.S11(i, j, k), S22 = S.S22(i, j, k), S33 = S.S33(i, j, k);
    FT q = sq(S11) + sq(S22) + sq(S33) + GBO_IXY(dxv2) + GBO_IXY(dyu2) + GBO_IXZ(dxw2) + GBO_IXZ(dzu2) +
           GBO_IYZ(dyw2) + GBO_IYZ(dzv2);
    FT d2 = FT(3) / (FT(1) / sq(A.Dfx()) + FT(1) / sq(A.Dfy()) + FT(1) / sq(A.Dfz(k)));
    FT nsgs = FT(0);
    if (q != FT(0)) {
        auto f_dxvS12 = [&](int a, int b, int c) { return A.n_dxv(a, b, c) * A.n_S12(a, b, c); };
        auto f_dxwS13 = [&](int a, int b, int c) { return A.n_dxw(a, b, c) * A.n_S13(a, b, c); };
        auto f_dxv = [&](int a, int b, int c) { return A.n_dxv(a, b, c); };
        auto f_dxw = [&](int a, int b, int c) { return A.n_dxw(a, b, c); };
        auto f_S23 = [&](int a, int b, int c) { return A.n_S23(a, b, c); };
        auto f_dyuS12 = [&](int a, int b, int c) { return A.n_dyu(a, b, c) * A.n_S12(a, b, c); };
        auto f_dyu = [&](int a, int b, int c) { return A.n_dyu(a, b, c); };
        auto f_dyw = [&](int a, int b, int c) { return A.n_dyw(a, b, c); };
        auto f_S13 = [&](int a, int b, int c) { return A.n_S13(a, b, c); };
        auto f_dywS23 = [&](int a, int b, int c) { return A.n_dyw(a, b, c) * A.n_S23(a, b, c); };
        auto f_dzu = [&](int a, int b, int c) { return A.n_dzu(a, b, c); };
        auto f_dzv = [&](int a, int b, int c) { return A.n_dzv(a, b, c); };
        auto f_S12 = [&](int a, int b, int c) { return A.n_S12(a, b, c); };
        auto f_dzuS13 = [&](int a, int b, int c) { return A.n_dzu(a, b, c) * A.n_S13(a, b, c); };
        auto f_dzvS23 = [&](int a, int b, int c) { return A.n_dzv(a, b, c) * A.n_S23(a, b, c); };
        FT r1 = S11 * sq(S11) + S22 * GBO_IXY(dxv2) + S33 * GBO_IXZ(dxw2) + FT(2) * S11 * GBO_IXY(f_dxvS12) +
                FT(2) * S11 * GBO_IXZ(f_dxwS13) + FT(2) * GBO_IXY(f_dxv) * GBO_IXZ(f_dxw) * GBO_IYZ(f_S23);
        FT r2 = S11 * GBO_IXY(dyu2) + S22 * sq(S22) + S33 * GBO_IYZ(dyw2) + FT(2) * S22 * GBO_IXY(f_dyuS12) +
                FT(2) * GBO_IXY(f_dyu) * GBO_IYZ(f_dyw) * GBO_IXZ(f_S13) + FT(2) * S22 * GBO_IYZ(f_dywS23);
        FT r3 = S11 * GBO_IXZ(dzu2) + S22 * GBO_IYZ(dzv2) + S33 * sq(S33) + FT(2) * GBO_IXZ(f_dzu) * GBO_IYZ(f_dzv) * GBO_IXY(f_S12) +
                FT(2) * S33 * GBO_IXZ(f_dzuS13) + FT(2) * S33 * GBO_IYZ(f_dzvS23);
        FT r = r1 + r2 + r3;
        nsgs = -P.C * d2 * (r - FT(0)) / q;
    }
    nu_out[idx] = fmax(FT(0), nsgs);
    if (kap_out && has_c) {
        // tracer gradients at faces, conditional ∂ on an immersed grid
        auto n_dxc = [&](int a, int b, int cc) {
            return A.Dfx() * (cond_zero(g, a - 1, b, cc, a, b, cc) ? FT(0) : (c(a, b, cc) - c(a - 1, b, cc)) * g.rdx);
        };
        auto n_dyc = [&](int a, int b, int cc) {
            return A.Dfy() * (cond_zero(g, a, b - 1, cc, a, b, cc) ? FT(0) : (c(a, b, cc) - c(a, b - 1, cc)) * g.rdy);
        };
        auto n_dzc = [&](int a, int b, int cc) {
            return A.Dfz(cc) * (cond_zero(g, a, b, cc - 1, a, b, cc) ? FT(0) : (c(a, b, cc) - c(a, b, cc - 1)) * M.rdzf(cc));
        };
        auto dxc2 = [&](int a, int b, int cc) { return sq(n_dxc(a, b, cc)); };
        auto dyc2 = [&](int a, int b, int cc) { return sq(n_dyc(a, b, cc)); };
        auto dzc2 = [&](int a, int b, int cc) { return sq(n_dzc(a, b, cc)); };
        FT sigma = GBO_IX(dxc2) + GBO_IY(dyc2) + GBO_IZ(dzc2);
        FT ksgs = FT(0);
        if (sigma != FT(0)) {
            auto f_dxv = [&](int a, int b, int cc) { return A.n_dxv(a, b, cc); };
            auto f_dxw = [&](int a, int b, int cc) { return A.n_dxw(a, b, cc); };
            auto f_dyu = [&](int a, int b, int cc) { return A.n_dyu(a, b, cc); };
            auto f_dyw = [&](int a, int b, int cc) { return A.n_dyw(a, b, cc); };
            auto f_dzu = [&](int a, int b, int cc) { return A.n_dzu(a, b, cc); };
            auto f_dzv = [&](int a, int b, int cc) { return A.n_dzv(a, b, cc); };
            FT cx_ux = S11 * GBO_IX(dxc2) + GBO_IXY(f_dxv) * GBO_IX(n_dxc) * GBO_IY(n_dyc) +
                       GBO_IXZ(f_dxw) * GBO_IX(n_dxc) * GBO_IZ(n_dzc);
            FT cy_uy = GBO_IXY(f_dyu) * GBO_IY(n_dyc) * GBO_IX(n_dxc) + S22 * GBO_IY(dyc2) +
                       GBO_IXZ(f_dyw) * GBO_IY(n_dyc) * GBO_IZ(n_dzc);
            FT cz_uz = GBO_IXZ(f_dzu) * GBO_IZ(n_dzc) * GBO_IX(n_dxc) + GBO_IYZ(f_dzv) * GBO_IZ(n_dzc) * GBO_IY(n_dyc) +
                       S33 * GBO_IZ(dzc2);
            FT theta = cx_ux + cy_uy + cz_uz;
            ksgs = -P.C * d2 * theta / sigma;
        }
        kap_out[idx] = fmax(FT(0), ksgs);
    }
}

template <typename FT>
__global__ void k_amd(StepP<FT> P, FT* __restrict__ nu_out, FT* __restrict__ kap_out) {
    const GridP<FT>& g = P.g;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y * blockDim.y + threadIdx.y;
    int k = blockIdx.z;
    if (i >= g.Nx || j >= g.Ny) return;
    Fields<FT> F{cfld(P.u, g), cfld(P.v, g), cfld(P.nu, g), cfld(P.phy, g), wfld(P.w, g)};
    Strain<FT> S(g, F);
    CFld<FT> c = cfld(P.c, g, P.cref);
    amd_point<FT>(P, g, S, c, P.c != nullptr, i, j, k, i + (size_t)g.Nx * (j + (size_t)g.Ny * k), nu_out, kap_out);
}

// ---------------------------------------------------------------------------
// Hydrostatic pressure anomaly: downward integral of ℑz(b)·Δzᶠ
// (update_hydrostatic_pressure.jl:11-21).  One thread per (i, j) column.
// When b is stored as departures from a reference profile, the integral runs over
// the departures only: the profile's part is the same in every column, and pHY′
// enters the momentum equations only through its horizontal differences
// (∂x pHY′, ∂y pHY′; w has no buoyancy term when pHY′ is present), so dropping it
// changes no tendency and keeps those differences free of the cancellation of two
// O(N² H²) column integrals.  Reading the field back adds the profile's part.
// ---------------------------------------------------------------------------
// With src (a stage's buoyancy predictor b*), the column is read from src and also stored
// into dst (the buoyancy state), which is then the stage's copy of b* into b: one pass
// instead of a copy kernel and this scan.
template <typename FT>
__global__ void k_hydrostatic(StepP<FT> P, FT* __restrict__ phy, const FT* __restrict__ src = nullptr,
                              FT* __restrict__ dst = nullptr) {
    const GridP<FT>& g = P.g;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    Met<FT> M(g);
    const FT* b = src ? src : P.b;
    const size_t col = i + (size_t)g.Nx * j, plane = (size_t)g.Nx * g.Ny;
    const int Nz = g.Nz;
    FT bk = b[col + plane * (Nz - 1)];
    if (dst) dst[col + plane * (Nz - 1)] = bk;
    // ℑz(b) at the top face uses the mirrored halo b[Nz+1] = b[Nz]
    FT pk = -(FT(0.5) * (bk + bk)) * M.dzf(Nz);
    phy[col + plane * (Nz - 1)] = pk;
    // one thread per column (few warps per SM): the levels are loaded eight at a time
    // ahead of the scan so that the loads overlap
    constexpr int U = 8;
    for (int ka = Nz - 2; ka >= 0; ka -= U) {
        FT bs[U];
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (ka - u >= 0) bs[u] = b[col + plane * (ka - u)];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int k = ka - u;
            if (k < 0) break;
            if (dst) dst[col + plane * k] = bs[u];
            pk -= (FT(0.5) * (bs[u] + bk)) * M.dzf(k + 1);
            phy[col + plane * k] = pk;
            bk = bs[u];
        }
    }
}
