// ocean_oracle.cpp -- FP64 CPU oracle for the NonhydrostaticModel RK3 time step.
//
// TEST INFRASTRUCTURE ONLY.  This file restates, in plain C++17 + OpenMP, the
// algorithm of Oceananigans.jl v0.110.19 for
//   time_step!(model::NonhydrostaticModel{<:RungeKutta3TimeStepper}, Δt)
// so that the CUDA library can be checked against it.  It is imported only by
// tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg; the product
// library never links or calls it.
//
// Unlike the CUDA kernels (which synthesise halos inside the stencil loads),
// the oracle stores every field with halo points laid out as the reference's
// OffsetArrays (1-based interior, H halo points per side) and fills halos with
// the reference's fill order: Flux/NormalFlow first, then Periodic
// (src/BoundaryConditions/boundary_condition_ordering.jl:84-104).  Halo points
// that the reference never writes stay zero, as they do there.
//
// Each function cites the reference file:line it follows (paths relative to the
// Oceananigans.jl source tree).  Parity with the reference itself is pinned by
// the golden fixtures and analytic tests under tests/ (the Julia reference
// cannot run in this environment; see the oracle tests' docstrings).
#include <cmath>
#include <cstdlib>
#include <complex>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/gbo.h"

namespace {

using cplx = std::complex<double>;

// ---------------------------------------------------------------------------
// Reconstruction constants (same derivation as gen_coefficients.py; FP64)
// src/Advection/weno_interpolants.jl:71-94,101-110,169-174
// ---------------------------------------------------------------------------
struct Coeffs {
    double p3[3][3], cstar3[3], p2[2][2], cstar2[2], c4[4], c2[2], eps;
    Coeffs() {
        // exact Shu (1998) weights; last = 1 - sum(others) in FP64
        const double e3[3][3] = {{1.0 / 3, 5.0 / 6, 0}, {-1.0 / 6, 5.0 / 6, 0}, {1.0 / 3, -7.0 / 6, 0}};
        for (int s = 0; s < 3; ++s) {
            p3[s][0] = e3[s][0]; p3[s][1] = e3[s][1];
            p3[s][2] = 1.0 - (p3[s][0] + p3[s][1]);
        }
        p2[0][0] = 0.5; p2[0][1] = 1.0 - 0.5;
        p2[1][0] = -0.5; p2[1][1] = 1.0 - (-0.5);
        cstar3[0] = 3.0 / 10; cstar3[1] = 3.0 / 5; cstar3[2] = 1.0 / 10;
        cstar2[0] = 2.0 / 3; cstar2[1] = 1.0 / 3;
        // Centered(order=4): stencil_coefficients(order=4, r=1) = (-1/12, 7/12, 7/12, 1-sum)
        double a = -1.0 / 12, b = 7.0 / 12, c = 7.0 / 12;
        double last = 1.0 - ((a + b) + c);
        // offsets -2,-1,0,+1 take coeff[4],coeff[3],coeff[2],coeff[1]
        c4[0] = last; c4[1] = c; c4[2] = b; c4[3] = a;
        c2[0] = 0.5; c2[1] = 1.0 - 0.5;
        eps = (double)1e-8f;  // Float32 literal promoted (weno_interpolants.jl:71)
    }
};
const Coeffs CF;

const double SM3[3][6] = {{10, -31, 11, 25, -19, 4}, {4, -13, 5, 13, -13, 4}, {4, -19, 11, 25, -31, 10}};

// ---------------------------------------------------------------------------
// Grid (src/Grids/rectilinear_grid.jl:266-305; grid_generation.jl:34-176)
// ---------------------------------------------------------------------------
struct Grid {
    int Nx = 0, Ny = 0, Nz = 0, H = 3, Hz = 3;
    bool flatz = false;
    double Lx = 0, Ly = 0, Lz = 0, dx = 0, dy = 0;
    double x0 = 0, y0 = 0;  // west and south domain edges
    // vertical spacings indexed k in [1-Hz, Nz+Hz+1] (Δzᵃᵃᶜ and Δzᵃᵃᶠ)
    std::vector<double> dzc_, dzf_, zf_, zc_;
    int zoff = 0;  // vector index = k + zoff
    bool immersed = false;
    bool stretched = false;  // z faces given explicitly
    std::vector<double> zb;  // numerical bottom height per (i,j) incl. halos, (Nx+2H)*(Ny+2H)

    double dzC(int k) const { return dzc_[k + zoff]; }
    double dzF(int k) const { return dzf_[k + zoff]; }
    double zC(int k) const { return zc_[k + zoff]; }
    double zF(int k) const { return zf_[k + zoff]; }
};

// generate_coordinate for a stretched Bounded coordinate (grid_generation.jl:34-90)
void build_stretched_z(Grid& g, const double* faces) {
    const int N = g.Nz, H = g.Hz;
    std::vector<double> Fi(faces, faces + N + 1);
    g.Lz = Fi[N] - Fi[0];
    // lower/upper exterior spacings wrap from the opposite end (:16,19)
    std::vector<double> dlow(H), dup(H);
    for (int i = 1; i <= H; ++i) dlow[i - 1] = Fi[N + 1 - H + i - 1] - Fi[N + 1 - H + i - 2];
    for (int i = 1; i <= H; ++i) dup[i - 1] = Fi[i] - Fi[i - 1];
    std::vector<double> dplus(dup.rbegin(), dup.rend());
    std::vector<double> F;
    for (int i = 1; i <= H; ++i) {
        double s = 0;
        for (int q = i; q <= H; ++q) s += dlow[q - 1];
        F.push_back(Fi[0] - s);
    }
    for (double f : Fi) F.push_back(f);
    std::vector<double> Fp;
    for (int i = 1; i <= H; ++i) {
        double s = 0;
        for (int q = i; q <= H; ++q) s += dplus[q - 1];
        Fp.push_back(Fi[N] + s);
    }
    std::reverse(Fp.begin(), Fp.end());
    for (double f : Fp) F.push_back(f);
    // TC = N + 2H centers; TF = N + 1 + 2H faces (Bounded)
    const int TC = N + 2 * H, TF = N + 1 + 2 * H;
    std::vector<double> C(TC);
    for (int i = 0; i < TC; ++i) C[i] = (F[i + 1] + F[i]) / 2;
    std::vector<double> Df(TC - 1);
    for (int i = 1; i < TC; ++i) Df[i - 1] = C[i] - C[i - 1];
    std::vector<double> Dc(TF - 1);
    for (int i = 0; i < TF - 1; ++i) Dc[i] = F[i + 1] - F[i];
    // Δᶠ = [Δᶠ[1], Δᶠ..., Δᶠ[end]] then shifted right by one (:83-86)
    std::vector<double> Dff;
    Dff.push_back(Df.front());
    for (double d : Df) Dff.push_back(d);
    Dff.push_back(Df.back());
    for (int i = (int)Dff.size() - 1; i >= 1; --i) Dff[i] = Dff[i - 1];
    // Offsets: Δᶜ is OffsetArray(-H) -> index k maps to position k+H-1 (1-based -> 0-based)
    //          Δᶠ is OffsetArray(-H-1) -> index k maps to position k+H
    const int kmin = 1 - H, kmax = N + H + 1;
    g.zoff = -kmin;
    const int len = kmax - kmin + 1;
    g.dzc_.assign(len, 0.0); g.dzf_.assign(len, 0.0); g.zf_.assign(len, 0.0); g.zc_.assign(len, 0.0);
    for (int k = kmin; k <= kmax; ++k) {
        int pc = k + H - 1;
        if (pc >= 0 && pc < (int)Dc.size()) g.dzc_[k + g.zoff] = Dc[pc];
        int pf = k + H;
        if (pf >= 0 && pf < (int)Dff.size()) g.dzf_[k + g.zoff] = Dff[pf];
        int pF = k + H - 1;
        if (pF >= 0 && pF < TF) g.zf_[k + g.zoff] = F[pF];
        if (pF >= 0 && pF < TC) g.zc_[k + g.zoff] = C[pF];
    }
}

void build_regular_z(Grid& g, double z0, double z1) {
    const int N = g.Nz, H = g.Hz;
    g.Lz = z1 - z0;
    const double d = g.Lz / N;
    const int kmin = 1 - H, kmax = N + H + 1;
    g.zoff = -kmin;
    const int len = kmax - kmin + 1;
    g.dzc_.assign(len, d); g.dzf_.assign(len, d);
    g.zf_.assign(len, 0.0); g.zc_.assign(len, 0.0);
    for (int k = kmin; k <= kmax; ++k) {
        g.zf_[k + g.zoff] = z0 + (k - 1) * d;
        g.zc_[k + g.zoff] = z0 + (k - 0.5) * d;
    }
}

// ---------------------------------------------------------------------------
// Field storage with halos (OffsetArray-like, 1-based interior)
// ---------------------------------------------------------------------------
struct Field {
    int nx = 0, ny = 0, nz = 0, ox = 0, oy = 0, oz = 0;  // parent sizes and offsets
    std::vector<double> d;
    void init(int Nx, int Ny, int NzLoc, int H, int Hz) {
        nx = Nx + 2 * H; ny = Ny + 2 * H; nz = NzLoc + 2 * Hz;
        ox = H - 1; oy = H - 1; oz = Hz - 1;
        d.assign((size_t)nx * ny * nz, 0.0);
    }
    inline double& at(int i, int j, int k) { return d[(size_t)(i + ox) + (size_t)nx * ((j + oy) + (size_t)ny * (k + oz))]; }
    inline double operator()(int i, int j, int k) const { return d[(size_t)(i + ox) + (size_t)nx * ((j + oy) + (size_t)ny * (k + oz))]; }
};

// ---------------------------------------------------------------------------
// The oracle model
// ---------------------------------------------------------------------------
struct Model {
    Grid g;
    gbo_model_desc desc;
    int ntr = 0;
    Field u, v, w, p, phy, nu;
    std::vector<Field> c, kappa;                    // tracers and AMD diffusivities
    Field sig, sigb;                                // DynamicSmagorinsky: Σ and Σ̄
    std::vector<double> dyn_cs2;                    // DynamicSmagorinsky: c² per level (1-based)
    Field jlm, jmm, jlm_prev, jmm_prev;             // Lagrangian averaging: 𝒥ᴸᴹ, 𝒥ᴹᴹ and their previous values
    double prev_compute_time = 0;                   // time of the last Lagrangian update
    bool velocities_set = false;                    // set! received u, v or w since the last finalize
    bool lagrangian() const {
        return desc.closure == GBO_CLOSURE_DYNAMIC_SMAGORINSKY && desc.closure_averaging == GBO_AVERAGING_LAGRANGIAN;
    }
    std::vector<Field> Gn, Gm;                      // tendencies (u,v,w,tracers...)
    double time = 0;
    int64_t iteration = 0;
    double last_dt = INFINITY;                      // clock.last_Δt (QAB2 Euler steps)
    bool has_phy = false;
    std::string err;
    // FT solver persistent storage (the reference keeps solver.storage between solves)
    std::vector<cplx> ft_storage;
    int last_cg_iters = 0;
    // CG work arrays
    Field cg_r, cg_p, cg_q, cg_z, cg_rhs, cg_x;

    int nfields() const { return 3 + ntr; }
    Field& fld(int n) { return n == 0 ? u : n == 1 ? v : n == 2 ? w : c[n - 3]; }
};

inline int wrap(int i, int N) {  // periodic 1-based wrap
    int r = (i - 1) % N;
    if (r < 0) r += N;
    return r + 1;
}

// ---------------------------------------------------------------------------
// Halo fills (src/BoundaryConditions/fill_halo_regions*.jl)
// kind: 0 = Center-in-z field with Flux (no-flux) z BCs, 1 = w (Face in z,
//       impenetrable NormalFlow), the latter filled only if normal_flow.
// ---------------------------------------------------------------------------
void fill_halos(Model& m, Field& f, int kind, bool normal_flow = true) {
    const Grid& g = m.g;
    const int Nx = g.Nx, Ny = g.Ny, Nz = g.Nz, H = g.H;
    const int kz_lo = 1 - g.Hz;
    const int kz_hi = ((kind == 1 && !g.flatz) ? Nz + 1 : Nz) + g.Hz;
    if (!g.flatz) {
        // 1) Flux / NormalFlow on z over the interior (Nx, Ny) (fill_halo_regions_flux.jl:9-27,
        //    fill_halo_regions_normal_flow.jl:2-7)
        for (int j = 1; j <= Ny; ++j)
            for (int i = 1; i <= Nx; ++i) {
                if (kind == 0) {
                    f.at(i, j, 0) = f(i, j, 1);
                    f.at(i, j, Nz + 1) = f(i, j, Nz);
                } else if (normal_flow) {
                    f.at(i, j, 1) = 0.0;
                    f.at(i, j, Nz + 1) = 0.0;
                }
            }
    }
    // 2) Periodic x over the full parent (y, z) extent (fill_halo_regions_periodic.jl:5-11)
    for (int k = kz_lo; k <= kz_hi; ++k)
        for (int j = 1 - H; j <= Ny + H; ++j)
            for (int i = 1; i <= H; ++i) {
                f.at(i - H, j, k) = f(Nx + i - H, j, k);
                f.at(Nx + i, j, k) = f(i, j, k);
            }
    // 3) Periodic y over the full parent (x, z) extent (:13-19)
    for (int k = kz_lo; k <= kz_hi; ++k)
        for (int j = 1; j <= H; ++j)
            for (int i = 1 - H; i <= Nx + H; ++i) {
                f.at(i, j - H, k) = f(i, Ny + j - H, k);
                f.at(i, Ny + j, k) = f(i, j, k);
            }
}

// ---------------------------------------------------------------------------
// Immersed boundary (GridFittedBottom): src/ImmersedBoundaries/grid_fitted_bottom.jl:118-158
// ---------------------------------------------------------------------------
inline double zb_at(const Grid& g, int i, int j) {
    int ii = wrap(i, g.Nx), jj = wrap(j, g.Ny);
    return g.zb[(size_t)(ii - 1) + (size_t)g.Nx * (jj - 1)];
}
// _immersed_cell: z at center ≤ bottom
inline bool immersed_cell(const Grid& g, int i, int j, int k) {
    if (!g.immersed) return false;
    return g.zC(k) <= zb_at(g, i, j);
}
// inactive_cell for Bounded z: cells outside 1..Nz are inactive (src/Grids/inactive_node.jl)
inline bool inactive_cell(const Grid& g, int i, int j, int k) {
    bool outside = (!g.flatz) && (k < 1 || k > g.Nz);
    return outside || immersed_cell(g, i, j, k);
}

// ---------------------------------------------------------------------------
// WENO / centered reconstructions (src/Advection/weno_interpolants.jl,
// centered_reconstruction.jl, topologically_conditional_interpolation.jl)
// ---------------------------------------------------------------------------
inline double beta3(const double* P, int s) {
    const double* C = SM3[s];
    // ψ1*(C1ψ1 + C2ψ2 + C3ψ3) + ψ2*(C4ψ2 + C5ψ3) + ψ3*ψ3*C6  (weno_interpolants.jl:196-213)
    return P[0] * (C[0] * P[0] + C[1] * P[1] + C[2] * P[2]) + P[1] * (C[3] * P[1] + C[4] * P[2]) + P[2] * P[2] * C[5];
}

// WENO5 biased reconstruction at a face from S[0..5] = ψ[f-3..f+2] (weno_interpolants.jl:296-321,515-562)
double weno5(const double* S, bool left) {
    double P[3][3];
    if (left) {
        P[0][0] = S[2]; P[0][1] = S[3]; P[0][2] = S[4];
        P[1][0] = S[1]; P[1][1] = S[2]; P[1][2] = S[3];
        P[2][0] = S[0]; P[2][1] = S[1]; P[2][2] = S[2];
    } else {
        P[0][0] = S[3]; P[0][1] = S[2]; P[0][2] = S[1];
        P[1][0] = S[4]; P[1][1] = S[3]; P[1][2] = S[2];
        P[2][0] = S[5]; P[2][1] = S[4]; P[2][2] = S[3];
    }
    double b[3];
    for (int s = 0; s < 3; ++s) b[s] = beta3(P[s], s);
    double tau = std::fabs(b[0] - b[2]);
    double a[3];
    for (int s = 0; s < 3; ++s) {
        double q = tau / (b[s] + CF.eps);
        a[s] = CF.cstar3[s] * (1 + q * q);
    }
    double inv = 1 / ((a[0] + a[1]) + a[2]);
    double w0 = a[0] * inv, w1 = a[1] * inv, w2 = a[2] * inv;
    double p0 = (CF.p3[0][0] * P[0][0] + CF.p3[0][1] * P[0][1]) + CF.p3[0][2] * P[0][2];
    double p1 = (CF.p3[1][0] * P[1][0] + CF.p3[1][1] * P[1][1]) + CF.p3[1][2] * P[1][2];
    double p2 = (CF.p3[2][0] * P[2][0] + CF.p3[2][1] * P[2][1]) + CF.p3[2][2] * P[2][2];
    return w0 * p0 + w1 * p1 + w2 * p2;
}

// WENO3 from S[0..3] = ψ[f-2..f+1]
double weno3(const double* S, bool left) {
    double P[2][2];
    if (left) {
        P[0][0] = S[1]; P[0][1] = S[2];
        P[1][0] = S[0]; P[1][1] = S[1];
    } else {
        P[0][0] = S[2]; P[0][1] = S[1];
        P[1][0] = S[3]; P[1][1] = S[2];
    }
    double b[2];
    for (int s = 0; s < 2; ++s) b[s] = P[s][0] * (1 * P[s][0] + -2 * P[s][1]) + P[s][1] * P[s][1] * 1;
    double tau = std::fabs(b[0] - b[1]);
    double a[2];
    for (int s = 0; s < 2; ++s) {
        double q = tau / (b[s] + CF.eps);
        a[s] = CF.cstar2[s] * (1 + q * q);
    }
    double inv = 1 / (a[0] + a[1]);
    double p0 = CF.p2[0][0] * P[0][0] + CF.p2[0][1] * P[0][1];
    double p1 = CF.p2[1][0] * P[1][0] + CF.p2[1][1] * P[1][1];
    return (a[0] * inv) * p0 + (a[1] * inv) * p1;
}

inline double c4(const double* q) { return CF.c4[0] * q[0] + CF.c4[1] * q[1] + CF.c4[2] * q[2] + CF.c4[3] * q[3]; }
inline double c2(double a, double b) { return CF.c2[0] * a + CF.c2[1] * b; }

// Buffer selection in a Bounded direction with N cells (topologically_conditional_interpolation.jl:52-58)
// R = required halo of the scheme (3 for WENO5, 2 for WENO3)
inline bool biased_ok_face(int i, int N, int R) { return (i >= R + 1) && (i <= N + 1 - (R - 1)) && (i >= R) && (i <= N + 1 - R); }
inline bool biased_ok_center(int i, int N, int R) { return (i >= R) && (i <= N + 1 - (R - 1)) && (i >= R - 1) && (i <= N + 1 - R); }
inline bool symm_ok_face(int i, int N, int R) { return (i >= R + 1) && (i <= N + 1 - R); }
inline bool symm_ok_center(int i, int N, int R) { return (i >= R) && (i <= N + 1 - R); }

// Generic accessor: a lambda q(o) returning the value at face-relative offset o.
template <class Q>
double biased_interp(Q q, bool left, int level) {
    // level 3 = WENO5, 2 = WENO3, 1 = Centered2 (biased == symmetric for Centered)
    if (level == 3) {
        double S[6];
        for (int o = -3; o <= 2; ++o) S[o + 3] = q(o);
        return weno5(S, left);
    } else if (level == 2) {
        double S[4];
        for (int o = -2; o <= 1; ++o) S[o + 2] = q(o);
        return weno3(S, left);
    }
    return c2(q(-1), q(0));
}
template <class Q>
double symm_interp(Q q, int level) {
    if (level == 3) {
        double S[4];
        for (int o = -2; o <= 1; ++o) S[o + 2] = q(o);
        return c4(S);
    }
    return c2(q(-1), q(0));
}

// level for a Bounded-z reconstruction; immersed reduction handled by the caller
inline int zlevel_biased(int k, int N, bool face) {
    if (face) return biased_ok_face(k, N, 3) ? 3 : biased_ok_face(k, N, 2) ? 2 : 1;
    return biased_ok_center(k, N, 3) ? 3 : biased_ok_center(k, N, 2) ? 2 : 1;
}
inline int zlevel_symm(int k, int N, bool face) {
    if (face) return symm_ok_face(k, N, 3) ? 3 : 1;
    return symm_ok_center(k, N, 3) ? 3 : 1;
}

inline bool bias_left(double u) { return u > 0; }

// ---------------------------------------------------------------------------
// Metrics (src/Operators/spacings_and_areas_and_volumes.jl:440-490)
// ---------------------------------------------------------------------------
struct Met {
    const Grid& g;
    explicit Met(const Grid& gg) : g(gg) {}
    double dzc(int k) const { return g.flatz ? 1.0 : g.dzC(k); }
    double dzf(int k) const { return g.flatz ? 1.0 : g.dzF(k); }
    // Ax at (f,c,c) / (c,c,c): Δy Δzᶜ ; at (f,c,f): Δy Δzᶠ
    double Ax_c(int k) const { return g.dy * dzc(k); }
    double Ax_f(int k) const { return g.dy * dzf(k); }
    double Ay_c(int k) const { return g.dx * dzc(k); }
    double Ay_f(int k) const { return g.dx * dzf(k); }
    double Az() const { return g.dx * g.dy; }
    double Vc(int k) const { return Az() * dzc(k); }
    double Vf(int k) const { return Az() * dzf(k); }
};

// ---------------------------------------------------------------------------
// Immersed-aware predicates for GridFittedBottom (src/ImmersedBoundaries/immersed_boundary_interface.jl:49-63)
// peripheral/immersed_peripheral node: a face between an active and an inactive cell.
// ---------------------------------------------------------------------------
inline bool imm(const Grid& g, int i, int j, int k) { return immersed_cell(g, i, j, k); }
// u-face (f,c,c) at (i,j,k): between cells (i-1,j,k) and (i,j,k)
inline bool imm_periph_fcc(const Grid& g, int i, int j, int k) {
    bool a = imm(g, i - 1, j, k), b = imm(g, i, j, k);
    return (a != b) || (a && b);  // peripheral or inactive
}

// Immersed cell strictly inside the domain (immersed_inactive_node of a Center node)
inline bool imm_in(const Grid& g, int i, int j, int k) {
    if (!g.immersed) return false;
    if (!g.flatz && (k < 1 || k > g.Nz)) return false;
    return immersed_cell(g, i, j, k);
}
// immersed_peripheral_node for the flux / velocity locations: a node is on the immersed
// periphery when one of its adjacent cells is immersed and none is outside the domain
// (immersed_boundary_interface.jl:49-63, inactive_node.jl:140-160).  fx, fy, fz = Face flags.
inline bool imm_periph(const Grid& g, int i, int j, int k, bool fx, bool fy, bool fz) {
    if (!g.immersed) return false;
    bool any_imm = false, any_out = false;
    for (int a = 0; a <= (fx ? 1 : 0); ++a)
        for (int b = 0; b <= (fy ? 1 : 0); ++b)
            for (int c = 0; c <= (fz ? 1 : 0); ++c) {
                int kk = k - c;
                bool out = !g.flatz && (kk < 1 || kk > g.Nz);
                any_out |= out;
                any_imm |= (!out) && immersed_cell(g, i - a, j - b, kk);
            }
    return any_imm && !any_out;
}
// immersed_inactive_node of a location with Face flags: every adjacent cell inactive on the
// immersed grid but not every one outside the domain (inactive_node.jl:127-137;
// immersed_boundary_interface.jl:59-60)
inline bool imm_inactive_node(const Grid& g, int i, int j, int k, bool fx, bool fy, bool fz) {
    if (!g.immersed) return false;
    bool all = true, all_out = true;
    for (int a = 0; a <= (fx ? 1 : 0); ++a)
        for (int b = 0; b <= (fy ? 1 : 0); ++b)
            for (int c = 0; c <= (fz ? 1 : 0); ++c) {
                int kk = k - c;
                bool out = !g.flatz && (kk < 1 || kk > g.Nz);
                all_out = all_out && out;
                all = all && (out || immersed_cell(g, i - a, j - b, kk));
            }
    return all && !all_out;
}
// inactive_node of the stencil nodes used by the immersed-aware reconstruction
// (immersed_advective_fluxes.jl:114-152): Center nodes are inactive cells; Face nodes
// are inactive when both adjacent cells are.
inline bool inactive_c(const Grid& g, int i, int j, int k) { return inactive_cell(g, i, j, k); }
// Level of a reconstruction of order 5 in direction d at index n (the face or centre index
// passed to the interpolation, loc_face = Face location) on an immersed grid: WENO5 / WENO3 /
// second order depending on whether the buffer's stencil nodes are all active.
int ibg_level(const Grid& g, int d, int i, int j, int k, bool loc_face) {
    auto node_inactive = [&](int off) {
        int ii = i + (d == 0 ? off : 0), jj = j + (d == 1 ? off : 0), kk = k + (d == 2 ? off : 0);
        if (loc_face) return inactive_c(g, ii, jj, kk);  // flipped to Center
        // flipped to Face: both cells adjacent in direction d inactive
        int ip = ii - (d == 0), jp = jj - (d == 1), kp = kk - (d == 2);
        return inactive_c(g, ii, jj, kk) && inactive_c(g, ip, jp, kp);
    };
    for (int B = 3; B >= 2; --B) {
        int lo = loc_face ? -B : -B + 1, hi = loc_face ? B - 1 : B;
        bool near = false;
        for (int o = lo; o <= hi && !near; ++o) near = node_inactive(o);
        if (!near) return B;
    }
    return 1;
}

// ---------------------------------------------------------------------------
// Tendencies (src/Models/NonhydrostaticModels/nonhydrostatic_tendency_kernel_functions.jl:71-302)
// ---------------------------------------------------------------------------
struct Ctx {
    Model& m;
    const Grid& g;
    Met M;
    int Nz;
    bool flatz;
    bool weno;
    explicit Ctx(Model& mm) : m(mm), g(mm.g), M(mm.g), Nz(mm.g.Nz), flatz(mm.g.flatz),
                              weno(mm.desc.advection == GBO_ADVECTION_WENO5) {}

    // --- immersed-aware WENO order reduction (immersed_advective_fluxes.jl:127-214):
    // if any node in the stencil is inactive, fall back to the buffer scheme.
    int reduce_x(int level, int i, int j, int k, int width_lo, int width_hi) const {
        if (!g.immersed) return level;
        while (level > 1) {
            int lo = level == 3 ? -3 : -2, hi = level == 3 ? 2 : 1;
            (void)width_lo; (void)width_hi;
            bool any = false;
            for (int o = lo; o <= hi && !any; ++o) any = inactive_cell(g, i + o, j, k);
            if (!any) break;
            level = level == 3 ? 2 : 1;
        }
        return level;
    }

    // Symmetric interpolation levels: 3 -> C4, 1 -> C2
    // ---- momentum advection ----
    // Flux Uu at (c,c,c) index (i,j,k): advective_momentum_flux_Uu (upwind_biased_advective_fluxes.jl:23-29)
    // level of a horizontal (periodic) reconstruction: WENO5 unless near an immersed node
    int hl(int d, int i, int j, int k, bool face) const { return g.immersed ? ibg_level(g, d, i, j, k, face) : 3; }
    int zl_b(int k, bool face) const { return g.immersed ? ibg_level(g, 2, 0, 0, k, face) : zlevel_biased(k, Nz, face); }
    int zl_s(int k, bool face) const { return g.immersed ? ibg_level(g, 2, 0, 0, k, face) : zlevel_symm(k, Nz, face); }
    int zlb(int i, int j, int k, bool face) const { return g.immersed ? ibg_level(g, 2, i, j, k, face) : zlevel_biased(k, Nz, face); }
    int zls(int i, int j, int k, bool face) const { return g.immersed ? (ibg_level(g, 2, i, j, k, face) == 3 ? 3 : 1) : zlevel_symm(k, Nz, face); }
    int hls(int d, int i, int j, int k, bool face) const { return hl(d, i, j, k, face) == 3 ? 3 : 1; }

    double F_Uu(int i, int j, int k) const {
        if (imm_periph(g, i, j, k, false, false, false)) return 0.0;
        const Field& U = m.u;
        double ut;
        // _symmetric_interpolate_xᶜᵃᵃ(i) and _biased_interpolate_xᶜᵃᵃ(i): Center location in x
        auto q = [&](int o) { return M.Ax_c(k) * U(i + 1 + o, j, k); };
        ut = symm_interp(q, hls(0, i, j, k, false));
        auto qb = [&](int o) { return U(i + 1 + o, j, k); };
        double ur = biased_interp(qb, bias_left(ut), hl(0, i, j, k, false));
        return ut * ur;
    }
    // Vu at (f,f,c): ṽ = sym_x face i of Ay v; uᴿ = biased_y face j of u
    double F_Vu(int i, int j, int k) const {
        if (imm_periph(g, i, j, k, true, true, false)) return 0.0;
        auto q = [&](int o) { return M.Ay_c(k) * m.v(i + o, j, k); };
        double vt = symm_interp(q, hls(0, i, j, k, true));
        auto qb = [&](int o) { return m.u(i, j + o, k); };
        double ur = biased_interp(qb, bias_left(vt), hl(1, i, j, k, true));
        return vt * ur;
    }
    // Wu at (f,c,f)
    double F_Wu(int i, int j, int k) const {
        if (imm_periph(g, i, j, k, true, false, true)) return 0.0;
        auto q = [&](int o) { return M.Az() * m.w(i + o, j, k); };
        double wt = symm_interp(q, hls(0, i, j, k, true));
        auto qb = [&](int o) { return m.u(i, j, k + o); };
        double ur = biased_interp(qb, bias_left(wt), zlb(i, j, k, true));
        return wt * ur;
    }
    // Uv at (f,f,c): ũ = sym_y face j of Ax u; vᴿ = biased_x face i of v
    double F_Uv(int i, int j, int k) const {
        if (imm_periph(g, i, j, k, true, true, false)) return 0.0;
        auto q = [&](int o) { return M.Ax_c(k) * m.u(i, j + o, k); };
        double ut = symm_interp(q, hls(1, i, j, k, true));
        auto qb = [&](int o) { return m.v(i + o, j, k); };
        double vr = biased_interp(qb, bias_left(ut), hl(0, i, j, k, true));
        return ut * vr;
    }
    // Vv at (c,c,c)
    double F_Vv(int i, int j, int k) const {
        if (imm_periph(g, i, j, k, false, false, false)) return 0.0;
        auto q = [&](int o) { return M.Ay_c(k) * m.v(i, j + 1 + o, k); };
        double vt = symm_interp(q, hls(1, i, j, k, false));
        auto qb = [&](int o) { return m.v(i, j + 1 + o, k); };
        double vr = biased_interp(qb, bias_left(vt), hl(1, i, j, k, false));
        return vt * vr;
    }
    // Wv at (c,f,f)
    double F_Wv(int i, int j, int k) const {
        if (imm_periph(g, i, j, k, false, true, true)) return 0.0;
        auto q = [&](int o) { return M.Az() * m.w(i, j + o, k); };
        double wt = symm_interp(q, hls(1, i, j, k, true));
        auto qb = [&](int o) { return m.v(i, j, k + o); };
        double vr = biased_interp(qb, bias_left(wt), zlb(i, j, k, true));
        return wt * vr;
    }
    // Uw at (f,c,f): ũ = sym_z face k of Ax u (Ax at centers k+o); wᴿ = biased_x face i of w
    double F_Uw(int i, int j, int k) const {
        if (imm_periph(g, i, j, k, true, false, true)) return 0.0;
        auto q = [&](int o) { return M.Ax_c(k + o) * m.u(i, j, k + o); };
        double ut = symm_interp(q, zls(i, j, k, true));
        auto qb = [&](int o) { return m.w(i + o, j, k); };
        double wr = biased_interp(qb, bias_left(ut), hl(0, i, j, k, true));
        return ut * wr;
    }
    // Vw at (c,f,f)
    double F_Vw(int i, int j, int k) const {
        if (imm_periph(g, i, j, k, false, true, true)) return 0.0;
        auto q = [&](int o) { return M.Ay_c(k + o) * m.v(i, j, k + o); };
        double vt = symm_interp(q, zls(i, j, k, true));
        auto qb = [&](int o) { return m.w(i, j + o, k); };
        double wr = biased_interp(qb, bias_left(vt), hl(1, i, j, k, true));
        return vt * wr;
    }
    // Ww at (c,c,c) index k: sym/biased at face k+1 with center conditions
    double F_Ww(int i, int j, int k) const {
        if (imm_periph(g, i, j, k, false, false, false)) return 0.0;
        auto q = [&](int o) { return M.Az() * m.w(i, j, k + 1 + o); };
        double wt = symm_interp(q, zls(i, j, k, false));
        auto qb = [&](int o) { return m.w(i, j, k + 1 + o); };
        double wr = biased_interp(qb, bias_left(wt), zlb(i, j, k, false));
        return wt * wr;
    }

    // ---- tracer advection (upwind_biased_advective_fluxes.jl:95-121) ----
    double F_cx(const Field& cc, int i, int j, int k) const {
        double ut = m.u(i, j, k);
        auto qb = [&](int o) { return cc(i + o, j, k); };
        double cr = biased_interp(qb, bias_left(ut), hl(0, i, j, k, true));
        return M.Ax_c(k) * ut * cr;
    }
    double F_cy(const Field& cc, int i, int j, int k) const {
        double vt = m.v(i, j, k);
        auto qb = [&](int o) { return cc(i, j + o, k); };
        double cr = biased_interp(qb, bias_left(vt), hl(1, i, j, k, true));
        return M.Ay_c(k) * vt * cr;
    }
    double F_cz(const Field& cc, int i, int j, int k) const {
        double wt = m.w(i, j, k);
        auto qb = [&](int o) { return cc(i, j, k + o); };
        double cr = biased_interp(qb, bias_left(wt), zlb(i, j, k, true));
        return M.Az() * wt * cr;
    }

    // ---- closure (abstract_scalar_diffusivity_closure.jl:214-262; velocity_tracer_gradients.jl) ----
    const Field& NU() const { return m.nu; }
    double nu_ffc(int i, int j, int k) const {
        const Field& n = NU();
        return 0.5 * (0.5 * (n(i - 1, j - 1, k) + n(i, j - 1, k)) + 0.5 * (n(i - 1, j, k) + n(i, j, k)));
    }
    double nu_fcf(int i, int j, int k) const {
        const Field& n = NU();
        return 0.5 * (0.5 * (n(i - 1, j, k - 1) + n(i, j, k - 1)) + 0.5 * (n(i - 1, j, k) + n(i, j, k)));
    }
    double nu_cff(int i, int j, int k) const {
        const Field& n = NU();
        return 0.5 * (0.5 * (n(i, j - 1, k - 1) + n(i, j, k - 1)) + 0.5 * (n(i, j - 1, k) + n(i, j, k)));
    }
    // Conditional ∂ on an immersed grid (conditional_differences.jl:15-43): zero when either
    // differenced node is an immersed-inactive node of the field's location.
    bool cu(int i0, int j0, int k0, int i1, int j1, int k1) const {
        return imm_inactive_node(g, i0, j0, k0, true, false, false) || imm_inactive_node(g, i1, j1, k1, true, false, false);
    }
    bool cv(int i0, int j0, int k0, int i1, int j1, int k1) const {
        return imm_inactive_node(g, i0, j0, k0, false, true, false) || imm_inactive_node(g, i1, j1, k1, false, true, false);
    }
    bool cw(int i0, int j0, int k0, int i1, int j1, int k1) const {
        return imm_inactive_node(g, i0, j0, k0, false, false, true) || imm_inactive_node(g, i1, j1, k1, false, false, true);
    }
    double S11(int i, int j, int k) const { return cu(i, j, k, i + 1, j, k) ? 0.0 : (m.u(i + 1, j, k) - m.u(i, j, k)) * (1 / g.dx); }
    double S22(int i, int j, int k) const { return cv(i, j, k, i, j + 1, k) ? 0.0 : (m.v(i, j + 1, k) - m.v(i, j, k)) * (1 / g.dy); }
    double S33(int i, int j, int k) const {
        return (flatz || cw(i, j, k, i, j, k + 1)) ? 0.0 : (m.w(i, j, k + 1) - m.w(i, j, k)) * (1 / M.dzc(k));
    }
    double dyu(int i, int j, int k) const { return cu(i, j - 1, k, i, j, k) ? 0.0 : (m.u(i, j, k) - m.u(i, j - 1, k)) * (1 / g.dy); }
    double dxv(int i, int j, int k) const { return cv(i - 1, j, k, i, j, k) ? 0.0 : (m.v(i, j, k) - m.v(i - 1, j, k)) * (1 / g.dx); }
    double dzu(int i, int j, int k) const {
        return (flatz || cu(i, j, k - 1, i, j, k)) ? 0.0 : (m.u(i, j, k) - m.u(i, j, k - 1)) * (1 / M.dzf(k));
    }
    double dxw(int i, int j, int k) const { return cw(i - 1, j, k, i, j, k) ? 0.0 : (m.w(i, j, k) - m.w(i - 1, j, k)) * (1 / g.dx); }
    double dzv(int i, int j, int k) const {
        return (flatz || cv(i, j, k - 1, i, j, k)) ? 0.0 : (m.v(i, j, k) - m.v(i, j, k - 1)) * (1 / M.dzf(k));
    }
    double dyw(int i, int j, int k) const { return cw(i, j - 1, k, i, j, k) ? 0.0 : (m.w(i, j, k) - m.w(i, j - 1, k)) * (1 / g.dy); }
    double S12(int i, int j, int k) const { return 0.5 * (dyu(i, j, k) + dxv(i, j, k)); }
    double S13(int i, int j, int k) const { return 0.5 * (dzu(i, j, k) + dxw(i, j, k)); }
    double S23(int i, int j, int k) const { return 0.5 * (dzv(i, j, k) + dyw(i, j, k)); }

    // viscous fluxes τ (-2 ν Σ)
    // each viscous flux is zero on the immersed periphery of its location (conditional_flux,
    // immersed_diffusive_fluxes.jl:25-40); the default immersed boundary condition adds none
    bool zp(int i, int j, int k, bool fx, bool fy, bool fz) const { return imm_periph(g, i, j, k, fx, fy, fz); }
    double tau_ux(int i, int j, int k) const { return zp(i, j, k, false, false, false) ? 0.0 : -2 * (NU()(i, j, k) * S11(i, j, k)); }
    double tau_uy(int i, int j, int k) const { return zp(i, j, k, true, true, false) ? 0.0 : -2 * (nu_ffc(i, j, k) * S12(i, j, k)); }
    double tau_uz(int i, int j, int k) const { return zp(i, j, k, true, false, true) ? 0.0 : -2 * (nu_fcf(i, j, k) * S13(i, j, k)); }
    double tau_vx(int i, int j, int k) const { return zp(i, j, k, true, true, false) ? 0.0 : -2 * (nu_ffc(i, j, k) * S12(i, j, k)); }
    double tau_vy(int i, int j, int k) const { return zp(i, j, k, false, false, false) ? 0.0 : -2 * (NU()(i, j, k) * S22(i, j, k)); }
    double tau_vz(int i, int j, int k) const { return zp(i, j, k, false, true, true) ? 0.0 : -2 * (nu_cff(i, j, k) * S23(i, j, k)); }
    double tau_wx(int i, int j, int k) const { return zp(i, j, k, true, false, true) ? 0.0 : -2 * (nu_fcf(i, j, k) * S13(i, j, k)); }
    double tau_wy(int i, int j, int k) const { return zp(i, j, k, false, true, true) ? 0.0 : -2 * (nu_cff(i, j, k) * S23(i, j, k)); }
    double tau_wz(int i, int j, int k) const { return zp(i, j, k, false, false, false) ? 0.0 : -2 * (NU()(i, j, k) * S33(i, j, k)); }

    // diffusive tracer fluxes; κ at faces = ℑ(κ_ccc) (/Pr for Smagorinsky)
    double kap_x(int n, int i, int j, int k) const {
        if (kappa_field()) { const Field& K = m.kappa[n]; return 0.5 * (K(i - 1, j, k) + K(i, j, k)); }
        return 0.5 * (m.nu(i - 1, j, k) + m.nu(i, j, k)) / m.desc.closure_Pr;
    }
    double kap_y(int n, int i, int j, int k) const {
        if (kappa_field()) { const Field& K = m.kappa[n]; return 0.5 * (K(i, j - 1, k) + K(i, j, k)); }
        return 0.5 * (m.nu(i, j - 1, k) + m.nu(i, j, k)) / m.desc.closure_Pr;
    }
    double kap_z(int n, int i, int j, int k) const {
        if (kappa_field()) { const Field& K = m.kappa[n]; return 0.5 * (K(i, j, k - 1) + K(i, j, k)); }
        return 0.5 * (m.nu(i, j, k - 1) + m.nu(i, j, k)) / m.desc.closure_Pr;
    }
    // conditional tracer gradients and zero flux on the immersed periphery of the flux
    // location (immersed_diffusive_fluxes.jl:42-44)
    double dcx(const Field& cc, int i, int j, int k) const {
        return (imm_in(g, i - 1, j, k) || imm_in(g, i, j, k)) ? 0.0 : (cc(i, j, k) - cc(i - 1, j, k)) * (1 / g.dx);
    }
    double dcy(const Field& cc, int i, int j, int k) const {
        return (imm_in(g, i, j - 1, k) || imm_in(g, i, j, k)) ? 0.0 : (cc(i, j, k) - cc(i, j - 1, k)) * (1 / g.dy);
    }
    double dcz(const Field& cc, int i, int j, int k) const {
        return (imm_in(g, i, j, k - 1) || imm_in(g, i, j, k)) ? 0.0 : (cc(i, j, k) - cc(i, j, k - 1)) * (1 / M.dzf(k));
    }
    double q_x(int n, const Field& cc, int i, int j, int k) const { return zp(i, j, k, true, false, false) ? 0.0 : -kap_x(n, i, j, k) * dcx(cc, i, j, k); }
    double q_y(int n, const Field& cc, int i, int j, int k) const { return zp(i, j, k, false, true, false) ? 0.0 : -kap_y(n, i, j, k) * dcy(cc, i, j, k); }
    double q_z(int n, const Field& cc, int i, int j, int k) const { return zp(i, j, k, false, false, true) ? 0.0 : -kap_z(n, i, j, k) * dcz(cc, i, j, k); }

    bool closure_on() const { return m.desc.closure != GBO_CLOSURE_NONE; }
    // AMD and ScalarDiffusivity carry per-tracer diffusivity fields
    bool kappa_field() const { return m.desc.closure == GBO_CLOSURE_AMD || m.desc.closure == GBO_CLOSURE_SCALAR_DIFFUSIVITY; }

    // --- immersed flux masking (immersed_advective_fluxes.jl:19-70; immersed_diffusive_fluxes.jl)
    // fluxes through faces on the immersed periphery are zero.
    bool periph_x(int i, int j, int k) const {  // x-face between (i-1) and i
        return g.immersed && (imm(g, i - 1, j, k) || imm(g, i, j, k));
    }
    bool periph_y(int i, int j, int k) const { return g.immersed && (imm(g, i, j - 1, k) || imm(g, i, j, k)); }
    bool periph_z(int i, int j, int k) const { return g.immersed && (imm(g, i, j, k - 1) || imm(g, i, j, k)); }

    double Gu(int i, int j, int k) const {
        double adv = 0;
        if (m.desc.advection != GBO_ADVECTION_NONE) {
            double dx_ = F_Uu(i, j, k) - F_Uu(i - 1, j, k);
            double dy_ = F_Vu(i, j + 1, k) - F_Vu(i, j, k);
            double dz_ = flatz ? 0.0 : (F_Wu(i, j, k + 1) - F_Wu(i, j, k));
            adv = (1 / M.Vc(k)) * (dx_ + dy_ + dz_);
        }
        double G = -adv;
        if (m.desc.has_coriolis) {
            double f = m.desc.coriolis_f;
            // masked_Ay_qᶜᶠᶜ: zero on the immersed periphery (coriolis_schemes.jl:55-58)
            auto AyV = [&](int ii, int jj) { return imm_periph(g, ii, jj, k, false, true, false) ? 0.0 : M.Ay_c(k) * m.v(ii, jj, k); };
            double ixy = 0.5 * (0.5 * (AyV(i - 1, j) + AyV(i, j)) + 0.5 * (AyV(i - 1, j + 1) + AyV(i, j + 1)));
            double xfu = -f * ixy * (1 / M.Ay_c(k));
            G = G - xfu;
        }
        // ∂xᶠᶜᶜ is conditional on an immersed grid (conditional_differences.jl:15-43)
        if (m.has_phy) G = G - ((imm_in(g, i - 1, j, k) || imm_in(g, i, j, k)) ? 0.0 : (m.phy(i, j, k) - m.phy(i - 1, j, k))) * (1 / g.dx);
        if (closure_on()) {
            double dx_ = M.Ax_c(k) * tau_ux(i, j, k) - M.Ax_c(k) * tau_ux(i - 1, j, k);
            double dy_ = M.Ay_c(k) * tau_uy(i, j + 1, k) - M.Ay_c(k) * tau_uy(i, j, k);
            double dz_ = flatz ? 0.0 : (M.Az() * tau_uz(i, j, k + 1) - M.Az() * tau_uz(i, j, k));
            G = G - (1 / M.Vc(k)) * (dx_ + dy_ + dz_);
        }
        return G;
    }
    double Gv(int i, int j, int k) const {
        double adv = 0;
        if (m.desc.advection != GBO_ADVECTION_NONE) {
            double dx_ = F_Uv(i + 1, j, k) - F_Uv(i, j, k);
            double dy_ = F_Vv(i, j, k) - F_Vv(i, j - 1, k);
            double dz_ = flatz ? 0.0 : (F_Wv(i, j, k + 1) - F_Wv(i, j, k));
            adv = (1 / M.Vc(k)) * (dx_ + dy_ + dz_);
        }
        double G = -adv;
        if (m.desc.has_coriolis) {
            double f = m.desc.coriolis_f;
            auto AxU = [&](int ii, int jj) { return imm_periph(g, ii, jj, k, true, false, false) ? 0.0 : M.Ax_c(k) * m.u(ii, jj, k); };
            double ixy = 0.5 * (0.5 * (AxU(i, j - 1) + AxU(i + 1, j - 1)) + 0.5 * (AxU(i, j) + AxU(i + 1, j)));
            double yfu = f * ixy * (1 / M.Ax_c(k));
            G = G - yfu;
        }
        if (m.has_phy) G = G - ((imm_in(g, i, j - 1, k) || imm_in(g, i, j, k)) ? 0.0 : (m.phy(i, j, k) - m.phy(i, j - 1, k))) * (1 / g.dy);
        if (closure_on()) {
            double dx_ = M.Ax_c(k) * tau_vx(i + 1, j, k) - M.Ax_c(k) * tau_vx(i, j, k);
            double dy_ = M.Ay_c(k) * tau_vy(i, j, k) - M.Ay_c(k) * tau_vy(i, j - 1, k);
            double dz_ = flatz ? 0.0 : (M.Az() * tau_vz(i, j, k + 1) - M.Az() * tau_vz(i, j, k));
            G = G - (1 / M.Vc(k)) * (dx_ + dy_ + dz_);
        }
        return G;
    }
    double Gw(int i, int j, int k) const {
        double adv = 0;
        if (m.desc.advection != GBO_ADVECTION_NONE) {
            double dx_ = F_Uw(i + 1, j, k) - F_Uw(i, j, k);
            double dy_ = F_Vw(i, j + 1, k) - F_Vw(i, j, k);
            double dz_ = F_Ww(i, j, k) - F_Ww(i, j, k - 1);
            adv = (1 / M.Vf(k)) * (dx_ + dy_ + dz_);
        }
        double G = -adv;
        // buoyancy: with a hydrostatic pressure anomaly w gets no buoyancy term (:171-173)
        if (closure_on()) {
            auto twx = [&](int ii) { return tau_wx(ii, j, k); };
            auto twy = [&](int jj) { return tau_wy(i, jj, k); };
            double dx_ = M.Ax_f(k) * twx(i + 1) - M.Ax_f(k) * twx(i);
            double dy_ = M.Ay_f(k) * twy(j + 1) - M.Ay_f(k) * twy(j);
            double dz_ = M.Az() * tau_wz(i, j, k) - M.Az() * tau_wz(i, j, k - 1);
            G = G - (1 / M.Vf(k)) * (dx_ + dy_ + dz_);
        }
        return G;
    }
    double Gc(int n, int i, int j, int k) const {
        const Field& cc = m.c[n];
        double adv = 0;
        if (m.desc.advection != GBO_ADVECTION_NONE) {
            double dx_ = F_cx(cc, i + 1, j, k) - F_cx(cc, i, j, k);
            double dy_ = F_cy(cc, i, j + 1, k) - F_cy(cc, i, j, k);
            double dz_ = flatz ? 0.0 : (F_cz(cc, i, j, k + 1) - F_cz(cc, i, j, k));
            adv = (1 / M.Vc(k)) * (dx_ + dy_ + dz_);
        }
        double G = -adv;
        if (closure_on()) {
            double dx_ = M.Ax_c(k) * q_x(n, cc, i + 1, j, k) - M.Ax_c(k) * q_x(n, cc, i, j, k);
            double dy_ = M.Ay_c(k) * q_y(n, cc, i, j + 1, k) - M.Ay_c(k) * q_y(n, cc, i, j, k);
            double dz_ = flatz ? 0.0 : (M.Az() * q_z(n, cc, i, j, k + 1) - M.Az() * q_z(n, cc, i, j, k));
            G = G - (1 / M.Vc(k)) * (dx_ + dy_ + dz_);
        }
        return G;
    }
};

// ---------------------------------------------------------------------------
// Closures
// ---------------------------------------------------------------------------
// Smagorinsky-Lilly (Smagorinskys/smagorinsky.jl:90-104; lilly_coefficient.jl:122-142;
// scale_invariant_operators.jl:10-13)
double smagorinsky_nu(const Ctx& C, int i, int j, int k) {
    const Model& m = C.m;
    auto S12sq = [&](int ii, int jj, int kk) { double s = C.S12(ii, jj, kk); return s * s; };
    auto S13sq = [&](int ii, int jj, int kk) { double s = C.S13(ii, jj, kk); return s * s; };
    auto S23sq = [&](int ii, int jj, int kk) { double s = C.S23(ii, jj, kk); return s * s; };
    double s11 = C.S11(i, j, k), s22 = C.S22(i, j, k), s33 = C.flatz ? 0.0 : C.S33(i, j, k);
    double tr = s11 * s11 + s22 * s22 + s33 * s33;
    double ixy = 0.5 * (0.5 * (S12sq(i, j, k) + S12sq(i + 1, j, k)) + 0.5 * (S12sq(i, j + 1, k) + S12sq(i + 1, j + 1, k)));
    double ixz, iyz;
    if (C.flatz) {
        ixz = 0.5 * (S13sq(i, j, k) + S13sq(i + 1, j, k));
        iyz = 0.5 * (S23sq(i, j, k) + S23sq(i, j + 1, k));
    } else {
        ixz = 0.5 * (0.5 * (S13sq(i, j, k) + S13sq(i + 1, j, k)) + 0.5 * (S13sq(i, j, k + 1) + S13sq(i + 1, j, k + 1)));
        iyz = 0.5 * (0.5 * (S23sq(i, j, k) + S23sq(i, j + 1, k)) + 0.5 * (S23sq(i, j, k + 1) + S23sq(i, j + 1, k + 1)));
    }
    double Sig2 = tr + 2 * ixy + 2 * ixz + 2 * iyz;
    double D3 = C.g.dx * C.g.dy * C.M.dzc(k);
    double Df = std::cbrt(D3);
    // N² = ℑz(∂z b) at the center
    double N2 = 0;
    if (m.desc.buoyancy_tracer && !C.flatz) {
        const Field& b = m.c[0];
        // N² = ℑz(∂z b), conditional ∂ on an immersed grid
        double b1 = (imm_in(C.g, i, j, k - 1) || imm_in(C.g, i, j, k)) ? 0.0 : (b(i, j, k) - b(i, j, k - 1)) * (1 / C.M.dzf(k));
        double b2 = (imm_in(C.g, i, j, k) || imm_in(C.g, i, j, k + 1)) ? 0.0 : (b(i, j, k + 1) - b(i, j, k)) * (1 / C.M.dzf(k + 1));
        N2 = 0.5 * (b1 + b2);
    }
    double c0 = m.desc.closure_C, cb = m.desc.closure_Cb;
    double N2p = std::max(0.0, N2);
    double r = cb * N2p / Sig2;
    double mn = (std::isnan(r)) ? r : std::min(1.0, r);  // Julia's min propagates NaN
    double vs2 = 1.0 - mn;
    double vs = (Sig2 == 0) ? 0.0 : std::sqrt(vs2);
    double cs2 = vs * (c0 * c0);
    return cs2 * (Df * Df) * std::sqrt(2 * Sig2);
}

// DynamicSmagorinsky with averaging = (1, 2) (Smagorinskys/dynamic_coefficient.jl:215-300;
// scale_invariant_operators.jl:8-13,94-188): Σ = √(ΣᵢⱼΣᵢⱼ) and Σ̄ of the test-filtered
// velocities, Lᵢⱼ and Mᵢⱼ per cell, their x-y means per level, c² = max(𝒥ᴸᴹ, min) / 𝒥ᴹᴹ
// (0 where 𝒥ᴹᴹ ≤ 0), νₑ = c² Δᶠ² √(2Σ²).  Halo reads follow the stored fields: one
// mirrored layer beyond the z walls, zeros further out.
template <class ST>
double strain_sq(const ST& S, int i, int j, int k) {
    auto sq = [](double x) { return x * x; };
    double s11 = S.S11(i, j, k), s22 = S.S22(i, j, k), s33 = S.S33(i, j, k);
    double tr = s11 * s11 + s22 * s22 + s33 * s33;
    double ixy = 0.5 * (0.5 * (sq(S.S12(i, j, k)) + sq(S.S12(i + 1, j, k))) + 0.5 * (sq(S.S12(i, j + 1, k)) + sq(S.S12(i + 1, j + 1, k))));
    double ixz = 0.5 * (0.5 * (sq(S.S13(i, j, k)) + sq(S.S13(i + 1, j, k))) + 0.5 * (sq(S.S13(i, j, k + 1)) + sq(S.S13(i + 1, j, k + 1))));
    double iyz = 0.5 * (0.5 * (sq(S.S23(i, j, k)) + sq(S.S23(i, j + 1, k))) + 0.5 * (sq(S.S23(i, j, k + 1)) + sq(S.S23(i, j + 1, k + 1))));
    return tr + 2 * ixy + 2 * ixz + 2 * iyz;
}

// filter(i, j, k, grid, f) = (6 f + the six face neighbours) / 12 (scale_invariant_operators.jl:94-104)
template <class F>
double test_filter(const F& f, int i, int j, int k) {
    return (6 * f(i, j, k) + f(i + 1, j, k) + f(i - 1, j, k) + f(i, j + 1, k) + f(i, j - 1, k) + f(i, j, k + 1) + f(i, j, k - 1)) / 12;
}

// Σ̄ᵢⱼ: the strain of the filtered velocities at the reference's locations (:110-150)
struct FiltStrain {
    const Ctx& C;
    double fu(int i, int j, int k) const { return test_filter([&](int a, int b, int c) { return C.m.u(a, b, c); }, i, j, k); }
    double fv(int i, int j, int k) const { return test_filter([&](int a, int b, int c) { return C.m.v(a, b, c); }, i, j, k); }
    double fw(int i, int j, int k) const { return test_filter([&](int a, int b, int c) { return C.m.w(a, b, c); }, i, j, k); }
    double S11(int i, int j, int k) const { return (fu(i + 1, j, k) - fu(i, j, k)) * (1 / C.g.dx); }
    double S22(int i, int j, int k) const { return (fv(i, j + 1, k) - fv(i, j, k)) * (1 / C.g.dy); }
    double S33(int i, int j, int k) const { return (fw(i, j, k + 1) - fw(i, j, k)) * (1 / C.M.dzc(k)); }
    double S12(int i, int j, int k) const {
        return 0.5 * ((fu(i, j, k) - fu(i, j - 1, k)) * (1 / C.g.dy) + (fv(i, j, k) - fv(i - 1, j, k)) * (1 / C.g.dx));
    }
    double S13(int i, int j, int k) const {
        return 0.5 * ((fu(i, j, k) - fu(i, j, k - 1)) * (1 / C.M.dzf(k)) + (fw(i, j, k) - fw(i - 1, j, k)) * (1 / C.g.dx));
    }
    double S23(int i, int j, int k) const {
        return 0.5 * ((fv(i, j, k) - fv(i, j, k - 1)) * (1 / C.M.dzf(k)) + (fw(i, j, k) - fw(i, j - 1, k)) * (1 / C.g.dy));
    }
};

// LM_and_MM (dynamic_coefficient.jl:254-276): Lᵢⱼ = ⟨uᵢuⱼ⟩ − ⟨uᵢ⟩⟨uⱼ⟩ from cell-centre
// products, Mᵢⱼ = 2Δᶠ² (⟨Σ Σᵢⱼ⟩ − ᾱ²β Σ̄ Σ̄ᵢⱼ) with ᾱ² = 4, β = 1 (scale_invariant_operators.jl:152-188)
void lm_mm(const Ctx& C, const FiltStrain& B, int i, int j, int k, double& LM, double& MM) {
    const Model& m = C.m;
    const Field &u = m.u, &v = m.v, &w = m.w, &sg = m.sig, &sb = m.sigb;
    auto sq = [](double x) { return x * x; };
    auto ixu = [&](int a, int b, int c) { return 0.5 * (u(a, b, c) + u(a + 1, b, c)); };
    auto iyv = [&](int a, int b, int c) { return 0.5 * (v(a, b, c) + v(a, b + 1, c)); };
    auto izw = [&](int a, int b, int c) { return 0.5 * (w(a, b, c) + w(a, b, c + 1)); };
    auto u1u1 = [&](int a, int b, int c) { return 0.5 * (sq(u(a, b, c)) + sq(u(a + 1, b, c))); };
    auto u2u2 = [&](int a, int b, int c) { return 0.5 * (sq(v(a, b, c)) + sq(v(a, b + 1, c))); };
    auto u3u3 = [&](int a, int b, int c) { return 0.5 * (sq(w(a, b, c)) + sq(w(a, b, c + 1))); };
    auto u1u2 = [&](int a, int b, int c) { return ixu(a, b, c) * iyv(a, b, c); };
    auto u1u3 = [&](int a, int b, int c) { return ixu(a, b, c) * izw(a, b, c); };
    auto u2u3 = [&](int a, int b, int c) { return iyv(a, b, c) * izw(a, b, c); };
    double fu0 = B.fu(i, j, k), fu1 = B.fu(i + 1, j, k);
    double fv0 = B.fv(i, j, k), fv1 = B.fv(i, j + 1, k);
    double fw0 = B.fw(i, j, k), fw1 = B.fw(i, j, k + 1);
    double ixfu = 0.5 * (fu0 + fu1), iyfv = 0.5 * (fv0 + fv1), izfw = 0.5 * (fw0 + fw1);
    double L11 = test_filter(u1u1, i, j, k) - 0.5 * (sq(fu0) + sq(fu1));
    double L22 = test_filter(u2u2, i, j, k) - 0.5 * (sq(fv0) + sq(fv1));
    double L33 = test_filter(u3u3, i, j, k) - 0.5 * (sq(fw0) + sq(fw1));
    double L12 = test_filter(u1u2, i, j, k) - ixfu * iyfv;
    double L13 = test_filter(u1u3, i, j, k) - ixfu * izfw;
    double L23 = test_filter(u2u3, i, j, k) - iyfv * izfw;
    // ℑxyᶜᶜᵃ = ℑyᵃᶜᵃ ∘ ℑxᶜᵃᵃ etc. (interpolation_operators.jl:45-53)
    auto ixy = [](auto f, int a, int b, int c) { return 0.5 * (0.5 * (f(a, b, c) + f(a + 1, b, c)) + 0.5 * (f(a, b + 1, c) + f(a + 1, b + 1, c))); };
    auto ixz = [](auto f, int a, int b, int c) { return 0.5 * (0.5 * (f(a, b, c) + f(a + 1, b, c)) + 0.5 * (f(a, b, c + 1) + f(a + 1, b, c + 1))); };
    auto iyz = [](auto f, int a, int b, int c) { return 0.5 * (0.5 * (f(a, b, c) + f(a, b + 1, c)) + 0.5 * (f(a, b, c + 1) + f(a, b + 1, c + 1))); };
    auto s12 = [&](int a, int b, int c) { return C.S12(a, b, c); };
    auto s13 = [&](int a, int b, int c) { return C.S13(a, b, c); };
    auto s23 = [&](int a, int b, int c) { return C.S23(a, b, c); };
    auto b12 = [&](int a, int b, int c) { return B.S12(a, b, c); };
    auto b13 = [&](int a, int b, int c) { return B.S13(a, b, c); };
    auto b23 = [&](int a, int b, int c) { return B.S23(a, b, c); };
    auto ss11 = [&](int a, int b, int c) { return sg(a, b, c) * C.S11(a, b, c); };
    auto ss22 = [&](int a, int b, int c) { return sg(a, b, c) * C.S22(a, b, c); };
    auto ss33 = [&](int a, int b, int c) { return sg(a, b, c) * C.S33(a, b, c); };
    auto ss12 = [&](int a, int b, int c) { return sg(a, b, c) * ixy(s12, a, b, c); };
    auto ss13 = [&](int a, int b, int c) { return sg(a, b, c) * ixz(s13, a, b, c); };
    auto ss23 = [&](int a, int b, int c) { return sg(a, b, c) * iyz(s23, a, b, c); };
    double sbar = sb(i, j, k);
    double bb11 = sbar * B.S11(i, j, k), bb22 = sbar * B.S22(i, j, k), bb33 = sbar * B.S33(i, j, k);
    double bb12 = sbar * ixy(b12, i, j, k), bb13 = sbar * ixz(b13, i, j, k), bb23 = sbar * iyz(b23, i, j, k);
    double Df = std::cbrt(C.g.dx * C.g.dy * C.M.dzc(k));  // ∛volume
    double f2 = 2 * (Df * Df);
    double M11 = f2 * (test_filter(ss11, i, j, k) - 4 * bb11);
    double M22 = f2 * (test_filter(ss22, i, j, k) - 4 * bb22);
    double M33 = f2 * (test_filter(ss33, i, j, k) - 4 * bb33);
    double M12 = f2 * (test_filter(ss12, i, j, k) - 4 * bb12);
    double M13 = f2 * (test_filter(ss13, i, j, k) - 4 * bb13);
    double M23 = f2 * (test_filter(ss23, i, j, k) - 4 * bb23);
    LM = L11 * M11 + L22 * M22 + L33 * M33 + 2 * L12 * M12 + 2 * L13 * M13 + 2 * L23 * M23;
    MM = M11 * M11 + M22 * M22 + M33 * M33 + 2 * M12 * M12 + 2 * M13 * M13 + 2 * M23 * M23;
}

// _compute_Σ!, _compute_Σ̄! over the interior from the velocities as they are (their
// halos included), then the halos of Σ and Σ̄
void compute_sigmas(Model& m, const Ctx& C, const FiltStrain& B) {
    const Grid& g = m.g;
#pragma omp parallel for collapse(2)
    for (int k = 1; k <= g.Nz; ++k)
        for (int j = 1; j <= g.Ny; ++j)
            for (int i = 1; i <= g.Nx; ++i) {
                m.sig.at(i, j, k) = std::sqrt(strain_sq(C, i, j, k));
                m.sigb.at(i, j, k) = std::sqrt(strain_sq(B, i, j, k));
            }
    fill_halos(m, m.sig, 0);
    fill_halos(m, m.sigb, 0);
}

void dynamic_smagorinsky(Model& m) {
    Ctx C(m);
    const Grid& g = m.g;
    FiltStrain B{C};
    compute_sigmas(m, C, B);
    const size_t plane = (size_t)g.Nx * g.Ny;
    std::vector<double> LM(plane * g.Nz), MM(plane * g.Nz);
#pragma omp parallel for collapse(2)
    for (int k = 1; k <= g.Nz; ++k)
        for (int j = 1; j <= g.Ny; ++j)
            for (int i = 1; i <= g.Nx; ++i) {
                size_t q = (size_t)(i - 1) + (size_t)g.Nx * (j - 1) + plane * (k - 1);
                lm_mm(C, B, i, j, k, LM[q], MM[q]);
            }
    // 𝒥ᴸᴹ, 𝒥ᴹᴹ = Average over x and y; square_smagorinsky_coefficient (dynamic_coefficient.jl:236-248)
    const double lmin = m.desc.closure_min_numerator;
    m.dyn_cs2.assign(g.Nz + 1, 0.0);
    for (int k = 1; k <= g.Nz; ++k) {
        double a = 0, b = 0;
        for (size_t q = 0; q < plane; ++q) {
            a += LM[plane * (k - 1) + q];
            b += MM[plane * (k - 1) + q];
        }
        double jlm = a / (double)plane, jmm = b / (double)plane;
        double num = std::isnan(jlm) ? jlm : std::max(jlm, lmin);  // Julia's max propagates NaN
        m.dyn_cs2[k] = jmm > 0 ? num / jmm : 0.0;                 // × (𝒥ᴹᴹ > 0), a strong zero
    }
    // _compute_smagorinsky_viscosity! (smagorinsky.jl:90-104)
#pragma omp parallel for collapse(2)
    for (int k = 1; k <= g.Nz; ++k)
        for (int j = 1; j <= g.Ny; ++j)
            for (int i = 1; i <= g.Nx; ++i) {
                double Df = std::cbrt(g.dx * g.dy * C.M.dzc(k));
                m.nu.at(i, j, k) = m.dyn_cs2[k] * (Df * Df) * std::sqrt(2 * strain_sq(C, i, j, k));
            }
    fill_halos(m, m.nu, 0);
}

// ---------------------------------------------------------------------------
// DynamicSmagorinsky with LagrangianAveraging (Smagorinskys/dynamic_coefficient.jl:322-487):
// 𝒥ᴸᴹ, 𝒥ᴹᴹ are relaxed towards LM, MM along trajectories once per time step
// (step_closure_prognostics!, after the step's last projection and before update_state!,
// so the velocities' halos still hold the values filled before that projection).
// ---------------------------------------------------------------------------
inline double jl_max(double a, double b) { return (std::isnan(a) || std::isnan(b)) ? NAN : std::max(a, b); }
inline double jl_clamp(double x, double lo, double hi) { return x > hi ? hi : (x < lo ? lo : x); }

// interpolator (Utils/interpolation.jl:34-42): i⁻ = unsafe_trunc(fi), ξ = mod(fi, 1)
inline void interpolator(double fi, int& lo, double& xi) {
    lo = (int)fi;
    double r = std::fmod(fi, 1.0);
    xi = (r == 0) ? 0.0 : (r < 0 ? r + 1.0 : r);
}

// fractional indices of a point (Fields/interpolate.jl:44-58,72-79,166-201): regular
// spacings by division, a z given by its faces by a binary search over the cell centres
double frac_x(const Grid& g, double x) { return (x - (g.x0 + 0.5 * g.dx)) / g.dx + 1; }
double frac_y(const Grid& g, double y) { return (y - (g.y0 + 0.5 * g.dy)) / g.dy + 1; }
double frac_z(const Grid& g, double z) {
    if (!g.stretched) return (z - g.zC(1)) / g.dzC(1) + 1;
    int low = 0, high = g.Nz - 1;
    while (low + 1 < high) {
        int mid = (low + high) / 2;
        double v = g.zC(mid + 1);
        if (v == z) return mid + 1;
        if (v < z) low = mid;
        else high = mid;
    }
    const int i1 = low + 1, i2 = high + 1;
    const double x1 = g.zC(i1), x2 = g.zC(i2);
    return (double)(i2 - i1) / (x2 - x1) * (z - x1) + i1;
}

// _interpolate (Utils/interpolation.jl:58-72): trilinear, the eight terms in this order
double trilinear(const Field& f, double fi, double fj, double fk) {
    int i0, j0, k0;
    double x, y, z;
    interpolator(fi, i0, x);
    interpolator(fj, j0, y);
    interpolator(fk, k0, z);
    const int i1 = i0 + 1, j1 = j0 + 1, k1 = k0 + 1;
    return (1 - x) * (1 - y) * (1 - z) * f(i0, j0, k0) + (1 - x) * (1 - y) * z * f(i0, j0, k1) +
           (1 - x) * y * (1 - z) * f(i0, j1, k0) + (1 - x) * y * z * f(i0, j1, k1) +
           x * (1 - y) * (1 - z) * f(i1, j0, k0) + x * (1 - y) * z * f(i1, j0, k1) +
           x * y * (1 - z) * f(i1, j1, k0) + x * y * z * f(i1, j1, k1);
}

// initialize_closure_fields! (:407-437): 𝒥ᴸᴹ = max(mean LM, min), 𝒥ᴹᴹ = mean MM everywhere
void lagrangian_initialize(Model& m) {
    Ctx C(m);
    const Grid& g = m.g;
    FiltStrain B{C};
    compute_sigmas(m, C, B);
    const size_t N = (size_t)g.Nx * g.Ny * g.Nz;
    std::vector<double> LM(N), MM(N);
#pragma omp parallel for collapse(2)
    for (int k = 1; k <= g.Nz; ++k)
        for (int j = 1; j <= g.Ny; ++j)
            for (int i = 1; i <= g.Nx; ++i) {
                size_t q = (size_t)(i - 1) + (size_t)g.Nx * ((j - 1) + (size_t)g.Ny * (k - 1));
                lm_mm(C, B, i, j, k, LM[q], MM[q]);
            }
    double a = 0, b = 0;
    for (size_t q = 0; q < N; ++q) {
        a += LM[q];
        b += MM[q];
    }
    std::fill(m.jlm.d.begin(), m.jlm.d.end(), jl_max(a / (double)N, m.desc.closure_min_numerator));
    std::fill(m.jmm.d.begin(), m.jmm.d.end(), b / (double)N);
    m.prev_compute_time = m.time;
}

// step_closure_prognostics! and _lagrangian_average_LM_MM! (:342-405,439-484)
void lagrangian_step(Model& m) {
    Ctx C(m);
    const Grid& g = m.g;
    FiltStrain B{C};
    compute_sigmas(m, C, B);
    m.jlm_prev.d = m.jlm.d;
    m.jmm_prev.d = m.jmm.d;
    const double dt = m.time - m.prev_compute_time;
    m.prev_compute_time = m.time;
    const double lmin = m.desc.closure_min_numerator;
#pragma omp parallel for collapse(2)
    for (int k = 1; k <= g.Nz; ++k)
        for (int j = 1; j <= g.Ny; ++j)
            for (int i = 1; i <= g.Nx; ++i) {
                double LM, MM;
                lm_mm(C, B, i, j, k, LM, MM);
                const double lmp = jl_max(m.jlm_prev(i, j, k), lmin), mmp = m.jmm_prev(i, j, k);
                const double Df = std::cbrt(g.dx * g.dy * C.M.dzc(k));
                const double Tm = 1.5 * Df / std::sqrt(std::sqrt(std::sqrt(lmp * mmp)));  // √∜
                const double tau = dt / Tm, eps = tau / (1 + tau);
                const double x = g.x0 + (i - 0.5) * g.dx, y = g.y0 + (j - 0.5) * g.dy, z = g.zC(k);
                const double dzk = C.M.dzc(k);
                const double ddx = jl_clamp(m.u(i, j, k) * dt, -g.dx, g.dx);
                const double ddy = jl_clamp(m.v(i, j, k) * dt, -g.dy, g.dy);
                const double ddz = jl_clamp(m.w(i, j, k) * dt, -dzk, dzk);
                const double fi = frac_x(g, x - ddx), fj = frac_y(g, y - ddy), fk = frac_z(g, z - ddz);
                const double imm = trilinear(m.jmm_prev, fi, fj, fk), ilm = trilinear(m.jlm_prev, fi, fj, fk);
                m.jmm.at(i, j, k) = eps * MM + (1 - eps) * imm;
                const double lms = eps * LM + (1 - eps) * jl_max(ilm, lmin);
                m.jlm.at(i, j, k) = jl_max(lms, lmin);
            }
}

// νₑ from the pointwise coefficient (square_smagorinsky_coefficient, :236-248), then the
// halos of every closure field (update_nonhydrostatic_model_state.jl:50)
void lagrangian_nu(Model& m) {
    Ctx C(m);
    const Grid& g = m.g;
    const double lmin = m.desc.closure_min_numerator;
#pragma omp parallel for collapse(2)
    for (int k = 1; k <= g.Nz; ++k)
        for (int j = 1; j <= g.Ny; ++j)
            for (int i = 1; i <= g.Nx; ++i) {
                const double lm = jl_max(m.jlm(i, j, k), lmin), mm = m.jmm(i, j, k);
                const double cs2 = mm > 0 ? lm / mm : 0.0;
                const double Df = std::cbrt(g.dx * g.dy * C.M.dzc(k));
                m.nu.at(i, j, k) = cs2 * (Df * Df) * std::sqrt(2 * strain_sq(C, i, j, k));
            }
    for (Field* f : {&m.nu, &m.jlm, &m.jmm, &m.jlm_prev, &m.jmm_prev, &m.sig, &m.sigb}) fill_halos(m, *f, 0);
}

// AMD (anisotropic_minimum_dissipation.jl:161-204,243-358; velocity_tracer_gradients.jl:120-250)
struct AMDops {
    const Ctx& C;
    explicit AMDops(const Ctx& c) : C(c) {}
    double Dfx() const { return 2 * C.g.dx; }
    double Dfy() const { return 2 * C.g.dy; }
    double Dfz(int k) const { return 2 * C.M.dzc(k); }
    // normalized gradients at their native locations
    double n_dxu(int i, int j, int k) const { return C.S11(i, j, k); }
    double n_dyv(int i, int j, int k) const { return C.S22(i, j, k); }
    double n_dzw(int i, int j, int k) const { return C.S33(i, j, k); }
    double n_dxv(int i, int j, int k) const { return Dfx() / Dfy() * C.dxv(i, j, k); }
    double n_dyu(int i, int j, int k) const { return Dfy() / Dfx() * C.dyu(i, j, k); }
    double n_dxw(int i, int j, int k) const { return Dfx() / Dfz(k) * C.dxw(i, j, k); }
    double n_dzu(int i, int j, int k) const { return Dfz(k) / Dfx() * C.dzu(i, j, k); }
    double n_dyw(int i, int j, int k) const { return Dfy() / Dfz(k) * C.dyw(i, j, k); }
    double n_dzv(int i, int j, int k) const { return Dfz(k) / Dfy() * C.dzv(i, j, k); }
    double n_S12(int i, int j, int k) const { return 0.5 * (n_dyu(i, j, k) + n_dxv(i, j, k)); }
    double n_S13(int i, int j, int k) const { return 0.5 * (n_dzu(i, j, k) + n_dxw(i, j, k)); }
    double n_S23(int i, int j, int k) const { return 0.5 * (n_dzv(i, j, k) + n_dyw(i, j, k)); }
    template <class F> double Ixy(F f, int i, int j, int k) const {  // ℑxyᶜᶜᵃ of an ffc quantity
        return 0.5 * (0.5 * (f(i, j, k) + f(i + 1, j, k)) + 0.5 * (f(i, j + 1, k) + f(i + 1, j + 1, k)));
    }
    template <class F> double Ixz(F f, int i, int j, int k) const {  // ℑxzᶜᵃᶜ of an fcf quantity
        return 0.5 * (0.5 * (f(i, j, k) + f(i + 1, j, k)) + 0.5 * (f(i, j, k + 1) + f(i + 1, j, k + 1)));
    }
    template <class F> double Iyz(F f, int i, int j, int k) const {  // ℑyzᵃᶜᶜ of a cff quantity
        return 0.5 * (0.5 * (f(i, j, k) + f(i, j + 1, k)) + 0.5 * (f(i, j, k + 1) + f(i, j + 1, k + 1)));
    }
    template <class F> double Ix(F f, int i, int j, int k) const { return 0.5 * (f(i, j, k) + f(i + 1, j, k)); }
    template <class F> double Iy(F f, int i, int j, int k) const { return 0.5 * (f(i, j, k) + f(i, j + 1, k)); }
    template <class F> double Iz(F f, int i, int j, int k) const { return 0.5 * (f(i, j, k) + f(i, j, k + 1)); }

    double nu(int i, int j, int k) const {
        auto sq = [](double x) { return x * x; };
        auto dxv2 = [&](int a, int b, int c) { return sq(n_dxv(a, b, c)); };
        auto dyu2 = [&](int a, int b, int c) { return sq(n_dyu(a, b, c)); };
        auto dxw2 = [&](int a, int b, int c) { return sq(n_dxw(a, b, c)); };
        auto dzu2 = [&](int a, int b, int c) { return sq(n_dzu(a, b, c)); };
        auto dyw2 = [&](int a, int b, int c) { return sq(n_dyw(a, b, c)); };
        auto dzv2 = [&](int a, int b, int c) { return sq(n_dzv(a, b, c)); };
        double q = sq(n_dxu(i, j, k)) + sq(n_dyv(i, j, k)) + sq(n_dzw(i, j, k)) + Ixy(dxv2, i, j, k) + Ixy(dyu2, i, j, k) +
                   Ixz(dxw2, i, j, k) + Ixz(dzu2, i, j, k) + Iyz(dyw2, i, j, k) + Iyz(dzv2, i, j, k);
        if (q == 0) return 0.0;
        double S11 = n_dxu(i, j, k), S22 = n_dyv(i, j, k), S33 = n_dzw(i, j, k);
        auto f_dxvS12 = [&](int a, int b, int c) { return n_dxv(a, b, c) * n_S12(a, b, c); };
        auto f_dxwS13 = [&](int a, int b, int c) { return n_dxw(a, b, c) * n_S13(a, b, c); };
        auto f_dxv = [&](int a, int b, int c) { return n_dxv(a, b, c); };
        auto f_dxw = [&](int a, int b, int c) { return n_dxw(a, b, c); };
        auto f_S23 = [&](int a, int b, int c) { return n_S23(a, b, c); };
        auto f_dyuS12 = [&](int a, int b, int c) { return n_dyu(a, b, c) * n_S12(a, b, c); };
        auto f_dyu = [&](int a, int b, int c) { return n_dyu(a, b, c); };
        auto f_dyw = [&](int a, int b, int c) { return n_dyw(a, b, c); };
        auto f_S13 = [&](int a, int b, int c) { return n_S13(a, b, c); };
        auto f_dywS23 = [&](int a, int b, int c) { return n_dyw(a, b, c) * n_S23(a, b, c); };
        auto f_dzu = [&](int a, int b, int c) { return n_dzu(a, b, c); };
        auto f_dzv = [&](int a, int b, int c) { return n_dzv(a, b, c); };
        auto f_S12 = [&](int a, int b, int c) { return n_S12(a, b, c); };
        auto f_dzuS13 = [&](int a, int b, int c) { return n_dzu(a, b, c) * n_S13(a, b, c); };
        auto f_dzvS23 = [&](int a, int b, int c) { return n_dzv(a, b, c) * n_S23(a, b, c); };
        double r1 = S11 * sq(n_dxu(i, j, k)) + S22 * Ixy(dxv2, i, j, k) + S33 * Ixz(dxw2, i, j, k) +
                    2 * n_dxu(i, j, k) * Ixy(f_dxvS12, i, j, k) + 2 * n_dxu(i, j, k) * Ixz(f_dxwS13, i, j, k) +
                    2 * Ixy(f_dxv, i, j, k) * Ixz(f_dxw, i, j, k) * Iyz(f_S23, i, j, k);
        double r2 = S11 * Ixy(dyu2, i, j, k) + S22 * sq(n_dyv(i, j, k)) + S33 * Iyz(dyw2, i, j, k) +
                    2 * n_dyv(i, j, k) * Ixy(f_dyuS12, i, j, k) + 2 * Ixy(f_dyu, i, j, k) * Iyz(f_dyw, i, j, k) * Ixz(f_S13, i, j, k) +
                    2 * n_dyv(i, j, k) * Iyz(f_dywS23, i, j, k);
        double r3 = S11 * Ixz(dzu2, i, j, k) + S22 * Iyz(dzv2, i, j, k) + S33 * sq(n_dzw(i, j, k)) +
                    2 * Ixz(f_dzu, i, j, k) * Iyz(f_dzv, i, j, k) * Ixy(f_S12, i, j, k) + 2 * n_dzw(i, j, k) * Ixz(f_dzuS13, i, j, k) +
                    2 * n_dzw(i, j, k) * Iyz(f_dzvS23, i, j, k);
        double r = r1 + r2 + r3;
        double Cb_zeta = 0.0;  // Cb = nothing (default)
        double d2 = 3 / (1 / sq(Dfx()) + 1 / sq(Dfy()) + 1 / sq(Dfz(k)));
        double nsgs = -C.m.desc.closure_C * d2 * (r - Cb_zeta) / q;
        return std::max(0.0, nsgs);
    }
    double kappa(const Field& c, int i, int j, int k) const {
        auto sq = [](double x) { return x * x; };
        // conditional ∂ of the tracer on an immersed grid
        auto n_dxc = [&](int a, int b, int cc) { return Dfx() * C.dcx(c, a, b, cc); };
        auto n_dyc = [&](int a, int b, int cc) { return Dfy() * C.dcy(c, a, b, cc); };
        auto n_dzc = [&](int a, int b, int cc) { return Dfz(cc) * C.dcz(c, a, b, cc); };
        auto dxc2 = [&](int a, int b, int cc) { return sq(n_dxc(a, b, cc)); };
        auto dyc2 = [&](int a, int b, int cc) { return sq(n_dyc(a, b, cc)); };
        auto dzc2 = [&](int a, int b, int cc) { return sq(n_dzc(a, b, cc)); };
        double sigma = Ix(dxc2, i, j, k) + Iy(dyc2, i, j, k) + Iz(dzc2, i, j, k);
        if (sigma == 0) return 0.0;
        auto f_dxv = [&](int a, int b, int cc) { return n_dxv(a, b, cc); };
        auto f_dxw = [&](int a, int b, int cc) { return n_dxw(a, b, cc); };
        auto f_dyu = [&](int a, int b, int cc) { return n_dyu(a, b, cc); };
        auto f_dyw = [&](int a, int b, int cc) { return n_dyw(a, b, cc); };
        auto f_dzu = [&](int a, int b, int cc) { return n_dzu(a, b, cc); };
        auto f_dzv = [&](int a, int b, int cc) { return n_dzv(a, b, cc); };
        double cx_ux = n_dxu(i, j, k) * Ix(dxc2, i, j, k) + Ixy(f_dxv, i, j, k) * Ix(n_dxc, i, j, k) * Iy(n_dyc, i, j, k) +
                       Ixz(f_dxw, i, j, k) * Ix(n_dxc, i, j, k) * Iz(n_dzc, i, j, k);
        double cy_uy = Ixy(f_dyu, i, j, k) * Iy(n_dyc, i, j, k) * Ix(n_dxc, i, j, k) + n_dyv(i, j, k) * Iy(dyc2, i, j, k) +
                       Ixz(f_dyw, i, j, k) * Iy(n_dyc, i, j, k) * Iz(n_dzc, i, j, k);
        double cz_uz = Ixz(f_dzu, i, j, k) * Iz(n_dzc, i, j, k) * Ix(n_dxc, i, j, k) + Iyz(f_dzv, i, j, k) * Iz(n_dzc, i, j, k) * Iy(n_dyc, i, j, k) +
                       n_dzw(i, j, k) * Iz(dzc2, i, j, k);
        double theta = cx_ux + cy_uy + cz_uz;
        double d2 = 3 / (1 / sq(Dfx()) + 1 / sq(Dfy()) + 1 / sq(Dfz(k)));
        double ksgs = -C.m.desc.closure_C * d2 * theta / sigma;
        return std::max(0.0, ksgs);
    }
};

// ---------------------------------------------------------------------------
// FFT utilities (FP64; mixed radix, recursive) -- oracle-only, validated
// against numpy.fft in the tests.
// ---------------------------------------------------------------------------
void fft_rec(cplx* a, int n, int stride, cplx* out, int sign, cplx* scratch) {
    if (n == 1) { out[0] = a[0]; return; }
    int p = 2;
    while (p * p <= n && n % p) ++p;
    if (n % p) p = n;
    int m = n / p;
    // decimation in time: sub-sequences a[r + p*t]
    for (int r = 0; r < p; ++r) fft_rec(a + r * stride, m, stride * p, scratch + r * m, sign, out + r * m);
    for (int k = 0; k < m; ++k)
        for (int q = 0; q < p; ++q) {
            cplx s = 0;
            for (int r = 0; r < p; ++r) {
                double ang = sign * 2.0 * M_PI * (double)r * (double)(k + q * m) / (double)n;
                s += scratch[r * m + k] * cplx(std::cos(ang), std::sin(ang));
            }
            out[k + q * m] = s;
        }
}
// in-place 1D transform of a strided line; sign -1 forward, +1 inverse (unnormalised)
void fft_line(cplx* base, int n, long stride, int sign, std::vector<cplx>& buf) {
    buf.resize(3 * (size_t)n);
    cplx* in = buf.data();
    cplx* out = in + n;
    cplx* scr = out + n;
    for (int t = 0; t < n; ++t) in[t] = base[t * stride];
    fft_rec(in, n, 1, out, sign, scr);
    for (int t = 0; t < n; ++t) base[t * stride] = out[t];
}

// DCT-II (FFTW REDFT10) and its inverse (REDFT01 / 2N) of a strided complex line,
// computed through the length-2N symmetric extension.
void dct2_line(cplx* base, int n, long stride, std::vector<cplx>& buf) {
    std::vector<cplx> ext(2 * (size_t)n);
    for (int t = 0; t < n; ++t) { ext[t] = base[t * stride]; ext[2 * n - 1 - t] = base[t * stride]; }
    fft_line(ext.data(), 2 * n, 1, -1, buf);
    for (int k = 0; k < n; ++k) {
        double ang = -M_PI * k / (2.0 * n);
        base[k * stride] = ext[k] * cplx(std::cos(ang), std::sin(ang));  // = 2 Σ x cos(...)
    }
}
void idct2_line(cplx* base, int n, long stride, std::vector<cplx>& buf) {
    // x_t = (1/2N) [X_0 + 2 Σ_{k≥1} X_k cos(π k (t+1/2)/N)], via the extension X_{2N-k} = -X_k
    std::vector<cplx> ext(2 * (size_t)n);
    for (int k = 0; k < n; ++k) {
        double ang = M_PI * k / (2.0 * n);
        ext[k] = base[k * stride] * cplx(std::cos(ang), std::sin(ang));
    }
    ext[n] = 0;
    for (int k = 1; k < n; ++k) {
        double ang = M_PI * (2 * n - k) / (2.0 * n);
        ext[2 * n - k] = -base[k * stride] * cplx(std::cos(ang), std::sin(ang));
    }
    fft_line(ext.data(), 2 * n, 1, +1, buf);
    for (int t = 0; t < n; ++t) base[t * stride] = ext[t] / (2.0 * n);
}

// Poisson eigenvalues (src/Solvers/poisson_eigenvalues.jl:8-23)
double lam_periodic(int i1, int N, double L) { double s = 2 * std::sin((i1 - 1) * M_PI / N) / (L / N); return s * s; }
double lam_bounded(int i1, int N, double L) { double s = 2 * std::sin((i1 - 1) * M_PI / (2 * N)) / (L / N); return s * s; }

// Forward x,y FFTs over a complex Nx*Ny*Nz array (x fastest)
void fft_xy(const Grid& g, std::vector<cplx>& A, int sign) {
    const int Nx = g.Nx, Ny = g.Ny, Nz = g.Nz;
#pragma omp parallel
    {
        std::vector<cplx> buf;
#pragma omp for collapse(2)
        for (int k = 0; k < Nz; ++k)
            for (int j = 0; j < Ny; ++j) fft_line(&A[(size_t)Nx * (j + (size_t)Ny * k)], Nx, 1, sign, buf);
#pragma omp for collapse(2)
        for (int k = 0; k < Nz; ++k)
            for (int i = 0; i < Nx; ++i) fft_line(&A[i + (size_t)Nx * Ny * k], Ny, Nx, sign, buf);
    }
}

// FFTBasedPoissonSolver.solve! restated (fft_based_poisson_solver.jl:94-124):
// ϕ = eigen-expansion solution of ∇²ϕ = b with the zero mode set to zero.
void fft_poisson(const Grid& g, std::vector<double>& phi, const std::vector<double>& b) {
    const int Nx = g.Nx, Ny = g.Ny, Nz = g.Nz;
    const size_t N = (size_t)Nx * Ny * Nz;
    std::vector<cplx> A(N);
    for (size_t n = 0; n < N; ++n) A[n] = b[n];
    if (!g.flatz) {
#pragma omp parallel
        {
            std::vector<cplx> buf;
#pragma omp for collapse(2)
            for (int j = 0; j < Ny; ++j)
                for (int i = 0; i < Nx; ++i) dct2_line(&A[i + (size_t)Nx * j], Nz, (long)Nx * Ny, buf);
        }
    }
    fft_xy(g, A, -1);
#pragma omp parallel for collapse(2)
    for (int k = 0; k < Nz; ++k)
        for (int j = 0; j < Ny; ++j)
            for (int i = 0; i < Nx; ++i) {
                double lx = lam_periodic(i + 1, Nx, g.Lx), ly = lam_periodic(j + 1, Ny, g.Ly);
                double lz = g.flatz ? 0.0 : lam_bounded(k + 1, Nz, g.Lz);
                size_t n = i + (size_t)Nx * (j + (size_t)Ny * k);
                A[n] = -A[n] / (lx + ly + lz);
                if (i == 0 && j == 0 && k == 0) A[n] = 0;
            }
    fft_xy(g, A, +1);
    const double s = 1.0 / ((double)Nx * Ny);
    for (size_t n = 0; n < N; ++n) A[n] *= s;
    if (!g.flatz) {
#pragma omp parallel
        {
            std::vector<cplx> buf;
#pragma omp for collapse(2)
            for (int j = 0; j < Ny; ++j)
                for (int i = 0; i < Nx; ++i) idct2_line(&A[i + (size_t)Nx * j], Nz, (long)Nx * Ny, buf);
        }
    }
    phi.resize(N);
    for (size_t n = 0; n < N; ++n) phi[n] = A[n].real();
}

// FourierTridiagonalPoissonSolver restated (fourier_tridiagonal_poisson_solver.jl:160-260;
// batched_tridiagonal_solver.jl:217-243).  b must already be multiplied by Δzᶜ.
void ft_poisson(Model& m, std::vector<double>& phi, const std::vector<double>& b) {
    const Grid& g = m.g;
    const int Nx = g.Nx, Ny = g.Ny, Nz = g.Nz;
    const size_t N = (size_t)Nx * Ny * Nz;
    std::vector<cplx> A(N);
    for (size_t n = 0; n < N; ++n) A[n] = b[n];
    fft_xy(g, A, -1);
    if (m.ft_storage.size() != N) m.ft_storage.assign(N, 0.0);
    std::vector<cplx>& S = m.ft_storage;
    const double tiny = 10 * 2.220446049250313e-16;
#pragma omp parallel for collapse(2)
    for (int j = 0; j < Ny; ++j)
        for (int i = 0; i < Nx; ++i) {
            double lx = lam_periodic(i + 1, Nx, g.Lx), ly = lam_periodic(j + 1, Ny, g.Ly);
            auto D = [&](int k) {  // k 1-based (:199-212)
                if (k == 1) return -1 / g.dzF(2) - g.dzC(1) * (lx + ly);
                if (k == Nz) return -1 / g.dzF(Nz) - g.dzC(Nz) * (lx + ly);
                return -(1 / g.dzF(k + 1) + 1 / g.dzF(k)) - g.dzC(k) * (lx + ly);
            };
            auto off = [&](int q) { return 1 / g.dzF(q + 1); };  // lower = upper diagonal (:225-229)
            std::vector<cplx> t(Nz + 1);
            auto idx = [&](int k) { return i + (size_t)Nx * (j + (size_t)Ny * (k - 1)); };
            double beta = D(1);
            S[idx(1)] = A[idx(1)] / beta;
            for (int k = 2; k <= Nz; ++k) {
                double c_ = off(k - 1), a_ = off(k - 1);
                t[k] = c_ / beta;
                beta = D(k) - a_ * t[k].real();
                cplx fk = A[idx(k)];
                bool dd = std::fabs(beta) > tiny;
                cplx star = (fk - a_ * S[idx(k - 1)]) / beta;
                if (dd) S[idx(k)] = star;
            }
            for (int k = Nz - 1; k >= 1; --k) S[idx(k)] -= t[k + 1] * S[idx(k + 1)];
        }
    std::vector<cplx> P(S);
    fft_xy(g, P, +1);
    const double s = 1.0 / ((double)Nx * Ny);
    cplx mean = 0;
    for (size_t n = 0; n < N; ++n) { P[n] *= s; mean += P[n]; }
    mean /= (double)N;
    phi.resize(N);
    for (size_t n = 0; n < N; ++n) phi[n] = (P[n] - mean).real();
    S = P;  // the reference transforms storage in place; keep the same state
}

// ---------------------------------------------------------------------------
// State update and time stepping
// ---------------------------------------------------------------------------
void compute_closure(Model& m) {
    if (m.desc.closure == GBO_CLOSURE_NONE) return;
    if (m.desc.closure == GBO_CLOSURE_SCALAR_DIFFUSIVITY) {
        // ScalarDiffusivity(ν, κ): numbers, the same at every point and halo point
        // (scalar_diffusivity.jl:8-12; νᶜᶜᶜ(i, j, k, grid, closure::ScalarDiffusivity, ...) = ν)
        std::fill(m.nu.d.begin(), m.nu.d.end(), m.desc.closure_nu);
        for (int n = 0; n < m.ntr; ++n) std::fill(m.kappa[n].d.begin(), m.kappa[n].d.end(), m.desc.closure_kappa[n]);
        return;
    }
    if (m.desc.closure == GBO_CLOSURE_DYNAMIC_SMAGORINSKY) {
        if (m.lagrangian()) lagrangian_nu(m);
        else dynamic_smagorinsky(m);
        return;
    }
    Ctx C(m);
    const Grid& g = m.g;
#pragma omp parallel for collapse(2)
    for (int k = 1; k <= g.Nz; ++k)
        for (int j = 1; j <= g.Ny; ++j)
            for (int i = 1; i <= g.Nx; ++i) {
                if (m.desc.closure == GBO_CLOSURE_SMAGORINSKY_LILLY) m.nu.at(i, j, k) = smagorinsky_nu(C, i, j, k);
                else {
                    AMDops A(C);
                    m.nu.at(i, j, k) = A.nu(i, j, k);
                    for (int n = 0; n < m.ntr; ++n) m.kappa[n].at(i, j, k) = A.kappa(m.c[n], i, j, k);
                }
            }
    fill_halos(m, m.nu, 0);
    for (auto& K : m.kappa) fill_halos(m, K, 0);
}

// _update_hydrostatic_pressure! (update_hydrostatic_pressure.jl:11-21)
void update_phy(Model& m) {
    if (!m.has_phy) return;
    const Grid& g = m.g;
    const Field& b = m.c[0];
    const int Nz = g.Nz;
#pragma omp parallel for collapse(2)
    for (int j = 1; j <= g.Ny; ++j)
        for (int i = 1; i <= g.Nx; ++i) {
            double pk = -(0.5 * (b(i, j, Nz) + b(i, j, Nz + 1))) * g.dzF(Nz + 1);
            m.phy.at(i, j, Nz) = pk;
            for (int k = Nz - 1; k >= 1; --k) {
                pk -= (0.5 * (b(i, j, k) + b(i, j, k + 1))) * g.dzF(k + 1);
                m.phy.at(i, j, k) = pk;
            }
        }
    fill_halos(m, m.phy, 0);
}

// _mask_immersed_field!: zero where immersed_peripheral_node holds at the field's location
// (mask_immersed_field.jl:65-77).  loc: 0 = (c,c,c), 1 = u (f,c,c), 2 = v (c,f,c), 3 = w (c,c,f)
void mask_immersed(Model& m, Field& f, int loc) {
    const Grid& g = m.g;
    if (!g.immersed) return;
    for (int k = 1; k <= g.Nz + (loc == 3 ? 1 : 0); ++k)
        for (int j = 1; j <= g.Ny; ++j)
            for (int i = 1; i <= g.Nx; ++i)
                if (imm_periph(g, i, j, k, loc == 1, loc == 2, loc == 3)) f.at(i, j, k) = 0.0;
}

void compute_tendencies(Model& m) {
    Ctx C(m);
    const Grid& g = m.g;
#pragma omp parallel for collapse(2)
    for (int k = 1; k <= g.Nz; ++k)
        for (int j = 1; j <= g.Ny; ++j)
            for (int i = 1; i <= g.Nx; ++i) {
                m.Gn[0].at(i, j, k) = C.Gu(i, j, k);
                m.Gn[1].at(i, j, k) = C.Gv(i, j, k);
                m.Gn[2].at(i, j, k) = g.flatz ? 0.0 : C.Gw(i, j, k);
                for (int n = 0; n < m.ntr; ++n) m.Gn[3 + n].at(i, j, k) = C.Gc(n, i, j, k);
            }
}

// update_state! (update_nonhydrostatic_model_state.jl:22-62)
void update_state(Model& m) {
    for (int n = 0; n < m.ntr; ++n) mask_immersed(m, m.c[n], 0);
    fill_halos(m, m.u, 0);
    fill_halos(m, m.v, 0);
    fill_halos(m, m.w, 1, /*normal_flow=*/false);
    for (int n = 0; n < m.ntr; ++n) fill_halos(m, m.c[n], 0);
    compute_closure(m);
    update_phy(m);
    compute_tendencies(m);
}

// compute_flux_bc_tendencies! (compute_flux_bcs.jl:113-162)
void flux_bc_tendencies(Model& m) {
    const Grid& g = m.g;
    if (g.flatz) return;
    Met M(g);
    for (int n = 0; n < m.ntr; ++n) {
        double qt = m.desc.tracer_flux_top[n], qb = m.desc.tracer_flux_bottom[n];
        if (qt == 0 && qb == 0) continue;
        Field& G = m.Gn[3 + n];
        for (int j = 1; j <= g.Ny; ++j)
            for (int i = 1; i <= g.Nx; ++i) {
                if (qb != 0) G.at(i, j, 1) += qb * M.Az() / M.Vc(1);
                if (qt != 0) G.at(i, j, g.Nz) -= qt * M.Az() / M.Vc(g.Nz);
            }
    }
}

// Solve for the pressure and correct the velocities (pressure_correction.jl:6-20,67-106;
// solve_for_pressure.jl:12-161)
int solve_cg(Model& m, double dt);
int pressure_correction(Model& m, double dtau) {
    const Grid& g = m.g;
    const int Nx = g.Nx, Ny = g.Ny, Nz = g.Nz;
    Met M(g);
    mask_immersed(m, m.u, 1);
    mask_immersed(m, m.v, 2);
    mask_immersed(m, m.w, 3);
    fill_halos(m, m.u, 0);
    fill_halos(m, m.v, 0);
    fill_halos(m, m.w, 1, true);
    const size_t N = (size_t)Nx * Ny * Nz;
    int rc = 0;
    if (m.desc.pressure_solver == GBO_SOLVER_CONJUGATE_GRADIENT) {
        rc = solve_cg(m, dtau);
    } else {
        std::vector<double> rhs(N), phi;
#pragma omp parallel for collapse(2)
        for (int k = 1; k <= Nz; ++k)
            for (int j = 1; j <= Ny; ++j)
                for (int i = 1; i <= Nx; ++i) {
                    double div = (1 / M.Vc(k)) * ((M.Ax_c(k) * m.u(i + 1, j, k) - M.Ax_c(k) * m.u(i, j, k)) +
                                                  (M.Ay_c(k) * m.v(i, j + 1, k) - M.Ay_c(k) * m.v(i, j, k)) +
                                                  (g.flatz ? 0.0 : (M.Az() * m.w(i, j, k + 1) - M.Az() * m.w(i, j, k))));
                    bool active = !inactive_cell(g, i, j, k);
                    double val = active ? div : 0.0;
                    if (m.desc.pressure_solver == GBO_SOLVER_FOURIER_TRIDIAGONAL) val = (active ? g.dzC(k) : 0.0) * div;
                    rhs[(i - 1) + (size_t)Nx * ((j - 1) + (size_t)Ny * (k - 1))] = val;
                }
        if (m.desc.pressure_solver == GBO_SOLVER_FOURIER_TRIDIAGONAL) ft_poisson(m, phi, rhs);
        else fft_poisson(g, phi, rhs);
        for (int k = 1; k <= Nz; ++k)
            for (int j = 1; j <= Ny; ++j)
                for (int i = 1; i <= Nx; ++i) m.p.at(i, j, k) = phi[(i - 1) + (size_t)Nx * ((j - 1) + (size_t)Ny * (k - 1))];
    }
    fill_halos(m, m.p, 0);
    // _make_pressure_correction!
#pragma omp parallel for collapse(2)
    for (int k = 1; k <= Nz; ++k)
        for (int j = 1; j <= Ny; ++j)
            for (int i = 1; i <= Nx; ++i) {
                // ∂ operators are conditional on an immersed grid (conditional_differences.jl:15-43)
                double dx_ = (imm_in(g, i - 1, j, k) || imm_in(g, i, j, k)) ? 0.0 : (m.p(i, j, k) - m.p(i - 1, j, k));
                double dy_ = (imm_in(g, i, j - 1, k) || imm_in(g, i, j, k)) ? 0.0 : (m.p(i, j, k) - m.p(i, j - 1, k));
                m.u.at(i, j, k) -= dx_ * (1 / g.dx);
                m.v.at(i, j, k) -= dy_ * (1 / g.dy);
                if (!g.flatz) {
                    double dz_ = (imm_in(g, i, j, k - 1) || imm_in(g, i, j, k)) ? 0.0 : (m.p(i, j, k) - m.p(i, j, k - 1));
                    m.w.at(i, j, k) -= dz_ * (1 / g.dzF(k));
                }
            }
    double dtp = std::max(2.220446049250313e-16, dtau);
    for (int k = 1; k <= Nz; ++k)
        for (int j = 1; j <= Ny; ++j)
            for (int i = 1; i <= Nx; ++i) m.p.at(i, j, k) /= dtp;
    return rc;
}

// One RK3 substep (nonhydrostatic_rk3_substep.jl:31-63; runge_kutta_3.jl:196-204)
int rk3_substep(Model& m, double dt, double gamma, double zeta, bool first) {
    const Grid& g = m.g;
    flux_bc_tendencies(m);
    for (int n = 0; n < m.nfields(); ++n) {
        Field& U = m.fld(n);
        Field& G = m.Gn[n];
        Field& Gm = m.Gm[n];
        int k0 = 1;
        if (n == 2 && !g.flatz) k0 = 2;  // w excludes the Bounded periphery (kernel_launching.jl:160-171)
        if (n == 2 && g.flatz) continue;
#pragma omp parallel for collapse(2)
        for (int k = k0; k <= g.Nz; ++k)
            for (int j = 1; j <= g.Ny; ++j)
                for (int i = 1; i <= g.Nx; ++i) {
                    if (first) U.at(i, j, k) += dt * gamma * G(i, j, k);
                    else U.at(i, j, k) += dt * (gamma * G(i, j, k) + zeta * Gm(i, j, k));
                }
    }
    double dtau = first ? dt * gamma : dt * (gamma + zeta);
    return pressure_correction(m, dtau);
}

// One QuasiAdamsBashforth2 step (quasi_adams_bashforth_2.jl:100-121, :134-147;
// nonhydrostatic_ab2_step.jl:29-58): U += Δt (α Gⁿ - β G⁻ not_euler) with α = 3/2 + χ,
// β = 1/2 + χ and χ = -1/2 for an Euler step, taken whenever Δt differs from
// clock.last_Δt; the projection uses Δτ = Δt; then G⁻ = Gⁿ, tick!, update_state!.
int time_step_ab2(Model& m, double dt) {
    const bool euler = dt != m.last_dt;
    if (m.iteration == 0) {  // maybe_prepare_first_time_step! (TimeSteppers.jl:41-48)
        m.last_dt = dt;
        update_state(m);
    }
    const double chi = euler ? -0.5 : m.desc.ab2_chi;
    const double alpha = 1.5 + chi, beta = 0.5 + chi;
    const Grid& g = m.g;
    flux_bc_tendencies(m);
    for (int n = 0; n < m.nfields(); ++n) {
        Field& U = m.fld(n);
        Field& G = m.Gn[n];
        Field& Gm = m.Gm[n];
        int k0 = 1;
        if (n == 2 && !g.flatz) k0 = 2;  // w excludes the Bounded periphery
        if (n == 2 && g.flatz) continue;
#pragma omp parallel for collapse(2)
        for (int k = k0; k <= g.Nz; ++k)
            for (int j = 1; j <= g.Ny; ++j)
                for (int i = 1; i <= g.Nx; ++i) {
                    double Gu = alpha * G(i, j, k) - (euler ? 0.0 : beta * Gm(i, j, k));
                    U.at(i, j, k) += dt * Gu;
                }
    }
    int rc = pressure_correction(m, dt);
    for (int n = 0; n < m.nfields(); ++n) m.Gm[n].d = m.Gn[n].d;
    m.time += dt;
    m.iteration += 1;
    m.last_dt = dt;
    if (m.lagrangian()) lagrangian_step(m);  // quasi_adams_bashforth_2.jl:117
    update_state(m);
    return rc;
}

int time_step(Model& m, double dt) {
    if (m.desc.timestepper == GBO_TIMESTEPPER_QAB2) return time_step_ab2(m, dt);
    const double g1 = 8.0 / 15, g2 = 5.0 / 12, g3 = 3.0 / 4, z2 = -17.0 / 60, z3 = -5.0 / 12;
    if (m.iteration == 0) update_state(m);
    double tnext = m.time + dt;
    int rc = 0;
    auto cache = [&]() { for (int n = 0; n < m.nfields(); ++n) m.Gm[n].d = m.Gn[n].d; };
    rc |= rk3_substep(m, dt, g1, 0, true);
    cache();
    m.time += dt * g1;
    update_state(m);
    rc |= rk3_substep(m, dt, g2, z2, false);
    cache();
    m.time += dt * (g2 + z2);
    update_state(m);
    rc |= rk3_substep(m, dt, g3, z3, false);
    cache();
    m.time = tnext;
    m.iteration += 1;
    if (m.lagrangian()) lagrangian_step(m);  // only when clock.stage == 1 again (runge_kutta_3.jl:163)
    update_state(m);
    return rc;
}

// ---------------------------------------------------------------------------
// Conjugate gradient Poisson solver on an immersed grid
// (conjugate_gradient_poisson_solver.jl:38-211; conjugate_gradient_solver.jl:177-284)
// ---------------------------------------------------------------------------
// Conditional difference: zero across a face touching an immersed / inactive cell
// (ImmersedBoundaries/conditional_differences.jl:15-43)
double Vlap(const Model& m, const Field& c, int i, int j, int k) {
    const Grid& g = m.g;
    Met M(g);
    auto fx = [&](int ii) {  // Ax ∂x at (ii-1/2)
        if (inactive_cell(g, ii - 1, j, k) || inactive_cell(g, ii, j, k)) return 0.0;
        return M.Ax_c(k) * ((c(ii, j, k) - c(ii - 1, j, k)) * (1 / g.dx));
    };
    auto fy = [&](int jj) {
        if (inactive_cell(g, i, jj - 1, k) || inactive_cell(g, i, jj, k)) return 0.0;
        return M.Ay_c(k) * ((c(i, jj, k) - c(i, jj - 1, k)) * (1 / g.dy));
    };
    auto fz = [&](int kk) {
        if (g.flatz) return 0.0;
        if (inactive_cell(g, i, j, kk - 1) || inactive_cell(g, i, j, kk)) return 0.0;
        return M.Az() * ((c(i, j, kk) - c(i, j, kk - 1)) * (1 / g.dzF(kk)));
    };
    return (fx(i + 1) - fx(i)) + (fy(j + 1) - fy(j)) + (fz(k + 1) - fz(k));
}

void apply_Vlap(Model& m, Field& out, Field& in) {
    fill_halos(m, in, 0);
    const Grid& g = m.g;
#pragma omp parallel for collapse(2)
    for (int k = 1; k <= g.Nz; ++k)
        for (int j = 1; j <= g.Ny; ++j)
            for (int i = 1; i <= g.Nx; ++i) out.at(i, j, k) = Vlap(m, in, i, j, k);
}

double field_dot(const Model& m, const Field& a, const Field& b) {
    const Grid& g = m.g;
    double s = 0;
    for (int k = 1; k <= g.Nz; ++k)
        for (int j = 1; j <= g.Ny; ++j)
            for (int i = 1; i <= g.Nx; ++i) s += a(i, j, k) * b(i, j, k);
    return s;
}
double field_mean(const Model& m, const Field& a) {
    const Grid& g = m.g;
    double s = 0;
    for (int k = 1; k <= g.Nz; ++k)
        for (int j = 1; j <= g.Ny; ++j)
            for (int i = 1; i <= g.Nx; ++i) s += a(i, j, k);
    return s / ((double)g.Nx * g.Ny * g.Nz);
}
// ||V⁻¹ r||
double vin_norm(const Model& m, const Field& r) {
    const Grid& g = m.g;
    Met M(g);
    double s = 0;
    for (int k = 1; k <= g.Nz; ++k)
        for (int j = 1; j <= g.Ny; ++j)
            for (int i = 1; i <= g.Nx; ++i) { double x = r(i, j, k) * (1 / M.Vc(k)); s += x * x; }
    return std::sqrt(s);
}

// FFT preconditioner: z = solve(V⁻¹ r) with the spectral solver of the underlying grid
// (conjugate_gradient_poisson_solver.jl:141-147,170-211): FFT on a regular grid,
// Fourier-tridiagonal on a stretched one, whose solve! multiplies the source by Δzᶜ
// (set_source_term!, fourier_tridiagonal_poisson_solver.jl:231-281)
void precondition_fft(Model& m, Field& z, const Field& r) {
    const Grid& g = m.g;
    Met M(g);
    const int Nx = g.Nx, Ny = g.Ny, Nz = g.Nz;
    std::vector<double> rhs((size_t)Nx * Ny * Nz), phi;
    for (int k = 1; k <= Nz; ++k)
        for (int j = 1; j <= Ny; ++j)
            for (int i = 1; i <= Nx; ++i) {
                double s = r(i, j, k) * (1 / M.Vc(k));
                if (g.stretched) s *= g.dzC(k);
                rhs[(i - 1) + (size_t)Nx * ((j - 1) + (size_t)Ny * (k - 1))] = s;
            }
    if (g.stretched) ft_poisson(m, phi, rhs);
    else fft_poisson(g, phi, rhs);
    for (int k = 1; k <= Nz; ++k)
        for (int j = 1; j <= Ny; ++j)
            for (int i = 1; i <= Nx; ++i) z.at(i, j, k) = phi[(i - 1) + (size_t)Nx * ((j - 1) + (size_t)Ny * (k - 1))];
}

// mean over the cells that are not immersed (immersed_reductions.jl: NotImmersed condition)
double active_mean(const Model& m, const Field& a) {
    const Grid& g = m.g;
    double s = 0;
    long n = 0;
    for (int k = 1; k <= g.Nz; ++k)
        for (int j = 1; j <= g.Ny; ++j)
            for (int i = 1; i <= g.Nx; ++i)
                if (!inactive_cell(g, i, j, k)) { s += a(i, j, k); ++n; }
    return n ? s / n : 0.0;
}

void gauge(Model& m, Field& x, Field& r) {
    const Grid& g = m.g;
    double mx = active_mean(m, x), mr = active_mean(m, r);
    for (int k = 1; k <= g.Nz; ++k)
        for (int j = 1; j <= g.Ny; ++j)
            for (int i = 1; i <= g.Nx; ++i) {
                double act = inactive_cell(g, i, j, k) ? 0.0 : 1.0;
                x.at(i, j, k) = (x(i, j, k) - mx) * act;
                r.at(i, j, k) = (r(i, j, k) - mr) * act;
            }
}

// Solve V∇²x = b (b = V·div) with preconditioned CG.  x (= m.p) holds p_prev·Δt on entry.
int cg_solve(Model& m, Field& x, const Field& b) {
    const Grid& g = m.g;
    const int Nx = g.Nx, Ny = g.Ny, Nz = g.Nz;
    double rel = m.desc.cg_reltol > 0 ? m.desc.cg_reltol : std::sqrt(2.220446049250313e-16);
    double abs_ = m.desc.cg_abstol > 0 ? m.desc.cg_abstol : std::sqrt(2.220446049250313e-16);
    int maxiter = m.desc.cg_maxiter > 0 ? m.desc.cg_maxiter : Nx * Ny * Nz;
    Field &r = m.cg_r, &p = m.cg_p, &q = m.cg_q, &z = m.cg_z;
    apply_Vlap(m, q, x);
    r.d = b.d;
    for (int k = 1; k <= Nz; ++k)
        for (int j = 1; j <= Ny; ++j)
            for (int i = 1; i <= Nx; ++i) r.at(i, j, k) = b(i, j, k) - q(i, j, k);
    double tol = std::max(rel * vin_norm(m, r), abs_);
    int it = 0;
    double rho_prev = 0;
    static const bool trace = std::getenv("GBO_ORACLE_CG_TRACE") != nullptr;
    while (it < maxiter && vin_norm(m, r) > tol) {
        if (trace && (it < 50 || it % 500 == 0)) std::fprintf(stderr, "cg %d |V^-1 r| = %.6e (tol %.3e)\n", it, vin_norm(m, r), tol);
        if (m.desc.preconditioner == GBO_PRECOND_NONE) z.d = r.d;
        else precondition_fft(m, z, r);
        double rho = field_dot(m, z, r);
        if (it == 0) p.d = z.d;
        else {
            double beta = rho / rho_prev;
            for (size_t n = 0; n < p.d.size(); ++n) p.d[n] = z.d[n] + beta * p.d[n];
        }
        apply_Vlap(m, q, p);
        double alpha = rho / field_dot(m, p, q);
        for (size_t n = 0; n < x.d.size(); ++n) { x.d[n] += alpha * p.d[n]; r.d[n] -= alpha * q.d[n]; }
        gauge(m, x, r);
        ++it;
        rho_prev = rho;
    }
    m.last_cg_iters = it;
    return (it >= maxiter && vin_norm(m, r) > tol) ? GBO_ERR_NOT_CONVERGED : GBO_OK;
}

int solve_cg(Model& m, double dt) {
    const Grid& g = m.g;
    Met M(g);
    double dtp = std::max(2.220446049250313e-16, dt) * (std::isfinite(dt) ? 1.0 : 0.0);
    for (auto& x : m.p.d) x *= dtp;
    Field& rhs = m.cg_rhs;
    for (int k = 1; k <= g.Nz; ++k)
        for (int j = 1; j <= g.Ny; ++j)
            for (int i = 1; i <= g.Nx; ++i) {
                double div = (1 / M.Vc(k)) * ((M.Ax_c(k) * m.u(i + 1, j, k) - M.Ax_c(k) * m.u(i, j, k)) +
                                              (M.Ay_c(k) * m.v(i, j + 1, k) - M.Ay_c(k) * m.v(i, j, k)) +
                                              (g.flatz ? 0.0 : (M.Az() * m.w(i, j, k + 1) - M.Az() * m.w(i, j, k))));
                bool active = !inactive_cell(g, i, j, k);
                rhs.at(i, j, k) = (active ? div : 0.0) * M.Vc(k);
            }
    return cg_solve(m, m.p, rhs);
}

}  // namespace

// ===========================================================================
// C ABI used by the Python test harness (oracle/oracle.py)
// ===========================================================================
extern "C" {

void* orc_create(const gbo_grid_desc* gd, const gbo_model_desc* md) {
    auto* m = new Model();
    Grid& g = m->g;
    g.Nx = gd->size[0]; g.Ny = gd->size[1]; g.Nz = gd->size[2];
    g.flatz = gd->topology[2] == GBO_FLAT;
    g.immersed = gd->bottom_height != nullptr;
    g.H = g.immersed ? 4 : 3;
    g.Hz = g.flatz ? 0 : g.H;
    if (g.flatz) g.Nz = 1;
    g.Lx = gd->x[1] - gd->x[0];
    g.Ly = gd->y[1] - gd->y[0];
    g.dx = g.Lx / g.Nx;
    g.dy = g.Ly / g.Ny;
    g.x0 = gd->x[0];
    g.y0 = gd->y[0];
    if (g.flatz) {
        g.Lz = 1;
        g.dzc_.assign(9, 1.0); g.dzf_.assign(9, 1.0); g.zc_.assign(9, 0.0); g.zf_.assign(9, 0.0);
        g.zoff = 4;
    } else if (gd->z_faces) {
        build_stretched_z(g, gd->z_faces);
        g.stretched = true;
    } else {
        build_regular_z(g, gd->z[0], gd->z[1]);
    }
    if (g.immersed) {
        // GridFittedBottom: numerical bottom = top face of the last immersed cell
        // (_compute_numerical_bottom_height!, grid_fitted_bottom.jl:118-148)
        g.zb.assign((size_t)g.Nx * g.Ny, 0.0);
        for (int j = 1; j <= g.Ny; ++j)
            for (int i = 1; i <= g.Nx; ++i) {
                double h = gd->bottom_height[(i - 1) + (size_t)g.Nx * (j - 1)];
                double zb = g.zF(1);
                for (int k = 1; k <= g.Nz; ++k) {
                    if (g.zC(k) <= h) zb = g.zF(k + 1);
                }
                g.zb[(i - 1) + (size_t)g.Nx * (j - 1)] = zb;
            }
    }
    m->desc = *md;
    m->ntr = md->ntracers;
    m->has_phy = (!g.flatz) && md->buoyancy_tracer && m->ntr > 0;
    const int H = g.H, Hz = g.Hz;
    m->u.init(g.Nx, g.Ny, g.Nz, H, Hz);
    m->v.init(g.Nx, g.Ny, g.Nz, H, Hz);
    m->w.init(g.Nx, g.Ny, g.flatz ? 1 : g.Nz + 1, H, Hz);
    m->p.init(g.Nx, g.Ny, g.Nz, H, Hz);
    m->phy.init(g.Nx, g.Ny, g.Nz, H, Hz);
    m->nu.init(g.Nx, g.Ny, g.Nz, H, Hz);
    if (md->closure == GBO_CLOSURE_DYNAMIC_SMAGORINSKY) {
        m->sig.init(g.Nx, g.Ny, g.Nz, H, Hz);
        m->sigb.init(g.Nx, g.Ny, g.Nz, H, Hz);
    }
    if (m->lagrangian())
        for (Field* f : {&m->jlm, &m->jmm, &m->jlm_prev, &m->jmm_prev}) f->init(g.Nx, g.Ny, g.Nz, H, Hz);
    m->c.resize(m->ntr);
    for (auto& f : m->c) f.init(g.Nx, g.Ny, g.Nz, H, Hz);
    if (md->closure == GBO_CLOSURE_AMD || md->closure == GBO_CLOSURE_SCALAR_DIFFUSIVITY) {
        m->kappa.resize(m->ntr);
        for (auto& f : m->kappa) f.init(g.Nx, g.Ny, g.Nz, H, Hz);
    }
    m->Gn.resize(m->nfields());
    m->Gm.resize(m->nfields());
    for (int n = 0; n < m->nfields(); ++n) {
        int nzl = (n == 2 && !g.flatz) ? g.Nz + 1 : g.Nz;
        m->Gn[n].init(g.Nx, g.Ny, nzl, H, Hz);
        m->Gm[n].init(g.Nx, g.Ny, nzl, H, Hz);
    }
    for (Field* f : {&m->cg_r, &m->cg_p, &m->cg_q, &m->cg_z, &m->cg_rhs}) f->init(g.Nx, g.Ny, g.Nz, H, Hz);
    // the constructor initializes the closure fields from the zero velocities
    // (nonhydrostatic_model.jl:310): 𝒥ᴸᴹ = minimum_numerator, 𝒥ᴹᴹ = 0
    if (m->lagrangian()) lagrangian_initialize(*m);
    return m;
}

void orc_destroy(void* h) { delete static_cast<Model*>(h); }

static Field* field_ptr(Model* m, int id, int* nzl) {
    const Grid& g = m->g;
    *nzl = g.Nz;
    if (id == GBO_FIELD_U) return &m->u;
    if (id == GBO_FIELD_V) return &m->v;
    if (id == GBO_FIELD_W) { *nzl = g.flatz ? 1 : g.Nz + 1; return &m->w; }
    if (id >= GBO_FIELD_TRACER && id < GBO_FIELD_TRACER + m->ntr) return &m->c[id - GBO_FIELD_TRACER];
    if (id == GBO_FIELD_PNHS) return &m->p;
    if (id == GBO_FIELD_PHY) return &m->phy;
    if (id == GBO_FIELD_NU) return &m->nu;
    if (id == GBO_FIELD_KAPPA && !m->kappa.empty()) return &m->kappa[0];
    if (id == 104 && m->lagrangian()) return &m->jlm;  // oracle only: 𝒥ᴸᴹ, 𝒥ᴹᴹ
    if (id == 105 && m->lagrangian()) return &m->jmm;
    return nullptr;
}

int orc_set_field(void* h, int id, const double* data, int64_t n) {
    Model* m = static_cast<Model*>(h);
    int nzl;
    Field* f = field_ptr(m, id, &nzl);
    const Grid& g = m->g;
    if (!f || n != (int64_t)g.Nx * g.Ny * nzl) return GBO_ERR_INVALID;
    for (int k = 1; k <= nzl; ++k)
        for (int j = 1; j <= g.Ny; ++j)
            for (int i = 1; i <= g.Nx; ++i) f->at(i, j, k) = data[(i - 1) + (size_t)g.Nx * ((j - 1) + (size_t)g.Ny * (k - 1))];
    // set! then fill_halo_regions!(ϕ) with normal-flow fills (set_nonhydrostatic_model.jl:57)
    fill_halos(*m, *f, id == GBO_FIELD_W ? 1 : 0, true);
    if (id == GBO_FIELD_U || id == GBO_FIELD_V || id == GBO_FIELD_W) m->velocities_set = true;
    return GBO_OK;
}

int orc_get_field(void* h, int id, double* out, int64_t n) {
    Model* m = static_cast<Model*>(h);
    int nzl;
    Field* f = field_ptr(m, id, &nzl);
    const Grid& g = m->g;
    if (!f || n != (int64_t)g.Nx * g.Ny * nzl) return GBO_ERR_INVALID;
    for (int k = 1; k <= nzl; ++k)
        for (int j = 1; j <= g.Ny; ++j)
            for (int i = 1; i <= g.Nx; ++i) out[(i - 1) + (size_t)g.Nx * ((j - 1) + (size_t)g.Ny * (k - 1))] = (*f)(i, j, k);
    return GBO_OK;
}

// Rest of set!(model; ...) (set_nonhydrostatic_model.jl:59-73)
int orc_set_finalize(void* h, int enforce) {
    Model* m = static_cast<Model*>(h);
    for (int n = 0; n < m->ntr; ++n) mask_immersed(*m, m->c[n], 0);
    mask_immersed(*m, m->u, 1);
    mask_immersed(*m, m->v, 2);
    mask_immersed(*m, m->w, 3);
    const bool init = m->lagrangian() && m->velocities_set;  // initialize_closure_fields! (:62,69)
    m->velocities_set = false;
    if (init) lagrangian_initialize(*m);
    update_state(*m);
    int rc = 0;
    if (enforce) {
        rc = pressure_correction(*m, 1.0);
        if (init) lagrangian_initialize(*m);
        update_state(*m);
    }
    return rc;
}

int orc_time_step(void* h, double dt, int nsteps) {
    Model* m = static_cast<Model*>(h);
    int rc = 0;
    for (int s = 0; s < nsteps; ++s) rc |= time_step(*m, dt);
    return rc;
}

// Checker access for the Lagrangian-averaging tests: a field's parent array (halos
// included, x fastest; dims = nx, ny, nz of the parent) and one Lagrangian update of
// 𝒥ᴸᴹ, 𝒥ᴹᴹ from the current state with the clock advanced by dt.
int orc_parent(void* h, int id, double* out, int64_t n, int* dims) {
    Model* m = static_cast<Model*>(h);
    int nzl;
    Field* f = field_ptr(m, id, &nzl);
    if (!f) return GBO_ERR_INVALID;
    dims[0] = f->nx; dims[1] = f->ny; dims[2] = f->nz;
    if (out) {
        if (n != (int64_t)f->d.size()) return GBO_ERR_INVALID;
        std::copy(f->d.begin(), f->d.end(), out);
    }
    return GBO_OK;
}

int orc_lagrangian_update(void* h, double dt) {
    Model* m = static_cast<Model*>(h);
    if (!m->lagrangian()) return GBO_ERR_INVALID;
    m->time += dt;
    lagrangian_step(*m);
    return GBO_OK;
}

int orc_clock(void* h, double* t, int64_t* it) {
    Model* m = static_cast<Model*>(h);
    *t = m->time;
    *it = m->iteration;
    return 0;
}

int orc_last_cg_iterations(void* h) { return static_cast<Model*>(h)->last_cg_iters; }

// Standalone Poisson solve with the model's solver: phi, rhs hold Nx*Ny*Nz interior values.
// For FourierTridiagonal the rhs is multiplied by Δzᶜ here (set_source_term!, :268-276).
int orc_poisson_solve(void* h, double* phi, const double* rhs) {
    Model* m = static_cast<Model*>(h);
    const Grid& g = m->g;
    const size_t N = (size_t)g.Nx * g.Ny * g.Nz;
    std::vector<double> b(rhs, rhs + N), out;
    if (m->desc.pressure_solver == GBO_SOLVER_CONJUGATE_GRADIENT) {
        // solve!(x, ::ConjugateGradientSolver, b): V∇²ϕ = rhs from the initial guess in ϕ
        Field& x = m->cg_x;
        x.init(g.Nx, g.Ny, g.Nz, g.H, g.Hz);
        Field& bb = m->cg_rhs;
        for (int k = 1; k <= g.Nz; ++k)
            for (int j = 1; j <= g.Ny; ++j)
                for (int i = 1; i <= g.Nx; ++i) {
                    size_t q = (i - 1) + (size_t)g.Nx * ((j - 1) + (size_t)g.Ny * (k - 1));
                    x.at(i, j, k) = phi[q];
                    bb.at(i, j, k) = rhs[q];
                }
        int rc = cg_solve(*m, x, bb);
        for (int k = 1; k <= g.Nz; ++k)
            for (int j = 1; j <= g.Ny; ++j)
                for (int i = 1; i <= g.Nx; ++i) phi[(i - 1) + (size_t)g.Nx * ((j - 1) + (size_t)g.Ny * (k - 1))] = x(i, j, k);
        return rc;
    }
    if (m->desc.pressure_solver == GBO_SOLVER_FOURIER_TRIDIAGONAL) {
        for (int k = 1; k <= g.Nz; ++k)
            for (size_t n = 0; n < (size_t)g.Nx * g.Ny; ++n) b[n + (size_t)g.Nx * g.Ny * (k - 1)] *= g.dzC(k);
        ft_poisson(*m, out, b);
    } else {
        fft_poisson(g, out, b);
    }
    std::memcpy(phi, out.data(), N * sizeof(double));
    return 0;
}

// Grid metrics for tests: writes Δzᶜ and Δzᶠ for k = 1-Hz .. Nz+Hz+1
int orc_z_spacings(void* h, double* dzc, double* dzf, int n) {
    Model* m = static_cast<Model*>(h);
    const Grid& g = m->g;
    int kmin = 1 - g.Hz, kmax = g.Nz + g.Hz + 1;
    if (n != kmax - kmin + 1) return GBO_ERR_INVALID;
    for (int k = kmin; k <= kmax; ++k) { dzc[k - kmin] = g.dzC(k); dzf[k - kmin] = g.dzF(k); }
    return 0;
}

// One WENO5 reconstruction (for unit tests): S = ψ[f-3..f+2]
double orc_weno5(const double* S, int left) { return weno5(S, left != 0); }

void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"
