// gbo_dynamic.cuh -- DynamicSmagorinsky (turbulence_closure_implementations/Smagorinskys/
// dynamic_coefficient.jl, scale_invariant_operators.jl:94-188) with either averaging.
//
// Averaged over x and y (averaging = (1, 2)), per state update:
//   k_dyn_sigma   Σ = √(ΣᵢⱼΣᵢⱼ) of the resolved strain and Σ̄ = √(Σ̄ᵢⱼΣ̄ᵢⱼ) of the strain of
//                 the test-filtered velocities, one cell per thread (_compute_Σ!, _compute_Σ̄!);
//   k_dyn_lm      Lᵢⱼ Mᵢⱼ and Mᵢⱼ Mᵢⱼ per cell (LM_and_MM), summed per block in FP64;
//   k_dyn_coef    per level: 𝒥ᴸᴹ, 𝒥ᴹᴹ = the x-y means of LM and MM (Field(Average(…, dims=(1, 2)))),
//                 c² = max(𝒥ᴸᴹ, minimum_numerator) / 𝒥ᴹᴹ, or 0 where 𝒥ᴹᴹ ≤ 0
//                 (square_smagorinsky_coefficient);
//   k_smagorinsky νₑ = c² Δᶠ² √(2Σ²) with the level's c² (_compute_smagorinsky_viscosity!).
//
// LagrangianAveraging (dynamic_coefficient.jl:364-487): 𝒥ᴸᴹ, 𝒥ᴹᴹ are fields relaxed along
// trajectories once per time step, after the step's last projection
// (step_closure_prognostics!):
//   k_dyn_sigma   Σ, Σ̄ of the velocities as they are at that point (see LagC);
//   k_lag_lm      LM, MM per cell, written over 𝒥 after 𝒥 was copied to 𝒥⁻;
//   k_lag_step    T = 1.5 Δᶠ (𝒥ᴸᴹ⁻𝒥ᴹᴹ⁻)^(-1/8),
//                 ε = τ / (1 + τ) with τ = Δt / T, the departure point x - clamp(u Δt, ±Δ),
//                 𝒥 = ε (LM, MM) + (1 - ε) trilinear(𝒥⁻ at the departure point)
//                 (_lagrangian_average_LM_MM!);
//   k_lag_tick    previous_compute_time = clock.time (the FP64 clock of the update);
// and per state update k_smagorinsky with the cell's c² = max(𝒥ᴸᴹ, min) / 𝒥ᴹᴹ.  At set!
// with velocities (initialize_closure_fields!, :407-437) both fields take the domain means
// of LM and MM (k_lag_lm, k_lag_sum, k_lag_init_mean, k_lag_fill).
//
// The stencil kernels (k_dyn_sigma, k_dyn_lm, k_lag_lm) are instantiated in gbo_dynamic_f32.cu / _f64.cu
// and launched through the dyn_launch_* functions declared at the end.
//
// The halo conventions are the stored fields' (CFld / WFld): one mirrored layer below and
// above the domain for Center fields and Σ, Σ̄ (fill_halo_regions_flux.jl:14-15), zero
// beyond it, zero for w on and beyond the walls.
#pragma once
#include "gbo_kernels.cuh"

namespace dyn {
constexpr int TX = 32, TY = 8;
constexpr int COEF_THREADS = 256;
}  // namespace dyn

// The test filter: ⟨f⟩ = (6 f + the six face neighbours) / 12 (scale_invariant_operators.jl:94-104).
template <typename FT, class F>
GBO_D FT test_filter(const F& f, int i, int j, int k) {
    return (FT(6) * f(i, j, k) + f(i + 1, j, k) + f(i - 1, j, k) + f(i, j + 1, k) + f(i, j - 1, k) + f(i, j, k + 1) +
            f(i, j, k - 1)) / FT(12);
}

template <typename FT, class A>
struct Filtered {
    A a;
    GBO_D FT operator()(int i, int j, int k) const { return test_filter<FT>(a, i, j, k); }
};

// The three velocity accessors a strain (StrainT) is taken of.
template <class CU, class CW>
struct Vel {
    CU u, v;
    CW w;
};
template <typename FT>
using PlainVel = Vel<CFld<FT>, WFld<FT>>;

// The velocities seen through the test filter: the strain of these (StrainT) is Σ̄ᵢⱼ,
// ∂ of ⟨u⟩ at the reference's locations (scale_invariant_operators.jl:110-150).
template <typename FT, class V>
using FiltVel = Vel<Filtered<FT, decltype(V::u)>, Filtered<FT, decltype(V::w)>>;
template <typename FT, class V>
GBO_D FiltVel<FT, V> filtered(const V& vel) {
    return FiltVel<FT, V>{{vel.u}, {vel.v}, {vel.w}};
}

// The velocities as step_closure_prognostics! sees them: the interior holds the projected
// velocities, while the halos still hold what they were filled with before the
// projection (compute_pressure_correction! fills the halos of the predictor; the
// correction writes the interior only).  `in` is read inside the domain, `halo` (with the
// stored-field halo rules) everywhere else.
template <typename FT>
struct LagC {
    CFld<FT> in, halo;
    GBO_D FT operator()(int i, int j, int k) const {
        return ((unsigned)i < (unsigned)in.Nx && (unsigned)j < (unsigned)in.Ny && (unsigned)k < (unsigned)in.Nz)
                   ? in(i, j, k)
                   : halo(i, j, k);
    }
};
template <typename FT>
struct LagW {
    WFld<FT> in, halo;
    GBO_D FT operator()(int i, int j, int k) const {
        return ((unsigned)i < (unsigned)in.Nx && (unsigned)j < (unsigned)in.Ny) ? in(i, j, k) : halo(i, j, k);
    }
};
template <typename FT>
using LagVel = Vel<LagC<FT>, LagW<FT>>;

// ΣᵢⱼΣᵢⱼ at a cell centre of a 3-D grid (ΣᵢⱼΣᵢⱼᶜᶜᶜ, Σ̄ᵢⱼΣ̄ᵢⱼᶜᶜᶜ)
template <typename FT, class ST>
GBO_D FT strain_sq(const ST& S, int i, int j, int k) {
    auto sq = [](FT x) { return x * x; };
    FT s11 = S.S11(i, j, k), s22 = S.S22(i, j, k), s33 = S.S33(i, j, k);
    FT tr = s11 * s11 + s22 * s22 + s33 * s33;
    FT ixy = FT(0.5) * (FT(0.5) * (sq(S.S12(i, j, k)) + sq(S.S12(i + 1, j, k))) +
                        FT(0.5) * (sq(S.S12(i, j + 1, k)) + sq(S.S12(i + 1, j + 1, k))));
    FT ixz = FT(0.5) * (FT(0.5) * (sq(S.S13(i, j, k)) + sq(S.S13(i + 1, j, k))) +
                        FT(0.5) * (sq(S.S13(i, j, k + 1)) + sq(S.S13(i + 1, j, k + 1))));
    FT iyz = FT(0.5) * (FT(0.5) * (sq(S.S23(i, j, k)) + sq(S.S23(i, j + 1, k))) +
                        FT(0.5) * (sq(S.S23(i, j, k + 1)) + sq(S.S23(i, j + 1, k + 1))));
    return tr + FT(2) * ixy + FT(2) * ixz + FT(2) * iyz;
}

template <typename FT, class V>
__global__ void k_dyn_sigma(GridP<FT> g, V vel, FT* __restrict__ sig, FT* __restrict__ sigb) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= g.Nx || j >= g.Ny) return;
    StrainT<FT, V> S(g, vel);
    const FiltVel<FT, V> FF = filtered<FT>(vel);
    StrainT<FT, FiltVel<FT, V>> SB(g, FF);
    const size_t idx = i + (size_t)g.Nx * (j + (size_t)g.Ny * k);
    sig[idx] = sqrt(strain_sq<FT>(S, i, j, k));
    sigb[idx] = sqrt(strain_sq<FT>(SB, i, j, k));
}

// Lᵢⱼ Mᵢⱼ and Mᵢⱼ Mᵢⱼ at a cell (LM_and_MM, dynamic_coefficient.jl:254-276) from the
// Leonard stresses Lᵢⱼ = ⟨uᵢuⱼ⟩ − ⟨uᵢ⟩⟨uⱼ⟩ and Mᵢⱼ = 2Δᶠ²(⟨ΣΣᵢⱼ⟩ − ᾱ²β Σ̄Σ̄ᵢⱼ), ᾱ² = 4, β = 1
// (scale_invariant_operators.jl:152-188); products of velocities are formed at cell
// centres from ℑ of the face values, as the reference does.
template <typename FT, class V>
GBO_D void lm_mm_point(const GridP<FT>& g, const V& vel, const FT* __restrict__ sig, const FT* __restrict__ sigb,
                       int i, int j, int k, FT& LM, FT& MM) {
    const auto& u = vel.u;
    const auto& v = vel.v;
    const auto& w = vel.w;
    const CFld<FT> sg = cfld(sig, g), sb = cfld(sigb, g);
    StrainT<FT, V> S(g, vel);
    const FiltVel<FT, V> FF = filtered<FT>(vel);
    StrainT<FT, FiltVel<FT, V>> SB(g, FF);
    Met<FT> M(g);
    const FT h = FT(0.5);
    auto sq = [](FT x) { return x * x; };

    // Leonard stresses
    auto ixu = [&](int a, int b, int c) { return h * (u(a, b, c) + u(a + 1, b, c)); };
    auto iyv = [&](int a, int b, int c) { return h * (v(a, b, c) + v(a, b + 1, c)); };
    auto izw = [&](int a, int b, int c) { return h * (w(a, b, c) + w(a, b, c + 1)); };
    auto u1u1 = [&](int a, int b, int c) { return h * (sq(u(a, b, c)) + sq(u(a + 1, b, c))); };
    auto u2u2 = [&](int a, int b, int c) { return h * (sq(v(a, b, c)) + sq(v(a, b + 1, c))); };
    auto u3u3 = [&](int a, int b, int c) { return h * (sq(w(a, b, c)) + sq(w(a, b, c + 1))); };
    auto u1u2 = [&](int a, int b, int c) { return ixu(a, b, c) * iyv(a, b, c); };
    auto u1u3 = [&](int a, int b, int c) { return ixu(a, b, c) * izw(a, b, c); };
    auto u2u3 = [&](int a, int b, int c) { return iyv(a, b, c) * izw(a, b, c); };
    const FT fu0 = FF.u(i, j, k), fu1 = FF.u(i + 1, j, k);
    const FT fv0 = FF.v(i, j, k), fv1 = FF.v(i, j + 1, k);
    const FT fw0 = FF.w(i, j, k), fw1 = FF.w(i, j, k + 1);
    const FT ixfu = h * (fu0 + fu1), iyfv = h * (fv0 + fv1), izfw = h * (fw0 + fw1);
    const FT L11 = test_filter<FT>(u1u1, i, j, k) - h * (sq(fu0) + sq(fu1));
    const FT L22 = test_filter<FT>(u2u2, i, j, k) - h * (sq(fv0) + sq(fv1));
    const FT L33 = test_filter<FT>(u3u3, i, j, k) - h * (sq(fw0) + sq(fw1));
    const FT L12 = test_filter<FT>(u1u2, i, j, k) - ixfu * iyfv;
    const FT L13 = test_filter<FT>(u1u3, i, j, k) - ixfu * izfw;
    const FT L23 = test_filter<FT>(u2u3, i, j, k) - iyfv * izfw;

    // Σ Σᵢⱼ at cell centres (off-diagonal strains interpolated from the edges) and their filter
    auto ss11 = [&](int a, int b, int c) { return sg(a, b, c) * S.S11(a, b, c); };
    auto ss22 = [&](int a, int b, int c) { return sg(a, b, c) * S.S22(a, b, c); };
    auto ss33 = [&](int a, int b, int c) { return sg(a, b, c) * S.S33(a, b, c); };
    auto ss12 = [&](int a, int b, int c) {
        return sg(a, b, c) * (h * (h * (S.S12(a, b, c) + S.S12(a + 1, b, c)) + h * (S.S12(a, b + 1, c) + S.S12(a + 1, b + 1, c))));
    };
    auto ss13 = [&](int a, int b, int c) {
        return sg(a, b, c) * (h * (h * (S.S13(a, b, c) + S.S13(a + 1, b, c)) + h * (S.S13(a, b, c + 1) + S.S13(a + 1, b, c + 1))));
    };
    auto ss23 = [&](int a, int b, int c) {
        return sg(a, b, c) * (h * (h * (S.S23(a, b, c) + S.S23(a, b + 1, c)) + h * (S.S23(a, b, c + 1) + S.S23(a, b + 1, c + 1))));
    };
    const FT sbar = sb(i, j, k);
    const FT bb11 = sbar * SB.S11(i, j, k);
    const FT bb22 = sbar * SB.S22(i, j, k);
    const FT bb33 = sbar * SB.S33(i, j, k);
    const FT bb12 = sbar * (h * (h * (SB.S12(i, j, k) + SB.S12(i + 1, j, k)) + h * (SB.S12(i, j + 1, k) + SB.S12(i + 1, j + 1, k))));
    const FT bb13 = sbar * (h * (h * (SB.S13(i, j, k) + SB.S13(i + 1, j, k)) + h * (SB.S13(i, j, k + 1) + SB.S13(i + 1, j, k + 1))));
    const FT bb23 = sbar * (h * (h * (SB.S23(i, j, k) + SB.S23(i, j + 1, k)) + h * (SB.S23(i, j, k + 1) + SB.S23(i, j + 1, k + 1))));
    const FT Df = cbrt(g.dx * g.dy * M.dzc(k));
    const FT f2 = FT(2) * (Df * Df);
    const FT M11 = f2 * (test_filter<FT>(ss11, i, j, k) - FT(4) * bb11);
    const FT M22 = f2 * (test_filter<FT>(ss22, i, j, k) - FT(4) * bb22);
    const FT M33 = f2 * (test_filter<FT>(ss33, i, j, k) - FT(4) * bb33);
    const FT M12 = f2 * (test_filter<FT>(ss12, i, j, k) - FT(4) * bb12);
    const FT M13 = f2 * (test_filter<FT>(ss13, i, j, k) - FT(4) * bb13);
    const FT M23 = f2 * (test_filter<FT>(ss23, i, j, k) - FT(4) * bb23);
    LM = L11 * M11 + L22 * M22 + L33 * M33 + FT(2) * L12 * M12 + FT(2) * L13 * M13 + FT(2) * L23 * M23;
    MM = M11 * M11 + M22 * M22 + M33 * M33 + FT(2) * M12 * M12 + FT(2) * M13 * M13 + FT(2) * M23 * M23;
}

// LM and MM of every cell of a 32×8 tile of one level, summed in FP64 in a fixed order;
// part[2 (k·nb + b)] and part[2 (k·nb + b) + 1] hold the tile's two sums.
template <typename FT, class V>
__global__ void __launch_bounds__(dyn::TX * dyn::TY) k_dyn_lm(GridP<FT> g, V vel, const FT* __restrict__ sig,
                                                               const FT* __restrict__ sigb, double* __restrict__ part) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    double lm = 0.0, mm = 0.0;
    if (i < g.Nx && j < g.Ny) {
        FT a, b;
        lm_mm_point<FT>(g, vel, sig, sigb, i, j, k, a, b);
        lm = (double)a;
        mm = (double)b;
    }
    for (int o = 16; o > 0; o >>= 1) {
        lm += __shfl_down_sync(0xffffffffu, lm, o);
        mm += __shfl_down_sync(0xffffffffu, mm, o);
    }
    __shared__ double sh[2][dyn::TY];
    if (threadIdx.x == 0) {
        sh[0][threadIdx.y] = lm;
        sh[1][threadIdx.y] = mm;
    }
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        double a = 0.0, b = 0.0;
        for (int r = 0; r < dyn::TY; ++r) {
            a += sh[0][r];
            b += sh[1][r];
        }
        const size_t nb = (size_t)gridDim.x * gridDim.y;
        const size_t q = (size_t)k * nb + blockIdx.x + (size_t)gridDim.x * blockIdx.y;
        part[2 * q] = a;
        part[2 * q + 1] = b;
    }
}

// One block per level: the x-y means 𝒥ᴸᴹ, 𝒥ᴹᴹ from the tile sums, then the squared
// coefficient max(𝒥ᴸᴹ, 𝒥ᴸᴹ_min) / 𝒥ᴹᴹ where 𝒥ᴹᴹ > 0, else 0 (the reference multiplies by
// the Bool (𝒥ᴹᴹ > 0), a strong zero).  max propagates NaN as Julia's does.
template <typename FT>
__global__ void __launch_bounds__(dyn::COEF_THREADS) k_dyn_coef(const double* __restrict__ part, int nb, double ncells,
                                                                 FT lm_min, FT* __restrict__ cs2, FT* __restrict__ jlm_out,
                                                                 FT* __restrict__ jmm_out) {
    const int k = blockIdx.x;
    double a = 0.0, b = 0.0;
    for (int q = threadIdx.x; q < nb; q += blockDim.x) {
        a += part[2 * ((size_t)k * nb + q)];
        b += part[2 * ((size_t)k * nb + q) + 1];
    }
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
    __shared__ double sh[2][dyn::COEF_THREADS / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        sh[0][wid] = a;
        sh[1][wid] = b;
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    a = 0.0;
    b = 0.0;
    for (int r = 0; r < dyn::COEF_THREADS / 32; ++r) {
        a += sh[0][r];
        b += sh[1][r];
    }
    const FT jlm = FT(a / ncells), jmm = FT(b / ncells);
    const FT num = isnan(jlm) ? jlm : (jlm > lm_min ? jlm : lm_min);
    cs2[k] = jmm > FT(0) ? num / jmm : FT(0);
    jlm_out[k] = jlm;
    jmm_out[k] = jmm;
}

// ---------------------------------------------------------------------------
// LagrangianAveraging (dynamic_coefficient.jl:364-487)
// ---------------------------------------------------------------------------
// FP64 slots of the Lagrangian clock (clock.time and previous_compute_time are Float64)
enum { LAG_TIME = 0, LAG_PREV, LAG_DT, LAG_LM0, LAG_MM0, LAG_NSLOTS };
constexpr int LAG_SUM_BLOCKS = 2 * 152;  // blocks of the domain sums at initialization

template <typename FT>
struct LagP {
    GridP<FT> g;
    LagVel<FT> vel;                       // projected interior, halos from the predictor
    const FT* __restrict__ jlm_prev;      // 𝒥ᴸᴹ⁻, 𝒥ᴹᴹ⁻ (interior, halos synthesised)
    const FT* __restrict__ jmm_prev;
    FT* jlm;                              // in: LM, MM of this step; out: 𝒥ᴸᴹ, 𝒥ᴹᴹ
    FT* jmm;
    FT lm_min;                            // minimum_numerator in FT
    double x0, y0, dx, dy;                // cell centres x0 + (i + 1/2) Δx (FP64)
    const double* __restrict__ zc;        // z of the Nz cell centres (FP64)
    double dz1;                           // Δzᶜ of the first cell (regular z)
    int stretched;
    const double* clock;                  // LAG_* slots
    const double* dtp;                    // Δt of this step (FP64)
};

// Julia's max / min propagate NaN
template <typename T>
GBO_D T jl_max(T a, T b) { return (isnan(a) || isnan(b)) ? a + b : (a > b ? a : b); }
GBO_D double jl_clamp(double x, double lo, double hi) { return x > hi ? hi : (x < lo ? lo : x); }

// interpolator (Utils/interpolation.jl:34-42): i⁻ = unsafe_trunc(Int, fi), ξ = mod(fi, 1)
// on a 1-based fractional index; returns the 0-based lower index.
GBO_D int lag_interpolator(double fi, double& xi) {
    const int lo = (int)fi;
    const double r = fmod(fi, 1.0);
    xi = (r == 0.0) ? 0.0 : (r < 0.0 ? r + 1.0 : r);
    return lo - 1;
}

// fractional z index of a point (Fields/interpolate.jl:44-58,166-201): regular spacing by
// division; explicit faces by the bracketing interval of the cell centres (the reference's
// binary search), extrapolated linearly beyond the first and last centres
template <typename FT>
GBO_D double lag_frac_z(const LagP<FT>& P, double z) {
    const int Nz = P.g.Nz;
    if (!P.stretched) return (z - P.zc[0]) / P.dz1 + 1.0;
    int low = 0, high = Nz - 1;
    while (low + 1 < high) {
        const int mid = (low + high) / 2;
        const double v = P.zc[mid];
        if (v == z) return mid + 1;
        if (v < z) low = mid;
        else high = mid;
    }
    const double x1 = P.zc[low], x2 = P.zc[high];
    return (double)(high - low) / (x2 - x1) * (z - x1) + (low + 1);
}

// 𝒥⁻ at a 0-based index: periodic in x and y, the mirrored layer in z (the trilinear
// stencil reaches one cell beyond the domain; its upper node beyond that carries weight 0)
template <typename FT>
GBO_D FT lag_prev(const FT* __restrict__ a, const GridP<FT>& g, int i, int j, int k) {
    i = wrapi(i, g.Nx);
    j = wrapi(j, g.Ny);
    k = k < 0 ? 0 : (k >= g.Nz ? g.Nz - 1 : k);
    return __ldg(a + i + (size_t)g.Nx * (j + (size_t)g.Ny * k));
}

// _interpolate (Utils/interpolation.jl:58-72): the eight weights in the reference's order
template <typename FT>
GBO_D double lag_trilinear(const FT* __restrict__ a, const GridP<FT>& g, int i0, int j0, int k0, double x, double y,
                           double z) {
    const int i1 = i0 + 1, j1 = j0 + 1, k1 = k0 + 1;
    return (1 - x) * (1 - y) * (1 - z) * (double)lag_prev(a, g, i0, j0, k0) +
           (1 - x) * (1 - y) * z * (double)lag_prev(a, g, i0, j0, k1) +
           (1 - x) * y * (1 - z) * (double)lag_prev(a, g, i0, j1, k0) +
           (1 - x) * y * z * (double)lag_prev(a, g, i0, j1, k1) +
           x * (1 - y) * (1 - z) * (double)lag_prev(a, g, i1, j0, k0) +
           x * (1 - y) * z * (double)lag_prev(a, g, i1, j0, k1) +
           x * y * (1 - z) * (double)lag_prev(a, g, i1, j1, k0) + x * y * z * (double)lag_prev(a, g, i1, j1, k1);
}

// LM and MM of every cell (_compute_LM_MM!), stored in FT as the reference's fields are
template <typename FT, class V>
__global__ void __launch_bounds__(dyn::TX * dyn::TY) k_lag_lm(GridP<FT> g, V vel, const FT* __restrict__ sig,
                                                               const FT* __restrict__ sigb, FT* __restrict__ lm,
                                                               FT* __restrict__ mm) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= g.Nx || j >= g.Ny) return;
    FT a, b;
    lm_mm_point<FT>(g, vel, sig, sigb, i, j, k, a, b);
    const size_t idx = i + (size_t)g.Nx * (j + (size_t)g.Ny * k);
    lm[idx] = a;
    mm[idx] = b;
}

// FP64 sums of two arrays per block (grid-stride, fixed order for a fixed launch):
// part[2 b], part[2 b + 1]
template <typename FT>
__global__ void __launch_bounds__(256) k_lag_sum(const FT* __restrict__ a, const FT* __restrict__ b, size_t n,
                                                 double* __restrict__ part) {
    double x = 0.0, y = 0.0;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
        x += (double)a[q];
        y += (double)b[q];
    }
    for (int o = 16; o > 0; o >>= 1) {
        x += __shfl_down_sync(0xffffffffu, x, o);
        y += __shfl_down_sync(0xffffffffu, y, o);
    }
    __shared__ double sh[2][8];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        sh[0][wid] = x;
        sh[1][wid] = y;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        x = 0.0;
        y = 0.0;
        for (int r = 0; r < (int)(blockDim.x >> 5); ++r) {
            x += sh[0][r];
            y += sh[1][r];
        }
        part[2 * (size_t)blockIdx.x] = x;
        part[2 * (size_t)blockIdx.x + 1] = y;
    }
}

// _lagrangian_average_LM_MM! (dynamic_coefficient.jl:364-405), one cell per thread.  The
// elapsed time Δt = clock.time - previous_compute_time is FP64 (the clock's type), so the
// relaxation weight and the departure point are formed in FP64 as the reference's
// promotion does; the fields are stored in FT.
// LM and MM of this step are read from jlm / jmm (k_lag_lm wrote them there after 𝒥 was
// copied to 𝒥⁻); each thread reads and then overwrites its own cell only.
template <typename FT>
__global__ void __launch_bounds__(dyn::TX * dyn::TY) k_lag_step(LagP<FT> P) {
    const GridP<FT>& g = P.g;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= g.Nx || j >= g.Ny) return;
    const double tnow = P.clock[LAG_TIME] + *P.dtp;
    const double dt = tnow - P.clock[LAG_PREV];
    const size_t idx = i + (size_t)g.Nx * (j + (size_t)g.Ny * k);
    const FT LM = P.jlm[idx], MM = P.jmm[idx];
    const FT lmp = jl_max(__ldg(P.jlm_prev + idx), P.lm_min), mmp = __ldg(P.jmm_prev + idx);
    Met<FT> M(g);
    const FT dzk = M.dzc(k);
    const FT Df = cbrt(g.dx * g.dy * dzk);
    const FT Tm = FT(1.5) * Df / sqrt(sqrt(sqrt(lmp * mmp)));  // 1.5 Δᶠ / √(∜(𝒥ᴸᴹ𝒥ᴹᴹ))
    const double tau = dt / (double)Tm;
    const double eps = tau / (1 + tau);
    // departure point: the node minus the displacement by the cell's own u[i, j, k],
    // v[i, j, k], w[i, j, k] over Δt, each clamped to one cell width
    const double x = P.x0 + (i + 0.5) * P.dx, y = P.y0 + (j + 0.5) * P.dy, z = P.zc[k];
    const double ddx = jl_clamp((double)P.vel.u.in(i, j, k) * dt, -(double)g.dx, (double)g.dx);
    const double ddy = jl_clamp((double)P.vel.v.in(i, j, k) * dt, -(double)g.dy, (double)g.dy);
    const double ddz = jl_clamp((double)P.vel.w.in(i, j, k) * dt, -(double)dzk, (double)dzk);
    const double fi = (x - ddx - (P.x0 + 0.5 * P.dx)) / P.dx + 1;
    const double fj = (y - ddy - (P.y0 + 0.5 * P.dy)) / P.dy + 1;
    const double fk = lag_frac_z(P, z - ddz);
    double xi, yi, zi;
    const int i0 = lag_interpolator(fi, xi), j0 = lag_interpolator(fj, yi), k0 = lag_interpolator(fk, zi);
    const double imm = lag_trilinear(P.jmm_prev, g, i0, j0, k0, xi, yi, zi);
    const double ilm = lag_trilinear(P.jlm_prev, g, i0, j0, k0, xi, yi, zi);
    P.jmm[idx] = FT(eps * (double)MM + (1 - eps) * imm);
    const double lms = eps * (double)LM + (1 - eps) * jl_max(ilm, (double)P.lm_min);
    P.jlm[idx] = FT(jl_max(lms, (double)P.lm_min));
}

// previous_compute_time = clock.time after the update (one thread, after k_lag_step)
static __global__ void k_lag_tick(double* clock, const double* dtp) {
    const double t = clock[LAG_TIME] + *dtp;
    clock[LAG_TIME] = t;
    clock[LAG_PREV] = t;
}

// Δt of the next steps (a plain time_step! call) into the clock's slot
static __global__ void k_lag_set_dt(double* clock, double dt, double time) {
    clock[LAG_DT] = dt;
    clock[LAG_TIME] = time;
}

// initialize_closure_fields! (:407-437): the domain means of LM and MM from the block sums
// of k_lag_sum, 𝒥ᴸᴹ₀ = max(mean LM, minimum_numerator), 𝒥ᴹᴹ₀ = mean MM, and
// previous_compute_time = clock.time.  One block.
template <typename FT>
__global__ void __launch_bounds__(dyn::COEF_THREADS) k_lag_init_mean(const double* __restrict__ part, int nparts,
                                                                      double ncells, double lm_min, double time,
                                                                      double* clock) {
    double a = 0.0, b = 0.0;
    for (int q = threadIdx.x; q < nparts; q += blockDim.x) {
        a += part[2 * (size_t)q];
        b += part[2 * (size_t)q + 1];
    }
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
    __shared__ double sh[2][dyn::COEF_THREADS / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        sh[0][wid] = a;
        sh[1][wid] = b;
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    a = 0.0;
    b = 0.0;
    for (int r = 0; r < dyn::COEF_THREADS / 32; ++r) {
        a += sh[0][r];
        b += sh[1][r];
    }
    // mean of the FT field LM, then max with minimum_numerator (both FT in the reference)
    const FT mlm = FT(a / ncells), mmm = FT(b / ncells);
    clock[LAG_LM0] = (double)jl_max(mlm, FT(lm_min));
    clock[LAG_MM0] = (double)mmm;
    clock[LAG_TIME] = time;
    clock[LAG_PREV] = time;
}

// parent(𝒥ᴸᴹ) .= 𝒥ᴸᴹ₀, parent(𝒥ᴹᴹ) .= 𝒥ᴹᴹ₀ (grid-stride)
template <typename FT>
__global__ void k_lag_fill(const double* __restrict__ clock, FT* __restrict__ jlm, FT* __restrict__ jmm, size_t n) {
    const FT a = FT(clock[LAG_LM0]), b = FT(clock[LAG_MM0]);
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
        jlm[q] = a;
        jmm[q] = b;
    }
}

// Launchers of the stencil kernels, instantiated for float and double in gbo_dynamic_f32.cu / _f64.cu
// (their own translation unit: the LM / MM stencil is large).
template <typename FT>
void dyn_launch_sigma(dim3 grid, dim3 block, cudaStream_t st, const GridP<FT>& g, const PlainVel<FT>& vel, FT* sig,
                      FT* sigb);
template <typename FT>
void dyn_launch_sigma(dim3 grid, dim3 block, cudaStream_t st, const GridP<FT>& g, const LagVel<FT>& vel, FT* sig,
                      FT* sigb);
template <typename FT>
void dyn_launch_lm_sums(dim3 grid, dim3 block, cudaStream_t st, const GridP<FT>& g, const PlainVel<FT>& vel,
                        const FT* sig, const FT* sigb, double* part);
template <typename FT>
void dyn_launch_lag_lm(dim3 grid, dim3 block, cudaStream_t st, const GridP<FT>& g, const LagVel<FT>& vel,
                       const FT* sig, const FT* sigb, FT* lm, FT* mm);
