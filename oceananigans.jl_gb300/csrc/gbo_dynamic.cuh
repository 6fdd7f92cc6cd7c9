// gbo_dynamic.cuh -- DynamicSmagorinsky with the coefficient averaged over x and y
// (turbulence_closure_implementations/Smagorinskys/dynamic_coefficient.jl:215-300,
// scale_invariant_operators.jl:94-188).
//
// Per state update:
//   k_dyn_sigma   Σ = √(ΣᵢⱼΣᵢⱼ) of the resolved strain and Σ̄ = √(Σ̄ᵢⱼΣ̄ᵢⱼ) of the strain of
//                 the test-filtered velocities, one cell per thread (_compute_Σ!, _compute_Σ̄!);
//   k_dyn_lm      Lᵢⱼ Mᵢⱼ and Mᵢⱼ Mᵢⱼ per cell (LM_and_MM), summed per block in FP64;
//   k_dyn_coef    per level: 𝒥ᴸᴹ, 𝒥ᴹᴹ = the x-y means of LM and MM (Field(Average(…, dims=(1, 2)))),
//                 c² = max(𝒥ᴸᴹ, minimum_numerator) / 𝒥ᴹᴹ, or 0 where 𝒥ᴹᴹ ≤ 0
//                 (square_smagorinsky_coefficient);
//   k_smagorinsky νₑ = c² Δᶠ² √(2Σ²) with the level's c² (_compute_smagorinsky_viscosity!).
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

// The velocities seen through the test filter: the strain of these (StrainT) is Σ̄ᵢⱼ,
// ∂ of ⟨u⟩ at the reference's locations (scale_invariant_operators.jl:110-150).
template <typename FT>
struct FiltFields {
    Filtered<FT, CFld<FT>> u, v;
    Filtered<FT, WFld<FT>> w;
};

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

template <typename FT>
__global__ void k_dyn_sigma(StepP<FT> P, FT* __restrict__ sig, FT* __restrict__ sigb) {
    const GridP<FT>& g = P.g;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= g.Nx || j >= g.Ny) return;
    const CFld<FT> u = cfld(P.u, g), v = cfld(P.v, g);
    const WFld<FT> w = wfld(P.w, g);
    Fields<FT> F{u, v, cfld(P.nu, g), cfld(P.phy, g), w};
    StrainT<FT> S(g, F);
    FiltFields<FT> FF{{u}, {v}, {w}};
    StrainT<FT, FiltFields<FT>> SB(g, FF);
    const size_t idx = i + (size_t)g.Nx * (j + (size_t)g.Ny * k);
    sig[idx] = sqrt(strain_sq<FT>(S, i, j, k));
    sigb[idx] = sqrt(strain_sq<FT>(SB, i, j, k));
}

// Lᵢⱼ Mᵢⱼ and Mᵢⱼ Mᵢⱼ at a cell (LM_and_MM, dynamic_coefficient.jl:254-276) from the
// Leonard stresses Lᵢⱼ = ⟨uᵢuⱼ⟩ − ⟨uᵢ⟩⟨uⱼ⟩ and Mᵢⱼ = 2Δᶠ²(⟨ΣΣᵢⱼ⟩ − ᾱ²β Σ̄Σ̄ᵢⱼ), ᾱ² = 4, β = 1
// (scale_invariant_operators.jl:152-188); products of velocities are formed at cell
// centres from ℑ of the face values, as the reference does.
template <typename FT>
GBO_D void lm_mm_point(const StepP<FT>& P, const FT* __restrict__ sig, const FT* __restrict__ sigb, int i, int j,
                       int k, FT& LM, FT& MM) {
    const GridP<FT>& g = P.g;
    const CFld<FT> u = cfld(P.u, g), v = cfld(P.v, g);
    const WFld<FT> w = wfld(P.w, g);
    const CFld<FT> sg = cfld(sig, g), sb = cfld(sigb, g);
    Fields<FT> F{u, v, cfld(P.nu, g), cfld(P.phy, g), w};
    StrainT<FT> S(g, F);
    FiltFields<FT> FF{{u}, {v}, {w}};
    StrainT<FT, FiltFields<FT>> SB(g, FF);
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
template <typename FT>
__global__ void __launch_bounds__(dyn::TX * dyn::TY) k_dyn_lm(StepP<FT> P, const FT* __restrict__ sig,
                                                               const FT* __restrict__ sigb, double* __restrict__ part) {
    const GridP<FT>& g = P.g;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    double lm = 0.0, mm = 0.0;
    if (i < g.Nx && j < g.Ny) {
        FT a, b;
        lm_mm_point<FT>(P, sig, sigb, i, j, k, a, b);
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
