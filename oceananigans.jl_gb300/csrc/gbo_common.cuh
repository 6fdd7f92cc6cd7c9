// gbo_common.cuh -- shared device-side definitions for the GB300 NonhydrostaticModel kernels.
//
// Data layout in HBM: every field stores interior points only, x fastest,
// index i + Nx*(j + Ny*k) with 0-based (i, j, k).  Halo points are never
// stored: the kernels synthesise them at load time with the semantics of the
// reference's halo fills (src/BoundaryConditions/fill_halo_regions*.jl):
//   * x and y are Periodic: indices wrap;
//   * Center-in-z fields on Bounded z (u, v, tracers, νₑ, κₑ, pHY′, p) carry a
//     no-flux halo of ONE mirrored layer (fill_halo_regions_flux.jl:9-27);
//     deeper halo layers are never written by the reference and read as zero;
//   * w (Face in z) stores faces k = 0..Nz-1; the bottom face k = 0 and the
//     top face k = Nz are impenetrable and always zero
//     (fill_halo_regions_normal_flow.jl:2-7); faces outside read as zero.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "gbo_coeffs.h"

#define GBO_HD __host__ __device__ __forceinline__
#define GBO_D __device__ __forceinline__

template <typename FT>
struct Cx {
    FT re, im;
};
template <typename FT> GBO_HD Cx<FT> cx(FT a, FT b) { return Cx<FT>{a, b}; }
template <typename FT> GBO_HD Cx<FT> operator+(Cx<FT> a, Cx<FT> b) { return {a.re + b.re, a.im + b.im}; }
template <typename FT> GBO_HD Cx<FT> operator-(Cx<FT> a, Cx<FT> b) { return {a.re - b.re, a.im - b.im}; }
template <typename FT> GBO_HD Cx<FT> operator*(Cx<FT> a, Cx<FT> b) {
    return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <typename FT> GBO_HD Cx<FT> operator*(FT s, Cx<FT> a) { return {s * a.re, s * a.im}; }
template <typename FT> GBO_HD Cx<FT> conj(Cx<FT> a) { return {a.re, -a.im}; }

// Grid description visible to kernels.  Vertical spacings are tables indexed
// by the reference's 1-based level kr in [1-Hz, Nz+Hz+1] at position kr + zoff.
template <typename FT>
struct GridP {
    int Nx, Ny, Nz;
    int flatz;        // 1: topology (Periodic, Periodic, Flat)
    int zoff;
    FT dx, dy;        // uniform horizontal spacings
    FT rdx, rdy;      // 1/Δx, 1/Δy evaluated in FT (Δx⁻¹ operators)
    const FT* dzc;    // Δzᵃᵃᶜ(kr)
    const FT* dzf;    // Δzᵃᵃᶠ(kr)
    const FT* rdzc;   // 1/Δzᵃᵃᶜ(kr)
    const FT* rdzf;   // 1/Δzᵃᵃᶠ(kr)
    const FT* rvc;    // 1/Vᶜᶜᶜ(kr) = 1/(Δx Δy Δzᵃᵃᶜ), formed in FT as the operators do
    // immersed boundary: per-column index of the first active cell (0 = none immersed)
    const int* kbot;  // Nx*Ny entries or nullptr
};

// Periodic index within one period of the domain (the per-point stencils: |offset| <= 4
// and N >= 8)
GBO_D int wrapi(int i, int N) { return i < 0 ? i + N : (i >= N ? i - N : i); }
// Periodic index for any offset: tile fills and tile-edge loads reach up to a tile width
// beyond the domain, which is more than one period when N is below the tile width plus
// its halo
GBO_D int wrapm(int i, int N) {
    const int r = i % N;
    return r < 0 ? r + N : r;
}
// The same with the one-period case first (tile fills: the modulo only on small grids)
GBO_D int wrapt(int i, int N) {
    i = i < 0 ? i + N : (i >= N ? i - N : i);
    return (unsigned)i < (unsigned)N ? i : wrapm(i, N);
}

template <typename FT>
GBO_D FT ldg(const FT* p) { return __ldg(p); }

// eps(FT) in double: the floor of Δτ in the pressure correction (pressure_correction.jl:102-104)
template <typename FT>
GBO_HD double machine_eps() { return sizeof(FT) == 4 ? 1.1920928955078125e-07 : 2.220446049250313e-16; }
// Δt and the projection factors of the three RK3 stages, in FT, as the stage kernels
// read them from device memory: Δτ = FT(Δt c) with c = γ₁ on the first stage and γ + ζ
// (summed in FT) on the others (nonhydrostatic_rk3_substep.jl:34-36); the correction
// uses 1 / max(eps, Δτ) and the CG initial guess pNHS max(eps, Δτ) (pressure_correction.jl:102-104).
enum { DTF_DT = 0, DTF_RDTAU = 1, DTF_SCALE = 4, DTF_N = 8 };
template <typename FT>
GBO_HD void stage_factors(double dt, double c0, double c1, double c2, FT* out) {
    const double c[3] = {c0, c1, c2};
    out[DTF_DT] = FT(dt);
    for (int s = 0; s < 3; ++s) {
        const double tau = (double)FT(dt * c[s]);
        const double e = machine_eps<FT>();
        const FT m = FT(tau > e ? tau : e);
        out[DTF_RDTAU + s] = FT(1) / m;
        out[DTF_SCALE + s] = m;
    }
}

// Accessor for a Center-in-z field.
//
// Tracers of single-precision models on a Bounded z are stored as departures from a
// per-level reference profile `ref` (Nz values, fixed when the tracer is set): a
// stratification b = N² z + b′ held in FP32 would round b′ at the ulp of N² z at
// every stage.  The accessor returns ref[k] + a[i, j, k], the field's value; the
// mirrored halo layer mirrors both, and the deeper layers (zero in the reference)
// stay zero.
template <typename FT>
struct CFld {
    const FT* __restrict__ a;
    int Nx, Ny, Nz, flatz;
    const FT* ref = nullptr;  // reference profile of a departure field (Bounded z only), or null
    // (i, j) any distance outside the domain (tile fills)
    GBO_D FT far(int i, int j, int k) const { return (*this)(wrapt(i, Nx), wrapt(j, Ny), k); }
    GBO_D FT at(size_t off, int k) const {
        const FT x = ldg(a + off);
        return ref ? ldg(ref + k) + x : x;
    }
    // the column at offset c = i + Nx j of the domain, at level k
    GBO_D FT col(size_t c, int k) const {
        if (flatz) return ldg(a + c);
        if (k < -1 || k > Nz) return FT(0);
        k = k < 0 ? 0 : (k >= Nz ? Nz - 1 : k);
        return at(c + (size_t)Nx * Ny * k, k);
    }
    GBO_D FT operator()(int i, int j, int k) const {
        i = wrapi(i, Nx);
        j = wrapi(j, Ny);
        if (flatz) return ldg(a + i + (size_t)Nx * j);
        if (k < -1 || k > Nz) return FT(0);
        k = k < 0 ? 0 : (k >= Nz ? Nz - 1 : k);
        return at(i + (size_t)Nx * (j + (size_t)Ny * k), k);
    }
};

// Accessor for w (Face in z): faces 0..Nz-1 stored, face 0 and Nz are walls.
template <typename FT>
struct WFld {
    const FT* __restrict__ a;
    int Nx, Ny, Nz;
    GBO_D FT far(int i, int j, int k) const { return (*this)(wrapt(i, Nx), wrapt(j, Ny), k); }
    // the column at offset c = i + Nx j of the domain, at face k
    GBO_D FT col(size_t c, int k) const {
        if (k <= 0 || k >= Nz) return FT(0);
        return ldg(a + c + (size_t)Nx * Ny * k);
    }
    GBO_D FT operator()(int i, int j, int k) const {
        if (k <= 0 || k >= Nz) return FT(0);
        i = wrapi(i, Nx);
        j = wrapi(j, Ny);
        return ldg(a + i + (size_t)Nx * (j + (size_t)Ny * k));
    }
};

template <typename FT>
GBO_D CFld<FT> cfld(const FT* a, const GridP<FT>& g, const FT* ref = nullptr) {
    return CFld<FT>{a, g.Nx, g.Ny, g.Nz, g.flatz, g.flatz ? nullptr : ref};
}
template <typename FT>
GBO_D WFld<FT> wfld(const FT* a, const GridP<FT>& g) { return WFld<FT>{a, g.Nx, g.Ny, g.Nz}; }

// Device-side error flags (bit mask) read back by the host after a step.
#define GBO_FLAG_NAN     1u
#define GBO_FLAG_TIMEOUT 2u
