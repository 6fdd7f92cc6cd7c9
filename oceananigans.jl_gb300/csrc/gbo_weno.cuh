// gbo_weno.cuh -- WENO5 / WENO3 / centered reconstructions on device.
//
// Z-WENO of order 5 with the buffer hierarchy WENO5 -> WENO3 -> Centered(2)
// used near Bounded walls, as Oceananigans' WENO() builds it
// (src/Advection/weno_reconstruction.jl:107-140):
//   * stencils S_r (left / right biased) ... weno_interpolants.jl:515-562
//   * smoothness β_r with integer coefficients ... weno_interpolants.jl:169-174,196-213;
//     in single precision every stencil is shifted by its centre value before
//     β is formed (weno_interpolants.jl:268-281) to avoid cancellation
//   * τ = |β₀ - β_{N-1}|, α_r = C★_r (1 + (τ/(β_r + ε))²), ω = α/Σα
//     (weno_interpolants.jl:296-328), ε the single-precision literal 1e-8
//   * ψ̂ = Σ ω_r p_r with p_r the order-N reconstruction of stencil r.
// Reconstruction weights come from gbo_coeffs.h (generated, exact rationals).
#pragma once
#include "gbo_common.cuh"

template <typename FT> struct IsF32 { static constexpr bool value = false; };
template <> struct IsF32<float> { static constexpr bool value = true; };

// Division used in the WENO weights.  FP64 keeps IEEE division (the reference's
// CPU semantics, the parity target).  FP32 forms a / b as the reference's GPU backend
// does for its default weight computation (newton_div with BackendOptimizedDivision,
// ext/OceananigansCUDAExt.jl:147,165-171): a times the approximate reciprocal
// rcp.approx.ftz.f32 of b; the normalisation 1 / Σα takes the same reciprocal.
GBO_D float rcp_approx(float b) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(b));
    return r;
}
GBO_D double weno_div(double a, double b) { return a / b; }
GBO_D float weno_div(float a, float b) { return a * rcp_approx(b); }
GBO_D double weno_inv(double b) { return 1.0 / b; }
GBO_D float weno_inv(float b) { return rcp_approx(b); }

template <typename FT>
GBO_D FT beta3(FT p0, FT p1, FT p2, int s) {
    if (IsF32<FT>::value) {
        // shift by the stencil centre; p1 - p1 is exactly +0 for finite values, so the
        // terms in p1 vanish without changing any bit of β
        FT c = p1;
        p0 -= c; p2 -= c;
        p1 = FT(0);
    }
    FT b;
    if (s == 0)
        b = p0 * (FT(10) * p0 + FT(-31) * p1 + FT(11) * p2) + p1 * (FT(25) * p1 + FT(-19) * p2) + p2 * p2 * FT(4);
    else if (s == 1)
        b = p0 * (FT(4) * p0 + FT(-13) * p1 + FT(5) * p2) + p1 * (FT(13) * p1 + FT(-13) * p2) + p2 * p2 * FT(4);
    else
        b = p0 * (FT(4) * p0 + FT(-19) * p1 + FT(11) * p2) + p1 * (FT(25) * p1 + FT(-31) * p2) + p2 * p2 * FT(10);
    return b;
}

// WENO5 inlined at every use (default) or as one out-of-line function (a smaller
// loop body for the instruction cache; measured equal speed on the fused kernel).
#ifndef GBO_WENO_NOINLINE
#define GBO_WENO_NOINLINE 0
#endif
#if GBO_WENO_NOINLINE
#define GBO_WENO_FN __device__ __noinline__
#else
#define GBO_WENO_FN GBO_D
#endif

// WENO5 biased reconstruction at a face from ψ at face offsets -3..+2.
template <typename FT>
GBO_WENO_FN FT weno5v(FT s0, FT s1, FT s2, FT s3, FT s4, FT s5, bool left) {
    using K = GboCoeffs<FT>;
    FT a0, a1, a2, b0, b1, b2, c0, c1, c2;  // stencils P0=(a), P1=(b), P2=(c)
    if (left) {
        a0 = s2; a1 = s3; a2 = s4;
        b0 = s1; b1 = s2; b2 = s3;
        c0 = s0; c1 = s1; c2 = s2;
    } else {
        a0 = s3; a1 = s2; a2 = s1;
        b0 = s4; b1 = s3; b2 = s2;
        c0 = s5; c1 = s4; c2 = s3;
    }
    FT be0 = beta3(a0, a1, a2, 0), be1 = beta3(b0, b1, b2, 1), be2 = beta3(c0, c1, c2, 2);
    FT tau = fabs(be0 - be2);
    FT q0 = weno_div(tau, be0 + K::eps), q1 = weno_div(tau, be1 + K::eps), q2 = weno_div(tau, be2 + K::eps);
    FT al0 = K::weno3_cstar[0] * (FT(1) + q0 * q0);
    FT al1 = K::weno3_cstar[1] * (FT(1) + q1 * q1);
    FT al2 = K::weno3_cstar[2] * (FT(1) + q2 * q2);
    FT inv = weno_inv((al0 + al1) + al2);
    FT p0 = (K::weno3_p0[0] * a0 + K::weno3_p0[1] * a1) + K::weno3_p0[2] * a2;
    FT p1 = (K::weno3_p1[0] * b0 + K::weno3_p1[1] * b1) + K::weno3_p1[2] * b2;
    FT p2 = (K::weno3_p2[0] * c0 + K::weno3_p2[1] * c1) + K::weno3_p2[2] * c2;
    return (al0 * inv) * p0 + (al1 * inv) * p1 + (al2 * inv) * p2;
}
// S[0..5] = ψ at face offsets -3..+2
template <typename FT>
GBO_D FT weno5(const FT S[6], bool left) {
    return weno5v<FT>(S[0], S[1], S[2], S[3], S[4], S[5], left);
}

// Two WENO5 reconstructions at once: (weno5(A, la), weno5(B, lb)).  The generic form
// evaluates them one after the other; the FP32 form below evaluates both in packed FP32
// (FFMA2 / FADD2 / FMUL2, sm_100 and later), component x for A and y for B, with the
// operations of weno5v in the same order (the β of a shifted stencil drops its terms in
// the centre value, which are exactly zero there), so each component equals the scalar
// result up to the contraction of products into FMAs.
template <typename FT>
GBO_D void weno5_2(const FT A[6], bool la, const FT B[6], bool lb, FT& ra, FT& rb) {
    ra = weno5<FT>(A, la);
    rb = weno5<FT>(B, lb);
}

namespace wenopk {
GBO_D float2 f2(float a, float b) { return make_float2(a, b); }
GBO_D float2 add(float2 a, float2 b) { return __fadd2_rn(a, b); }
GBO_D float2 sub(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
GBO_D float2 mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
GBO_D float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
GBO_D float2 sc(float c) { return make_float2(c, c); }
// β of a shifted 3-point stencil (weno_interpolants.jl:169-174, shift :268-281):
// p0, p2 are the outer values minus the centre value
GBO_D float2 beta(float2 p0, float2 p2, float c00, float c02, float c22) {
    // p0 (c00 p0 + c02 p2) + c22 p2 p2, as weno5v's polynomial with its centre terms removed
    return fma2(p0, fma2(sc(c02), p2, mul(sc(c00), p0)), mul(mul(p2, p2), sc(c22)));
}
}  // namespace wenopk

template <>
GBO_D void weno5_2<float>(const float A[6], bool la, const float B[6], bool lb, float& ra, float& rb) {
    using namespace wenopk;
    using K = GboCoeffs<float>;
    // a right-biased reconstruction is the left-biased one of the reversed stencil
    float2 t[6];
#pragma unroll
    for (int j = 0; j < 6; ++j) t[j] = f2(la ? A[j] : A[5 - j], lb ? B[j] : B[5 - j]);
    // stencils P0 = (t2, t3, t4), P1 = (t1, t2, t3), P2 = (t0, t1, t2)
    const float2 be0 = beta(sub(t[2], t[3]), sub(t[4], t[3]), 10.f, 11.f, 4.f);
    const float2 be1 = beta(sub(t[1], t[2]), sub(t[3], t[2]), 4.f, 5.f, 4.f);
    const float2 be2 = beta(sub(t[0], t[1]), sub(t[2], t[1]), 4.f, 11.f, 10.f);
    const float2 d = sub(be0, be2);
    const float2 tau = f2(fabsf(d.x), fabsf(d.y));
    const float2 e0 = add(be0, sc(K::eps)), e1 = add(be1, sc(K::eps)), e2 = add(be2, sc(K::eps));
    const float2 q0 = mul(tau, f2(rcp_approx(e0.x), rcp_approx(e0.y)));
    const float2 q1 = mul(tau, f2(rcp_approx(e1.x), rcp_approx(e1.y)));
    const float2 q2 = mul(tau, f2(rcp_approx(e2.x), rcp_approx(e2.y)));
    const float2 al0 = mul(sc(K::weno3_cstar[0]), fma2(q0, q0, sc(1.f)));
    const float2 al1 = mul(sc(K::weno3_cstar[1]), fma2(q1, q1, sc(1.f)));
    const float2 al2 = mul(sc(K::weno3_cstar[2]), fma2(q2, q2, sc(1.f)));
    const float2 sum = add(add(al0, al1), al2);
    const float2 inv = f2(rcp_approx(sum.x), rcp_approx(sum.y));
    const float2 p0 = fma2(sc(K::weno3_p0[2]), t[4], fma2(sc(K::weno3_p0[1]), t[3], mul(sc(K::weno3_p0[0]), t[2])));
    const float2 p1 = fma2(sc(K::weno3_p1[2]), t[3], fma2(sc(K::weno3_p1[1]), t[2], mul(sc(K::weno3_p1[0]), t[1])));
    const float2 p2 = fma2(sc(K::weno3_p2[2]), t[2], fma2(sc(K::weno3_p2[1]), t[1], mul(sc(K::weno3_p2[0]), t[0])));
    const float2 r = fma2(mul(al2, inv), p2, fma2(mul(al1, inv), p1, mul(mul(al0, inv), p0)));
    ra = r.x;
    rb = r.y;
}

// WENO3 biased reconstruction at a face; S[0..3] = ψ at face offsets -2..+1.
template <typename FT>
GBO_D FT weno3(const FT S[4], bool left) {
    using K = GboCoeffs<FT>;
    FT a0, a1, b0, b1;
    if (left) { a0 = S[1]; a1 = S[2]; b0 = S[0]; b1 = S[1]; }
    else      { a0 = S[2]; a1 = S[1]; b0 = S[3]; b1 = S[2]; }
    FT sa0 = a0, sa1 = a1, sb0 = b0, sb1 = b1;
    if (IsF32<FT>::value) { sa0 -= a1; sa1 = FT(0); sb0 -= b1; sb1 = FT(0); }
    FT be0 = sa0 * (FT(1) * sa0 + FT(-2) * sa1) + sa1 * sa1 * FT(1);
    FT be1 = sb0 * (FT(1) * sb0 + FT(-2) * sb1) + sb1 * sb1 * FT(1);
    FT tau = fabs(be0 - be1);
    FT q0 = weno_div(tau, be0 + K::eps), q1 = weno_div(tau, be1 + K::eps);
    FT al0 = K::weno2_cstar[0] * (FT(1) + q0 * q0);
    FT al1 = K::weno2_cstar[1] * (FT(1) + q1 * q1);
    FT inv = weno_inv(al0 + al1);
    FT p0 = K::weno2_p0[0] * a0 + K::weno2_p0[1] * a1;
    FT p1 = K::weno2_p1[0] * b0 + K::weno2_p1[1] * b1;
    return (al0 * inv) * p0 + (al1 * inv) * p1;
}

template <typename FT>
GBO_D FT cen4(FT q0, FT q1, FT q2, FT q3) {  // offsets -2, -1, 0, +1
    using K = GboCoeffs<FT>;
    return K::c4[0] * q0 + K::c4[1] * q1 + K::c4[2] * q2 + K::c4[3] * q3;
}
template <typename FT>
GBO_D FT cen2(FT qm, FT q0) {  // offsets -1, 0
    using K = GboCoeffs<FT>;
    return K::c2[0] * qm + K::c2[1] * q0;
}

// Buffer-scheme selection in Bounded z (topologically_conditional_interpolation.jl:52-58),
// kr = 1-based level, N = Nz.  Returns 3 (WENO5 / C4), 2 (WENO3) or 1 (C2).
GBO_D int zlev_biased_face(int kr, int N) {
    if (kr >= 4 && kr <= N - 2) return 3;
    if (kr >= 3 && kr <= N - 1) return 2;
    return 1;
}
GBO_D int zlev_biased_center(int kr, int N) {
    if (kr >= 3 && kr <= N - 2) return 3;
    if (kr >= 2 && kr <= N - 1) return 2;
    return 1;
}
GBO_D int zlev_symm_face(int kr, int N) { return (kr >= 4 && kr <= N - 2) ? 3 : 1; }
GBO_D int zlev_symm_center(int kr, int N) { return (kr >= 3 && kr <= N - 2) ? 3 : 1; }

// Biased reconstruction with level selection; q(o) gives ψ at face offset o.
template <typename FT, class Q>
GBO_D FT biased(Q q, bool left, int level) {
    if (level == 3) {
        FT S[6];
#pragma unroll
        for (int o = -3; o <= 2; ++o) S[o + 3] = q(o);
        return weno5<FT>(S, left);
    }
    if (level == 2) {
        FT S[4];
#pragma unroll
        for (int o = -2; o <= 1; ++o) S[o + 2] = q(o);
        return weno3<FT>(S, left);
    }
    return cen2<FT>(q(-1), q(0));
}
template <typename FT, class Q>
GBO_D FT symm(Q q, int level) {
    if (level == 3) return cen4<FT>(q(-2), q(-1), q(0), q(1));
    return cen2<FT>(q(-1), q(0));
}
