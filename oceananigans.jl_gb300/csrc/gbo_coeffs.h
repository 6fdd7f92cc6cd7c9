// Generated by gen_coefficients.py -- do not edit by hand.
// Uniform finite-volume reconstruction weights (Shu 1998, eq. 2.21) rounded to the
// working precision with the last weight of each stencil = 1 - sum(others) in that
// precision, as Oceananigans' stencil_coefficients does
// (src/Advection/reconstruction_coefficients.jl:58-77).
#pragma once

template <typename FT> struct GboCoeffs;

template <> struct GboCoeffs<double> {
  // WENO{3} (order 5) stencil 0
  static constexpr double weno3_p0[3] = {3.33333333333333315e-01, 8.33333333333333370e-01, -1.66666666666666741e-01};
  // WENO{3} (order 5) stencil 1
  static constexpr double weno3_p1[3] = {-1.66666666666666657e-01, 8.33333333333333370e-01, 3.33333333333333259e-01};
  // WENO{3} (order 5) stencil 2
  static constexpr double weno3_p2[3] = {3.33333333333333315e-01, -1.16666666666666674e+00, 1.83333333333333348e+00};
  static constexpr double weno3_cstar[3] = {2.99999999999999989e-01, 5.99999999999999978e-01, 1.00000000000000006e-01};
  // WENO{2} (order 3) stencil 0
  static constexpr double weno2_p0[2] = {5.00000000000000000e-01, 5.00000000000000000e-01};
  // WENO{2} (order 3) stencil 1
  static constexpr double weno2_p1[2] = {-5.00000000000000000e-01, 1.50000000000000000e+00};
  static constexpr double weno2_cstar[2] = {6.66666666666666630e-01, 3.33333333333333315e-01};
  // Centered(order=4) weights for offsets -2, -1, 0, +1 relative to the face
  static constexpr double c4[4] = {-8.33333333333334814e-02, 5.83333333333333370e-01, 5.83333333333333370e-01, -8.33333333333333287e-02};
  // Centered(order=2) weights for offsets -1, 0
  static constexpr double c2[2] = {5.00000000000000000e-01, 5.00000000000000000e-01};
  // WENO regulariser: the single-precision literal 1e-8 promoted (weno_interpolants.jl:71)
  static constexpr double eps = 9.99999993922529029e-09;
  static constexpr double rk3_gamma1 = 5.33333333333333326e-01;
  static constexpr double rk3_zeta1 = 0.00000000000000000e+00;
  static constexpr double rk3_gamma2 = 4.16666666666666685e-01;
  static constexpr double rk3_zeta2 = -2.83333333333333326e-01;
  static constexpr double rk3_gamma3 = 7.50000000000000000e-01;
  static constexpr double rk3_zeta3 = -4.16666666666666685e-01;
};

template <> struct GboCoeffs<float> {
  // WENO{3} (order 5) stencil 0
  static constexpr float weno3_p0[3] = {3.333333433e-01f, 8.333333135e-01f, -1.666666269e-01f};
  // WENO{3} (order 5) stencil 1
  static constexpr float weno3_p1[3] = {-1.666666716e-01f, 8.333333135e-01f, 3.333333731e-01f};
  // WENO{3} (order 5) stencil 2
  static constexpr float weno3_p2[3] = {3.333333433e-01f, -1.166666627e+00f, 1.833333254e+00f};
  static constexpr float weno3_cstar[3] = {3.000000119e-01f, 6.000000238e-01f, 1.000000015e-01f};
  // WENO{2} (order 3) stencil 0
  static constexpr float weno2_p0[2] = {5.000000000e-01f, 5.000000000e-01f};
  // WENO{2} (order 3) stencil 1
  static constexpr float weno2_p1[2] = {-5.000000000e-01f, 1.500000000e+00f};
  static constexpr float weno2_cstar[2] = {6.666666865e-01f, 3.333333433e-01f};
  // Centered(order=4) weights for offsets -2, -1, 0, +1 relative to the face
  static constexpr float c4[4] = {-8.333325386e-02f, 5.833333135e-01f, 5.833333135e-01f, -8.333333582e-02f};
  // Centered(order=2) weights for offsets -1, 0
  static constexpr float c2[2] = {5.000000000e-01f, 5.000000000e-01f};
  // WENO regulariser: the single-precision literal 1e-8 promoted (weno_interpolants.jl:71)
  static constexpr float eps = 9.999999939e-09f;
  static constexpr float rk3_gamma1 = 5.333333611e-01f;
  static constexpr float rk3_zeta1 = 0.000000000e+00f;
  static constexpr float rk3_gamma2 = 4.166666567e-01f;
  static constexpr float rk3_zeta2 = -2.833333313e-01f;
  static constexpr float rk3_gamma3 = 7.500000000e-01f;
  static constexpr float rk3_zeta3 = -4.166666567e-01f;
};

// Smoothness-indicator coefficients (weno_interpolants.jl:169-174), exact integers
#define GBO_WENO3_BETA0 {10, -31, 11, 25, -19, 4}
#define GBO_WENO3_BETA1 {4, -13, 5, 13, -13, 4}
#define GBO_WENO3_BETA2 {4, -19, 11, 25, -31, 10}
#define GBO_WENO2_BETA0 {1, -2, 1}
#define GBO_WENO2_BETA1 {1, -2, 1}
