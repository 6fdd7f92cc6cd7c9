// gbo_dynamic.cuh -- DynamicSmagorinsky (turbulence_closure_implementations/Smagorinskys/
// dynamic_coefficient.jl, scale_invariant_operators.jl:94-188) with either averaging.
//
// The test filter ⟨f⟩ = (6 f + the six face neighbours) / 12 (scale_invariant_operators.jl:
// 94-104) of products of interpolated strains makes LM and MM wide stencils; the tiled
// kernels at the end of this file (k_dyn_sigma_tiled, k_lm_mm_tiled) stage a block's
// velocities, filtered velocities and centre products in shared memory and evaluate them
// once per point (see there).
//
// Averaged over x and y (averaging = (1, 2)), per state update:
//   k_dyn_sigma_tiled  Σ = √(ΣᵢⱼΣᵢⱼ) of the resolved strain and Σ̄ = √(Σ̄ᵢⱼΣ̄ᵢⱼ) of the strain
//                      of the test-filtered velocities (_compute_Σ!, _compute_Σ̄!);
//   k_lm_mm_tiled      Lᵢⱼ Mᵢⱼ and Mᵢⱼ Mᵢⱼ per cell (LM_and_MM);
//   k_dyn_tile_sums    their FP64 sums per 32 × 8 tile of a level;
//   k_dyn_coef         per level: 𝒥ᴸᴹ, 𝒥ᴹᴹ = the x-y means of LM and MM
//                      (Field(Average(…, dims=(1, 2)))), c² = max(𝒥ᴸᴹ, minimum_numerator) / 𝒥ᴹᴹ,
//                      or 0 where 𝒥ᴹᴹ ≤ 0 (square_smagorinsky_coefficient);
//   k_smagorinsky      νₑ = c² Δᶠ² √(2Σ²) with the level's c² (_compute_smagorinsky_viscosity!).
//
// LagrangianAveraging (dynamic_coefficient.jl:364-487): 𝒥ᴸᴹ, 𝒥ᴹᴹ are fields relaxed along
// trajectories once per time step, after the step's last projection
// (step_closure_prognostics!):
//   k_dyn_sigma_tiled  Σ, Σ̄ of the velocities as they are at that point (see LagC);
//   k_lm_mm_tiled      LM, MM per cell, written over 𝒥 after 𝒥 was copied to 𝒥⁻;
//   k_lag_step         T = 1.5 Δᶠ (𝒥ᴸᴹ⁻𝒥ᴹᴹ⁻)^(-1/8), ε = τ / (1 + τ) with τ = Δt / T, the
//                      departure point x - clamp(u Δt, ±Δ), 𝒥 = ε (LM, MM) + (1 - ε)
//                      trilinear(𝒥⁻ at the departure point) (_lagrangian_average_LM_MM!);
//   k_lag_tick         previous_compute_time = clock.time (the FP64 clock of the update);
// and per state update k_smagorinsky with the cell's c² = max(𝒥ᴸᴹ, min) / 𝒥ᴹᴹ.  At set!
// with velocities (initialize_closure_fields!, :407-437) both fields take the domain means
// of LM and MM (k_lm_mm_tiled, k_lag_sum, k_lag_init_mean, k_lag_fill).
//
// The tiled kernels are instantiated in gbo_dynamic_f32.cu / _f64.cu and launched through
// the dyn_launch_* functions.
//
// The halo conventions are the stored fields' (CFld / WFld): one mirrored layer below and
// above the domain for Center fields and Σ, Σ̄ (fill_halo_regions_flux.jl:14-15), zero
// beyond it, zero for w on and beyond the walls.
#pragma once
#include "gbo_kernels.cuh"
#include "gbo_fused.cuh"  // 16-byte copies and the halo levels of the tile fills

namespace dyn {
constexpr int TX = 32, TY = 8;
constexpr int COEF_THREADS = 256;
}  // namespace dyn

// The three velocity accessors the tiled kernels stage their tiles through.
template <class CU, class CW>
struct Vel {
    CU u, v;
    CW w;
};
template <typename FT>
using PlainVel = Vel<CFld<FT>, WFld<FT>>;

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
    double xc0, yc0;                      // the first centres x0 + 0.5 Δx, y0 + 0.5 Δy (FT values)
    double rdx, rdy, rdz1;                // 1 / Δx, 1 / Δy, 1 / Δzᶜ of the first cell (of the FT spacings)
    const double* __restrict__ zc;        // z of the Nz cell centres (FT values, stored as FP64)
    double dz1;                           // Δzᶜ of the first cell (regular z; FT value)
    int stretched;
    const double* clock;                  // LAG_* slots
    const double* dtp;                    // Δt of this step (FP64)
};

// Julia's max / min propagate NaN
template <typename T>
GBO_D T jl_max(T a, T b) { return (isnan(a) || isnan(b)) ? a + b : (a > b ? a : b); }
GBO_D double jl_clamp(double x, double lo, double hi) { return x > hi ? hi : (x < lo ? lo : x); }

// interpolator (Utils/interpolation.jl:34-42): i⁻ = unsafe_trunc(Int, fi), ξ = mod(fi, 1)
// on a 1-based fractional index; returns the 0-based lower index.  The remainder of
// fi / 1 is fi - trunc(fi): both are exact (the fractional bits of fi are representable),
// so this is fmod(fi, 1) without its general-divisor reduction
GBO_D int lag_interpolator(double fi, double& xi) {
    const int lo = (int)fi;
    const double r = fi - trunc(fi);
    xi = (r == 0.0) ? 0.0 : (r < 0.0 ? r + 1.0 : r);
    return lo - 1;
}
GBO_D int lag_interpolator(float fi, float& xi) {
    const int lo = (int)fi;
    const float r = fi - truncf(fi);
    xi = (r == 0.f) ? 0.f : (r < 0.f ? r + 1.f : r);
    return lo - 1;
}

// fractional z index of a point (Fields/interpolate.jl:44-58,166-201): regular spacing by
// division; explicit faces by the bracketing interval of the cell centres (the reference's
// binary search), extrapolated linearly beyond the first and last centres
template <typename FT>
GBO_D double lag_frac_z(const LagP<FT>& P, double z) {
    const int Nz = P.g.Nz;
    if (!P.stretched) return (z - P.zc[0]) * P.rdz1 + 1.0;
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

// _interpolate (Utils/interpolation.jl:58-72): the eight weights in the reference's order,
// ϕ = (1 - ξ or ξ) (1 - η or η) (1 - ζ or ζ) left to right.  ξ, η have the type of the
// fractional x and y indices (FT) and ζ that of the z index (ZT); the product of the x and
// y factors is taken in FT, then promoted with ζ, as the reference's promotion does.
template <typename FT, typename ZT>
GBO_D ZT lag_trilinear(const FT* __restrict__ a, const GridP<FT>& g, int i0, int j0, int k0, FT x, FT y, ZT z) {
    const int i1 = i0 + 1, j1 = j0 + 1, k1 = k0 + 1;
    const FT ax = FT(1) - x, ay = FT(1) - y;
    const ZT az = ZT(1) - z;
    return ZT(ax * ay) * az * ZT(lag_prev(a, g, i0, j0, k0)) + ZT(ax * ay) * z * ZT(lag_prev(a, g, i0, j0, k1)) +
           ZT(ax * y) * az * ZT(lag_prev(a, g, i0, j1, k0)) + ZT(ax * y) * z * ZT(lag_prev(a, g, i0, j1, k1)) +
           ZT(x * ay) * az * ZT(lag_prev(a, g, i1, j0, k0)) + ZT(x * ay) * z * ZT(lag_prev(a, g, i1, j0, k1)) +
           ZT(x * y) * az * ZT(lag_prev(a, g, i1, j1, k0)) + ZT(x * y) * z * ZT(lag_prev(a, g, i1, j1, k1));
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
// promotion does; the fields are stored in FT.  FP64 division is the costly operation
// here, so ε = τ / (1 + τ) with τ = Δt / T is formed as Δt / (T + Δt) and the fractional
// indices multiply by the reciprocal spacings (both equal to the reference's forms up to
// FP64 rounding).
// LM and MM of this step are read from jlm / jmm (k_lm_mm_tiled wrote them there after 𝒥
// was copied to 𝒥⁻); each thread reads and then overwrites its own cell only.
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
    const double Td = (double)Tm;
    // the reference's form where T is 0, infinite or NaN (τ infinite or NaN)
    const double eps = (Td > 0.0 && Td < INFINITY) ? dt / (Td + dt) : (dt / Td) / (1 + dt / Td);
    // departure point: the node minus the displacement by the cell's own u[i, j, k],
    // v[i, j, k], w[i, j, k] over Δt, each clamped to one cell width.  The nodes and
    // spacings are the grid's (FT; zc and the first centres rounded to FT on the host), the
    // displaced point FP64; the fractional x and y indices are converted to FT
    // (fractional_x_index, Fields/interpolate.jl:60-66), the z index keeps FP64 on a
    // regular grid (the type of z, :190-194) and is converted to FT on a stretched one (:196-201)
    const double x = (double)FT(P.x0 + (i + 0.5) * P.dx), y = (double)FT(P.y0 + (j + 0.5) * P.dy), z = P.zc[k];
    const double ddx = jl_clamp((double)P.vel.u.in(i, j, k) * dt, -(double)g.dx, (double)g.dx);
    const double ddy = jl_clamp((double)P.vel.v.in(i, j, k) * dt, -(double)g.dy, (double)g.dy);
    const double ddz = jl_clamp((double)P.vel.w.in(i, j, k) * dt, -(double)dzk, (double)dzk);
    const FT fi = FT((x - ddx - P.xc0) * P.rdx) + FT(1);
    const FT fj = FT((y - ddy - P.yc0) * P.rdy) + FT(1);
    FT xi, yi;
    const int i0 = lag_interpolator(fi, xi), j0 = lag_interpolator(fj, yi);
    double imm, ilm;
    if (!P.stretched) {
        double zi;
        const int k0 = lag_interpolator(lag_frac_z(P, z - ddz), zi);
        imm = lag_trilinear<FT, double>(P.jmm_prev, g, i0, j0, k0, xi, yi, zi);
        ilm = lag_trilinear<FT, double>(P.jlm_prev, g, i0, j0, k0, xi, yi, zi);
    } else {
        FT zi;
        const int k0 = lag_interpolator(FT(lag_frac_z(P, z - ddz)), zi);
        imm = (double)lag_trilinear<FT, FT>(P.jmm_prev, g, i0, j0, k0, xi, yi, zi);
        ilm = (double)lag_trilinear<FT, FT>(P.jlm_prev, g, i0, j0, k0, xi, yi, zi);
    }
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

// Launchers of the stencil kernels (the tiled forms below), instantiated for float and
// double in gbo_dynamic_f32.cu / _f64.cu (their own translation units: the stencils are large).
template <typename FT>
void dyn_launch_sigma(cudaStream_t st, const GridP<FT>& g, const PlainVel<FT>& vel, FT* sig, FT* sigb);
template <typename FT>
void dyn_launch_sigma(cudaStream_t st, const GridP<FT>& g, const LagVel<FT>& vel, FT* sig, FT* sigb);
template <typename FT>
void dyn_launch_lm(cudaStream_t st, const GridP<FT>& g, const PlainVel<FT>& vel, const FT* sig, const FT* sigb, FT* lm,
                   FT* mm);
template <typename FT>
void dyn_launch_lm(cudaStream_t st, const GridP<FT>& g, const LagVel<FT>& vel, const FT* sig, const FT* sigb, FT* lm,
                   FT* mm);
template <typename FT>
cudaError_t dyn_set_smem();

// ---------------------------------------------------------------------------
// Tiled Σ, Σ̄ and LM, MM.  LM_and_MM evaluates the test filter of products of
// interpolated strains: evaluated point by point, every cell would recompute the
// filtered velocities and the centre products of its neighbours many times over.  A
// 32 × 4 × 2 block instead stages the
// velocities of its cells and two points around them (through the same accessors, so
// every halo rule, the predictor halos of the Lagrangian update included, is the
// accessor's), forms the filtered velocities and the twelve centre products of the
// Leonard and model tensors once per point of the tile and one point around it, and then
// every cell evaluates LM_and_MM's expressions (the reference's order of operations, each
// strain as StrainT forms it) from those values.
// Positions beyond one point outside the domain feed only cells outside it; their
// indices are clamped so that every read stays in bounds.
// ---------------------------------------------------------------------------
namespace dtile {
constexpr int TX = 32, TY = 4, KT = 2, NT = TX * TY * KT;
// velocities: -2 .. +1 beyond the tile in y and z; in x from -4 (rows of 16-byte chunks
// that start on a multiple of four columns) to TX + 3
constexpr int RHX = 4;
constexpr int RX = TX + 2 * RHX, RY = TY + 4, RZ = KT + 4, RS = RX * RY * RZ;
constexpr int QX = TX + 2, QY = TY + 2, QZ = KT + 2, QS = QX * QY * QZ;  // filtered velocities, products: -1 .. +1
GBO_D int ri(int x, int y, int z) { return ((z + 2) * RY + (y + 2)) * RX + (x + RHX); }
GBO_D int qi(int x, int y, int z) { return ((z + 1) * QY + (y + 1)) * QX + (x + 1); }
enum { Q11 = 0, Q22, Q33, Q12, Q13, Q23, M11, M22, M33, M12, M13, M23, NQ };
template <typename FT>
struct __align__(16) SmemS {
    FT u[RS], v[RS], w[RS];
    FT fu[QS], fv[QS], fw[QS];
};
template <typename FT>
struct SmemL : SmemS<FT> {
    FT q[NQ][QS];
};
// a domain index for a tile position: at most one point beyond the domain is a real halo
// point; farther ones only feed cells outside the domain
GBO_D int clamp_far(int i, int n) { return i > n + 1 ? n + 1 : i; }
}  // namespace dtile

// The first of the V values of a 16-byte chunk of a row at (gi, gj, gk) (gi a multiple of
// V, Nx a multiple of V: the chunk lies in one period), read through each accessor's
// halo rules; zero: the accessor's value there is zero (the copy writes zeros).
template <typename FT>
GBO_D const FT* chunk_src(const CFld<FT>& f, int gi, int gj, int gk, bool& zero) {
    const int zc = fused::zsrc_c(gk, f.Nz, f.flatz);
    zero = zc < 0;
    return f.a + wrapt(gi, f.Nx) + (size_t)f.Nx * (wrapt(gj, f.Ny) + (size_t)f.Ny * (zc < 0 ? 0 : zc));
}
template <typename FT>
GBO_D const FT* chunk_src(const WFld<FT>& f, int gi, int gj, int gk, bool& zero) {
    zero = gk <= 0 || gk >= f.Nz;
    return f.a + wrapt(gi, f.Nx) + (size_t)f.Nx * (wrapt(gj, f.Ny) + (size_t)f.Ny * (zero ? 0 : gk));
}
template <typename FT>
GBO_D const FT* chunk_src(const LagC<FT>& f, int gi, int gj, int gk, bool& zero) {
    const bool in = (unsigned)gi < (unsigned)f.in.Nx && (unsigned)gj < (unsigned)f.in.Ny && (unsigned)gk < (unsigned)f.in.Nz;
    return in ? chunk_src(f.in, gi, gj, gk, zero) : chunk_src(f.halo, gi, gj, gk, zero);
}
template <typename FT>
GBO_D const FT* chunk_src(const LagW<FT>& f, int gi, int gj, int gk, bool& zero) {
    const bool in = (unsigned)gi < (unsigned)f.in.Nx && (unsigned)gj < (unsigned)f.in.Ny;
    return in ? chunk_src(f.in, gi, gj, gk, zero) : chunk_src(f.halo, gi, gj, gk, zero);
}
// whether an accessor's rows can be copied in 16-byte chunks: aligned storage, no
// reference profile to add
template <typename FT>
GBO_D bool chunk_ok(const CFld<FT>& f) { return f.ref == nullptr && ((size_t)f.a & 15) == 0; }
template <typename FT>
GBO_D bool chunk_ok(const WFld<FT>& f) { return ((size_t)f.a & 15) == 0; }
template <typename FT>
GBO_D bool chunk_ok(const LagC<FT>& f) { return chunk_ok(f.in) && chunk_ok(f.halo); }
template <typename FT>
GBO_D bool chunk_ok(const LagW<FT>& f) { return chunk_ok(f.in) && chunk_ok(f.halo); }

// stage u, v, w of the tile and two points around it (in x four: whole chunks), then the
// filtered velocities over the tile and one point around it
template <typename FT, class V>
GBO_D void dtile_stage(dtile::SmemS<FT>& s, const GridP<FT>& g, const V& vel, int i0, int j0, int k0, int tid) {
    using namespace dtile;
    constexpr int CW = fused::VW<FT>, CR = RX / CW;
    const bool vec = g.Nx % CW == 0 && chunk_ok(vel.u) && chunk_ok(vel.v) && chunk_ok(vel.w);
    if (vec) {
        for (int e = tid; e < CR * RY * RZ; e += NT) {
            const int gi = i0 + (e % CR) * CW - RHX, gj = j0 + (e / CR) % RY - 2, gk = k0 + e / (CR * RY) - 2;
            bool zu, zv, zw;
            const FT* pu = chunk_src(vel.u, gi, gj, gk, zu);
            const FT* pv = chunk_src(vel.v, gi, gj, gk, zv);
            const FT* pw = chunk_src(vel.w, gi, gj, gk, zw);
            fused::cp_async16(&s.u[e * CW], pu, zu);
            fused::cp_async16(&s.v[e * CW], pv, zv);
            fused::cp_async16(&s.w[e * CW], pw, zw);
        }
        fused::cp_async_commit();
        fused::cp_async_wait_all();
    } else {
        for (int e = tid; e < RS; e += NT) {
            const int x = e % RX - RHX, y = (e / RX) % RY - 2, z = e / (RX * RY) - 2;
            const int gi = clamp_far(i0 + x, g.Nx), gj = clamp_far(j0 + y, g.Ny), gk = k0 + z;
            s.u[e] = vel.u(gi, gj, gk);
            s.v[e] = vel.v(gi, gj, gk);
            s.w[e] = vel.w(gi, gj, gk);
        }
    }
    __syncthreads();
    // the test filter ⟨f⟩ = (6 f + the six face neighbours) / 12, the neighbours in the order x, y, z
    auto tf = [&](const FT* a, int x, int y, int z) {
        return (FT(6) * a[ri(x, y, z)] + a[ri(x + 1, y, z)] + a[ri(x - 1, y, z)] + a[ri(x, y + 1, z)] + a[ri(x, y - 1, z)] +
                a[ri(x, y, z + 1)] + a[ri(x, y, z - 1)]) / FT(12);
    };
    for (int e = tid; e < QS; e += NT) {
        const int x = e % QX - 1, y = (e / QX) % QY - 1, z = e / (QX * QY) - 1;
        s.fu[e] = tf(s.u, x, y, z);
        s.fv[e] = tf(s.v, x, y, z);
        s.fw[e] = tf(s.w, x, y, z);
    }
}

// ΣᵢⱼΣᵢⱼ of the strain of velocities held at tile positions (index function ix), at cell
// (x, y, z) of level k: Σ₁₁² + Σ₂₂² + Σ₃₃² + 2 ℑxy(Σ₁₂²) + 2 ℑxz(Σ₁₃²) + 2 ℑyz(Σ₂₃²)
template <typename FT, class IX>
GBO_D FT dtile_strain_sq(const FT* u, const FT* v, const FT* w, IX ix, const GridP<FT>& g, const Met<FT>& M, int x,
                         int y, int z, int k0) {
    auto sq = [](FT a) { return a * a; };
    const int k = k0 + z;
    const FT s11 = (u[ix(x + 1, y, z)] - u[ix(x, y, z)]) * g.rdx;
    const FT s22 = (v[ix(x, y + 1, z)] - v[ix(x, y, z)]) * g.rdy;
    const FT s33 = (w[ix(x, y, z + 1)] - w[ix(x, y, z)]) * M.rdzc(k);
    const FT tr = s11 * s11 + s22 * s22 + s33 * s33;
    auto S12 = [&](int a, int b) {
        return FT(0.5) * ((u[ix(a, b, z)] - u[ix(a, b - 1, z)]) * g.rdy + (v[ix(a, b, z)] - v[ix(a - 1, b, z)]) * g.rdx);
    };
    auto S13 = [&](int a, int c) {
        return FT(0.5) * ((u[ix(a, y, c)] - u[ix(a, y, c - 1)]) * M.rdzf(k0 + c) + (w[ix(a, y, c)] - w[ix(a - 1, y, c)]) * g.rdx);
    };
    auto S23 = [&](int b, int c) {
        return FT(0.5) * ((v[ix(x, b, c)] - v[ix(x, b, c - 1)]) * M.rdzf(k0 + c) + (w[ix(x, b, c)] - w[ix(x, b - 1, c)]) * g.rdy);
    };
    const FT ixy = FT(0.5) * (FT(0.5) * (sq(S12(x, y)) + sq(S12(x + 1, y))) + FT(0.5) * (sq(S12(x, y + 1)) + sq(S12(x + 1, y + 1))));
    const FT ixz = FT(0.5) * (FT(0.5) * (sq(S13(x, z)) + sq(S13(x + 1, z))) + FT(0.5) * (sq(S13(x, z + 1)) + sq(S13(x + 1, z + 1))));
    const FT iyz = FT(0.5) * (FT(0.5) * (sq(S23(y, z)) + sq(S23(y + 1, z))) + FT(0.5) * (sq(S23(y, z + 1)) + sq(S23(y + 1, z + 1))));
    return tr + FT(2) * ixy + FT(2) * ixz + FT(2) * iyz;
}

// Σ = √(ΣᵢⱼΣᵢⱼ) and Σ̄ = √(Σ̄ᵢⱼΣ̄ᵢⱼ) of every cell (_compute_Σ!, _compute_Σ̄!)
template <typename FT, class V>
__global__ void __launch_bounds__(dtile::NT) k_dyn_sigma_tiled(GridP<FT> g, V vel, FT* __restrict__ sig,
                                                                FT* __restrict__ sigb) {
    using namespace dtile;
    extern __shared__ __align__(16) unsigned char dyn_smem[];
    SmemS<FT>& s = *reinterpret_cast<SmemS<FT>*>(dyn_smem);
    const int tid = threadIdx.x + TX * (threadIdx.y + TY * threadIdx.z);
    const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY, k0 = blockIdx.z * KT;
    dtile_stage<FT>(s, g, vel, i0, j0, k0, tid);
    __syncthreads();
    const int x = threadIdx.x, y = threadIdx.y, z = threadIdx.z;
    const int i = i0 + x, j = j0 + y, k = k0 + z;
    if (i >= g.Nx || j >= g.Ny || k >= g.Nz) return;
    Met<FT> M(g);
    const size_t idx = i + (size_t)g.Nx * (j + (size_t)g.Ny * k);
    sig[idx] = sqrt(dtile_strain_sq<FT>(s.u, s.v, s.w, ri, g, M, x, y, z, k0));
    sigb[idx] = sqrt(dtile_strain_sq<FT>(s.fu, s.fv, s.fw, qi, g, M, x, y, z, k0));
}

// LM and MM of every cell (LM_and_MM, dynamic_coefficient.jl:254-276) into lm, mm
template <typename FT, class V>
__global__ void __launch_bounds__(dtile::NT) k_lm_mm_tiled(GridP<FT> g, V vel, const FT* __restrict__ sig,
                                                            const FT* __restrict__ sigb, FT* __restrict__ lm,
                                                            FT* __restrict__ mm) {
    using namespace dtile;
    extern __shared__ __align__(16) unsigned char dyn_smem[];
    SmemL<FT>& s = *reinterpret_cast<SmemL<FT>*>(dyn_smem);
    const int tid = threadIdx.x + TX * (threadIdx.y + TY * threadIdx.z);
    const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY, k0 = blockIdx.z * KT;
    dtile_stage<FT>(s, g, vel, i0, j0, k0, tid);
    Met<FT> M(g);
    const CFld<FT> sg = cfld(sig, g);
    const FT h = FT(0.5);
    auto sq = [](FT a) { return a * a; };
    const FT* U = s.u;
    const FT* Vv = s.v;
    const FT* W = s.w;
    // the centre products of the tile and one point around it, each formed once
    for (int e = tid; e < QS; e += NT) {
        const int a = e % QX - 1, b = (e / QX) % QY - 1, c = e / (QX * QY) - 1;
        const int gk = k0 + c;
        const FT ua = U[ri(a, b, c)], ua1 = U[ri(a + 1, b, c)];
        const FT vb = Vv[ri(a, b, c)], vb1 = Vv[ri(a, b + 1, c)];
        const FT wc = W[ri(a, b, c)], wc1 = W[ri(a, b, c + 1)];
        s.q[Q11][e] = h * (sq(ua) + sq(ua1));
        s.q[Q22][e] = h * (sq(vb) + sq(vb1));
        s.q[Q33][e] = h * (sq(wc) + sq(wc1));
        const FT ixu = h * (ua + ua1), iyv = h * (vb + vb1), izw = h * (wc + wc1);
        s.q[Q12][e] = ixu * iyv;
        s.q[Q13][e] = ixu * izw;
        s.q[Q23][e] = iyv * izw;
        const FT sgv = sg(dtile::clamp_far(i0 + a, g.Nx), dtile::clamp_far(j0 + b, g.Ny), gk);
        s.q[M11][e] = sgv * ((ua1 - ua) * g.rdx);
        s.q[M22][e] = sgv * ((vb1 - vb) * g.rdy);
        s.q[M33][e] = sgv * ((wc1 - wc) * M.rdzc(gk));
        auto S12 = [&](int p, int r) {
            return FT(0.5) * ((U[ri(p, r, c)] - U[ri(p, r - 1, c)]) * g.rdy + (Vv[ri(p, r, c)] - Vv[ri(p - 1, r, c)]) * g.rdx);
        };
        auto S13 = [&](int p, int t) {
            return FT(0.5) * ((U[ri(p, b, t)] - U[ri(p, b, t - 1)]) * M.rdzf(k0 + t) + (W[ri(p, b, t)] - W[ri(p - 1, b, t)]) * g.rdx);
        };
        auto S23 = [&](int r, int t) {
            return FT(0.5) * ((Vv[ri(a, r, t)] - Vv[ri(a, r, t - 1)]) * M.rdzf(k0 + t) + (W[ri(a, r, t)] - W[ri(a, r - 1, t)]) * g.rdy);
        };
        s.q[M12][e] = sgv * (h * (h * (S12(a, b) + S12(a + 1, b)) + h * (S12(a, b + 1) + S12(a + 1, b + 1))));
        s.q[M13][e] = sgv * (h * (h * (S13(a, c) + S13(a + 1, c)) + h * (S13(a, c + 1) + S13(a + 1, c + 1))));
        s.q[M23][e] = sgv * (h * (h * (S23(b, c) + S23(b + 1, c)) + h * (S23(b, c + 1) + S23(b + 1, c + 1))));
    }
    __syncthreads();
    const int x = threadIdx.x, y = threadIdx.y, z = threadIdx.z;
    const int i = i0 + x, j = j0 + y, k = k0 + z;
    if (i >= g.Nx || j >= g.Ny || k >= g.Nz) return;
    auto TF = [&](int qn) {
        const FT* a = s.q[qn];
        return (FT(6) * a[qi(x, y, z)] + a[qi(x + 1, y, z)] + a[qi(x - 1, y, z)] + a[qi(x, y + 1, z)] + a[qi(x, y - 1, z)] +
                a[qi(x, y, z + 1)] + a[qi(x, y, z - 1)]) / FT(12);
    };
    const FT* FU = s.fu;
    const FT* FV = s.fv;
    const FT* FW = s.fw;
    const FT fu0 = FU[qi(x, y, z)], fu1 = FU[qi(x + 1, y, z)];
    const FT fv0 = FV[qi(x, y, z)], fv1 = FV[qi(x, y + 1, z)];
    const FT fw0 = FW[qi(x, y, z)], fw1 = FW[qi(x, y, z + 1)];
    const FT ixfu = h * (fu0 + fu1), iyfv = h * (fv0 + fv1), izfw = h * (fw0 + fw1);
    const FT L11 = TF(Q11) - h * (sq(fu0) + sq(fu1));
    const FT L22 = TF(Q22) - h * (sq(fv0) + sq(fv1));
    const FT L33 = TF(Q33) - h * (sq(fw0) + sq(fw1));
    const FT L12 = TF(Q12) - ixfu * iyfv;
    const FT L13 = TF(Q13) - ixfu * izfw;
    const FT L23 = TF(Q23) - iyfv * izfw;
    // the strain of the filtered velocities at the cell and its edges
    auto SB12 = [&](int p, int r) {
        return FT(0.5) * ((FU[qi(p, r, z)] - FU[qi(p, r - 1, z)]) * g.rdy + (FV[qi(p, r, z)] - FV[qi(p - 1, r, z)]) * g.rdx);
    };
    auto SB13 = [&](int p, int t) {
        return FT(0.5) * ((FU[qi(p, y, t)] - FU[qi(p, y, t - 1)]) * M.rdzf(k0 + t) + (FW[qi(p, y, t)] - FW[qi(p - 1, y, t)]) * g.rdx);
    };
    auto SB23 = [&](int r, int t) {
        return FT(0.5) * ((FV[qi(x, r, t)] - FV[qi(x, r, t - 1)]) * M.rdzf(k0 + t) + (FW[qi(x, r, t)] - FW[qi(x, r - 1, t)]) * g.rdy);
    };
    const size_t idx = i + (size_t)g.Nx * (j + (size_t)g.Ny * k);
    const FT sbar = __ldg(sigb + idx);
    const FT bb11 = sbar * ((fu1 - fu0) * g.rdx);
    const FT bb22 = sbar * ((fv1 - fv0) * g.rdy);
    const FT bb33 = sbar * ((fw1 - fw0) * M.rdzc(k));
    const FT bb12 = sbar * (h * (h * (SB12(x, y) + SB12(x + 1, y)) + h * (SB12(x, y + 1) + SB12(x + 1, y + 1))));
    const FT bb13 = sbar * (h * (h * (SB13(x, z) + SB13(x + 1, z)) + h * (SB13(x, z + 1) + SB13(x + 1, z + 1))));
    const FT bb23 = sbar * (h * (h * (SB23(y, z) + SB23(y + 1, z)) + h * (SB23(y, z + 1) + SB23(y + 1, z + 1))));
    const FT Df = cbrt(g.dx * g.dy * M.dzc(k));
    const FT f2 = FT(2) * (Df * Df);
    const FT m11 = f2 * (TF(M11) - FT(4) * bb11);
    const FT m22 = f2 * (TF(M22) - FT(4) * bb22);
    const FT m33 = f2 * (TF(M33) - FT(4) * bb33);
    const FT m12 = f2 * (TF(M12) - FT(4) * bb12);
    const FT m13 = f2 * (TF(M13) - FT(4) * bb13);
    const FT m23 = f2 * (TF(M23) - FT(4) * bb23);
    lm[idx] = L11 * m11 + L22 * m22 + L33 * m33 + FT(2) * L12 * m12 + FT(2) * L13 * m13 + FT(2) * L23 * m23;
    mm[idx] = m11 * m11 + m22 * m22 + m33 * m33 + FT(2) * m12 * m12 + FT(2) * m13 * m13 + FT(2) * m23 * m23;
}

// The per-level sums of the per-cell LM, MM arrays: a 32 × 8 block per tile of a level,
// each warp's row summed by a shuffle tree in FP64, the rows in order; k_dyn_coef sums the
// tiles of a level in order (a fixed order, so the mean is reproducible)
template <typename FT>
__global__ void __launch_bounds__(dyn::TX * dyn::TY) k_dyn_tile_sums(const FT* __restrict__ lmv, const FT* __restrict__ mmv,
                                                                     int Nx, int Ny, double* __restrict__ part) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    double lm = 0.0, mm = 0.0;
    if (i < Nx && j < Ny) {
        const size_t idx = i + (size_t)Nx * (j + (size_t)Ny * k);
        lm = (double)lmv[idx];
        mm = (double)mmv[idx];
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
