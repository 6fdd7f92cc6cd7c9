// gbo_cg.cuh -- conjugate-gradient Poisson solver kernels for an immersed grid
// (src/Solvers/conjugate_gradient_poisson_solver.jl:38-211;
//  src/Solvers/conjugate_gradient_solver.jl:177-284).
//
// The iteration runs without the host: every scalar (ρ, p·q, the active-cell sums
// of the gauge, ‖V⁻¹r‖, the iteration count and the stop flag) lives in a small
// FP64 array on the device.  k_cg_begin and k_cg_check evaluate the stopping rule
// of `iterating` (conjugate_gradient_solver.jl:278-283) on the device and, inside a
// CUDA graph, drive a conditional WHILE node with cudaGraphSetConditional, so a
// whole time step with three CG solves is one graph launch.  Dot products and
// norms accumulate in FP64 (warp shuffles, one atomic per block).
#pragma once
#include "gbo_tendency.cuh"

// scalar slots
enum {
    CG_RHO0 = 0, CG_RHO1,  // ρ = z·r of even / odd iterations
    CG_PQ,                 // p·q
    CG_SX, CG_SR,          // Σx and Σr over active cells (zero-mean gauge)
    CG_NORM2,              // ‖V⁻¹r‖² of the current residual
    CG_NACT,               // number of active cells
    CG_IT,                 // iterations of the current solve
    CG_TOL,                // max(reltol ‖V⁻¹r₀‖, abstol)
    CG_CONT,               // 1 while iterating
    CG_FAIL,               // set when a solve stops at maxiter above tolerance (sticky)
    CG_NORM,               // ‖V⁻¹r‖ at the last check
    CG_SOLVES, CG_ITERS,   // running totals (instrumentation)
    CG_NSLOTS
};

// z-slices per launch of the 3-D CG kernels: blocks march over k so that each
// kernel issues a few thousand block reductions, not one per (tile, level)
constexpr int CG_ZSLICES = 8;

GBO_D double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
// block-reduce one or two doubles and add them to device scalars
GBO_D void block_add(double a, double* da, double b = 0.0, double* db = nullptr) {
    __shared__ double sa[32], sb[32];
    int lane = (threadIdx.x + threadIdx.y * blockDim.x) & 31;
    int wid = (threadIdx.x + threadIdx.y * blockDim.x) >> 5;
    int nw = (blockDim.x * blockDim.y + 31) >> 5;
    a = warp_sum(a);
    b = warp_sum(b);
    if (lane == 0) { sa[wid] = a; sb[wid] = b; }
    __syncthreads();
    if (wid == 0) {
        a = lane < nw ? sa[lane] : 0.0;
        b = lane < nw ? sb[lane] : 0.0;
        a = warp_sum(a);
        b = warp_sum(b);
        if (lane == 0) {
            atomicAdd(da, a);
            if (db) atomicAdd(db, b);
        }
    }
}

GBO_D int cg_parity(const double* s) { return ((int)s[CG_IT]) & 1; }

// q = V∇²x with differences set to zero across faces touching immersed cells
// (_symmetric_laplacian_operator!, conjugate_gradient_poisson_solver.jl:62-79 with
// conditional_differences.jl:15-43).  With s, accumulates x·q into s[CG_PQ].
template <typename FT>
__global__ void k_cg_laplacian(GridP<FT> g, const FT* __restrict__ x, FT* __restrict__ q, double* s) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const bool in = i < g.Nx && j < g.Ny;
    CFld<FT> X = cfld(x, g);
    Met<FT> M(g);
    double acc = 0.0;
    for (int k = blockIdx.z; k < g.Nz; k += gridDim.z) {
        if (!in) continue;
        const FT Ax = M.Ax(k), Ay = M.Ay(k), Az = M.Az();
        auto fx = [&](int ii) { return cond_zero(g, ii - 1, j, k, ii, j, k) ? FT(0) : Ax * ((X(ii, j, k) - X(ii - 1, j, k)) * g.rdx); };
        auto fy = [&](int jj) { return cond_zero(g, i, jj - 1, k, i, jj, k) ? FT(0) : Ay * ((X(i, jj, k) - X(i, jj - 1, k)) * g.rdy); };
        auto fz = [&](int kk) {
            if (g.flatz) return FT(0);
            return cond_zero(g, i, j, kk - 1, i, j, kk) ? FT(0) : Az * ((X(i, j, kk) - X(i, j, kk - 1)) * M.rdzf(kk));
        };
        const FT val = (fx(i + 1) - fx(i)) + (fy(j + 1) - fy(j)) + (fz(k + 1) - fz(k));
        const size_t idx = i + (size_t)g.Nx * (j + (size_t)g.Ny * k);
        q[idx] = val;
        acc += (double)x[idx] * (double)val;
    }
    if (s) block_add(acc, s + CG_PQ);
}

// elementwise helpers over N values (1-D grid-stride)
template <typename FT>
__global__ void k_cg_init(const FT* __restrict__ b, const FT* __restrict__ q, FT* __restrict__ r, size_t n) {
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) r[t] = b[t] - q[t];
}
template <typename FT>
__global__ void k_cg_scale(const FT* __restrict__ a, FT* __restrict__ out, FT sc, size_t n) {
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) out[t] = a[t] * sc;
}
// V⁻¹r of one cell; times Δzᶜ for the Fourier-tridiagonal preconditioner, whose solve!
// applies set_source_term! (fourier_tridiagonal_poisson_solver.jl:231-281)
template <typename FT>
GBO_D FT precond_source(const Met<FT>& M, FT vr, int k, int dz_scale) { return dz_scale ? vr * M.dzc(k) : vr; }

// ‖V⁻¹r‖² (VolumeInverseNorm, conjugate_gradient_poisson_solver.jl:13-34) into s[CG_NORM2]
// and, if out, the preconditioner's right-hand side
template <typename FT>
__global__ void k_cg_vinv(GridP<FT> g, const FT* __restrict__ r, FT* __restrict__ out, double* s, int dz_scale) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const bool in = i < g.Nx && j < g.Ny;
    Met<FT> M(g);
    double acc = 0.0;
    for (int k = blockIdx.z; k < g.Nz; k += gridDim.z) {
        if (!in) continue;
        const size_t idx = i + (size_t)g.Nx * (j + (size_t)g.Ny * k);
        const FT vr = r[idx] * M.rVc(k);
        if (out) out[idx] = precond_source(M, vr, k, dz_scale);
        acc += (double)vr * (double)vr;
    }
    block_add(acc, s + CG_NORM2);
}

// Stopping rule before the first iteration: tolerance, counters, stop flag.
__global__ void k_cg_begin(double* s, double reltol, double abstol, double maxiter, cudaGraphConditionalHandle h,
                           int use_handle) {
    const double norm = sqrt(s[CG_NORM2]);
    const double tol = fmax(reltol * norm, abstol);
    const bool cont = 0.0 < maxiter && norm > tol;
    s[CG_TOL] = tol;
    s[CG_IT] = 0.0;
    s[CG_NORM] = norm;
    s[CG_CONT] = cont ? 1.0 : 0.0;
    s[CG_RHO0] = s[CG_RHO1] = s[CG_PQ] = s[CG_SX] = s[CG_SR] = s[CG_NORM2] = 0.0;
    s[CG_SOLVES] += 1.0;
    if (use_handle) cudaGraphSetConditional(h, cont ? 1u : 0u);
}

// ρ = z·r into the ρ slot of this iteration
template <typename FT>
__global__ void k_cg_dot(const FT* __restrict__ a, const FT* __restrict__ b, size_t n, double* s) {
    double acc = 0.0;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
        acc += (double)a[t] * (double)b[t];
    block_add(acc, s + CG_RHO0 + cg_parity(s));
}
// p = z (first iteration) or z + (ρ/ρ_prev) p (conjugate_gradient_solver.jl:246-263)
template <typename FT>
__global__ void k_cg_update_p(const FT* __restrict__ z, FT* __restrict__ p, const double* s, size_t n) {
    const int par = cg_parity(s);
    const bool first = s[CG_IT] == 0.0;
    const FT beta = first ? FT(0) : FT(s[CG_RHO0 + par] / s[CG_RHO0 + (par ^ 1)]);
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
        p[t] = first ? z[t] : z[t] + beta * p[t];
}
// x += α p, r -= α q with α = ρ / (p·q); accumulates the active-cell sums of x and r
template <typename FT>
__global__ void k_cg_update_xr(GridP<FT> g, FT* __restrict__ x, FT* __restrict__ r, const FT* __restrict__ p,
                               const FT* __restrict__ q, double* s) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const bool in = i < g.Nx && j < g.Ny;
    const FT alpha = FT(s[CG_RHO0 + cg_parity(s)] / s[CG_PQ]);
    double ax = 0.0, ar = 0.0;
    for (int k = blockIdx.z; k < g.Nz; k += gridDim.z) {
        if (!in) continue;
        const size_t idx = i + (size_t)g.Nx * (j + (size_t)g.Ny * k);
        const FT xv = x[idx] + alpha * p[idx];
        const FT rv = r[idx] - alpha * q[idx];
        x[idx] = xv;
        r[idx] = rv;
        if (!inactive_cell(g, i, j, k)) { ax += xv; ar += rv; }
    }
    block_add(ax, s + CG_SX, ar, s + CG_SR);
}
// zero-mean gauge over active cells with immersed cells zeroed (enforce_zero_mean_gauge!,
// conjugate_gradient_poisson_solver.jl:81-96); accumulates ‖V⁻¹r‖² and, if out, writes
// the next iteration's preconditioner right-hand side
template <typename FT>
__global__ void k_cg_gauge(GridP<FT> g, FT* __restrict__ x, FT* __restrict__ r, FT* __restrict__ out, double* s,
                           int dz_scale) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const bool in = i < g.Nx && j < g.Ny;
    const FT mx = FT(s[CG_SX] / s[CG_NACT]), mr = FT(s[CG_SR] / s[CG_NACT]);
    Met<FT> M(g);
    double acc = 0.0;
    for (int k = blockIdx.z; k < g.Nz; k += gridDim.z) {
        if (!in) continue;
        const size_t idx = i + (size_t)g.Nx * (j + (size_t)g.Ny * k);
        const FT act = inactive_cell(g, i, j, k) ? FT(0) : FT(1);
        x[idx] = (x[idx] - mx) * act;
        const FT rv = (r[idx] - mr) * act;
        r[idx] = rv;
        const FT vr = rv * M.rVc(k);
        if (out) out[idx] = precond_source(M, vr, k, dz_scale);
        acc += (double)vr * (double)vr;
    }
    block_add(acc, s + CG_NORM2);
}
// Stopping rule after an iteration (conjugate_gradient_solver.jl:278-283); clears the
// accumulators of the next iteration.
__global__ void k_cg_check(double* s, double maxiter, cudaGraphConditionalHandle h, int use_handle) {
    const double it = s[CG_IT] + 1.0;
    const double norm = sqrt(s[CG_NORM2]);
    const bool cont = it < maxiter && norm > s[CG_TOL];
    if (!cont && norm > s[CG_TOL]) s[CG_FAIL] = 1.0;
    s[CG_IT] = it;
    s[CG_NORM] = norm;
    s[CG_ITERS] += 1.0;
    s[CG_CONT] = cont ? 1.0 : 0.0;
    s[CG_PQ] = s[CG_SX] = s[CG_SR] = s[CG_NORM2] = 0.0;
    s[CG_RHO0 + (((int)it) & 1)] = 0.0;  // ρ slot of the next iteration (its ρ_prev is kept)
    if (use_handle) cudaGraphSetConditional(h, cont ? 1u : 0u);
}
// number of active cells (for the gauge means)
template <typename FT>
__global__ void k_cg_count(GridP<FT> g, double* s) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    double a = 0.0;
    for (int k = blockIdx.z; k < g.Nz; k += gridDim.z)
        if (i < g.Nx && j < g.Ny && !inactive_cell(g, i, j, k)) a += 1.0;
    block_add(a, s + CG_NACT);
}
