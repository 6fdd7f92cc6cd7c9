// gbo_cg.cuh -- conjugate-gradient Poisson solver kernels for an immersed grid
// (src/Solvers/conjugate_gradient_poisson_solver.jl:38-211;
//  src/Solvers/conjugate_gradient_solver.jl:177-284).
//
// The iteration runs without the host: every scalar (ρ, p·q, the active-cell sums
// of the gauge, ‖V⁻¹r‖, the iteration count and the stop flag) lives in a small
// FP64 array on the device.  k_cg_begin and the last block of k_cg_gauge evaluate
// the stopping rule of `iterating` (conjugate_gradient_solver.jl:278-283) on the
// device and, inside a CUDA graph, drive a conditional WHILE node with
// cudaGraphSetConditional, so a whole time step with three CG solves is one graph
// launch.  Dot products and norms accumulate in FP64 (warp shuffles, one atomic
// per block); the last block of each reduction forms the derived scalar (β, α,
// the gauge means) once instead of every thread dividing.
#pragma once
#include <type_traits>

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
    CG_BETA,               // ρ/ρ_prev of this iteration (0 on the first)
    CG_ALPHA,              // ρ/(p·q)
    CG_MX, CG_MR,          // active-cell means of x and r
    CG_ZRP,                // z·r_prev (flexible CG)
    CG_NSLOTS
};
// block-completion counters of the loop kernels (last block finalises the scalars)
enum {
    CC_DOT = 0, CC_LAP, CC_XR, CC_GAUGE, CC_VINV, CC_COUNT,
    CC_N
};

// z-slices per launch of the 3-D CG kernels: blocks march over a contiguous slice of
// levels so that each kernel issues a few thousand block reductions, not one per
// (tile, level); the streaming kernels load CG_UNROLL levels before storing them
constexpr int CG_ZSLICES = 8;
constexpr int CG_UNROLL = 4;

GBO_D double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
// Block sums in a fixed order (no floating-point atomics, so a solve is bitwise
// reproducible): every block reduces its threads' values, stores the two partial sums at
// its own index of part (the array after the scalar slots, s + CG_NSLOTS), and takes a
// completion ticket; the block holding the last ticket adds all partials in block order to
// *da (and *db) and resets the ticket.  Returns true in that block, once the totals are
// written by its thread 0.
GBO_D bool block_sum(double a, double* da, double b, double* db, double* part, unsigned int* ticket) {
    __shared__ double sa[32], sb[32];
    __shared__ bool last;
    const int tid = threadIdx.x + threadIdx.y * blockDim.x;
    const int lane = tid & 31, wid = tid >> 5, nt = blockDim.x * blockDim.y, nw = (nt + 31) >> 5;
    const unsigned nb = gridDim.x * gridDim.y * gridDim.z;
    a = warp_sum(a);
    b = warp_sum(b);
    if (lane == 0) { sa[wid] = a; sb[wid] = b; }
    __syncthreads();
    if (tid == 0) {
        double ta = 0.0, tb = 0.0;
        for (int w = 0; w < nw; ++w) { ta += sa[w]; tb += sb[w]; }
        const unsigned bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
        part[2 * (size_t)bid] = ta;
        part[2 * (size_t)bid + 1] = tb;
        __threadfence();
        last = atomicAdd(ticket, 1u) == nb - 1;
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double xa = 0.0, xb = 0.0;
    for (unsigned q = tid; q < nb; q += nt) {
        xa += __ldcg(part + 2 * (size_t)q);
        xb += __ldcg(part + 2 * (size_t)q + 1);
    }
    xa = warp_sum(xa);
    xb = warp_sum(xb);
    __syncthreads();  // sa / sb are reused
    if (lane == 0) { sa[wid] = xa; sb[wid] = xb; }
    __syncthreads();
    if (tid == 0) {
        double ta = 0.0, tb = 0.0;
        for (int w = 0; w < nw; ++w) { ta += sa[w]; tb += sb[w]; }
        *da += ta;
        if (db) *db += tb;
        *ticket = 0u;  // ready for the next launch
        __threadfence();
    }
    __syncthreads();
    return true;
}
// partial sums of one CG reduction launch live after the scalar slots
GBO_D double* cg_part(double* s) { return s + CG_NSLOTS; }

GBO_D int cg_parity(const double* s) { return ((int)s[CG_IT]) & 1; }

// q = V∇²x with differences set to zero across faces touching immersed cells
// (_symmetric_laplacian_operator!, conjugate_gradient_poisson_solver.jl:62-79 with
// conditional_differences.jl:15-43).
template <typename FT>
__global__ void k_cg_laplacian(GridP<FT> g, const FT* __restrict__ x, FT* __restrict__ q) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const bool in = i < g.Nx && j < g.Ny;
    CFld<FT> X = cfld(x, g);
    Met<FT> M(g);
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
    }
}

// elementwise helpers over N values (1-D grid-stride)
template <typename FT>
__global__ void k_cg_init(const FT* __restrict__ b, const FT* __restrict__ q, FT* __restrict__ r, size_t n) {
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) r[t] = b[t] - q[t];
}
template <typename FT>
__global__ void k_cg_scale(const FT* __restrict__ a, FT* __restrict__ out, FT sc, size_t n,
                           const FT* scp = nullptr) {
    if (scp) sc = __ldg(scp);
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) out[t] = a[t] * sc;
}
// V⁻¹r of one cell; times Δzᶜ for the Fourier-tridiagonal preconditioner, whose solve!
// applies set_source_term! (fourier_tridiagonal_poisson_solver.jl:231-281)
template <typename FT>
GBO_D FT precond_source(const Met<FT>& M, FT vr, int k, int dz_scale) { return dz_scale ? vr * M.dzc(k) : vr; }

// ‖V⁻¹r‖² (VolumeInverseNorm, conjugate_gradient_poisson_solver.jl:13-34) into s[CG_NORM2]
// and, if out, the preconditioner's right-hand side
template <typename FT>
__global__ void k_cg_vinv(GridP<FT> g, const FT* __restrict__ r, FT* __restrict__ out, double* s, int dz_scale,
                          unsigned int* cnt) {
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
    block_sum(acc, s + CG_NORM2, 0.0, nullptr, cg_part(s), cnt + CC_VINV);
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

// True in exactly one block: the one whose completion ticket is the last.  Each block's
// writes of its own partial results (thread 0) are made visible before its ticket; the
// last block then reads them all with L2 loads.
GBO_D bool last_block(unsigned int* counter) {
    __shared__ bool last;
    const unsigned int total = gridDim.x * gridDim.y * gridDim.z;
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        __threadfence();
        last = atomicAdd(counter, 1u) == total - 1;
        if (last) *counter = 0u;  // ready for the next launch
    }
    __syncthreads();
    return last;
}
GBO_D double ldcg(const double* p) { return __ldcg(p); }

// ρ = z·r into the ρ slot of this iteration; the last block sets β = ρ/ρ_prev
// (conjugate_gradient_solver.jl:246-263; 0 on the first iteration)
//
// Fail-safe for the loop: the first thread clears the stop flag and the loop
// condition at the start of every iteration; only the last block of k_cg_gauge
// sets them again, so an iteration whose stopping test did not run ends the loop
// instead of repeating it.
template <typename FT>
__global__ void k_cg_dot(const FT* __restrict__ a, const FT* __restrict__ b, size_t n, double* s, unsigned int* cnt,
                         cudaGraphConditionalHandle h, int use_handle, const FT* __restrict__ rprev = nullptr) {
    const int par = cg_parity(s);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        s[CG_CONT] = 0.0;
        if (use_handle) cudaGraphSetConditional(h, 0u);
    }
    // 16-byte vectors (4 floats or 2 doubles): each vector's products summed in FT, the
    // running sums in FP64
    double acc = 0.0, acc2 = 0.0;
    const size_t gid = blockIdx.x * (size_t)blockDim.x + threadIdx.x, stride = (size_t)gridDim.x * blockDim.x;
    constexpr int W = 16 / sizeof(FT);
    const bool aligned = ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b) |
                           reinterpret_cast<uintptr_t>(rprev)) & 15) == 0;
    size_t head = 0;
    if (aligned) {
        using V = typename std::conditional<sizeof(FT) == 4, float4, double2>::type;
        const V* av = reinterpret_cast<const V*>(a);
        const V* bv = reinterpret_cast<const V*>(b);
        const V* pv = reinterpret_cast<const V*>(rprev);
        const size_t nv = n / W;
        auto dot = [](const V& x, const V& y) {
            if constexpr (sizeof(FT) == 4) return (double)(x.x * y.x + x.y * y.y + x.z * y.z + x.w * y.w);
            else return x.x * y.x + x.y * y.y;
        };
#pragma unroll 2
        for (size_t t = gid; t < nv; t += stride) {
            const V x = av[t];
            acc += dot(x, bv[t]);
            if (rprev) acc2 += dot(x, pv[t]);
        }
        head = nv * W;
    }
    for (size_t t = head + gid; t < n; t += stride) {
        acc += (double)(a[t] * b[t]);
        if (rprev) acc2 += (double)(a[t] * rprev[t]);
    }
    if (block_sum(acc, s + CG_RHO0 + par, acc2, rprev ? s + CG_ZRP : nullptr, cg_part(s), cnt + CC_DOT) &&
        threadIdx.x == 0) {
        const bool first = s[CG_IT] == 0.0;
        const double rho = ldcg(s + CG_RHO0 + par), prev = ldcg(s + CG_RHO0 + (par ^ 1));
        // flexible (Polak-Ribière) CG for a preconditioner that varies: β = z·(r - r_prev) / ρ_prev
        const double num = rprev ? rho - ldcg(s + CG_ZRP) : rho;
        s[CG_BETA] = first ? 0.0 : num / prev;
        s[CG_ZRP] = 0.0;
    }
}

// Per-thread column context of the 3-D CG kernels: the wrapped neighbour columns and
// their numbers of immersed cells, constant along k (a cell (c, k) is immersed iff
// k < kb[c]).
struct CgCol {
    size_t C, W, E, S, N;  // column offsets of (i, j) and its x / y neighbours
    int kC, kW, kE, kS, kN;
};
template <typename FT>
GBO_D CgCol cg_col(const GridP<FT>& g, int i, int j) {
    CgCol c;
    const int iw = i == 0 ? g.Nx - 1 : i - 1, ie = i == g.Nx - 1 ? 0 : i + 1;
    const int js = j == 0 ? g.Ny - 1 : j - 1, jn = j == g.Ny - 1 ? 0 : j + 1;
    c.C = i + (size_t)g.Nx * j;
    c.W = iw + (size_t)g.Nx * j;
    c.E = ie + (size_t)g.Nx * j;
    c.S = i + (size_t)g.Nx * js;
    c.N = i + (size_t)g.Nx * jn;
    c.kC = c.kW = c.kE = c.kS = c.kN = 0;
    if (g.kbot) {
        c.kC = __ldg(g.kbot + c.C); c.kW = __ldg(g.kbot + c.W); c.kE = __ldg(g.kbot + c.E);
        c.kS = __ldg(g.kbot + c.S); c.kN = __ldg(g.kbot + c.N);
    }
    return c;
}

// p = z + β p_prev (p = z on the first iteration) fused with q = V∇²p: the new
// search direction is formed at every point of the 7-point stencil from z and
// the previous direction, so no separate pass writes p before the Laplacian reads
// it.  Differences across a face touching an immersed cell are zero
// (conditional_differences.jl:15-43); at the walls the mirrored halo makes them
// zero.  The two directions alternate between p0 and p1 by iteration parity.
// Accumulates p·q; the last block sets α = ρ/(p·q).
template <typename FT>
__global__ void k_cg_direction(GridP<FT> g, const FT* __restrict__ z, FT* __restrict__ p0, FT* __restrict__ p1,
                               FT* __restrict__ q, double* s, unsigned int* cnt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const bool in = i < g.Nx && j < g.Ny;
    const int par = cg_parity(s);
    const bool first = s[CG_IT] == 0.0;
    const FT beta = FT(s[CG_BETA]);
    const FT* __restrict__ pold = par ? p0 : p1;
    FT* __restrict__ pnew = par ? p1 : p0;
    const size_t plane = (size_t)g.Nx * g.Ny;
    Met<FT> M(g);
    FT acc = FT(0);
    if (in) {
        const CgCol c = cg_col(g, i, j);
        auto pn = [&](size_t col, int kk) {
            const size_t at = col + plane * kk;
            return first ? z[at] : z[at] + beta * pold[at];
        };
        // this block's contiguous slice of levels; p below, at and above the level roll
        // through registers
        const int per = (g.Nz + (int)gridDim.z - 1) / (int)gridDim.z;
        const int k0 = blockIdx.z * per, k1 = min(g.Nz, k0 + per);
        FT pc = k0 < k1 ? pn(c.C, k0) : FT(0);
        FT pb = k0 > 0 && k0 < k1 ? pn(c.C, k0 - 1) : pc;
        for (int k = k0; k < k1; ++k) {
            const FT Ax = M.Ax(k), Ay = M.Ay(k), Az = M.Az();
            const FT pt = k < g.Nz - 1 ? pn(c.C, k + 1) : pc;
            const FT pw = pn(c.W, k), pe = pn(c.E, k), ps = pn(c.S, k), pnn = pn(c.N, k);
            const bool im = k < c.kC;
            const FT fw = (im || k < c.kW) ? FT(0) : Ax * ((pc - pw) * g.rdx);
            const FT fe = (im || k < c.kE) ? FT(0) : Ax * ((pe - pc) * g.rdx);
            const FT fs = (im || k < c.kS) ? FT(0) : Ay * ((pc - ps) * g.rdy);
            const FT fn = (im || k < c.kN) ? FT(0) : Ay * ((pnn - pc) * g.rdy);
            FT dz = FT(0);
            if (!g.flatz) {
                const FT fb = (im || k - 1 < c.kC) ? FT(0) : Az * ((pc - pb) * M.rdzf(k));
                const FT ft = (im || k + 1 < c.kC) ? FT(0) : Az * ((pt - pc) * M.rdzf(k + 1));
                dz = ft - fb;
            }
            const FT val = (fe - fw) + (fn - fs) + dz;
            const size_t idx = c.C + plane * k;
            pnew[idx] = pc;
            q[idx] = val;
            acc += pc * val;
            pb = pc;
            pc = pt;
        }
    }
    if (block_sum((double)acc, s + CG_PQ, 0.0, nullptr, cg_part(s), cnt + CC_LAP) && threadIdx.x == 0 &&
        threadIdx.y == 0)
        s[CG_ALPHA] = ldcg(s + CG_RHO0 + par) / ldcg(s + CG_PQ);
}

// x += α p, r -= α q; accumulates the active-cell sums of x and r, the last block
// sets their means
template <typename FT>
__global__ void k_cg_update_xr(GridP<FT> g, FT* __restrict__ x, FT* __restrict__ r, const FT* __restrict__ p0,
                               const FT* __restrict__ p1, const FT* __restrict__ q, double* s, unsigned int* cnt,
                               FT* __restrict__ rprev = nullptr) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const bool in = i < g.Nx && j < g.Ny;
    const FT alpha = FT(s[CG_ALPHA]);
    const FT* p = cg_parity(s) ? p1 : p0;
    FT ax = FT(0), ar = FT(0);
    if (in) {
        const int kb = g.kbot ? __ldg(g.kbot + i + (size_t)g.Nx * j) : 0;
        const size_t plane = (size_t)g.Nx * g.Ny, c = i + (size_t)g.Nx * j;
        const int per = (g.Nz + (int)gridDim.z - 1) / (int)gridDim.z;
        const int k0 = blockIdx.z * per, k1 = min(g.Nz, k0 + per);
        // groups of CG_UNROLL levels: every load of the group before its stores
        for (int ka = k0; ka < k1; ka += CG_UNROLL) {
            FT xs[CG_UNROLL], rs[CG_UNROLL], ps[CG_UNROLL], qs[CG_UNROLL];
#pragma unroll
            for (int u = 0; u < CG_UNROLL; ++u) {
                const size_t idx = c + plane * (ka + u);
                if (ka + u < k1) { xs[u] = x[idx]; rs[u] = r[idx]; ps[u] = p[idx]; qs[u] = q[idx]; }
            }
#pragma unroll
            for (int u = 0; u < CG_UNROLL; ++u) {
                const int k = ka + u;
                if (k >= k1) break;
                const size_t idx = c + plane * k;
                const FT xv = xs[u] + alpha * ps[u];
                const FT rv = rs[u] - alpha * qs[u];
                if (rprev) rprev[idx] = rs[u];
                x[idx] = xv;
                r[idx] = rv;
                if (k >= kb) { ax += xv; ar += rv; }
            }
        }
    }
    if (block_sum((double)ax, s + CG_SX, (double)ar, s + CG_SR, cg_part(s), cnt + CC_XR) && threadIdx.x == 0 &&
        threadIdx.y == 0) {
        const double n = s[CG_NACT];
        s[CG_MX] = ldcg(s + CG_SX) / n;
        s[CG_MR] = ldcg(s + CG_SR) / n;
    }
}

// Zero-mean gauge over active cells with immersed cells zeroed (enforce_zero_mean_gauge!,
// conjugate_gradient_poisson_solver.jl:81-96); accumulates ‖V⁻¹r‖², writes the next
// preconditioner input (if out) and, in the last block, applies the stopping rule
// (conjugate_gradient_solver.jl:278-283), clears the next iteration's accumulators
// and sets the loop condition.
template <typename FT>
__global__ void k_cg_gauge(GridP<FT> g, FT* __restrict__ x, FT* __restrict__ r, FT* __restrict__ out, double* s,
                           int dz_scale, unsigned int* cnt, double maxiter, cudaGraphConditionalHandle h,
                           int use_handle) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const bool in = i < g.Nx && j < g.Ny;
    const FT mx = FT(s[CG_MX]), mr = FT(s[CG_MR]);
    Met<FT> M(g);
    FT acc = FT(0);
    if (in) {
        const int kb = g.kbot ? __ldg(g.kbot + i + (size_t)g.Nx * j) : 0;
        const size_t plane = (size_t)g.Nx * g.Ny, c = i + (size_t)g.Nx * j;
        const int per = (g.Nz + (int)gridDim.z - 1) / (int)gridDim.z;
        const int k0 = blockIdx.z * per, k1 = min(g.Nz, k0 + per);
        for (int ka = k0; ka < k1; ka += CG_UNROLL) {
            FT xs[CG_UNROLL], rs[CG_UNROLL];
#pragma unroll
            for (int u = 0; u < CG_UNROLL; ++u) {
                const size_t idx = c + plane * (ka + u);
                if (ka + u < k1) { xs[u] = x[idx]; rs[u] = r[idx]; }
            }
#pragma unroll
            for (int u = 0; u < CG_UNROLL; ++u) {
                const int k = ka + u;
                if (k >= k1) break;
                const size_t idx = c + plane * k;
                const FT act = k < kb ? FT(0) : FT(1);
                x[idx] = (xs[u] - mx) * act;
                const FT rv = (rs[u] - mr) * act;
                r[idx] = rv;
                const FT vr = rv * M.rVc(k);
                if (out) out[idx] = precond_source(M, vr, k, dz_scale);
                acc += vr * vr;
            }
        }
    }
    if (block_sum((double)acc, s + CG_NORM2, 0.0, nullptr, cg_part(s), cnt + CC_GAUGE) && threadIdx.x == 0 &&
        threadIdx.y == 0) {
        const double it = s[CG_IT] + 1.0;
        const double norm = sqrt(ldcg(s + CG_NORM2));
        const bool cont = it < maxiter && norm > s[CG_TOL];
        // stopped above tolerance, or on a NaN residual (which no comparison passes)
        if (!cont && !(norm <= s[CG_TOL])) s[CG_FAIL] = 1.0;
        s[CG_IT] = it;
        s[CG_NORM] = norm;
        s[CG_ITERS] += 1.0;
        s[CG_CONT] = cont ? 1.0 : 0.0;
        s[CG_PQ] = s[CG_SX] = s[CG_SR] = s[CG_NORM2] = 0.0;
        s[CG_RHO0 + (((int)it) & 1)] = 0.0;  // ρ slot of the next iteration (its ρ_prev is kept)
        __threadfence();
        if (use_handle) cudaGraphSetConditional(h, cont ? 1u : 0u);
    }
}

// number of active cells (for the gauge means)
template <typename FT>
__global__ void k_cg_count(GridP<FT> g, double* s, unsigned int* cnt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    double a = 0.0;
    for (int k = blockIdx.z; k < g.Nz; k += gridDim.z)
        if (i < g.Nx && j < g.Ny && !inactive_cell(g, i, j, k)) a += 1.0;
    block_sum(a, s + CG_NACT, 0.0, nullptr, cg_part(s), cnt + CC_COUNT);
}
