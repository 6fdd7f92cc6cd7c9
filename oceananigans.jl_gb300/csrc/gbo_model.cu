// gbo_model.cu -- model lifecycle, RK3 orchestration and the C ABI of libgb300ocean.so.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gbo.h"
#include "gbo_fft.cuh"
#include "gbo_cg.cuh"
#include "gbo_sim.cuh"
#include "gbo_learned.cuh"
#include "gbo_fused.cuh"
#include "gbo_dynamic.cuh"
#include "gbo_launch_table.h"

// ===========================================================================
// Pressure source and projection kernels
// ===========================================================================
enum { SRC_FFT = 0, SRC_FT = 1, SRC_CG = 2 };

// Levels marched by one thread of the column kernels (k_source, k_correct): the z
// neighbour of one level is the value of the previous one, and the index arithmetic
// and the immersed-column lookups are done once per column
constexpr int COL_LEVELS = 8;

// rhs = divᶜᶜᶜ(u*) (solve_for_pressure.jl:12-50): × Δzᶜ for the Fourier-tridiagonal
// solver, × Vᶜᶜᶜ for CG.
template <typename FT>
__global__ void __launch_bounds__(256) k_source(GridP<FT> g, const FT* __restrict__ u, const FT* __restrict__ v,
                                                const FT* __restrict__ w, FT* __restrict__ rhs, int mode) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    const int k0 = blockIdx.z * COL_LEVELS, k1 = min(g.Nz, k0 + COL_LEVELS);
    const size_t plane = (size_t)g.Nx * g.Ny, c = i + (size_t)g.Nx * j;
    const size_t cx = wrapi(i + 1, g.Nx) + (size_t)g.Nx * j, cy = i + (size_t)g.Nx * wrapi(j + 1, g.Ny);
    Met<FT> M(g);
    const FT Az = M.Az();
    const int kb = g.kbot ? __ldg(g.kbot + c) : 0;
    // all loads of the column first (w at faces k0 .. k1; face 0 and Nz are walls)
    FT ru[COL_LEVELS], rux[COL_LEVELS], rv[COL_LEVELS], rvy[COL_LEVELS], rw[COL_LEVELS + 1];
    rw[0] = (g.flatz || k0 <= 0) ? FT(0) : w[c + plane * k0];
#pragma unroll
    for (int l = 0; l < COL_LEVELS; ++l) {
        const int k = k0 + l;
        if (k < k1) {
            const size_t o = plane * k;
            ru[l] = u[c + o];
            rux[l] = u[cx + o];
            rv[l] = v[c + o];
            rvy[l] = v[cy + o];
            rw[l + 1] = (g.flatz || k + 1 >= g.Nz) ? FT(0) : w[c + o + plane];
        }
    }
#pragma unroll
    for (int l = 0; l < COL_LEVELS; ++l) {
        const int k = k0 + l;
        if (k < k1) {
            const FT Ax = M.Ax(k), Ay = M.Ay(k);
            const FT div = M.rVc(k) * ((Ax * rux[l] - Ax * ru[l]) + (Ay * rvy[l] - Ay * rv[l]) +
                                       (g.flatz ? FT(0) : (Az * rw[l + 1] - Az * rw[l])));
            const bool active = k >= kb;
            FT r = active ? div : FT(0);
            if (mode == SRC_FT) r = (active ? M.dzc(k) : FT(0)) * div;
            if (mode == SRC_CG) r = r * (Az * M.dzc(k));
            rhs[c + plane * k] = r;
        }
    }
}

// u = u* - ∂x(pΔτ), ... (pressure_correction.jl:67-73), p = pΔτ / max(eps, Δτ)
// (:102-104), and the tracer predictor copied to the state.  In place is allowed
// (every point reads only its own u*).  ∂ operators are conditional on an immersed
// grid (conditional_differences.jl:15-43): zero across a face touching an immersed cell.
template <typename FT>
__global__ void __launch_bounds__(256) k_correct(GridP<FT> g, const FT* us, const FT* vs, const FT* ws,
                                                 const FT* __restrict__ phi, FT* u, FT* v, FT* w, FT* __restrict__ p,
                                                 FT rdtau, FT phi_shift, const FT* rdp = nullptr) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    const int k0 = blockIdx.z * COL_LEVELS, k1 = min(g.Nz, k0 + COL_LEVELS);
    const size_t plane = (size_t)g.Nx * g.Ny, c = i + (size_t)g.Nx * j;
    const size_t cw = wrapi(i - 1, g.Nx) + (size_t)g.Nx * j, cs = i + (size_t)g.Nx * wrapi(j - 1, g.Ny);
    Met<FT> M(g);
    if (rdp) rdtau = __ldg(rdp);
    const bool ibg = g.kbot != nullptr;
    const int kbC = ibg ? __ldg(g.kbot + c) : 0, kbW = ibg ? __ldg(g.kbot + cw) : 0, kbS = ibg ? __ldg(g.kbot + cs) : 0;
    auto imm = [&](int kb, int k) { return ibg && k >= 0 && k < g.Nz && k < kb; };
    // all loads of the column first: u* may alias u (in place), so loads issued after a
    // store could not move ahead of it
    FT rp[COL_LEVELS + 1], rw[COL_LEVELS], rs[COL_LEVELS], ru[COL_LEVELS], rv[COL_LEVELS], rz[COL_LEVELS];
    rp[0] = phi[c + plane * (k0 > 0 ? k0 - 1 : 0)];  // ϕ below the first level (mirrored at the bottom)
#pragma unroll
    for (int l = 0; l < COL_LEVELS; ++l) {
        const int k = k0 + l;
        if (k < k1) {
            const size_t o = plane * k;
            rp[l + 1] = phi[c + o];
            rw[l] = phi[cw + o];
            rs[l] = phi[cs + o];
            ru[l] = us[c + o];
            rv[l] = vs[c + o];
            rz[l] = g.flatz ? FT(0) : ws[c + o];
        }
    }
#pragma unroll
    for (int l = 0; l < COL_LEVELS; ++l) {
        const int k = k0 + l;
        if (k < k1) {
            const size_t o = plane * k;
            const FT pc = rp[l + 1] - phi_shift;
            const FT dx_ = (imm(kbW, k) || imm(kbC, k)) ? FT(0) : (pc - (rw[l] - phi_shift));
            const FT dy_ = (imm(kbS, k) || imm(kbC, k)) ? FT(0) : (pc - (rs[l] - phi_shift));
            u[c + o] = ru[l] - dx_ * g.rdx;
            v[c + o] = rv[l] - dy_ * g.rdy;
            if (!g.flatz) {
                const FT dz_ = (imm(kbC, k - 1) || imm(kbC, k)) ? FT(0) : (pc - (rp[l] - phi_shift));
                w[c + o] = rz[l] - dz_ * M.rdzf(k);
            }
            p[c + o] = pc * rdtau;
        }
    }
}

// mask_immersed_field! (mask_immersed_field.jl:65-77): zero on the immersed periphery
// of each field's location.  which: bit 0 u, bit 1 v, bit 2 w, bit 3 tracer c (stored
// as departures from cref when cref is given: the masked value is then -cref[k]).
template <typename FT>
__global__ void k_mask(GridP<FT> g, FT* u, FT* v, FT* w, FT* c, int which, const FT* cref = nullptr) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y * blockDim.y + threadIdx.y;
    int k = blockIdx.z;
    if (i >= g.Nx || j >= g.Ny) return;
    const size_t idx = i + (size_t)g.Nx * (j + (size_t)g.Ny * k);
    if ((which & 1) && imm_periph(g, i, j, k, true, false, false)) u[idx] = FT(0);
    if ((which & 2) && imm_periph(g, i, j, k, false, true, false)) v[idx] = FT(0);
    if ((which & 4) && !g.flatz && imm_periph(g, i, j, k, false, false, true)) w[idx] = FT(0);
    if ((which & 8) && imm_periph(g, i, j, k, false, false, false)) c[idx] = cref ? -cref[k] : FT(0);
}

// Tracers of single-precision Bounded-z models are stored as departures from a per-level
// reference profile, the horizontal mean of the values they were last set to.
// k_level_mean: that mean in FP64 (one block per level); k_to_departure: the profile in
// FT and the departures from it; k_from_departure: profile + departure in the output type.
constexpr int LM_THREADS = 256;
template <typename T>
__global__ void __launch_bounds__(LM_THREADS) k_level_mean(const T* __restrict__ a, size_t plane, double* __restrict__ mean) {
    __shared__ double red[LM_THREADS];
    const size_t base = plane * blockIdx.x;
    double sum = 0;
    for (size_t q = threadIdx.x; q < plane; q += LM_THREADS) sum += (double)a[base + q];
    red[threadIdx.x] = sum;
    __syncthreads();
    for (int h = LM_THREADS / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) mean[blockIdx.x] = red[0] / (double)plane;
}
template <typename FT, typename T>
__global__ void k_to_departure(const T* __restrict__ a, const double* __restrict__ mean, FT* __restrict__ ref,
                               FT* __restrict__ c, size_t plane, size_t n) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += stride) {
        const size_t k = q / plane;
        const FT r = FT(mean[k]);
        c[q] = FT((double)a[q] - (double)r);
        if (q == k * plane) ref[k] = r;
    }
}
template <typename FT, typename T>
__global__ void k_from_departure(const FT* __restrict__ c, const FT* __restrict__ ref, T* __restrict__ out, size_t plane,
                                 size_t n) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += stride)
        out[q] = T((double)ref[q / plane] + (double)c[q]);
}

template <typename FT>
__global__ void k_scale_dzc(GridP<FT> g, FT* __restrict__ a) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y * blockDim.y + threadIdx.y;
    int k = blockIdx.z;
    if (i >= g.Nx || j >= g.Ny) return;
    a[i + (size_t)g.Nx * (j + (size_t)g.Ny * k)] *= Met<FT>(g).dzc(k);
}

template <typename FT>
__global__ void k_copy(const FT* __restrict__ a, FT* __restrict__ b, size_t n) {
    const size_t gid = blockIdx.x * (size_t)blockDim.x + threadIdx.x, stride = (size_t)gridDim.x * blockDim.x;
    // 16-byte vectors where both arrays allow it, then the remainder
    size_t head = 0;
    if (((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b)) & 15) == 0) {
        const size_t nv = n * sizeof(FT) / 16;
        const uint4* av = reinterpret_cast<const uint4*>(a);
        uint4* bv = reinterpret_cast<uint4*>(b);
        for (size_t t = gid; t < nv; t += stride) bv[t] = av[t];
        head = nv * 16 / sizeof(FT);
    }
    for (size_t t = head + gid; t < n; t += stride) b[t] = a[t];
}

template <typename FT>
__global__ void k_nan_check(const FT* __restrict__ a, size_t n, unsigned int* flags) {
    size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    size_t stride = (size_t)gridDim.x * blockDim.x;
    bool bad = false;
    for (; t < n; t += stride) bad |= !isfinite(a[t]);
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(flags, GBO_FLAG_NAN);
}


// ===========================================================================
// Host helpers
// ===========================================================================
namespace {

thread_local std::string g_last_error = "";

// Conjugate-gradient stopping parameters with the reference's defaults filled in:
// reltol = abstol = sqrt(eps(FT)) (conjugate_gradient_poisson_solver.jl:134-137) and
// maxiter = the number of cells (conjugate_gradient_solver.jl:91).
void cg_parameters(int32_t float_type, const gbo_model_desc& d, int64_t cells, double* rel, double* abs_,
                   double* maxiter) {
    const double eps = float_type == GBO_FLOAT32 ? 1.1920928955078125e-07 : 2.220446049250313e-16;
    *rel = d.cg_reltol > 0 ? d.cg_reltol : std::sqrt(eps);
    *abs_ = d.cg_abstol > 0 ? d.cg_abstol : std::sqrt(eps);
    *maxiter = d.cg_maxiter > 0 ? (double)d.cg_maxiter : (double)cells;
}

struct CudaError {
    cudaError_t e;
    const char* what;
};

#define GBO_CUDA(call)                                                  \
    do {                                                                \
        cudaError_t e_ = (call);                                        \
        if (e_ != cudaSuccess) throw CudaError{e_, #call};              \
    } while (0)

struct InvalidArg {
    std::string msg;
};

// FFT radix plan: radix-4 stages, then 2, 3, 5.  Returns false if n has other factors.
bool make_plan(int n, FFTPlan1D& p) {
    p.n = n;
    p.nrad = 0;
    int m = n;
    while (m % 4 == 0 && p.nrad < GBO_MAX_RADICES) { p.rad[p.nrad++] = 4; m /= 4; }
    for (int r : {2, 3, 5})
        while (m % r == 0 && p.nrad < GBO_MAX_RADICES) { p.rad[p.nrad++] = r; m /= r; }
    return m == 1 && n >= 1;
}

// Vertical grid following generate_coordinate (src/Grids/grid_generation.jl:34-176),
// evaluated in the working precision FT.  Tables cover kr in [1-H, Nz+H+1].
template <typename FT>
struct ZGrid {
    int Nz = 1, H = 3, zoff = 0;
    FT Lz = 1;
    std::vector<FT> dzc, dzf, zc, zf;
    bool flat = false;
    FT at(const std::vector<FT>& a, int kr) const { return a[kr + zoff]; }
};

template <typename FT>
ZGrid<FT> make_zgrid(int Nz, int H, bool flat, const double* faces, double z0, double z1) {
    ZGrid<FT> Z;
    Z.Nz = Nz;
    Z.H = H;
    Z.flat = flat;
    const int kmin = 1 - H, kmax = Nz + H + 1;
    Z.zoff = -kmin;
    const int len = kmax - kmin + 1;
    Z.dzc.assign(len, FT(1));
    Z.dzf.assign(len, FT(1));
    Z.zc.assign(len, FT(0));
    Z.zf.assign(len, FT(0));
    if (flat) return Z;
    if (!faces) {
        // regular: Δ = FT(L/N), faces F₋ + (k-1)Δ (grid_generation.jl:124-156)
        double L = z1 - z0;
        FT d = FT(L / Nz);
        Z.Lz = FT(L);
        for (int k = kmin; k <= kmax; ++k) {
            Z.dzc[k + Z.zoff] = d;
            Z.dzf[k + Z.zoff] = d;
            Z.zf[k + Z.zoff] = FT(z0 + (k - 1) * (L / Nz));
            Z.zc[k + Z.zoff] = FT(z0 + (k - 0.5) * (L / Nz));
        }
        return Z;
    }
    std::vector<FT> Fi(Nz + 1);
    for (int i = 0; i <= Nz; ++i) Fi[i] = FT(faces[i]);
    Z.Lz = Fi[Nz] - Fi[0];
    std::vector<FT> dlow(H), dup(H);
    for (int i = 1; i <= H; ++i) dlow[i - 1] = Fi[Nz + 1 - H + i - 1] - Fi[Nz + 1 - H + i - 2];
    for (int i = 1; i <= H; ++i) dup[i - 1] = Fi[i] - Fi[i - 1];
    std::vector<FT> dplus(dup.rbegin(), dup.rend());
    std::vector<FT> F;
    for (int i = 1; i <= H; ++i) {
        FT s = 0;
        for (int q = i; q <= H; ++q) s += dlow[q - 1];
        F.push_back(Fi[0] - s);
    }
    for (FT f : Fi) F.push_back(f);
    std::vector<FT> Fp;
    for (int i = 1; i <= H; ++i) {
        FT s = 0;
        for (int q = i; q <= H; ++q) s += dplus[q - 1];
        Fp.push_back(Fi[Nz] + s);
    }
    std::reverse(Fp.begin(), Fp.end());
    for (FT f : Fp) F.push_back(f);
    const int TC = Nz + 2 * H, TF = Nz + 1 + 2 * H;
    std::vector<FT> C(TC), Df, Dc(TF - 1);
    for (int i = 0; i < TC; ++i) C[i] = (F[i + 1] + F[i]) / FT(2);
    for (int i = 1; i < TC; ++i) Df.push_back(C[i] - C[i - 1]);
    for (int i = 0; i < TF - 1; ++i) Dc[i] = F[i + 1] - F[i];
    std::vector<FT> Dff;
    Dff.push_back(Df.front());
    for (FT d : Df) Dff.push_back(d);
    Dff.push_back(Df.back());
    for (int i = (int)Dff.size() - 1; i >= 1; --i) Dff[i] = Dff[i - 1];
    for (int k = kmin; k <= kmax; ++k) {
        int pc = k + H - 1, pf = k + H;
        if (pc >= 0 && pc < (int)Dc.size()) Z.dzc[k + Z.zoff] = Dc[pc];
        if (pf >= 0 && pf < (int)Dff.size()) Z.dzf[k + Z.zoff] = Dff[pf];
        if (pc >= 0 && pc < TF) Z.zf[k + Z.zoff] = F[pc];
        if (pc >= 0 && pc < TC) Z.zc[k + Z.zoff] = C[pc];
    }
    return Z;
}

template <typename FT>
std::vector<Cx<FT>> twiddles(int n, double frac = 1.0) {
    // exp(-2πi m frac / n), m = 0..n-1, evaluated in double on the host
    std::vector<Cx<FT>> t(n);
    for (int m = 0; m < n; ++m) {
        double a = -2.0 * M_PI * frac * (double)m / (double)n;
        t[m] = Cx<FT>{FT(std::cos(a)), FT(std::sin(a))};
    }
    return t;
}

// Poisson eigenvalues (src/Solvers/poisson_eigenvalues.jl:8-23), computed in FP64
double eig_periodic(int i1, int N, double L) { double s = 2 * std::sin((i1 - 1) * M_PI / N) / (L / N); return s * s; }
double eig_bounded(int i1, int N, double L) { double s = 2 * std::sin((i1 - 1) * M_PI / (2 * N)) / (L / N); return s * s; }

}  // namespace

// ===========================================================================
// Model
// ===========================================================================
struct gbo_model {
    virtual ~gbo_model() {}
    std::string err;
    int dtype = GBO_FLOAT64;
    gbo_grid_desc grid{};
    gbo_model_desc desc{};
    int Nx = 0, Ny = 0, Nz = 0;
    bool flat = false;
    double time = 0;
    int64_t iteration = 0;
    int last_iters = 0;
    int device = 0;
    virtual int set_field(int field, const void* host, int dtype, int64_t count) = 0;
    virtual int get_field(int field, void* host, int dtype, int64_t count) = 0;
    virtual int set_finalize(int enforce) = 0;
    virtual int step(double dt, int nsteps) = 0;
    virtual int sync() = 0;
    virtual int device_pointer(int field, void** p, int64_t* n) = 0;
    virtual int reference_profile(int field, double* out, int64_t n) = 0;
    virtual int poisson_device(void* phi, const void* rhs) = 0;
    virtual int64_t state_bytes() const = 0;
    virtual int get_state(void* buf, int64_t bytes) = 0;
    virtual int set_state(const void* buf, int64_t bytes) = 0;
    virtual int run(const gbo_run_desc* d, gbo_run_result* out) = 0;
    virtual int set_learned(const float* weights, int64_t count) = 0;
    virtual int operator_device(const void* x, void* out) = 0;
    virtual int precondition_device(const void* r, void* z) = 0;
    virtual void abort_capture() = 0;
    bool ensemble_member = false;
    virtual int timescales(double* adv, double* dif) = 0;
    virtual int timed_steps(double dt, int nsteps, double* ms, int nmax) = 0;
    virtual int timing_counts(int64_t* n, int nmax) const = 0;
    virtual void* stream_ptr() = 0;
    virtual int64_t capture_step(const float* dtf32, const double* dtf64) = 0;
    virtual void add_launches(int64_t n) = 0;
    virtual int finish_steps(double dt, int nsteps) = 0;
    virtual int64_t launch_count() const = 0;
    virtual int launch_shape(gbo_launch_shape* s) const = 0;
    virtual int set_launch_shape(const gbo_launch_shape* s) = 0;
    int64_t count(int field) const {
        int64_t plane = (int64_t)Nx * Ny;
        if (field == GBO_FIELD_W) return flat ? plane : plane * (Nz + 1);
        return plane * Nz;
    }
};

enum { G_MOMENTUM = 0, G_TRACER, G_CLOSURE, G_HYDROSTATIC, G_SOURCE, G_DCT_Z, G_FFT_X, G_FFT_Y, G_THOMAS,
       G_CORRECT, G_COPY, G_NAN, G_MASK, G_CG, G_CG_DOT, G_CG_DIR, G_CG_XR, G_CG_GAUGE, G_SIM, G_LEARNED, GROUPS };
const char* const GROUP_NAMES[GROUPS] = {"k_momentum", "k_tracer", "k_closure", "k_hydrostatic", "k_source",
                                         "k_dct_z", "k_rfft_x", "k_fft_y", "k_thomas_z", "k_correct", "k_copy",
                                         "k_nan_check", "k_mask", "k_cg", "k_cg_dot", "k_cg_direction",
                                         "k_cg_update_xr", "k_cg_gauge", "k_simulation", "k_cg_learned"};

// The fused momentum kernel is compiled per closure kind in its own translation units
// (gbo_fused_*.cu, compiled in parallel); these pick the instance.
template <typename FT, bool TR>
void launch_fused(int closure, bool ibg, dim3 grid, dim3 block, cudaStream_t st, const StepP<FT>& P, int kchunk);
template <typename FT, bool TR>
cudaError_t fused_set_smem_tr();
template <typename FT>
cudaError_t fused_set_smem() {
    cudaError_t a = fused_set_smem_tr<FT, true>(), b = fused_set_smem_tr<FT, false>();
    return a != cudaSuccess ? a : b;
}

namespace {

template <typename FT>
struct DBuf {
    FT* p = nullptr;
    size_t n = 0;
    void alloc(size_t count) {
        n = count;
        GBO_CUDA(cudaMalloc(&p, std::max<size_t>(1, count) * sizeof(FT)));
        GBO_CUDA(cudaMemset(p, 0, std::max<size_t>(1, count) * sizeof(FT)));
    }
    void free_() {
        if (p) cudaFree(p);
        p = nullptr;
    }
    template <typename T>
    void upload(const std::vector<T>& h) {
        alloc(h.size());
        GBO_CUDA(cudaMemcpy(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
    }
};

template <typename FT>
struct ModelImpl : gbo_model {
    using C = Cx<FT>;
    cudaStream_t stream = nullptr;
    int ntr = 0;
    bool has_phy = false;
    size_t N = 0;  // Nx*Ny*Nz
    // state and work arrays
    DBuf<FT> u, v, w, us, vs, ws, Gu, Gv, Gw, nu, phy, p;
    std::vector<DBuf<FT>> c, cs, Gc, kap;
    // tracer departures (single precision on a Bounded z): per-level reference profiles on
    // the device and on the host, and a staging buffer for set / get conversions
    bool departures = false;
    std::vector<DBuf<FT>> cref;
    std::vector<std::vector<double>> cref_h;
    DBuf<double> tstage, tmean;
    // DynamicSmagorinsky: Σ, Σ̄, per-tile LM/MM sums, and per level c², 𝒥ᴸᴹ, 𝒥ᴹᴹ
    DBuf<FT> dyn_sig, dyn_sigb, dyn_cs2, dyn_jlm, dyn_jmm, dyn_lmv, dyn_mmv;  // lmv, mmv: per-cell LM, MM (x-y average)
    DBuf<double> dyn_part;
    // DynamicSmagorinsky with LagrangianAveraging: 𝒥ᴸᴹ, 𝒥ᴹᴹ and their previous values, the
    // FP64 clock slots (LAG_*), the cell-centre z, and where the step being recorded reads
    // its FP64 Δt (the plain step's slot, or the simulation loop's)
    bool lagrangian = false, velocities_set = false, stretched_z = false;
    DBuf<FT> lag_jlm, lag_jmm, lag_jlm_prev, lag_jmm_prev;
    DBuf<double> lag_s, lag_zc;
    const double* lag_dtp = nullptr;
    double lag_x0 = 0, lag_y0 = 0;
    // grid tables
    DBuf<FT> t_dzc, t_dzf, t_rdzc, t_rdzf, t_rvc;
    DBuf<double> t_rdzf64, t_dzc64, t_lx64, t_ly64, t_ws;
    DBuf<int> t_kbot;
    ZGrid<FT> Z;
    GridP<FT> gp{};
    // Poisson solver
    DBuf<FT> rb, lx, ly, lz;
    DBuf<C> cb, tw_xh, tw_x, tw_y, tw_z, tq_z;
    // immersed boundary and conjugate-gradient solver
    bool ibg = false, cg = false;
    int precond_solver = GBO_SOLVER_FFT;  // spectral solver of the underlying grid
    DBuf<FT> cg_b, cg_r, cg_q, cg_d, cg_p1, cg_x;  // cg_d / cg_p1: search directions by parity
    DBuf<double> cg_s;
    DBuf<unsigned int> cg_cnt;
    double* h_cgs = nullptr;
    int cg_status = GBO_OK;
    cudaStream_t body_stream = nullptr;  // captures the CG loop body into a conditional node
    int64_t body_launches = 0;           // kernels per CG iteration
    double iters_seen = 0;               // CG_ITERS already accounted in `launches`
    PassP<FT> pp{};
    ThomasP tp{};
    int ZT = GBO_DCT_TILE, XL = 8, YT = 16;
    int kchunk = 16;  // levels marched per block by the fused momentum kernel
    size_t smem_z = 0, smem_x = 0, smem_y = 0;
    // flags
    unsigned int* d_flags = nullptr;
    unsigned int* h_flags = nullptr;
    // graph of one time step (Δt is read from the stage factors dtf, so one graph serves every Δt)
    cudaGraphExec_t graph = nullptr;
    cudaGraphExec_t graph_euler = nullptr;  // QAB2: the Euler step
    bool use_graph = true;
    bool qab2 = false;
    double last_dt = INFINITY;           // clock.last_Δt
    // simulation loop (gbo_run): state slots, block partials, graph of the loop
    DBuf<FT> dtf;                        // stage factors of the current Δt (DTF_*)
    LearnedNet* net = nullptr;           // learned correction of the CG preconditioner
    DBuf<FT> cg_rp;                      // previous residual (flexible CG)
    DBuf<double> run_s, run_part;
    DBuf<unsigned int> run_cnt;
    double* h_run = nullptr;
    cudaStream_t run_stream = nullptr;   // captures the loop body into a conditional node
    cudaStream_t if_stream = nullptr;    // captures the Euler / AB2 branches (QAB2)
    cudaGraphExec_t run_graph = nullptr;
    int64_t run_iter_launches = 0;       // kernels per loop iteration (CG iterations apart)

    ~ModelImpl() override {
        if (graph) cudaGraphExecDestroy(graph);
        if (graph_euler) cudaGraphExecDestroy(graph_euler);
        if (run_graph) cudaGraphExecDestroy(run_graph);
        if (net) learned_destroy(net);
        cg_rp.free_();
        dtf.free_();
        run_s.free_();
        run_part.free_();
        run_cnt.free_();
        if (h_run) cudaFreeHost(h_run);
        if (run_stream) cudaStreamDestroy(run_stream);
        if (if_stream) cudaStreamDestroy(if_stream);
        for (DBuf<FT>* b : {&u, &v, &w, &us, &vs, &ws, &Gu, &Gv, &Gw, &nu, &phy, &p, &t_dzc, &t_dzf, &t_rdzc, &t_rdzf, &t_rvc, &rb, &lx, &ly, &lz,
                            &cg_b, &cg_r, &cg_q, &cg_d, &cg_p1, &cg_x})
            b->free_();
        cg_s.free_();
        cg_cnt.free_();
        if (h_cgs) cudaFreeHost(h_cgs);
        if (body_stream) cudaStreamDestroy(body_stream);
        for (auto* vec : {&c, &cs, &Gc, &kap, &cref})
            for (auto& b : *vec) b.free_();
        tstage.free_();
        tmean.free_();
        t_rdzf64.free_(); t_dzc64.free_(); t_lx64.free_(); t_ly64.free_(); t_ws.free_(); t_kbot.free_();
        for (DBuf<C>* b : {&cb, &tw_xh, &tw_x, &tw_y, &tw_z, &tq_z}) b->free_();
        for (DBuf<FT>* b : {&dyn_sig, &dyn_sigb, &dyn_cs2, &dyn_jlm, &dyn_jmm, &dyn_lmv, &dyn_mmv, &lag_jlm, &lag_jmm,
                            &lag_jlm_prev, &lag_jmm_prev})
            b->free_();
        dyn_part.free_();
        lag_s.free_();
        lag_zc.free_();
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (join_ev) cudaEventDestroy(join_ev);
        if (d_flags) cudaFree(d_flags);
        if (h_flags) cudaFreeHost(h_flags);
        if (stream) cudaStreamDestroy(stream);
    }

    void init(const gbo_grid_desc* gd, const gbo_model_desc* md) {
        grid = *gd;
        grid.z_faces = nullptr;
        grid.bottom_height = nullptr;
        desc = *md;
        dtype = sizeof(FT) == 4 ? GBO_FLOAT32 : GBO_FLOAT64;
        Nx = gd->size[0];
        Ny = gd->size[1];
        flat = gd->topology[2] == GBO_FLAT;
        Nz = flat ? 1 : gd->size[2];
        ntr = md->ntracers;
        has_phy = !flat && md->buoyancy_tracer && ntr > 0;
        N = (size_t)Nx * Ny * Nz;
        GBO_CUDA(cudaGetDevice(&device));
        GBO_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        // grid tables
        const int H = gd->bottom_height ? 4 : 3;
        Z = make_zgrid<FT>(Nz, H, flat, gd->z_faces, gd->z[0], gd->z[1]);
        stretched_z = gd->z_faces != nullptr;
        std::vector<FT> rdzc(Z.dzc.size()), rdzf(Z.dzf.size());
        std::vector<double> rdzf64(Z.dzf.size()), dzc64(Z.dzc.size());
        for (size_t q = 0; q < Z.dzc.size(); ++q) {
            rdzc[q] = FT(1) / Z.dzc[q];
            rdzf[q] = FT(1) / Z.dzf[q];
            rdzf64[q] = 1.0 / (double)Z.dzf[q];
            dzc64[q] = (double)Z.dzc[q];
        }
        t_dzc.upload(Z.dzc); t_dzf.upload(Z.dzf); t_rdzc.upload(rdzc); t_rdzf.upload(rdzf);
        t_rdzf64.upload(rdzf64); t_dzc64.upload(dzc64);
        double Lx = gd->x[1] - gd->x[0], Ly = gd->y[1] - gd->y[0];
        gp.Nx = Nx; gp.Ny = Ny; gp.Nz = Nz; gp.flatz = flat; gp.zoff = Z.zoff;
        gp.dx = FT(Lx / Nx); gp.dy = FT(Ly / Ny);
        gp.rdx = FT(1) / gp.dx; gp.rdy = FT(1) / gp.dy;
        gp.dzc = t_dzc.p; gp.dzf = t_dzf.p; gp.rdzc = t_rdzc.p; gp.rdzf = t_rdzf.p;
        {
            // 1/Vᶜᶜᶜ = FT(1) / ((Δx Δy) Δzᶜ), the operation order of Met::rVc
            std::vector<FT> rvc(Z.dzc.size());
            const FT az = gp.dx * gp.dy;
            for (size_t q = 0; q < rvc.size(); ++q) rvc[q] = FT(1) / (az * Z.dzc[q]);
            t_rvc.upload(rvc);
            gp.rvc = t_rvc.p;
        }
        gp.kbot = nullptr;
        if (gd->bottom_height) {
            // GridFittedBottom: a cell is immersed iff its centre lies at or below the bottom
            // (grid_fitted_bottom.jl:118-158); kbot = index of the first active level.
            std::vector<int> kb((size_t)Nx * Ny);
            for (size_t q = 0; q < kb.size(); ++q) {
                double h = gd->bottom_height[q];
                int first = 0;
                for (int k = 0; k < Nz; ++k)
                    if ((double)Z.at(Z.zc, k + 1) <= h) first = k + 1;
                kb[q] = first;
            }
            t_kbot.upload(kb);
            gp.kbot = t_kbot.p;
            ibg = true;
        }
        cg = md->pressure_solver == GBO_SOLVER_CONJUGATE_GRADIENT;
        // the FFT preconditioner is the spectral solver of the underlying grid
        // (conjugate_gradient_poisson_solver.jl:141-147): Fourier-tridiagonal when z is stretched
        precond_solver = gd->z_faces ? GBO_SOLVER_FOURIER_TRIDIAGONAL : GBO_SOLVER_FFT;
        // fields
        for (DBuf<FT>* b : {&u, &v, &us, &vs, &Gu, &Gv, &p, &rb}) b->alloc(N);
        if (!flat) { w.alloc(N); ws.alloc(N); Gw.alloc(N); }
        const bool scalar = md->closure == GBO_CLOSURE_SCALAR_DIFFUSIVITY;
        if (md->closure != GBO_CLOSURE_NONE && !scalar) nu.alloc(N);
        if (has_phy) phy.alloc(N);
        c.resize(ntr); cs.resize(ntr); Gc.resize(ntr);
        for (int n = 0; n < ntr; ++n) { c[n].alloc(N); cs[n].alloc(N); Gc[n].alloc(N); }
        departures = sizeof(FT) == 4 && !flat && ntr > 0;
        if (departures) {
            cref.resize(ntr);
            cref_h.assign(ntr, std::vector<double>(Nz, 0.0));
            for (int n = 0; n < ntr; ++n) cref[n].upload(std::vector<FT>(Nz, FT(0)));
            tstage.alloc(N);
            tmean.alloc(Nz);
        }
        if (md->closure == GBO_CLOSURE_AMD) {
            kap.resize(ntr);
            for (int n = 0; n < ntr; ++n) kap[n].alloc(N);
        }
        if (md->closure == GBO_CLOSURE_DYNAMIC_SMAGORINSKY) {
            dyn_sig.alloc(N);
            dyn_sigb.alloc(N);
            dyn_part.alloc(std::max<size_t>((size_t)2 * Nz * ((Nx + dyn::TX - 1) / dyn::TX) * ((Ny + dyn::TY - 1) / dyn::TY),
                                            (size_t)2 * LAG_SUM_BLOCKS));
            for (DBuf<FT>* b : {&dyn_cs2, &dyn_jlm, &dyn_jmm}) b->alloc(Nz);
            lagrangian = md->closure_averaging == GBO_AVERAGING_LAGRANGIAN;
            GBO_CUDA(dyn_set_smem<FT>());
            if (!lagrangian) {
                dyn_lmv.alloc(N);
                dyn_mmv.alloc(N);
            }
        }
        if (lagrangian) {
            for (DBuf<FT>* b : {&lag_jlm, &lag_jmm, &lag_jlm_prev, &lag_jmm_prev}) b->alloc(N);
            std::vector<double> zc(Nz);
            // the grid's FT nodes (the reference interpolates on eltype(grid) coordinates)
            for (int k = 0; k < Nz; ++k) zc[k] = (double)(FT)Z.at(Z.zc, k + 1);
            lag_zc.upload(zc);
            lag_x0 = gd->x[0];
            lag_y0 = gd->y[0];
            // the constructor's initialize_closure_fields! sees zero velocities (LM = MM = 0):
            // 𝒥ᴸᴹ = max(0, minimum_numerator), 𝒥ᴹᴹ = 0, previous_compute_time = 0
            std::vector<double> s0(LAG_NSLOTS, 0.0);
            const FT lmin = FT(md->closure_min_numerator);
            s0[LAG_LM0] = (double)(lmin > FT(0) ? lmin : FT(0));
            lag_s.upload(s0);
            k_lag_fill<FT><<<conv_blocks(), 256, 0, stream>>>(lag_s.p, lag_jlm.p, lag_jmm.p, N);
            GBO_CUDA(cudaGetLastError());
            lag_dtp = lag_s.p + LAG_DT;
        }
        if (scalar) {
            kap.resize(ntr);
            // constant ν and κ held as fields: the AMD flux code reads them, and ν at
            // edges, ½(a + a) and ¼(4a), is a exactly as the reference's constant
            nu.upload(std::vector<FT>(N, FT(md->closure_nu)));
            for (int n = 0; n < ntr; ++n) kap[n].upload(std::vector<FT>(N, FT(md->closure_kappa[n])));
        }
        qab2 = md->timestepper == GBO_TIMESTEPPER_QAB2;
        GBO_CUDA(cudaMalloc(&d_flags, sizeof(unsigned int)));
        GBO_CUDA(cudaMemset(d_flags, 0, sizeof(unsigned int)));
        GBO_CUDA(cudaMallocHost(&h_flags, sizeof(unsigned int)));
        dtf.alloc(DTF_N);
        run_s.alloc(RUN_NSLOTS);
        run_part.alloc((size_t)SIM_BLOCKS * SIM_PARTS);
        run_cnt.alloc(1);
        GBO_CUDA(cudaMallocHost(&h_run, RUN_NSLOTS * sizeof(double)));
        init_poisson(Lx, Ly);
        if (cg) {
            for (DBuf<FT>* b : {&cg_b, &cg_r, &cg_q, &cg_d, &cg_p1, &cg_x}) b->alloc(N);
            // the scalar slots, then two partial sums per block of the largest CG reduction launch
            const dim3 cgg = cg_grid();
            cg_s.alloc(CG_NSLOTS + 2 * std::max<size_t>((size_t)cgg.x * cgg.y * cgg.z, 152 * 8));
            cg_cnt.alloc(CC_N);
            GBO_CUDA(cudaMallocHost(&h_cgs, CG_NSLOTS * sizeof(double)));
            GBO_CUDA(cudaStreamCreateWithFlags(&body_stream, cudaStreamNonBlocking));
            k_cg_count<FT><<<cg_grid(), blk(), 0, stream>>>(gp, cg_s.p, cg_cnt.p);
            GBO_CUDA(cudaGetLastError());
            GBO_CUDA(cudaStreamSynchronize(stream));
        }
    }

    void init_poisson(double Lx, double Ly) {
        const int Nh = Nx / 2 + 1;
        pp.Nx = Nx; pp.Ny = Ny; pp.Nz = Nz; pp.Nh = Nh;
        if (!make_plan(Nx / 2, pp.px_half) || !make_plan(Ny, pp.py) || !make_plan(Nz, pp.pz))
            throw InvalidArg{"grid sizes must factor into 2, 3 and 5 for the spectral Poisson solvers"};
        cb.alloc((size_t)Nh * Ny * Nz);
        pp.rb = rb.p;
        pp.cb = cb.p;
        tw_xh.upload(twiddles<FT>(Nx / 2));
        tw_x.upload(twiddles<FT>(Nx));
        tw_y.upload(twiddles<FT>(Ny));
        tw_z.upload(twiddles<FT>(Nz));
        tq_z.upload(twiddles<FT>(Nz, 0.25));  // exp(-iπk/(2Nz))
        pp.tw_xh = tw_xh.p; pp.tw_x = tw_x.p; pp.tw_y = tw_y.p; pp.tw_z = tw_z.p; pp.tq_z = tq_z.p;
        const double Lxf = (double)FT(Lx), Lyf = (double)FT(Ly), Lzf = (double)Z.Lz;
        std::vector<FT> hx(Nh), hy(Ny), hz(Nz);
        std::vector<double> hx64(Nh), hy64(Ny);
        for (int q = 0; q < Nh; ++q) { hx64[q] = eig_periodic(q + 1, Nx, Lxf); hx[q] = FT(hx64[q]); }
        for (int q = 0; q < Ny; ++q) { hy64[q] = eig_periodic(q + 1, Ny, Lyf); hy[q] = FT(hy64[q]); }
        for (int q = 0; q < Nz; ++q) hz[q] = flat ? FT(0) : FT(eig_bounded(q + 1, Nz, Lzf));
        lx.upload(hx); ly.upload(hy); lz.upload(hz);
        t_lx64.upload(hx64); t_ly64.upload(hy64);
        pp.lx = lx.p; pp.ly = ly.p; pp.lz = lz.p;
        pp.has_z = !flat;
        pp.scale = flat ? FT(1.0 / ((double)Nx * Ny)) : FT(1.0 / ((double)Nx * Ny * Nz));
        tp.Nh = Nh; tp.Ny = Ny; tp.Nz = Nz;
        tp.rdzf = t_rdzf64.p; tp.dzc = t_dzc64.p; tp.zoff = Z.zoff;
        tp.lx = t_lx64.p; tp.ly = t_ly64.p;
        tp.scale = 1.0 / ((double)Nx * Ny);
        // FP64 work space of the Thomas sweep, for models that use the Fourier-tridiagonal solver
        // (as the pressure solver or as the CG preconditioner on a stretched grid)
        if (desc.pressure_solver == GBO_SOLVER_FOURIER_TRIDIAGONAL ||
            (desc.pressure_solver == GBO_SOLVER_CONJUGATE_GRADIENT && precond_solver == GBO_SOLVER_FOURIER_TRIDIAGONAL)) {
            const size_t cl = (size_t)Nz * Nh * Ny;
            t_ws.alloc(4 * cl);  // forward-sweep re, im; then the pivot tables
            tp.ws = t_ws.p;
            tp.tab_s = t_ws.p + 2 * cl;
            tp.tab_t = t_ws.p + 3 * cl;
            launch_thomas_tables(tp, stream);
            GBO_CUDA(cudaGetLastError());
        }
        // shared-memory tiles: the tuned shape of this size class, else keep each block at
        // or below ~100 KB
        const size_t lim = GBO_PASS_SMEM_LIMIT;
        ZT = GBO_DCT_TILE;
        while (ZT > 2 && dct_smem<FT>(ZT, Nz) > lim) ZT /= 2;
        XL = 8;
        // two buffers of XL lines of Nx/2 coefficients, plus XL for staging Nx/2+1 per line
        while (XL > 1 && rfft_smem<FT>(XL, Nx) > lim) XL /= 2;
        YT = 16;
        while (YT > 1 && ffty_smem<FT>(YT, Ny) > lim) YT /= 2;
        kchunk = flat ? 1 : std::min(16, Nz);
        if (const LaunchShapeEntry* t = tuned_shape(Nx, Ny, Nz, sizeof(FT) == 8, ibg)) {
            ZT = t->dct_columns;
            XL = t->x_lines;
            YT = t->y_columns;
            if (!flat) kchunk = std::min(t->levels, Nz);
        }
        pass_smem();
        GBO_CUDA(fused_set_smem<FT>());
        GBO_CUDA(cudaFuncSetAttribute(k_smagorinsky_tiled<FT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(smag::SmemS<FT>)));
        GBO_CUDA(cudaFuncSetAttribute(k_amd_tiled<FT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(smag::SmemA<FT>)));
        GBO_CUDA(cudaFuncSetAttribute(k_amd_tiled_ibg<FT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(smag::Smem<FT>)));
        // The pass kernels are shared by every model in the process: allow them the device's
        // opt-in maximum rather than this model's sizes, so a model created later never
        // lowers the limit an earlier, larger model needs.
        int optin = 0;
        GBO_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
        if ((size_t)optin < std::max({smem_z, smem_x, smem_y}))
            throw InvalidArg{"grid too large for the shared-memory tiles of the spectral Poisson solver"};
        GBO_CUDA(fft_set_smem<FT>(optin, optin, optin));
    }

    // shared memory of the pass kernels at the current tiles
    void pass_smem() {
        smem_z = dct_smem<FT>(ZT, Nz);
        smem_x = rfft_smem<FT>(XL, Nx);
        smem_y = ffty_smem<FT>(YT, Ny);
    }
    int launch_shape(gbo_launch_shape* s) const override {
        *s = gbo_launch_shape{ZT, XL, YT, kchunk};
        return GBO_OK;
    }
    int set_launch_shape(const gbo_launch_shape* s) override {
        if (ensemble_member) { err = "the launch shape of an ensemble member cannot change"; return GBO_ERR_INVALID; }
        if (s->dct_columns < 2 || s->dct_columns > 64 || !pow2(s->dct_columns) || s->x_lines < 1 || s->x_lines > 32 ||
            s->y_columns < 1 || s->y_columns > 64 || !pow2(s->y_columns) || s->levels < 1 || s->levels > Nz ||
            (flat && s->levels != 1)) {
            err = "launch shape out of range (DCT and y-FFT tiles are powers of two)";
            return GBO_ERR_INVALID;
        }
        int optin = 0;
        GBO_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
        if (dct_smem<FT>(s->dct_columns, Nz) > (size_t)optin || rfft_smem<FT>(s->x_lines, Nx) > (size_t)optin ||
            ffty_smem<FT>(s->y_columns, Ny) > (size_t)optin) {
            err = "launch shape needs more shared memory per block than the device has";
            return GBO_ERR_INVALID;
        }
        GBO_CUDA(cudaStreamSynchronize(stream));
        drop_graphs();
        ZT = s->dct_columns;
        XL = s->x_lines;
        YT = s->y_columns;
        kchunk = s->levels;
        pass_smem();
        return GBO_OK;
    }

    // ------------------------------------------------------------------
    dim3 blk() const { return dim3(32, 8, 1); }
    dim3 grd() const { return dim3((Nx + 31) / 32, (Ny + 7) / 8, Nz); }
    dim3 cg_grid() const { return dim3((Nx + 31) / 32, (Ny + 7) / 8, std::min(Nz, CG_ZSLICES)); }
    dim3 col_grid() const { return dim3((Nx + 31) / 32, (Ny + 7) / 8, (Nz + COL_LEVELS - 1) / COL_LEVELS); }

    // kernel accounting: group of the next launch, launches per captured step,
    // optional per-group CUDA events (timing mode)
    int64_t launches = 0, graph_launches_per_step = 0;
    bool timing = false;
    int cur_group = 0;
    std::vector<double> group_ms = std::vector<double>(GROUPS, 0.0);
    std::vector<int64_t> group_n = std::vector<int64_t>(GROUPS, 0);
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;

    void pre(int group) {
        cur_group = group;
        if (timing) GBO_CUDA(cudaEventRecord(ev0, stream));
    }
    void check_launch() {
        GBO_CUDA(cudaGetLastError());
        launches += 1;
        if (timing) {
            GBO_CUDA(cudaEventRecord(ev1, stream));
            GBO_CUDA(cudaEventSynchronize(ev1));
            float ms = 0;
            GBO_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
            group_ms[cur_group] += ms;
            group_n[cur_group] += 1;
        }
    }

    // Flux code of the closure: ScalarDiffusivity runs the AMD fluxes on its constant
    // ν and κ fields (viscous fluxes 2νΣᵢⱼ and diffusive fluxes κ∂c of
    // abstract_scalar_diffusivity_closure.jl:214-262 for every AbstractScalarDiffusivity)
    int kernel_closure() const {
        if (desc.closure == GBO_CLOSURE_DYNAMIC_SMAGORINSKY) return CL_SMAG;  // the νₑ fluxes of every Smagorinsky
        return desc.closure == GBO_CLOSURE_SCALAR_DIFFUSIVITY ? (int)CL_AMD : desc.closure;
    }

    const FT* tracer_ref(int n) const { return departures && n < ntr ? cref[n].p : nullptr; }

    StepP<FT> params() {
        StepP<FT> P{};
        P.g = gp;
        P.u = u.p; P.v = v.p; P.w = flat ? nullptr : w.p;
        P.nu = nu.p; P.phy = phy.p;
        P.b = (desc.buoyancy_tracer && ntr > 0) ? c[0].p : nullptr;
        P.bref = (desc.buoyancy_tracer && departures) ? cref[0].p : nullptr;
        P.cref = nullptr;
        P.uo = us.p; P.vo = vs.p; P.wo = flat ? nullptr : ws.p;
        P.Gu = Gu.p; P.Gv = Gv.p; P.Gw = flat ? nullptr : Gw.p;
        P.f = FT(desc.coriolis_f);
        P.has_cor = desc.has_coriolis;
        P.has_phy = has_phy;
        P.closure = kernel_closure();
        P.buoyancy = desc.buoyancy_tracer && ntr > 0;
        P.Pr = FT(desc.closure_Pr);
        P.C = FT(desc.closure_C);
        P.Cb = FT(desc.closure_Cb);
        return P;
    }

    // Spectral solve of ∇²ϕ = rb in place (rb holds the source on entry, ϕ on exit)
    // with the FFT or the Fourier-tridiagonal solver.
    void poisson_solve(int solver) {
        if (solver == GBO_SOLVER_FOURIER_TRIDIAGONAL) {
            pre(G_FFT_X);
            launch_rfft_x<FT>(pp, 0, XL, smem_x, stream);
            check_launch();
            pre(G_FFT_Y);
            launch_fft_y<FT>(pp, 1, YT, smem_y, stream);
            check_launch();
            pre(G_THOMAS);
            launch_thomas_z<FT>(pp, tp, stream);
            check_launch();
            pre(G_FFT_Y);
            launch_fft_y<FT>(pp, 2, YT, smem_y, stream);
            check_launch();
            pre(G_FFT_X);
            launch_rfft_x<FT>(pp, 1, XL, smem_x, stream);
            check_launch();
            return;
        }
        if (!flat) {
            pre(G_DCT_Z);
            launch_dct_z<FT>(pp, 0, ZT, smem_z, stream);
            check_launch();
        }
        pre(G_FFT_X);
        launch_rfft_x<FT>(pp, 0, XL, smem_x, stream);
        check_launch();
        pre(G_FFT_Y);
        launch_fft_y<FT>(pp, 0, YT, smem_y, stream);
        check_launch();
        pre(G_FFT_X);
        launch_rfft_x<FT>(pp, 1, XL, smem_x, stream);
        check_launch();
        if (!flat) {
            pre(G_DCT_Z);
            launch_dct_z<FT>(pp, 1, ZT, smem_z, stream);
            check_launch();
        }
    }

    // compute_pressure_correction! + make_pressure_correction! on the predictor (us, vs, ws)
    // writing the state (u, v, w) and p; in == out is allowed.
    // With rdp / scp set, 1/max(eps, Δτ) and max(eps, Δτ) are read on the device.
    void project(FT* ui, FT* vi, FT* wi, double dtau, const FT* rdp = nullptr, const FT* scp = nullptr) {
        const double eps = machine_eps<FT>();
        if (ibg) {  // mask_immersed_field! on the velocities (pressure_correction.jl:9)
            pre(G_MASK);
            k_mask<FT><<<grd(), blk(), 0, stream>>>(gp, ui, vi, wi, nullptr, flat ? 3 : 7);
            check_launch();
        }
        const FT* phi = rb.p;
        if (cg) {
            cg_status = cg_solve(ui, vi, wi, std::max(eps, dtau) * (std::isfinite(dtau) ? 1.0 : 0.0), scp);
            phi = cg_x.p;
        } else {
            int mode = desc.pressure_solver == GBO_SOLVER_FOURIER_TRIDIAGONAL ? SRC_FT : SRC_FFT;
            pre(G_SOURCE);
            k_source<FT><<<col_grid(), blk(), 0, stream>>>(gp, ui, vi, wi, rb.p, mode);
            check_launch();
            poisson_solve(desc.pressure_solver);
        }
        FT rdtau = FT(1) / FT(std::max(eps, dtau));
        pre(G_CORRECT);
        k_correct<FT><<<col_grid(), blk(), 0, stream>>>(gp, ui, vi, wi, phi, u.p, v.p, flat ? nullptr : w.p, p.p, rdtau, FT(0),
                                                   rdp);
        check_launch();
    }

    // Preconditioned conjugate gradient for V∇²x = V·div u* with x₀ = p·Δτ
    // (solve_for_pressure.jl:52-72; conjugate_gradient_solver.jl:177-284).  Each
    // iteration reads ‖V⁻¹r‖ back to the host for the stopping test.
    int cg_solve(const FT* ui, const FT* vi, const FT* wi, double dtp, const FT* scp = nullptr) {
        const unsigned lin = (unsigned)std::min<size_t>((N + 255) / 256, 4 * 152 * 8);
        pre(G_CG);
        k_cg_scale<FT><<<lin, 256, 0, stream>>>(p.p, cg_x.p, FT(dtp), N, scp);
        check_launch();
        pre(G_SOURCE);
        k_source<FT><<<col_grid(), blk(), 0, stream>>>(gp, ui, vi, wi, cg_b.p, SRC_CG);
        check_launch();
        return cg_iterate();
    }

    // One CG iteration (iterate!, conjugate_gradient_solver.jl:202-235) and the stopping
    // test; rb holds the preconditioner's right-hand side on entry.
    void cg_body(double maxiter, cudaGraphConditionalHandle h, int use_handle) {
        const unsigned lin = (unsigned)std::min<size_t>((N + 255) / 256, 4 * 152 * 8);
        const bool pc = desc.preconditioner == GBO_PRECOND_FFT;
        const int dzs = precond_solver == GBO_SOLVER_FOURIER_TRIDIAGONAL;
        double* s = cg_s.p;
        const FT* z = cg_r.p;
        if (pc) {
            poisson_solve(precond_solver);
            z = rb.p;
            learned_correction(cg_r.p, rb.p);
        }
        FT* rprev = net ? cg_rp.p : nullptr;
        pre(G_CG_DOT);
        // one block per SM × 8: each thread sums several 16-byte vectors before the block
        // reduction, so few blocks reach the FP64 atomics and the completion ticket
        const unsigned dot_blocks = (unsigned)std::min<size_t>((N / 4 + 255) / 256 + 1, 152 * 8);
        k_cg_dot<FT><<<dot_blocks, 256, 0, stream>>>(z, cg_r.p, N, s, cg_cnt.p, h, use_handle, rprev);
        check_launch();
        pre(G_CG_DIR);
        k_cg_direction<FT><<<cg_grid(), blk(), 0, stream>>>(gp, z, cg_d.p, cg_p1.p, cg_q.p, s, cg_cnt.p);
        check_launch();
        pre(G_CG_XR);
        k_cg_update_xr<FT><<<cg_grid(), blk(), 0, stream>>>(gp, cg_x.p, cg_r.p, cg_d.p, cg_p1.p, cg_q.p, s, cg_cnt.p, rprev);
        check_launch();
        pre(G_CG_GAUGE);
        k_cg_gauge<FT><<<cg_grid(), blk(), 0, stream>>>(gp, cg_x.p, cg_r.p, pc ? rb.p : nullptr, s, dzs, cg_cnt.p,
                                                         maxiter, h, use_handle);
        check_launch();
    }

    // z += s · net(r / s, z / s, active) when a learned correction is loaded
    void learned_correction(const FT* r, FT* z) {
        if (!net) return;
        pre(G_LEARNED);
        const int nk = learned_apply(net, r, z, gp.kbot, sizeof(FT) == 8, stream, d_flags);
        check_launch();
        launches += nk - 1;
    }

    // The device-pointer entry points read buffers their caller has just written: order
    // this model's (non-blocking) stream after the work already issued to the legacy
    // default stream, where PyTorch and most callers issue theirs, without a host wait.
    cudaEvent_t join_ev = nullptr;
    void join_caller() {
        if (!join_ev) GBO_CUDA(cudaEventCreateWithFlags(&join_ev, cudaEventDisableTiming));
        GBO_CUDA(cudaEventRecord(join_ev, cudaStreamLegacy));
        GBO_CUDA(cudaStreamWaitEvent(stream, join_ev, 0));
    }

    void drop_graphs() {
        if (graph) { GBO_CUDA(cudaGraphExecDestroy(graph)); graph = nullptr; }
        if (graph_euler) { GBO_CUDA(cudaGraphExecDestroy(graph_euler)); graph_euler = nullptr; }
        if (run_graph) { GBO_CUDA(cudaGraphExecDestroy(run_graph)); run_graph = nullptr; }
    }

    int set_learned(const float* weights, int64_t count) override {
        if (!cg || desc.preconditioner != GBO_PRECOND_FFT) {
            err = "the learned correction needs the ConjugateGradientPoissonSolver with its FFT preconditioner";
            return GBO_ERR_INVALID;
        }
        if (ensemble_member) { err = "the preconditioner of an ensemble member cannot change"; return GBO_ERR_INVALID; }
        GBO_CUDA(cudaStreamSynchronize(stream));
        drop_graphs();  // the captured CG loops change
        if (net) { learned_destroy(net); net = nullptr; }
        if (!weights) return GBO_OK;
        std::string why;
        net = learned_create(Nx, Ny, Nz, weights, count, &why);
        if (!net) { err = why; return GBO_ERR_INVALID; }
        if (!cg_rp.p) cg_rp.alloc(N);
        return GBO_OK;
    }

    // V∇²x with the conditional differences of the CG operator (out must not alias x)
    int operator_device(const void* x, void* out) override {
        if (!ibg && !cg) { err = "the CG operator needs an immersed grid or the CG solver"; return GBO_ERR_INVALID; }
        join_caller();
        pre(G_CG);
        k_cg_laplacian<FT><<<cg_grid(), blk(), 0, stream>>>(gp, static_cast<const FT*>(x), static_cast<FT*>(out));
        check_launch();
        return sync();
    }

    // z = M r with the CG preconditioner (FFT solve of V⁻¹r on the underlying grid plus the
    // learned correction when loaded)
    int precondition_device(const void* r, void* z) override {
        if (!cg || desc.preconditioner != GBO_PRECOND_FFT) { err = "the model has no CG preconditioner"; return GBO_ERR_INVALID; }
        const int dzs = precond_solver == GBO_SOLVER_FOURIER_TRIDIAGONAL;
        join_caller();
        GBO_CUDA(cudaMemcpyAsync(cg_r.p, r, N * sizeof(FT), cudaMemcpyDeviceToDevice, stream));
        pre(G_CG);
        k_cg_vinv<FT><<<cg_grid(), blk(), 0, stream>>>(gp, cg_r.p, rb.p, cg_s.p, dzs, cg_cnt.p);
        check_launch();
        poisson_solve(precond_solver);
        learned_correction(cg_r.p, rb.p);
        GBO_CUDA(cudaMemcpyAsync(z, rb.p, N * sizeof(FT), cudaMemcpyDeviceToDevice, stream));
        // k_cg_vinv accumulated ‖V⁻¹r‖² into the solver's scalars: clear it for the next solve
        GBO_CUDA(cudaMemsetAsync(cg_s.p + CG_NORM2, 0, sizeof(double), stream));
        return sync();
    }

    void read_cg_scalars() {
        GBO_CUDA(cudaMemcpyAsync(h_cgs, cg_s.p, CG_NSLOTS * sizeof(double), cudaMemcpyDeviceToHost, stream));
        GBO_CUDA(cudaStreamSynchronize(stream));
    }

    // solve!(x, ::ConjugateGradientSolver, b) on x = cg_x, b = cg_b
    // (conjugate_gradient_solver.jl:177-197).  Under stream capture the loop becomes a
    // conditional WHILE node whose body is captured on body_stream; otherwise the host
    // reads the stop flag after each iteration.  Non-convergence is reported through
    // CG_FAIL when the step (or solve) is synchronised.
    int cg_iterate() {
        double rel, abs_, maxiter;
        cg_parameters(sizeof(FT) == 4 ? GBO_FLOAT32 : GBO_FLOAT64, desc, (int64_t)N, &rel, &abs_, &maxiter);
        // the device loop is additionally capped so that a stagnating solve ends in bounded time
        maxiter = std::min((double)GBO_CG_MAX_ITERATIONS, maxiter);
        const unsigned lin = (unsigned)std::min<size_t>((N + 255) / 256, 4 * 152 * 8);
        const bool pc = desc.preconditioner == GBO_PRECOND_FFT;
        const int dzs = precond_solver == GBO_SOLVER_FOURIER_TRIDIAGONAL;
        double* s = cg_s.p;
        pre(G_CG);
        k_cg_laplacian<FT><<<cg_grid(), blk(), 0, stream>>>(gp, cg_x.p, cg_q.p);
        check_launch();
        pre(G_CG);
        k_cg_init<FT><<<lin, 256, 0, stream>>>(cg_b.p, cg_q.p, cg_r.p, N);
        check_launch();
        pre(G_CG);
        k_cg_vinv<FT><<<cg_grid(), blk(), 0, stream>>>(gp, cg_r.p, pc ? rb.p : nullptr, s, dzs, cg_cnt.p);
        check_launch();
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        GBO_CUDA(cudaStreamIsCapturing(stream, &cs));
        if (cs == cudaStreamCaptureStatusActive) {
            cudaGraph_t g = nullptr;
            const cudaGraphNode_t* deps = nullptr;
            size_t nd = 0;
            GBO_CUDA(cudaStreamGetCaptureInfo(stream, &cs, nullptr, &g, nullptr, nullptr, nullptr));
            cudaGraphConditionalHandle h;
            GBO_CUDA(cudaGraphConditionalHandleCreate(&h, g, 0, 0));
            pre(G_CG);
            k_cg_begin<<<1, 1, 0, stream>>>(s, rel, abs_, maxiter, h, 1);
            check_launch();
            GBO_CUDA(cudaStreamGetCaptureInfo(stream, &cs, nullptr, &g, &deps, nullptr, &nd));
            cudaGraphNodeParams cp = {};
            cp.type = cudaGraphNodeTypeConditional;
            cp.conditional.handle = h;
            cp.conditional.type = cudaGraphCondTypeWhile;
            cp.conditional.size = 1;
            cudaGraphNode_t node;
            GBO_CUDA(cudaGraphAddNode(&node, g, deps, nullptr, nd, &cp));
            cudaGraph_t body = cp.conditional.phGraph_out[0];
            GBO_CUDA(cudaStreamUpdateCaptureDependencies(stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
            GBO_CUDA(cudaStreamBeginCaptureToGraph(body_stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
            struct Swap {  // launches go to `stream`: point it at the body stream meanwhile
                cudaStream_t& a; cudaStream_t& b;
                Swap(cudaStream_t& x, cudaStream_t& y) : a(x), b(y) { std::swap(a, b); }
                ~Swap() { std::swap(a, b); }
            };
            const int64_t before = launches;
            {
                Swap sw(stream, body_stream);
                cg_body(maxiter, h, 1);
            }
            body_launches = launches - before;
            launches = before;  // counted per executed iteration after the step
            cudaGraph_t captured = nullptr;
            GBO_CUDA(cudaStreamEndCapture(body_stream, &captured));
            // the body must hold the dot kernel (clears the loop condition) and the gauge
            // kernel (sets it): every kernel of cg_body is a node of the body graph
            size_t nodes = 0;
            GBO_CUDA(cudaGraphGetNodes(body, nullptr, &nodes));
            if ((int64_t)nodes != body_launches || body_launches < 2)
                throw CudaError{cudaErrorInvalidValue, "CG loop body capture"};
            return GBO_OK;
        }
        pre(G_CG);
        k_cg_begin<<<1, 1, 0, stream>>>(s, rel, abs_, maxiter, 0, 0);
        check_launch();
        read_cg_scalars();
        for (double n = 0; h_cgs[CG_CONT] != 0.0 && n <= maxiter; n += 1.0) {
            cg_body(maxiter, 0, 0);
            read_cg_scalars();
        }
        iters_seen = h_cgs[CG_ITERS];
        last_iters = (int)h_cgs[CG_IT];
        return cg_outcome();
    }

    // CG_FAIL (sticky) -> status; clears it
    int cg_outcome() {
        if (h_cgs[CG_FAIL] != 0.0) {
            GBO_CUDA(cudaMemsetAsync(cg_s.p + CG_FAIL, 0, sizeof(double), stream));
            GBO_CUDA(cudaStreamSynchronize(stream));
            err = "conjugate-gradient Poisson solver did not reach its tolerance within maxiter iterations";
            return GBO_ERR_NOT_CONVERGED;
        }
        return GBO_OK;
    }

    CFld<FT> host_cfld(const FT* a) const { return CFld<FT>{a, Nx, Ny, Nz, flat ? 1 : 0, nullptr}; }
    WFld<FT> host_wfld(const FT* a) const { return WFld<FT>{a, Nx, Ny, Nz}; }
    // the velocities with interior u, v, w and halos from hu, hv, hw
    LagVel<FT> lag_vel(const FT* hu, const FT* hv, const FT* hw) const {
        return LagVel<FT>{{host_cfld(u.p), host_cfld(hu)}, {host_cfld(v.p), host_cfld(hv)}, {host_wfld(w.p), host_wfld(hw)}};
    }
    dim3 dyn_grid() const { return dim3((Nx + dyn::TX - 1) / dyn::TX, (Ny + dyn::TY - 1) / dyn::TY, Nz); }

    // initialize_closure_fields! (dynamic_coefficient.jl:407-437): Σ, Σ̄, LM and MM of the
    // velocities (interior u, v, w; halos from hu, hv, hw) into 𝒥ᴸᴹ, 𝒥ᴹᴹ, then both = their
    // domain means everywhere and previous_compute_time = clock.time
    void lag_initialize(const FT* hu, const FT* hv, const FT* hw) {
        const LagVel<FT> V = lag_vel(hu, hv, hw);
        const dim3 dg = dyn_grid(), db(dyn::TX, dyn::TY);
        pre(G_CLOSURE);
        dyn_launch_sigma<FT>(stream, gp, V, dyn_sig.p, dyn_sigb.p);
        check_launch();
        pre(G_CLOSURE);
        dyn_launch_lm<FT>(stream, gp, V, dyn_sig.p, dyn_sigb.p, lag_jlm.p, lag_jmm.p);
        check_launch();
        const int nparts = LAG_SUM_BLOCKS;
        pre(G_CLOSURE);
        k_lag_sum<FT><<<nparts, 256, 0, stream>>>(lag_jlm.p, lag_jmm.p, N, dyn_part.p);
        check_launch();
        pre(G_CLOSURE);
        k_lag_init_mean<FT><<<1, dyn::COEF_THREADS, 0, stream>>>(dyn_part.p, nparts, (double)N,
                                                                 desc.closure_min_numerator, time, lag_s.p);
        check_launch();
        pre(G_CLOSURE);
        k_lag_fill<FT><<<conv_blocks(), 256, 0, stream>>>(lag_s.p, lag_jlm.p, lag_jmm.p, N);
        check_launch();
    }

    // step_closure_prognostics! (dynamic_coefficient.jl:439-484) after the step's last
    // projection: the projected interior with the predictor's halos, 𝒥⁻ = 𝒥, one
    // Lagrangian update over Δt = clock.time - previous_compute_time, then the clock
    void lag_step() {
        const LagVel<FT> V = lag_vel(us.p, vs.p, ws.p);
        const dim3 dg = dyn_grid(), db(dyn::TX, dyn::TY);
        pre(G_CLOSURE);
        dyn_launch_sigma<FT>(stream, gp, V, dyn_sig.p, dyn_sigb.p);
        check_launch();
        const unsigned cb = (unsigned)std::min<size_t>((N * sizeof(FT) / 16 + 255) / 256 + 1, 4 * 152 * 8);
        pre(G_COPY);
        k_copy<FT><<<cb, 256, 0, stream>>>(lag_jlm.p, lag_jlm_prev.p, N);
        check_launch();
        pre(G_COPY);
        k_copy<FT><<<cb, 256, 0, stream>>>(lag_jmm.p, lag_jmm_prev.p, N);
        check_launch();
        pre(G_CLOSURE);
        dyn_launch_lm<FT>(stream, gp, V, dyn_sig.p, dyn_sigb.p, lag_jlm.p, lag_jmm.p);
        check_launch();
        LagP<FT> L{};
        L.g = gp;
        L.vel = V;
        L.jlm_prev = lag_jlm_prev.p;
        L.jmm_prev = lag_jmm_prev.p;
        L.jlm = lag_jlm.p;
        L.jmm = lag_jmm.p;
        L.lm_min = FT(desc.closure_min_numerator);
        L.x0 = lag_x0;
        L.y0 = lag_y0;
        L.dx = (grid.x[1] - grid.x[0]) / Nx;
        L.dy = (grid.y[1] - grid.y[0]) / Ny;
        // the grid's FT first centres and spacings, promoted
        L.xc0 = (double)(FT)(L.x0 + 0.5 * L.dx);
        L.yc0 = (double)(FT)(L.y0 + 0.5 * L.dy);
        L.rdx = 1.0 / (double)(FT)L.dx;
        L.rdy = 1.0 / (double)(FT)L.dy;
        L.zc = lag_zc.p;
        L.dz1 = (double)(FT)Z.at(Z.dzc, 1);
        L.rdz1 = 1.0 / L.dz1;
        L.stretched = stretched_z ? 1 : 0;
        L.clock = lag_s.p;
        L.dtp = lag_dtp;
        pre(G_CLOSURE);
        k_lag_step<FT><<<dg, db, 0, stream>>>(L);
        check_launch();
        pre(G_CLOSURE);
        k_lag_tick<<<1, 1, 0, stream>>>(lag_s.p, lag_dtp);
        check_launch();
    }
    // Δt (FP64) of the next plain steps, and the clock the updates start from
    void lag_set_dt(double dt) {
        if (!lagrangian) return;
        pre(G_SIM);
        k_lag_set_dt<<<1, 1, 0, stream>>>(lag_s.p, dt, time);
        check_launch();
    }

    // Closure fields and the hydrostatic pressure anomaly of the current state: the part
    // of update_state! (update_nonhydrostatic_model_state.jl:64-83) that the next stage's
    // tendencies read.  Run after every projection, as the reference does.
    // b_pred: the buoyancy predictor still to be stored into b (the hydrostatic scan does it,
    // first, since the closures read b)
    void auxiliaries(const FT* b_pred = nullptr) {
        StepP<FT> P = params();
        if (b_pred) {
            pre(G_HYDROSTATIC);
            k_hydrostatic<FT><<<dim3((Nx + 31) / 32, (Ny + 7) / 8), blk(), 0, stream>>>(P, phy.p, b_pred, c[0].p);
            check_launch();
        }
        const dim3 sgrid((Nx + smag::TX - 1) / smag::TX, (Ny + smag::TY - 1) / smag::TY, (Nz + smag::KT - 1) / smag::KT);
        const dim3 sblock(smag::TX, smag::TY);
        if (desc.closure == GBO_CLOSURE_SMAGORINSKY_LILLY && ibg) {
            // conditional strain rates near the immersed boundary: the per-point kernel
            pre(G_CLOSURE);
            k_smagorinsky<FT><<<grd(), blk(), 0, stream>>>(P, nu.p);
            check_launch();
        } else if (desc.closure == GBO_CLOSURE_SMAGORINSKY_LILLY) {
            pre(G_CLOSURE);
            k_smagorinsky_tiled<FT><<<sgrid, sblock, sizeof(smag::SmemS<FT>), stream>>>(P, nu.p);
            check_launch();
        } else if (lagrangian) {
            // νₑ from the cell's own coefficient max(𝒥ᴸᴹ, minimum_numerator) / 𝒥ᴹᴹ
            StepP<FT> Q = P;
            Q.jlm = lag_jlm.p;
            Q.jmm = lag_jmm.p;
            Q.lm_min = FT(desc.closure_min_numerator);
            pre(G_CLOSURE);
            k_smagorinsky_tiled<FT><<<sgrid, sblock, sizeof(smag::SmemS<FT>), stream>>>(Q, nu.p);
            check_launch();
        } else if (desc.closure == GBO_CLOSURE_DYNAMIC_SMAGORINSKY) {
            // Σ and Σ̄, the tile sums of LM and MM, the per-level coefficient, then νₑ
            // (compute_coefficient_fields!, dynamic_coefficient.jl:225-250; smagorinsky.jl:90-104)
            const dim3 dg((Nx + dyn::TX - 1) / dyn::TX, (Ny + dyn::TY - 1) / dyn::TY, Nz), db(dyn::TX, dyn::TY);
            pre(G_CLOSURE);
            const PlainVel<FT> V{host_cfld(u.p), host_cfld(v.p), host_wfld(w.p)};
            dyn_launch_sigma<FT>(stream, gp, V, dyn_sig.p, dyn_sigb.p);
            check_launch();
            pre(G_CLOSURE);
            dyn_launch_lm<FT>(stream, gp, V, dyn_sig.p, dyn_sigb.p, dyn_lmv.p, dyn_mmv.p);
            check_launch();
            pre(G_CLOSURE);
            k_dyn_tile_sums<FT><<<dg, db, 0, stream>>>(dyn_lmv.p, dyn_mmv.p, Nx, Ny, dyn_part.p);
            check_launch();
            pre(G_CLOSURE);
            k_dyn_coef<FT><<<Nz, dyn::COEF_THREADS, 0, stream>>>(dyn_part.p, (int)(dg.x * dg.y), (double)Nx * (double)Ny,
                                                                 FT(desc.closure_min_numerator), dyn_cs2.p, dyn_jlm.p,
                                                                 dyn_jmm.p);
            check_launch();
            StepP<FT> Q = P;
            Q.cs2 = dyn_cs2.p;
            pre(G_CLOSURE);
            k_smagorinsky_tiled<FT><<<sgrid, sblock, sizeof(smag::SmemS<FT>), stream>>>(Q, nu.p);
            check_launch();
        } else if (desc.closure == GBO_CLOSURE_AMD) {
            StepP<FT> Q = P;
            auto amd = [&](FT* kap_out) {
                pre(G_CLOSURE);
                if (ibg) k_amd_tiled_ibg<FT><<<sgrid, sblock, sizeof(smag::Smem<FT>), stream>>>(Q, nu.p, kap_out);
                else k_amd_tiled<FT><<<sgrid, sblock, sizeof(smag::SmemA<FT>), stream>>>(Q, nu.p, kap_out);
                check_launch();
            };
            Q.c = ntr > 0 ? c[0].p : nullptr;
            Q.cref = tracer_ref(0);
            amd(ntr > 0 ? kap[0].p : nullptr);
            for (int n = 1; n < ntr; ++n) {
                Q.c = c[n].p;
                Q.cref = tracer_ref(n);
                amd(kap[n].p);  // viscosity recomputed identically; only κₑ of tracer n is new
            }
        }
        if (has_phy && !b_pred) {
            pre(G_HYDROSTATIC);
            k_hydrostatic<FT><<<dim3((Nx + 31) / 32, (Ny + 7) / 8), blk(), 0, stream>>>(P, phy.p);
            check_launch();
        }
    }

    // One RK3 stage: Gⁿ from the current state, predictor, projection.  Δt is read
    // on the device from the stage factors at dtf, so a captured step serves every Δt.
    void stage(const FT* dtf, int s, double gamma, double zeta, bool first, bool last) {
        StepP<FT> P = params();
        P.dt = FT(0);
        P.dtf = dtf;
        P.gamma = FT(gamma);
        P.zeta = FT(zeta);
        P.first = first;
        // momentum and tracer 0 in one march; further tracers use the per-point tracer kernel
        StepP<FT> M0 = P;
        const dim3 fgrid((Nx + fused::TX - 1) / fused::TX, (Ny + fused::TY - 1) / fused::TY, (Nz + kchunk - 1) / kchunk);
        const dim3 fblock(fused::TX, fused::TY);
        int tracer0 = 1;
        if (ibg && desc.closure != GBO_CLOSURE_NONE) {
            // closures on an immersed grid: the per-point kernels carry the conditional strain rates
            pre(G_MOMENTUM);
            k_momentum<FT><<<grd(), blk(), 0, stream>>>(P);
            check_launch();
            tracer0 = 0;
        } else if (ntr > 0) {
            M0.c = c[0].p;
            M0.cref = tracer_ref(0);
            M0.co = cs[0].p;
            M0.Gc = Gc[0].p;
            M0.kap = kap.empty() ? nullptr : kap[0].p;
            M0.flux_top = FT(desc.tracer_flux_top[0]);
            M0.flux_bot = FT(desc.tracer_flux_bottom[0]);
            pre(G_MOMENTUM);
            launch_fused<FT, true>(kernel_closure(), ibg, fgrid, fblock, stream, M0, kchunk);
            check_launch();
        } else {
            pre(G_MOMENTUM);
            launch_fused<FT, false>(kernel_closure(), ibg, fgrid, fblock, stream, M0, kchunk);
            check_launch();
        }
        for (int n = tracer0; n < ntr; ++n) {
            StepP<FT> Q = P;
            Q.c = c[n].p;
            Q.cref = tracer_ref(n);
            Q.co = cs[n].p;
            Q.Gc = Gc[n].p;
            Q.kap = kap.empty() ? nullptr : kap[n].p;
            Q.flux_top = FT(desc.tracer_flux_top[n]);
            Q.flux_bot = FT(desc.tracer_flux_bottom[n]);
            pre(G_TRACER);
            k_tracer<FT><<<grd(), blk(), 0, stream>>>(Q);
            check_launch();
        }
        // Δτ = Δt γ (first stage) or Δt (γ + ζ) with γ, ζ in the working precision
        // (nonhydrostatic_rk3_substep.jl:34-36; runge_kutta_3.jl:186-187)
        project(us.p, vs.p, flat ? nullptr : ws.p, 0.0, dtf + DTF_RDTAU + s, dtf + DTF_SCALE + s);
        // the buoyancy predictor is stored into the state by the hydrostatic scan, which reads
        // it anyway (no immersed masks to apply in between on a rectilinear grid)
        const bool b_in_scan = has_phy && !ibg;
        for (int n = b_in_scan ? 1 : 0; n < ntr; ++n) {
            pre(G_COPY);
            k_copy<FT><<<(unsigned)std::min<size_t>((N * sizeof(FT) / 16 + 255) / 256 + 1, 4 * 152 * 8), 256, 0, stream>>>(cs[n].p, c[n].p, N);
            check_launch();
        }
        mask_tracers();
        // the Lagrangian average steps once per time step, after its last projection and
        // before update_state! (runge_kutta_3.jl:163; quasi_adams_bashforth_2.jl:117)
        if (lagrangian && last) lag_step();
        auxiliaries(b_in_scan ? cs[0].p : nullptr);
    }

    // mask_immersed_field!(model.tracers) (update_nonhydrostatic_model_state.jl:25)
    void mask_tracers() {
        if (!ibg) return;
        for (int n = 0; n < ntr; ++n) {
            pre(G_MASK);
            k_mask<FT><<<grd(), blk(), 0, stream>>>(gp, nullptr, nullptr, nullptr, c[n].p, 8, tracer_ref(n));
            check_launch();
        }
    }

    // One time step.  RK3: three stages.  QAB2 (quasi_adams_bashforth_2.jl:100-121,
    // nonhydrostatic_ab2_step.jl:29-58): one stage U* = U + Δt (α Gⁿ - β G⁻) with
    // α = 3/2 + χ, β = 1/2 + χ in FT, projected with Δτ = Δt; `euler` (χ = -1/2) takes
    // U + Δt Gⁿ and reads no G⁻.
    void full_step(const FT* dtf, bool euler = false) {
        using K = GboCoeffs<double>;
        if (qab2) {
            const FT chi = FT(desc.ab2_chi);
            const FT alpha = FT(1.5) + chi, beta = FT(0.5) + chi;
            if (euler) stage(dtf, 0, 1.0, 0.0, true, true);
            else stage(dtf, 0, (double)alpha, -(double)beta, false, true);
            return;
        }
        stage(dtf, 0, K::rk3_gamma1, 0.0, true, false);
        stage(dtf, 1, K::rk3_gamma2, K::rk3_zeta2, false, false);
        stage(dtf, 2, K::rk3_gamma3, K::rk3_zeta3, false, true);
    }
    // c of Δτ = FT(Δt c) per stage: γ₁, and γ + ζ summed in FT (runge_kutta_3.jl:186-187)
    static StageC rk3_stage_c() {
        using K = GboCoeffs<double>;
        return StageC{(double)FT(K::rk3_gamma1), (double)(FT(K::rk3_gamma2) + FT(K::rk3_zeta2)),
                      (double)(FT(K::rk3_gamma3) + FT(K::rk3_zeta3))};
    }
    // QAB2 projects with Δτ = FT(Δt) (kernel_Δt, nonhydrostatic_ab2_step.jl:30,56-57)
    StageC stage_c() const { return qab2 ? StageC{1.0, 1.0, 1.0} : rk3_stage_c(); }

    // After a failure inside a capture: end every capture this model's streams are in,
    // so that the thread's later CUDA calls (allocations included) are not refused
    void abort_capture() override {
        for (cudaStream_t s : {stream, body_stream, run_stream, if_stream}) {
            if (!s) continue;
            cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
            if (cudaStreamIsCapturing(s, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) {
                cudaGraph_t g = nullptr;
                cudaStreamEndCapture(s, &g);
                if (g) cudaGraphDestroy(g);
            }
        }
        cudaGetLastError();
    }

    cudaGraphExec_t capture_graph(bool euler) {
        cudaGraph_t gph;
        cudaGraphExec_t exec = nullptr;
        GBO_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        int64_t before = launches;
        if (lagrangian) lag_dtp = lag_s.p + LAG_DT;
        try {
            full_step(dtf.p, euler);
        } catch (...) {
            launches = before;
            abort_capture();
            throw;
        }
        graph_launches_per_step = launches - before;
        launches = before;
        GBO_CUDA(cudaStreamEndCapture(stream, &gph));
        GBO_CUDA(cudaGraphInstantiate(&exec, gph, 0));
        GBO_CUDA(cudaGraphDestroy(gph));
        return exec;
    }
    // QAB2 takes an Euler step whenever Δt differs from the last one, the first
    // step included (last_Δt = Inf; quasi_adams_bashforth_2.jl:101)
    bool euler_step(double dt) const { return qab2 && dt != last_dt; }

    // Δt of the next steps into the stage factors the stage kernels read
    void set_dt(double dt, cudaStream_t st) {
        pre(G_SIM);
        k_set_dt<FT><<<1, 1, 0, st>>>(dtf.p, dt, stage_c());
        check_launch();
    }

    int step(double dt, int nsteps) override {
        if (nsteps <= 0) return GBO_OK;
        cg_status = GBO_OK;
        set_dt(dt, stream);
        lag_set_dt(dt);
        if (use_graph) {
            if (!graph) graph = capture_graph(false);
            if (qab2 && !graph_euler) graph_euler = capture_graph(true);
            for (int s = 0; s < nsteps; ++s) {
                GBO_CUDA(cudaGraphLaunch(euler_step(dt) ? graph_euler : graph, stream));
                last_dt = dt;
            }
            launches += graph_launches_per_step * nsteps;
        } else {
            int worst = GBO_OK;
            for (int s = 0; s < nsteps; ++s) {
                full_step(dtf.p, euler_step(dt));
                last_dt = dt;
                if (cg_status != GBO_OK) worst = cg_status;
            }
            cg_status = worst;
        }
        return finish_steps(dt, nsteps);
    }

    // Record one time step on this model's stream while it is joined to another
    // stream's capture (ensemble graphs), reading Δt from dtp; returns the kernels recorded.
    int64_t capture_step(const float* dtf32, const double* dtf64) override {
        const int64_t before = launches;
        if constexpr (sizeof(FT) == 4) full_step(dtf32);
        else full_step(dtf64);
        const int64_t n = launches - before;
        launches = before;
        return n;
    }
    void add_launches(int64_t n) override { launches += n; }

    // After nsteps steps were issued: clock, NaN check, synchronisation, CG bookkeeping.
    int finish_steps(double dt, int nsteps) override {
        for (int s = 0; s < nsteps; ++s) {
            // clock: tⁿ⁺¹ = tⁿ + Δt computed a priori (runge_kutta_3.jl:122,160-161)
            time = time + dt;
            iteration += 1;
        }
        pre(G_NAN);
        k_nan_check<FT><<<std::min<size_t>((N + 255) / 256, 1024), 256, 0, stream>>>(u.p, N, d_flags);
        check_launch();
        int rc = sync();
        if (cg) {  // iterations run inside the graph: account for them now
            read_cg_scalars();
            launches += body_launches * (int64_t)(h_cgs[CG_ITERS] - iters_seen);
            iters_seen = h_cgs[CG_ITERS];
            last_iters = (int)h_cgs[CG_IT];
            int st = cg_outcome();
            if (st != GBO_OK) cg_status = st;
        }
        return rc != GBO_OK ? rc : cg_status;
    }

    int timing_counts(int64_t* n, int nmax) const override {
        for (int g = 0; g < std::min(nmax, (int)GROUPS); ++g) n[g] = group_n[g];
        return GBO_OK;
    }

    int timed_steps(double dt, int nsteps, double* ms, int nmax) override {
        if (!ev0) { GBO_CUDA(cudaEventCreate(&ev0)); GBO_CUDA(cudaEventCreate(&ev1)); }
        std::fill(group_ms.begin(), group_ms.end(), 0.0);
        std::fill(group_n.begin(), group_n.end(), 0);
        timing = true;
        try {
            set_dt(dt, stream);
            lag_set_dt(dt);
            for (int s = 0; s < nsteps; ++s) {
                full_step(dtf.p, euler_step(dt));
                last_dt = dt;
                time += dt;
                iteration += 1;
            }
        } catch (...) {
            timing = false;
            throw;
        }
        timing = false;
        for (int g = 0; g < std::min(nmax, (int)GROUPS); ++g) ms[g] = group_n[g] ? group_ms[g] / group_n[g] : 0.0;
        return sync();
    }

    void* stream_ptr() override { return (void*)stream; }
    int64_t launch_count() const override { return launches; }

    int sync() override {
        GBO_CUDA(cudaMemcpyAsync(h_flags, d_flags, sizeof(unsigned int), cudaMemcpyDeviceToHost, stream));
        GBO_CUDA(cudaStreamSynchronize(stream));
        if (*h_flags & GBO_FLAG_NAN) {
            err = "NaN or Inf found in the prognostic state";
            GBO_CUDA(cudaMemset(d_flags, 0, sizeof(unsigned int)));
            return GBO_ERR_NAN;
        }
        return GBO_OK;
    }

    FT* field_ptr(int field) {
        if (field == GBO_FIELD_U) return u.p;
        if (field == GBO_FIELD_V) return v.p;
        if (field == GBO_FIELD_W) return flat ? nullptr : w.p;
        if (field >= GBO_FIELD_TRACER && field < GBO_FIELD_TRACER + ntr) return c[field - GBO_FIELD_TRACER].p;
        if (field == GBO_FIELD_PNHS) return p.p;
        if (field == GBO_FIELD_PHY) return has_phy ? phy.p : nullptr;
        if (field == GBO_FIELD_NU) return nu.p;
        if (field == GBO_FIELD_KAPPA) return kap.empty() ? nullptr : kap[0].p;
        if (field == GBO_FIELD_JLM) return lagrangian ? lag_jlm.p : nullptr;
        if (field == GBO_FIELD_JMM) return lagrangian ? lag_jmm.p : nullptr;
        return nullptr;
    }

    // index of a tracer stored as departures from its reference profile, or -1
    int departure_tracer(int field) const {
        const int n = field - GBO_FIELD_TRACER;
        return (departures && field >= GBO_FIELD_TRACER && n < ntr) ? n : -1;
    }
    unsigned conv_blocks() const { return (unsigned)std::min<size_t>((N + 255) / 256, (size_t)4 * 152 * 8); }
    // The hydrostatic pressure anomaly of the buoyancy profile alone (the part the kernels
    // leave out, see k_hydrostatic): the same downward integral in FP64.
    std::vector<double> phy_reference() const {
        const std::vector<double>& r = cref_h[0];
        std::vector<double> ph(Nz);
        double pk = -(0.5 * (r[Nz - 1] + r[Nz - 1])) * (double)Z.at(Z.dzf, Nz + 1);
        ph[Nz - 1] = pk;
        for (int k = Nz - 2; k >= 0; --k) {
            pk -= (0.5 * (r[k] + r[k + 1])) * (double)Z.at(Z.dzf, k + 2);
            ph[k] = pk;
        }
        return ph;
    }
    void download_profile(int n) {
        std::vector<FT> r(Nz);
        GBO_CUDA(cudaMemcpyAsync(r.data(), cref[n].p, Nz * sizeof(FT), cudaMemcpyDeviceToHost, stream));
        GBO_CUDA(cudaStreamSynchronize(stream));
        for (int k = 0; k < Nz; ++k) cref_h[n][k] = (double)r[k];
    }

    // Interior transfer with type conversion; w carries Nz+1 faces at the boundary.
    int set_field(int field, const void* host, int dt_, int64_t count) override {
        FT* d = field_ptr(field);
        if (field == GBO_FIELD_W && flat) { err = "w does not exist on a Flat-z grid"; return GBO_ERR_INVALID; }
        if (!d) { err = "unknown field id"; return GBO_ERR_INVALID; }
        if (count != this->count(field)) { err = "element count does not match the field size"; return GBO_ERR_INVALID; }
        const int dn = departure_tracer(field);
        if (dn >= 0) {
            // the profile is the horizontal mean of the new values; the field stores departures
            const size_t plane = (size_t)Nx * Ny;
            if (dt_ == GBO_FLOAT32) {
                float* st = reinterpret_cast<float*>(tstage.p);
                GBO_CUDA(cudaMemcpyAsync(st, host, N * sizeof(float), cudaMemcpyHostToDevice, stream));
                k_level_mean<float><<<Nz, LM_THREADS, 0, stream>>>(st, plane, tmean.p);
                k_to_departure<FT, float><<<conv_blocks(), 256, 0, stream>>>(st, tmean.p, cref[dn].p, d, plane, N);
            } else {
                GBO_CUDA(cudaMemcpyAsync(tstage.p, host, N * sizeof(double), cudaMemcpyHostToDevice, stream));
                k_level_mean<double><<<Nz, LM_THREADS, 0, stream>>>(tstage.p, plane, tmean.p);
                k_to_departure<FT, double><<<conv_blocks(), 256, 0, stream>>>(tstage.p, tmean.p, cref[dn].p, d, plane, N);
            }
            GBO_CUDA(cudaGetLastError());
            download_profile(dn);
            return GBO_OK;
        }
        const bool same = (dt_ == GBO_FLOAT32) == (sizeof(FT) == 4);
        if (same) {
            GBO_CUDA(cudaMemcpyAsync(d, host, N * sizeof(FT), cudaMemcpyHostToDevice, stream));
        } else {
            std::vector<FT> h(N);
            for (size_t q = 0; q < N; ++q)
                h[q] = dt_ == GBO_FLOAT32 ? FT(static_cast<const float*>(host)[q]) : FT(static_cast<const double*>(host)[q]);
            GBO_CUDA(cudaMemcpyAsync(d, h.data(), N * sizeof(FT), cudaMemcpyHostToDevice, stream));
            GBO_CUDA(cudaStreamSynchronize(stream));
        }
        if (field == GBO_FIELD_W)  // impenetrable walls: the bottom face is zero (set! + fill_halo_regions!)
            GBO_CUDA(cudaMemsetAsync(d, 0, (size_t)Nx * Ny * sizeof(FT), stream));
        if (field == GBO_FIELD_U || field == GBO_FIELD_V || field == GBO_FIELD_W) velocities_set = true;
        GBO_CUDA(cudaStreamSynchronize(stream));
        return GBO_OK;
    }

    int get_field(int field, void* host, int dt_, int64_t count) override {
        FT* d = field_ptr(field);
        if (count != this->count(field)) { err = "element count does not match the field size"; return GBO_ERR_INVALID; }
        const int dn = departure_tracer(field);
        if (dn >= 0) {  // reference profile + departure
            const size_t plane = (size_t)Nx * Ny;
            if (dt_ == GBO_FLOAT32) {
                float* st = reinterpret_cast<float*>(tstage.p);
                k_from_departure<FT, float><<<conv_blocks(), 256, 0, stream>>>(d, cref[dn].p, st, plane, N);
                GBO_CUDA(cudaGetLastError());
                GBO_CUDA(cudaMemcpyAsync(host, st, N * sizeof(float), cudaMemcpyDeviceToHost, stream));
            } else {
                k_from_departure<FT, double><<<conv_blocks(), 256, 0, stream>>>(d, cref[dn].p, tstage.p, plane, N);
                GBO_CUDA(cudaGetLastError());
                GBO_CUDA(cudaMemcpyAsync(host, tstage.p, N * sizeof(double), cudaMemcpyDeviceToHost, stream));
            }
            GBO_CUDA(cudaStreamSynchronize(stream));
            return GBO_OK;
        }
        if (field == GBO_FIELD_PHY && d && departures && desc.buoyancy_tracer) {
            // the kernels hold pHY′ of the departures; add that of the buoyancy profile
            std::vector<FT> h(N);
            GBO_CUDA(cudaMemcpyAsync(h.data(), d, N * sizeof(FT), cudaMemcpyDeviceToHost, stream));
            GBO_CUDA(cudaStreamSynchronize(stream));
            const std::vector<double> ph = phy_reference();
            const size_t plane = (size_t)Nx * Ny;
            for (size_t q = 0; q < N; ++q) {
                const double x = ph[q / plane] + (double)h[q];
                if (dt_ == GBO_FLOAT32) static_cast<float*>(host)[q] = (float)x;
                else static_cast<double*>(host)[q] = x;
            }
            return GBO_OK;
        }
        const bool same = (dt_ == GBO_FLOAT32) == (sizeof(FT) == 4);
        if (d && same) {
            GBO_CUDA(cudaMemcpyAsync(host, d, N * sizeof(FT), cudaMemcpyDeviceToHost, stream));
            GBO_CUDA(cudaStreamSynchronize(stream));
            if ((size_t)count > N) std::memset(static_cast<char*>(host) + N * sizeof(FT), 0, ((size_t)count - N) * sizeof(FT));
            return GBO_OK;
        }
        std::vector<FT> h(N, FT(0));
        if (d) {
            GBO_CUDA(cudaMemcpyAsync(h.data(), d, N * sizeof(FT), cudaMemcpyDeviceToHost, stream));
            GBO_CUDA(cudaStreamSynchronize(stream));
        } else if (field != GBO_FIELD_W) {
            err = "field not present in this model";
            return GBO_ERR_INVALID;
        }
        const size_t total = (size_t)count;
        for (size_t q = 0; q < total; ++q) {
            FT x = q < N ? h[q] : FT(0);  // the top w face (index Nz) is the wall
            if (dt_ == GBO_FLOAT32) static_cast<float*>(host)[q] = (float)x;
            else static_cast<double*>(host)[q] = (double)x;
        }
        return GBO_OK;
    }

    int set_finalize(int enforce) override {
        // set_nonhydrostatic_model.jl:59-73: mask tracers and velocities, then project
        cg_status = GBO_OK;
        const bool init = lagrangian && velocities_set;  // velocities_are_set && initialize_closure_fields!
        velocities_set = false;
        mask_tracers();
        if (ibg) {
            pre(G_MASK);
            k_mask<FT><<<grd(), blk(), 0, stream>>>(gp, u.p, v.p, flat ? nullptr : w.p, nullptr, flat ? 3 : 7);
            check_launch();
        }
        if (init) lag_initialize(u.p, v.p, w.p);
        if (enforce && init) {
            // the projection corrects the interior after the halos were filled from the set
            // values; the second initialization sees both, so keep the set values
            const unsigned cb = (unsigned)std::min<size_t>((N * sizeof(FT) / 16 + 255) / 256 + 1, 4 * 152 * 8);
            FT* const from[3] = {u.p, v.p, w.p};
            FT* const to[3] = {us.p, vs.p, ws.p};
            for (int q = 0; q < 3; ++q) {
                pre(G_COPY);
                k_copy<FT><<<cb, 256, 0, stream>>>(from[q], to[q], N);
                check_launch();
            }
            project(us.p, vs.p, ws.p, 1.0);
            lag_initialize(us.p, vs.p, ws.p);
        } else if (enforce) {
            project(u.p, v.p, flat ? nullptr : w.p, 1.0);
        }
        auxiliaries();
        int rc = sync();
        return rc != GBO_OK ? rc : cg_status;
    }

    int reference_profile(int field, double* out, int64_t n) override {
        if (n != Nz) { err = "the profile has Nz values"; return GBO_ERR_INVALID; }
        const int t = field - GBO_FIELD_TRACER;
        if (field < GBO_FIELD_TRACER || t >= ntr) { err = "reference profiles exist for tracers only"; return GBO_ERR_INVALID; }
        for (int k = 0; k < Nz; ++k) out[k] = departures ? cref_h[t][k] : 0.0;
        return GBO_OK;
    }

    int device_pointer(int field, void** ptr, int64_t* n) override {
        FT* d = field_ptr(field);
        if (!d) { err = "field not present in this model"; return GBO_ERR_INVALID; }
        *ptr = d;
        *n = (int64_t)N;
        return GBO_OK;
    }

    // ---- prognostic state (prognostic_state / restore_prognostic_state!,
    // nonhydrostatic_model.jl:354-377): clock, velocities, tracers and pNHS (the CG
    // initial guess).  RK3 keeps no tendency history across steps (ζ₁ = 0), and the
    // closure fields and pHY′ are recomputed from the restored state, except the
    // Lagrangian-averaged 𝒥ᴸᴹ, 𝒥ᴹᴹ and previous_compute_time, which are prognostic
    // (dynamic_coefficient.jl:524-539).
    struct StateHeader {
        uint64_t magic;
        int32_t version, dtype, Nx, Ny, Nz, ntr, timestepper;
        double time;
        int64_t iteration;
        double last_dt;
    };
    static constexpr uint64_t kStateMagic = 0x31657461747362ULL;  // "bstate1"
    static constexpr int32_t kStateVersion = 3;
    // QAB2 also keeps G⁻ (prognostic_state of its timestepper): the next step reads it
    std::vector<const FT*> state_fields() const {
        std::vector<const FT*> f{u.p, v.p};
        if (!flat) f.push_back(w.p);
        for (int n = 0; n < ntr; ++n) f.push_back(c[n].p);
        f.push_back(p.p);
        if (qab2) {
            f.push_back(Gu.p);
            f.push_back(Gv.p);
            if (!flat) f.push_back(Gw.p);
            for (int n = 0; n < ntr; ++n) f.push_back(Gc[n].p);
        }
        if (lagrangian) {
            f.push_back(lag_jlm.p);
            f.push_back(lag_jmm.p);
        }
        return f;
    }
    // after the fields: the tracers' reference profiles (Nz values each) when tracers are
    // stored as departures
    int64_t profile_bytes() const { return departures ? (int64_t)ntr * Nz * (int64_t)sizeof(FT) : 0; }
    // then previous_compute_time (FP64) of a Lagrangian average
    int64_t lag_bytes() const { return lagrangian ? (int64_t)sizeof(double) : 0; }
    int64_t state_bytes() const override {
        return (int64_t)sizeof(StateHeader) + (int64_t)state_fields().size() * (int64_t)N * (int64_t)sizeof(FT) +
               profile_bytes() + lag_bytes();
    }
    int get_state(void* buf, int64_t bytes) override {
        if (bytes != state_bytes()) { err = "state buffer size does not match gbo_state_bytes"; return GBO_ERR_INVALID; }
        StateHeader h{kStateMagic, kStateVersion, dtype, Nx, Ny, Nz, ntr, desc.timestepper, time, iteration, last_dt};
        std::memcpy(buf, &h, sizeof(h));
        char* at = static_cast<char*>(buf) + sizeof(h);
        for (const FT* f : state_fields()) {
            GBO_CUDA(cudaMemcpyAsync(at, f, N * sizeof(FT), cudaMemcpyDeviceToHost, stream));
            at += N * sizeof(FT);
        }
        for (int n = 0; departures && n < ntr; ++n) {
            GBO_CUDA(cudaMemcpyAsync(at, cref[n].p, Nz * sizeof(FT), cudaMemcpyDeviceToHost, stream));
            at += Nz * sizeof(FT);
        }
        if (lagrangian) GBO_CUDA(cudaMemcpyAsync(at, lag_s.p + LAG_PREV, sizeof(double), cudaMemcpyDeviceToHost, stream));
        GBO_CUDA(cudaStreamSynchronize(stream));
        return GBO_OK;
    }
    int set_state(const void* buf, int64_t bytes) override {
        if (bytes != state_bytes()) { err = "state buffer size does not match gbo_state_bytes"; return GBO_ERR_INVALID; }
        StateHeader h;
        std::memcpy(&h, buf, sizeof(h));
        if (h.magic != kStateMagic || h.version != kStateVersion) { err = "not a state written by gbo_get_state"; return GBO_ERR_INVALID; }
        if (h.dtype != dtype || h.Nx != Nx || h.Ny != Ny || h.Nz != Nz || h.ntr != ntr || h.timestepper != desc.timestepper) {
            err = "state was written by a model of another size, float type, tracer count or timestepper";
            return GBO_ERR_INVALID;
        }
        const char* at = static_cast<const char*>(buf) + sizeof(h);
        for (const FT* f : state_fields()) {
            GBO_CUDA(cudaMemcpyAsync(const_cast<FT*>(f), at, N * sizeof(FT), cudaMemcpyHostToDevice, stream));
            at += N * sizeof(FT);
        }
        for (int n = 0; departures && n < ntr; ++n) {
            GBO_CUDA(cudaMemcpyAsync(cref[n].p, at, Nz * sizeof(FT), cudaMemcpyHostToDevice, stream));
            at += Nz * sizeof(FT);
            download_profile(n);
        }
        if (lagrangian) {
            double clk[2];
            std::memcpy(&clk[1], at, sizeof(double));
            clk[0] = h.time;  // LAG_TIME, LAG_PREV
            GBO_CUDA(cudaMemcpyAsync(lag_s.p + LAG_TIME, clk, sizeof clk, cudaMemcpyHostToDevice, stream));
            GBO_CUDA(cudaStreamSynchronize(stream));
        }
        time = h.time;
        iteration = h.iteration;
        last_dt = h.last_dt;
        mask_tracers();
        auxiliaries();
        return sync();
    }

    // ---- simulation loop (run!(sim), src/Simulations/run.jl:165-262) ----
    SimP<FT> sim_params() {
        SimP<FT> S{};
        S.g = gp;
        S.u = u.p; S.v = v.p; S.w = flat ? nullptr : w.p;
        S.nu = nu.p;
        for (int n = 0; n < ntr; ++n) S.kap[n] = kap.empty() ? nullptr : kap[n].p;
        S.ntr = ntr;
        S.closure = desc.closure;
        S.run = run_s.p;
        S.part = run_part.p;
        S.cnt = run_cnt.p;
        return S;
    }
    // Δ² = min(Δx, Δy, min Δz)² and max(1, 1/Pr) of the diffusion timescale, in FT
    // (turbulence_closure_diagnostics.jl:8-13,48-53; min_Pr = 1 without tracers)
    void diffusion_constants(double* d2, double* prf) const {
        FT D = std::min(gp.dx, gp.dy);
        if (!flat)
            for (int kr = 1; kr <= Nz; ++kr) D = std::min(D, Z.at(Z.dzc, kr));
        *d2 = (double)(D * D);
        const FT pr = ntr > 0 ? FT(desc.closure_Pr) : FT(1);
        *prf = (double)std::max(FT(1), FT(1) / pr);
    }
    void read_run() {
        GBO_CUDA(cudaMemcpyAsync(h_run, run_s.p, RUN_NSLOTS * sizeof(double), cudaMemcpyDeviceToHost, stream));
        GBO_CUDA(cudaStreamSynchronize(stream));
    }

    int timescales(double* adv, double* dif) override {
        diffusion_constants(&h_run[RUN_DELTA2], &h_run[RUN_PR_FACTOR]);
        GBO_CUDA(cudaMemcpyAsync(run_s.p + RUN_DELTA2, h_run + RUN_DELTA2, 2 * sizeof(double), cudaMemcpyHostToDevice, stream));
        pre(G_SIM);
        k_sim_callbacks<FT><<<SIM_BLOCKS, 256, 0, stream>>>(sim_params(), SIM_TIMESCALES, 0, 0);
        check_launch();
        read_run();
        if (adv) *adv = h_run[RUN_TAU_ADV];
        if (dif) *dif = h_run[RUN_TAU_DIF];
        return GBO_OK;
    }

    // Add a conditional node (WHILE, or IF with an ELSE body) after the work captured so
    // far on `stream` and record each body with body(i) while `stream` points at a
    // stream capturing into that body.
    template <class F>
    void capture_conditional(cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type, unsigned nbodies,
                             cudaStream_t& aux, F&& body) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        cudaGraph_t g = nullptr;
        const cudaGraphNode_t* deps = nullptr;
        size_t nd = 0;
        GBO_CUDA(cudaStreamGetCaptureInfo(stream, &cs, nullptr, &g, &deps, nullptr, &nd));
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h;
        cp.conditional.type = type;
        cp.conditional.size = nbodies;
        cudaGraphNode_t node;
        GBO_CUDA(cudaGraphAddNode(&node, g, deps, nullptr, nd, &cp));
        GBO_CUDA(cudaStreamUpdateCaptureDependencies(stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
        for (unsigned b = 0; b < nbodies; ++b) {
            GBO_CUDA(cudaStreamBeginCaptureToGraph(aux, cp.conditional.phGraph_out[b], nullptr, nullptr, 0,
                                                   cudaStreamCaptureModeThreadLocal));
            std::swap(stream, aux);
            try {
                body(b);
            } catch (...) {
                std::swap(stream, aux);
                throw;
            }
            std::swap(stream, aux);
            cudaGraph_t captured = nullptr;
            GBO_CUDA(cudaStreamEndCapture(aux, &captured));
        }
    }
    cudaGraphConditionalHandle new_handle(unsigned dflt, unsigned flags) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        cudaGraph_t g = nullptr;
        GBO_CUDA(cudaStreamGetCaptureInfo(stream, &cs, nullptr, &g, nullptr, nullptr, nullptr));
        cudaGraphConditionalHandle h;
        GBO_CUDA(cudaGraphConditionalHandleCreate(&h, g, dflt, flags));
        return h;
    }

    // The loop graph: k_sim_start, then WHILE { k_sim_begin, one time step reading Δt
    // from the stage factors, k_sim_callbacks }.  The condition starts at 1 on every
    // launch (a time_step!(sim) always steps once); k_sim_begin clears it and only the
    // last block of k_sim_callbacks sets it again, to 1 while running and below
    // RUN_MAX_TAKEN iterations.  With QAB2 the step is an IF node whose bodies are the
    // Euler step and the AB2 step, chosen by k_sim_begin.
    void build_run_graph() {
        if (!run_stream) GBO_CUDA(cudaStreamCreateWithFlags(&run_stream, cudaStreamNonBlocking));
        if (qab2 && !if_stream) GBO_CUDA(cudaStreamCreateWithFlags(&if_stream, cudaStreamNonBlocking));
        const SimP<FT> S = sim_params();
        cudaGraph_t gph;
        if (lagrangian) lag_dtp = run_s.p + RUN_DT;  // the loop's aligned Δt
        GBO_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        k_sim_start<<<1, 1, 0, stream>>>(run_s.p);
        GBO_CUDA(cudaGetLastError());
        const cudaGraphConditionalHandle h = new_handle(1, cudaGraphCondAssignDefault);
        const int64_t before = launches;
        int64_t branch = 0;  // kernels of the branch not taken (QAB2)
        try {
        capture_conditional(h, cudaGraphCondTypeWhile, 1, run_stream, [&](unsigned) {
            const cudaGraphConditionalHandle he = qab2 ? new_handle(0, 0) : 0;
            pre(G_SIM);
            k_sim_begin<FT><<<1, 1, 0, stream>>>(run_s.p, dtf.p, stage_c(), h, he, 1, qab2 ? 1 : 0);
            check_launch();
            if (qab2) {
                capture_conditional(he, cudaGraphCondTypeIf, 2, if_stream, [&](unsigned b) {
                    const int64_t at = launches;
                    full_step(dtf.p, b == 0);
                    if (b == 1) branch = launches - at;
                });
            } else {
                full_step(dtf.p);
            }
            pre(G_SIM);
            k_sim_callbacks<FT><<<SIM_BLOCKS, 256, 0, stream>>>(S, SIM_AFTER_STEP, h, 1);
            check_launch();
        });
        } catch (...) {
            launches = before;
            if (lagrangian) lag_dtp = lag_s.p + LAG_DT;
            abort_capture();
            throw;
        }
        run_iter_launches = launches - before - branch;
        launches = before;
        if (lagrangian) lag_dtp = lag_s.p + LAG_DT;
        GBO_CUDA(cudaStreamEndCapture(stream, &gph));
        GBO_CUDA(cudaGraphInstantiate(&run_graph, gph, 0));
        GBO_CUDA(cudaGraphDestroy(gph));
    }

    int run(const gbo_run_desc* d, gbo_run_result* out) override {
        if (!(d->dt > 0) || !std::isfinite(d->dt)) { err = "dt must be positive and finite"; return GBO_ERR_INVALID; }
        if (d->minimum_relative_step != 0.0) { err = "minimum_relative_step > 0 (skipped time steps) is not supported"; return GBO_ERR_INVALID; }
        if (d->iterations_per_launch < 1) { err = "iterations_per_launch must be at least 1"; return GBO_ERR_INVALID; }
        if (d->nan_check_interval < 0 || d->wizard_interval < 0) { err = "callback intervals must be >= 0"; return GBO_ERR_INVALID; }
        if (std::isnan(d->stop_time) || std::isnan(d->stop_iteration) || std::isnan(d->wall_time_limit)) {
            err = "stop criteria must not be NaN";
            return GBO_ERR_INVALID;
        }
        if (d->wizard_interval > 0) {
            // TimeStepWizard's own checks (time_step_wizard.jl:75-77)
            if (!(d->min_change < 1)) { err = "min_change must be < 1"; return GBO_ERR_INVALID; }
            if (!(d->max_change > 1)) { err = "max_change must be > 1"; return GBO_ERR_INVALID; }
        }
        double* H = h_run;
        std::fill(H, H + RUN_NSLOTS, 0.0);
        // Simulation converts Δt and stop_time to the model's float type (simulation.jl:97-104)
        H[RUN_SIM_DT] = (double)FT(d->dt);
        H[RUN_DT] = H[RUN_SIM_DT];
        H[RUN_TIME] = time;
        H[RUN_ITER] = (double)iteration;
        H[RUN_STOP_TIME] = (double)FT(d->stop_time);
        H[RUN_STOP_ITER] = d->stop_iteration;
        H[RUN_ALIGN] = d->align_time_step ? 1.0 : 0.0;
        H[RUN_RUNNING] = 1.0;
        H[RUN_MAX_TAKEN] = (double)d->iterations_per_launch;
        H[RUN_WIZ_EVERY] = (double)d->wizard_interval;
        H[RUN_CFL] = d->cfl;
        H[RUN_DCFL] = d->diffusive_cfl;
        H[RUN_MAX_CHANGE] = d->max_change;
        H[RUN_MIN_CHANGE] = d->min_change;
        H[RUN_MAX_DT] = d->max_dt;
        H[RUN_MIN_DT] = d->min_dt;
        H[RUN_NAN_EVERY] = (double)d->nan_check_interval;
        diffusion_constants(&H[RUN_DELTA2], &H[RUN_PR_FACTOR]);
        H[RUN_TAU_ADV] = H[RUN_TAU_DIF] = INFINITY;
        H[RUN_LAST_DT] = last_dt;
        GBO_CUDA(cudaMemcpyAsync(run_s.p, H, RUN_NSLOTS * sizeof(double), cudaMemcpyHostToDevice, stream));
        GBO_CUDA(cudaStreamSynchronize(stream));  // H is reused for the read-back
        cg_status = GBO_OK;
        if (iteration == 0) {  // initialize!(sim) of a fresh simulation: every callback once
            pre(G_SIM);
            k_sim_callbacks<FT><<<SIM_BLOCKS, 256, 0, stream>>>(sim_params(), SIM_INIT, 0, 0);
            check_launch();
        }
        if (!run_graph) build_run_graph();
        lag_set_dt(0.0);  // the Lagrangian clock starts from the model's time (Δt comes from the loop)
        const auto t0 = std::chrono::steady_clock::now();
        int64_t steps = 0;
        int reason = GBO_STOP_NONE;
        for (;;) {
            GBO_CUDA(cudaGraphLaunch(run_graph, stream));
            read_run();
            const int64_t taken = (int64_t)H[RUN_TAKEN];
            steps += taken;
            launches += 1 + run_iter_launches * taken;
            time = H[RUN_TIME];
            iteration = (int64_t)H[RUN_ITER];
            last_dt = H[RUN_LAST_DT];
            if (cg) {  // CG iterations ran inside the graph: account for them now
                read_cg_scalars();
                launches += body_launches * (int64_t)(h_cgs[CG_ITERS] - iters_seen);
                iters_seen = h_cgs[CG_ITERS];
                last_iters = (int)h_cgs[CG_IT];
                int st = cg_outcome();
                if (st != GBO_OK) cg_status = st;
            }
            if (taken < 1) { err = "the simulation loop took no step"; return GBO_ERR_STATE; }
            if (H[RUN_RUNNING] == 0.0) {
                reason = (int)H[RUN_REASON];
                break;
            }
            // wall_time_limit_exceeded (simulation.jl:257-269), checked once per launch
            const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            if (wall >= d->wall_time_limit) {
                reason = GBO_STOP_WALL_TIME;
                break;
            }
        }
        if (out) {
            out->dt = H[RUN_SIM_DT];
            out->time = time;
            out->iteration = iteration;
            out->steps = steps;
            out->stop_reason = reason;
            out->nan_detected = H[RUN_NAN] != 0.0;
        }
        if (H[RUN_NAN] != 0.0 && d->nan_erroring) {
            char msg[160];
            std::snprintf(msg, sizeof msg, "time = %.17g, iteration = %lld: NaN found in field u. Aborting simulation.", time,
                          (long long)iteration);
            err = msg;
            return GBO_ERR_NAN;
        }
        return cg_status;
    }

    int poisson_device(void* phi, const void* rhs) override {
        join_caller();
        if (cg) {
            // V∇²ϕ = rhs by preconditioned CG from the initial guess in ϕ
            GBO_CUDA(cudaMemcpyAsync(cg_x.p, phi, N * sizeof(FT), cudaMemcpyDeviceToDevice, stream));
            GBO_CUDA(cudaMemcpyAsync(cg_b.p, rhs, N * sizeof(FT), cudaMemcpyDeviceToDevice, stream));
            int st = cg_iterate();
            GBO_CUDA(cudaMemcpyAsync(phi, cg_x.p, N * sizeof(FT), cudaMemcpyDeviceToDevice, stream));
            int rc = sync();
            return rc != GBO_OK ? rc : st;
        }
        GBO_CUDA(cudaMemcpyAsync(rb.p, rhs, N * sizeof(FT), cudaMemcpyDeviceToDevice, stream));
        if (desc.pressure_solver == GBO_SOLVER_FOURIER_TRIDIAGONAL) {
            // set_source_term!: b ← b Δzᶜ (fourier_tridiagonal_poisson_solver.jl:268-290)
            pre(G_SOURCE);
            k_scale_dzc<FT><<<grd(), blk(), 0, stream>>>(gp, rb.p);
            check_launch();
        }
        poisson_solve(desc.pressure_solver);
        GBO_CUDA(cudaMemcpyAsync(phi, rb.p, N * sizeof(FT), cudaMemcpyDeviceToDevice, stream));
        return sync();
    }
};

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
namespace {

template <class F>
int guarded(gbo_model* m, F&& f) {
    try {
        return f();
    } catch (const CudaError& e) {
        std::string msg = std::string("CUDA error in ") + e.what + ": " + cudaGetErrorString(e.e);
        if (m) m->err = msg;
        g_last_error = msg;
        return GBO_ERR_CUDA;
    } catch (const InvalidArg& e) {
        if (m) m->err = e.msg;
        g_last_error = e.msg;
        return GBO_ERR_INVALID;
    } catch (const std::exception& e) {
        if (m) m->err = e.what();
        g_last_error = e.what();
        return GBO_ERR_INVALID;
    }
}

std::string validate(const gbo_grid_desc* g, const gbo_model_desc* d) {
    if (!g || !d) return "null descriptor";
    if (g->topology[0] != GBO_PERIODIC || g->topology[1] != GBO_PERIODIC)
        return "x and y must be Periodic";
    if (g->topology[2] != GBO_BOUNDED && g->topology[2] != GBO_FLAT) return "z must be Bounded or Flat";
    if (g->float_type != GBO_FLOAT32 && g->float_type != GBO_FLOAT64) return "float_type must be GBO_FLOAT32 or GBO_FLOAT64";
    int nz = g->topology[2] == GBO_FLAT ? 1 : g->size[2];
    if (g->size[0] < 8 || g->size[1] < 8 || nz < 1) return "Nx and Ny must be at least 8";
    if (g->size[0] % 2) return "Nx must be even";
    if (g->topology[2] == GBO_BOUNDED && nz < 6) return "Nz must be at least 6 on a Bounded z";
    if (g->x[1] <= g->x[0] || g->y[1] <= g->y[0]) return "x and y extents must be increasing";
    if (g->topology[2] == GBO_BOUNDED && !g->z_faces && g->z[1] <= g->z[0]) return "z extent must be increasing";
    if (g->z_faces)
        for (int k = 0; k < nz; ++k)
            if (!(g->z_faces[k + 1] > g->z_faces[k])) return "z_faces must be increasing";
    if (d->advection != GBO_ADVECTION_WENO5) return "only WENO(order=5) advection is implemented";
    if (d->closure < 0 || d->closure > 4) return "unknown closure";
    if (d->closure == GBO_CLOSURE_DYNAMIC_SMAGORINSKY) {
        if (g->topology[2] != GBO_BOUNDED) return "DynamicSmagorinsky requires a three-dimensional grid with Bounded z";
        if (g->bottom_height) return "DynamicSmagorinsky is not available on an ImmersedBoundaryGrid";
        if (!std::isfinite(d->closure_min_numerator)) return "DynamicSmagorinsky minimum_numerator must be finite";
        if (d->closure_averaging != GBO_AVERAGING_XY && d->closure_averaging != GBO_AVERAGING_LAGRANGIAN)
            return "unknown DynamicSmagorinsky averaging";
    }
    if (d->closure == GBO_CLOSURE_SCALAR_DIFFUSIVITY) {
        if (!(d->closure_nu >= 0) || !std::isfinite(d->closure_nu)) return "ScalarDiffusivity ν must be finite and >= 0";
        for (int n = 0; n < d->ntracers && n < GBO_MAX_TRACERS; ++n)
            if (!(d->closure_kappa[n] >= 0) || !std::isfinite(d->closure_kappa[n]))
                return "ScalarDiffusivity κ must be finite and >= 0";
    }
    if (d->timestepper != GBO_TIMESTEPPER_RK3 && d->timestepper != GBO_TIMESTEPPER_QAB2) return "unknown timestepper";
    if (d->timestepper == GBO_TIMESTEPPER_QAB2 && !std::isfinite(d->ab2_chi)) return "QuasiAdamsBashforth2 χ must be finite";
    if (d->ntracers < 0 || d->ntracers > GBO_MAX_TRACERS) return "ntracers out of range";
    if (d->buoyancy_tracer && d->ntracers < 1) return "BuoyancyTracer requires tracer b (tracer 0)";
    if (d->pressure_solver == GBO_SOLVER_FFT && g->z_faces) return "FFTBasedPoissonSolver requires a regular grid";
    if (d->pressure_solver == GBO_SOLVER_FOURIER_TRIDIAGONAL && g->topology[2] != GBO_BOUNDED)
        return "FourierTridiagonalPoissonSolver requires Bounded z";
    if (d->pressure_solver < 0 || d->pressure_solver > 2) return "pressure_solver not available";
    if (d->pressure_solver == GBO_SOLVER_CONJUGATE_GRADIENT) {
        if (d->preconditioner == GBO_PRECOND_LEARNED) return "the learned preconditioner is not available";
        if (d->preconditioner < 0 || d->preconditioner > 1) return "unknown preconditioner";
        if (d->cg_reltol < 0 || d->cg_abstol < 0 || d->cg_maxiter < 0) return "CG tolerances and maxiter must be non-negative";
    }
    if (g->bottom_height) {
        if (g->topology[2] != GBO_BOUNDED) return "GridFittedBottom requires Bounded z";
        for (int q = 0; q < g->size[0] * g->size[1]; ++q)
            if (std::isnan(g->bottom_height[q])) return "bottom_height must not be NaN";
    }
    return "";
}

}  // namespace

// Message for gbo_last_error(NULL) from entry points in other translation units.
void gbo_record_error(const char* msg) { g_last_error = msg; }

extern "C" {

int gbo_cg_parameters(const gbo_grid_desc* grid, const gbo_model_desc* desc, double* reltol, double* abstol,
                      double* maxiter) {
    if (!grid || !desc || !reltol || !abstol || !maxiter) return GBO_ERR_INVALID;
    const int64_t cells = (int64_t)grid->size[0] * grid->size[1] * (grid->topology[2] == GBO_FLAT ? 1 : grid->size[2]);
    cg_parameters(grid->float_type, *desc, cells, reltol, abstol, maxiter);
    return GBO_OK;
}

void gbo_model_desc_default(gbo_model_desc* d) {
    std::memset(d, 0, sizeof(*d));
    d->advection = GBO_ADVECTION_WENO5;
    d->closure = GBO_CLOSURE_NONE;
    d->closure_C = 0.16;
    d->closure_Cb = 1.0;
    d->closure_Pr = 1.0;
    d->pressure_solver = GBO_SOLVER_FFT;
    d->preconditioner = GBO_PRECOND_FFT;
    d->timestepper = GBO_TIMESTEPPER_RK3;
    d->ab2_chi = 0.1;
    d->closure_min_numerator = 1e-32;
    d->closure_averaging = GBO_AVERAGING_LAGRANGIAN;
}

int gbo_model_create(const gbo_grid_desc* grid, const gbo_model_desc* desc, gbo_model** out) {
    if (!out) { g_last_error = "null output handle"; return GBO_ERR_INVALID; }
    *out = nullptr;
    std::string why = validate(grid, desc);
    if (!why.empty()) { g_last_error = why; return GBO_ERR_INVALID; }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        g_last_error = "no CUDA device visible";
        return GBO_ERR_NO_DEVICE;
    }
    gbo_model* m = nullptr;
    int rc = guarded(nullptr, [&]() {
        if (grid->float_type == GBO_FLOAT32) {
            auto* mm = new ModelImpl<float>();
            m = mm;
            mm->init(grid, desc);
        } else {
            auto* mm = new ModelImpl<double>();
            m = mm;
            mm->init(grid, desc);
        }
        return GBO_OK;
    });
    if (rc != GBO_OK) {
        delete m;
        return rc;
    }
    *out = m;
    return GBO_OK;
}

void gbo_model_destroy(gbo_model* m) { delete m; }

int gbo_set_field(gbo_model* m, int32_t field, const void* host, int32_t dtype, int64_t count) {
    if (!m || !host) return GBO_ERR_INVALID;
    if (dtype != GBO_FLOAT32 && dtype != GBO_FLOAT64) { m->err = "dtype must be GBO_FLOAT32 or GBO_FLOAT64"; return GBO_ERR_INVALID; }
    return guarded(m, [&]() { return m->set_field(field, host, dtype, count); });
}

int gbo_set_finalize(gbo_model* m, int32_t enforce) {
    if (!m) return GBO_ERR_INVALID;
    return guarded(m, [&]() { return m->set_finalize(enforce); });
}

int gbo_get_field(gbo_model* m, int32_t field, void* host, int32_t dtype, int64_t count) {
    if (!m || !host) return GBO_ERR_INVALID;
    if (dtype != GBO_FLOAT32 && dtype != GBO_FLOAT64) { m->err = "dtype must be GBO_FLOAT32 or GBO_FLOAT64"; return GBO_ERR_INVALID; }
    return guarded(m, [&]() { return m->get_field(field, host, dtype, count); });
}

int64_t gbo_field_count(const gbo_model* m, int32_t field) { return m ? m->count(field) : -1; }

int64_t gbo_state_bytes(const gbo_model* m) { return m ? m->state_bytes() : 0; }

int gbo_field_reference_profile(gbo_model* m, int32_t field, double* out, int64_t count) {
    if (!m || !out) return GBO_ERR_INVALID;
    return guarded(m, [&]() { return m->reference_profile(field, out, count); });
}

int gbo_get_state(gbo_model* m, void* buf, int64_t bytes) {
    if (!m || !buf) return GBO_ERR_INVALID;
    return guarded(m, [&]() { return m->get_state(buf, bytes); });
}

int gbo_set_state(gbo_model* m, const void* buf, int64_t bytes) {
    if (!m || !buf) return GBO_ERR_INVALID;
    return guarded(m, [&]() { return m->set_state(buf, bytes); });
}

void gbo_run_desc_default(gbo_run_desc* d) {
    if (!d) return;
    std::memset(d, 0, sizeof(*d));
    d->dt = 1.0;
    d->stop_time = INFINITY;
    d->stop_iteration = INFINITY;
    d->wall_time_limit = INFINITY;
    d->align_time_step = 1;
    d->minimum_relative_step = 0.0;
    d->nan_check_interval = 100;
    d->nan_erroring = 0;
    d->wizard_interval = 0;
    d->cfl = 0.2;
    d->diffusive_cfl = INFINITY;
    d->max_change = 1.1;
    d->min_change = 0.5;
    d->max_dt = INFINITY;
    d->min_dt = 0.0;
    d->iterations_per_launch = 100;
}

int gbo_run(gbo_model* m, const gbo_run_desc* d, gbo_run_result* out) {
    if (!m || !d) return GBO_ERR_INVALID;
    return guarded(m, [&]() { return m->run(d, out); });
}

int gbo_cell_advection_timescale(gbo_model* m, double* out) {
    if (!m || !out) return GBO_ERR_INVALID;
    return guarded(m, [&]() { return m->timescales(out, nullptr); });
}

int gbo_cell_diffusion_timescale(gbo_model* m, double* out) {
    if (!m || !out) return GBO_ERR_INVALID;
    return guarded(m, [&]() { return m->timescales(nullptr, out); });
}

int gbo_field_device_pointer(gbo_model* m, int32_t field, void** dptr, int64_t* count) {
    if (!m || !dptr || !count) return GBO_ERR_INVALID;
    return guarded(m, [&]() { return m->device_pointer(field, dptr, count); });
}

int gbo_time_step(gbo_model* m, double dt, int32_t nsteps) {
    if (!m) return GBO_ERR_INVALID;
    if (!(dt > 0) || !std::isfinite(dt)) { m->err = "dt must be positive and finite"; return GBO_ERR_INVALID; }
    return guarded(m, [&]() { return m->step(dt, nsteps); });
}

// ---------------------------------------------------------------------------
// Ensemble: independent models advanced together.  One time step of every member
// is captured into one CUDA graph as parallel branches (each member's stream is
// forked from the ensemble's stream with an event and joined back), so a single
// graph launch advances all members and the members of different sizes fill the
// GPU together.  No reference counterpart (the reference steps models one by one).
// ---------------------------------------------------------------------------
}  // extern "C"

struct gbo_ensemble {
    std::vector<gbo_model*> members;
    cudaStream_t stream = nullptr;
    cudaEvent_t fork = nullptr, done = nullptr;
    std::vector<cudaEvent_t> joins;
    cudaGraphExec_t graph = nullptr;
    float* d_f32 = nullptr;         // stage factors of Δt for the FP32 and the FP64 members
    double* d_f64 = nullptr;
    std::vector<int64_t> per_step;  // kernels each member records per step
    std::string err;

    ~gbo_ensemble() {
        if (graph) cudaGraphExecDestroy(graph);
        if (d_f32) cudaFree(d_f32);
        if (d_f64) cudaFree(d_f64);
        for (cudaEvent_t e : joins) cudaEventDestroy(e);
        if (fork) cudaEventDestroy(fork);
        if (done) cudaEventDestroy(done);
        if (stream) cudaStreamDestroy(stream);
        for (gbo_model* mm : members) delete mm;
    }

    void build() {
        if (!d_f32) GBO_CUDA(cudaMalloc(&d_f32, DTF_N * sizeof(float)));
        if (!d_f64) GBO_CUDA(cudaMalloc(&d_f64, DTF_N * sizeof(double)));
        cudaGraph_t g;
        GBO_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        GBO_CUDA(cudaEventRecord(fork, stream));
        try {
            for (size_t i = 0; i < members.size(); ++i) {
                cudaStream_t ms = static_cast<cudaStream_t>(members[i]->stream_ptr());
                GBO_CUDA(cudaStreamWaitEvent(ms, fork, 0));
                per_step[i] = members[i]->capture_step(d_f32, d_f64);
                GBO_CUDA(cudaEventRecord(joins[i], ms));
                GBO_CUDA(cudaStreamWaitEvent(stream, joins[i], 0));
            }
        } catch (...) {
            cudaGraph_t partial = nullptr;
            cudaStreamEndCapture(stream, &partial);
            if (partial) cudaGraphDestroy(partial);
            for (gbo_model* mm : members) mm->abort_capture();
            throw;
        }
        GBO_CUDA(cudaStreamEndCapture(stream, &g));
        GBO_CUDA(cudaGraphInstantiate(&graph, g, 0));
        GBO_CUDA(cudaGraphDestroy(g));
    }

    int step(double dt, int nsteps) {
        if (nsteps <= 0) return GBO_OK;
        if (!graph) build();
        k_set_dt_pair<<<1, 1, 0, stream>>>(d_f32, ModelImpl<float>::rk3_stage_c(), d_f64, ModelImpl<double>::rk3_stage_c(), dt);
        GBO_CUDA(cudaGetLastError());
        for (int s = 0; s < nsteps; ++s) GBO_CUDA(cudaGraphLaunch(graph, stream));
        members[0]->add_launches(1);  // k_set_dt_pair
        GBO_CUDA(cudaEventRecord(done, stream));
        int rc = GBO_OK;
        for (size_t i = 0; i < members.size(); ++i) {
            GBO_CUDA(cudaStreamWaitEvent(static_cast<cudaStream_t>(members[i]->stream_ptr()), done, 0));
            members[i]->add_launches(per_step[i] * nsteps);
            int r = members[i]->finish_steps(dt, nsteps);
            if (r != GBO_OK && rc == GBO_OK) {
                rc = r;
                err = "member " + std::to_string(i) + ": " + members[i]->err;
            }
        }
        return rc;
    }
};

namespace {
template <class F>
int eguarded(gbo_ensemble* e, F&& f) {
    try {
        return f();
    } catch (const CudaError& x) {
        std::string msg = std::string("CUDA error in ") + x.what + ": " + cudaGetErrorString(x.e);
        if (e) e->err = msg;
        g_last_error = msg;
        return GBO_ERR_CUDA;
    } catch (const std::exception& x) {
        if (e) e->err = x.what();
        g_last_error = x.what();
        return GBO_ERR_INVALID;
    }
}
}  // namespace

extern "C" {

int gbo_ensemble_create(int32_t n, const gbo_grid_desc* grids, const gbo_model_desc* descs, gbo_ensemble** out) {
    if (!out || !grids || !descs || n < 1) { g_last_error = "invalid ensemble arguments"; return GBO_ERR_INVALID; }
    *out = nullptr;
    for (int32_t i = 0; i < n; ++i)
        if (descs[i].timestepper != GBO_TIMESTEPPER_RK3) {
            g_last_error = "member " + std::to_string(i) + ": ensembles step RungeKutta3 models only";
            return GBO_ERR_INVALID;
        } else if (descs[i].closure == GBO_CLOSURE_DYNAMIC_SMAGORINSKY && descs[i].closure_averaging == GBO_AVERAGING_LAGRANGIAN) {
            // its FP64 clock advances with the member's own time_step! calls, not the ensemble's
            g_last_error = "member " + std::to_string(i) + ": a Lagrangian-averaged DynamicSmagorinsky cannot join an ensemble";
            return GBO_ERR_INVALID;
        }
    auto* e = new gbo_ensemble();
    for (int32_t i = 0; i < n; ++i) {
        gbo_model* mm = nullptr;
        int rc = gbo_model_create(&grids[i], &descs[i], &mm);
        if (rc != GBO_OK) {
            g_last_error = "member " + std::to_string(i) + ": " + g_last_error;
            delete e;
            return rc;
        }
        mm->ensemble_member = true;
        e->members.push_back(mm);
    }
    int rc = eguarded(e, [&]() {
        GBO_CUDA(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking));
        GBO_CUDA(cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming));
        GBO_CUDA(cudaEventCreateWithFlags(&e->done, cudaEventDisableTiming));
        e->joins.resize(n);
        for (auto& ev : e->joins) GBO_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        e->per_step.assign(n, 0);
        return GBO_OK;
    });
    if (rc != GBO_OK) {
        delete e;
        return rc;
    }
    *out = e;
    return GBO_OK;
}

void gbo_ensemble_destroy(gbo_ensemble* e) { delete e; }

int32_t gbo_ensemble_size(const gbo_ensemble* e) { return e ? (int32_t)e->members.size() : 0; }

gbo_model* gbo_ensemble_member(gbo_ensemble* e, int32_t i) {
    if (!e || i < 0 || i >= (int32_t)e->members.size()) return nullptr;
    return e->members[i];
}

int gbo_ensemble_stream(gbo_ensemble* e, void** stream) {
    if (!e || !stream) return GBO_ERR_INVALID;
    *stream = (void*)e->stream;
    return GBO_OK;
}

int gbo_ensemble_time_step(gbo_ensemble* e, double dt, int32_t nsteps) {
    if (!e) return GBO_ERR_INVALID;
    if (!(dt > 0) || !std::isfinite(dt)) { e->err = "dt must be positive and finite"; g_last_error = e->err; return GBO_ERR_INVALID; }
    int rc = eguarded(e, [&]() { return e->step(dt, nsteps); });
    if (rc != GBO_OK) g_last_error = e->err;
    return rc;
}

int gbo_clock(const gbo_model* m, double* time, int64_t* iteration) {
    if (!m) return GBO_ERR_INVALID;
    if (time) *time = m->time;
    if (iteration) *iteration = m->iteration;
    return GBO_OK;
}

int gbo_synchronize(gbo_model* m) {
    if (!m) return GBO_ERR_INVALID;
    return guarded(m, [&]() { return m->sync(); });
}

int32_t gbo_last_solver_iterations(const gbo_model* m) { return m ? m->last_iters : 0; }

const char* gbo_last_error(const gbo_model* m) {
    if (m && !m->err.empty()) return m->err.c_str();
    return g_last_error.c_str();
}

const char* gbo_version(void) { return "gb300ocean 0.1.0 (sm_103a)"; }

int gbo_model_stream(gbo_model* m, void** stream) {
    if (!m || !stream) return GBO_ERR_INVALID;
    *stream = m->stream_ptr();
    return GBO_OK;
}

int64_t gbo_kernel_launches(const gbo_model* m) { return m ? m->launch_count() : -1; }

int gbo_kernel_timings(gbo_model* m, double dt, int32_t nsteps, double* ms, int32_t nmax) {
    if (!m || !ms) return GBO_ERR_INVALID;
    if (!(dt > 0) || !std::isfinite(dt)) { m->err = "dt must be positive and finite"; return GBO_ERR_INVALID; }
    return guarded(m, [&]() { return m->timed_steps(dt, nsteps, ms, nmax); });
}

int32_t gbo_kernel_group_count(void) { return GROUPS; }

int gbo_get_launch_shape(const gbo_model* m, gbo_launch_shape* out) {
    if (!m || !out) return GBO_ERR_INVALID;
    return m->launch_shape(out);
}

int gbo_set_launch_shape(gbo_model* m, const gbo_launch_shape* shape) {
    if (!m || !shape) return GBO_ERR_INVALID;
    return guarded(m, [&]() { return m->set_launch_shape(shape); });
}

int gbo_kernel_timing_counts(const gbo_model* m, int64_t* n, int32_t nmax) {
    if (!m || !n || nmax < 0) return GBO_ERR_INVALID;
    return m->timing_counts(n, nmax);
}

const char* gbo_kernel_group_name(int32_t g) { return (g >= 0 && g < GROUPS) ? GROUP_NAMES[g] : ""; }

int gbo_poisson_solve_device(gbo_model* m, void* phi, const void* rhs) {
    if (!m || !phi || !rhs) return GBO_ERR_INVALID;
    return guarded(m, [&]() { return m->poisson_device(phi, rhs); });
}

int64_t gbo_learned_weight_count(void) { return learned::file_count(); }

int gbo_learned_preconditioner(gbo_model* m, const float* weights, int64_t count) {
    if (!m) return GBO_ERR_INVALID;
    return guarded(m, [&]() { return m->set_learned(weights, count); });
}

int gbo_poisson_operator_device(gbo_model* m, const void* x, void* out) {
    if (!m || !x || !out || x == out) return GBO_ERR_INVALID;
    return guarded(m, [&]() { return m->operator_device(x, out); });
}

int gbo_precondition_device(gbo_model* m, const void* r, void* z) {
    if (!m || !r || !z) return GBO_ERR_INVALID;
    return guarded(m, [&]() { return m->precondition_device(r, z); });
}

}  // extern "C"
