// gbo_static_poisson.cu -- gbo_poisson_solve_fft_static: the FFT-based Poisson
// solve of gbo_poisson_solve_device with its work space in one fixed device
// array instead of memory allocated for a model.
//
// The solve is the same pass chain as the model's FFT solver (DCT-II in z on a
// Bounded z, real FFT in x, FFT + eigenvalue divide + inverse FFT in y,
// inverse real FFT in x, inverse DCT in z) and launches the same kernels.  The
// real work buffer is the caller's ϕ; the complex spectrum, the twiddle tables
// and the eigenvalue tables live in g_scratch.  Nothing in g_scratch has to
// start at zero: every table is rewritten at the start of every call and every
// spectral coefficient is written by a forward pass before any pass reads it.
//
// This translation unit is its own device module, so the static array is
// reserved only in processes that call this entry point (the module is loaded
// on first use).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <mutex>

#include "../../include/gbo.h"
#include "gbo_fft.cuh"

void gbo_record_error(const char* msg);  // gbo_model.cu: message for gbo_last_error(NULL)

namespace {

static_assert(GBO_STATIC_SCRATCH_BYTES % 256 == 0, "scratch size must be a multiple of 256 bytes");
static __device__ __align__(256) unsigned char g_scratch[GBO_STATIC_SCRATCH_BYTES];

std::mutex g_setup_mutex;
// per-context set-up already done: the ID of the CUDA context (unique for the life of the
// process) and its opt-in shared-memory limit
constexpr int kMaxContexts = 64;
unsigned long long g_ctx_ids[kMaxContexts] = {};
int g_ctx_optin[kMaxContexts] = {};
int g_nctx = 0;

thread_local char g_msg[256];

int fail(int code, const char* fmt, long long a = 0, long long b = 0) {
    std::snprintf(g_msg, sizeof(g_msg), fmt, a, b);
    gbo_record_error(g_msg);
    return code;
}
int fail_msg(int code, const char* msg) {
    gbo_record_error(msg);
    return code;
}

// Radix plan with the same factor order as the model's solver (4s, then 2, 3, 5),
// so both solves run identical butterflies.
bool plan(int n, FFTPlan1D& p) {
    p.n = n;
    p.nrad = 0;
    int m = n;
    while (m % 4 == 0 && p.nrad < GBO_MAX_RADICES) { p.rad[p.nrad++] = 4; m /= 4; }
    for (int r : {2, 3, 5})
        while (m % r == 0 && p.nrad < GBO_MAX_RADICES) { p.rad[p.nrad++] = r; m /= r; }
    return m == 1 && n >= 1;
}

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

// Byte layout of the scratch for one grid: spectrum, twiddles, eigenvalues.
template <typename FT>
struct Layout {
    size_t cb, tw_xh, tw_x, tw_y, tw_z, tq_z, lx, ly, lz, total;
    Layout(int Nx, int Ny, int Nz) {
        const size_t C = sizeof(Cx<FT>), Nh = (size_t)Nx / 2 + 1;
        size_t at = 0;
        auto take = [&](size_t bytes) { size_t o = at; at += align256(bytes); return o; };
        cb = take(Nh * Ny * Nz * C);
        tw_xh = take((size_t)(Nx / 2) * C);
        tw_x = take((size_t)Nx * C);
        tw_y = take((size_t)Ny * C);
        tw_z = take((size_t)Nz * C);
        tq_z = take((size_t)Nz * C);
        lx = take(Nh * sizeof(FT));
        ly = take((size_t)Ny * sizeof(FT));
        lz = take((size_t)Nz * sizeof(FT));
        total = at;
    }
};

// Twiddles exp(-2πi f m / n) and Poisson eigenvalues (poisson_eigenvalues.jl:8-23)
// evaluated in FP64 and rounded to FT, as the model computes them on the host.
template <typename FT>
__global__ void k_static_tables(PassP<FT> P, Cx<FT>* tw_xh, Cx<FT>* tw_x, Cx<FT>* tw_y, Cx<FT>* tw_z, Cx<FT>* tq_z,
                                FT* lx, FT* ly, FT* lz, double Lx, double Ly, double Lz) {
    const int Nx = P.Nx, Ny = P.Ny, Nz = P.Nz, Nh = P.Nh;
    auto twiddle = [](Cx<FT>* t, int m, int n, double f) {
        double s, c;
        sincospi(-2.0 * f * (double)m / (double)n, &s, &c);
        t[m] = Cx<FT>{FT(c), FT(s)};
    };
    const int total = Nx / 2 + Nx + Ny + 2 * Nz + Nh + Ny + Nz;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < total; q += gridDim.x * blockDim.x) {
        int m = q;
        if (m < Nx / 2) { twiddle(tw_xh, m, Nx / 2, 1.0); continue; }
        m -= Nx / 2;
        if (m < Nx) { twiddle(tw_x, m, Nx, 1.0); continue; }
        m -= Nx;
        if (m < Ny) { twiddle(tw_y, m, Ny, 1.0); continue; }
        m -= Ny;
        if (m < Nz) { twiddle(tw_z, m, Nz, 1.0); continue; }
        m -= Nz;
        if (m < Nz) { twiddle(tq_z, m, Nz, 0.25); continue; }
        m -= Nz;
        if (m < Nh) {
            double s = 2 * sinpi((double)m / Nx) / (Lx / Nx);
            lx[m] = FT(s * s);
            continue;
        }
        m -= Nh;
        if (m < Ny) {
            double s = 2 * sinpi((double)m / Ny) / (Ly / Ny);
            ly[m] = FT(s * s);
            continue;
        }
        m -= Ny;
        double s = 2 * sinpi((double)m / (2.0 * Nz)) / (Lz / Nz);
        lz[m] = P.has_z ? FT(s * s) : FT(0);
    }
}

// The address of g_scratch in the current context, looked up on every call (a host-side
// lookup): the array belongs to the module loaded in a context, and a context reset
// (cudaDeviceReset, a primary-context reset, or another context made current) loads the
// module again, possibly elsewhere.  Once per context, with that context current: the
// opt-in shared-memory limit and the pass kernels' dynamic shared-memory attribute
// (function attributes are per context too).  The context is identified by its ID from
// the driver (cuCtxGetId, fetched through the runtime's driver entry point so the library
// needs no link to libcuda).
typedef int (*CtxGetCurrentFn)(void** ctx);
typedef int (*CtxGetIdFn)(void* ctx, unsigned long long* id);

int setup(int dev, unsigned char** base, int* optin) {
    void* p = nullptr;
    cudaError_t rc = cudaGetSymbolAddress(&p, g_scratch);  // also makes the context current
    if (rc != cudaSuccess) return fail(GBO_ERR_CUDA, "cudaGetSymbolAddress of the static scratch failed (error %lld)", (long long)rc);
    *base = static_cast<unsigned char*>(p);
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!get_current || !get_id) {
        cudaDriverEntryPointQueryResult q1, q2;
        void* f1 = nullptr;
        void* f2 = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
            q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess)
            return fail_msg(GBO_ERR_CUDA, "the driver does not provide cuCtxGetCurrent / cuCtxGetId");
        get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
        get_id = reinterpret_cast<CtxGetIdFn>(f2);
    }
    void* ctx = nullptr;
    unsigned long long id = 0;
    if (get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0)
        return fail_msg(GBO_ERR_CUDA, "no current CUDA context after the scratch lookup");
    for (int q = 0; q < g_nctx; ++q)
        if (g_ctx_ids[q] == id) {
            *optin = g_ctx_optin[q];
            return GBO_OK;
        }
    int v = 0;
    rc = cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (rc != cudaSuccess) return fail(GBO_ERR_CUDA, "cudaDeviceGetAttribute failed (error %lld)", (long long)rc);
    // Raise (never lower) the pass kernels' dynamic shared-memory limit, for both float
    // types, to the opt-in maximum: models set the same value when they are created, so
    // no later call lowers it.
    rc = fft_set_smem<float>(v, v, v);
    if (rc == cudaSuccess) rc = fft_set_smem<double>(v, v, v);
    if (rc != cudaSuccess) return fail(GBO_ERR_CUDA, "cudaFuncSetAttribute failed (error %lld)", (long long)rc);
    if (g_nctx < kMaxContexts) {
        g_ctx_ids[g_nctx] = id;
        g_ctx_optin[g_nctx] = v;
        ++g_nctx;
    }
    *optin = v;
    return GBO_OK;
}

template <typename FT>
int solve(const gbo_grid_desc* gd, void* phi, const void* rhs, cudaStream_t st) {
    const bool flat = gd->topology[2] == GBO_FLAT;
    const int Nx = gd->size[0], Ny = gd->size[1], Nz = flat ? 1 : gd->size[2];
    const Layout<FT> L(Nx, Ny, Nz);
    if (L.total > (size_t)GBO_STATIC_SCRATCH_BYTES)
        return fail(GBO_ERR_INVALID,
                    "grid needs %lld bytes of scratch but the static scratch holds %lld bytes (GBO_STATIC_SCRATCH_BYTES); "
                    "use gbo_poisson_solve_device on a model for larger grids",
                    (long long)L.total, (long long)GBO_STATIC_SCRATCH_BYTES);
    PassP<FT> P{};
    P.Nx = Nx; P.Ny = Ny; P.Nz = Nz; P.Nh = Nx / 2 + 1;
    if (!plan(Nx / 2, P.px_half) || !plan(Ny, P.py) || !plan(Nz, P.pz))
        return fail_msg(GBO_ERR_INVALID, "grid sizes must factor into 2, 3 and 5 for the FFT-based Poisson solver");

    int dev = 0;
    cudaError_t rc = cudaGetDevice(&dev);
    if (rc != cudaSuccess) return fail(GBO_ERR_NO_DEVICE, "no CUDA device (error %lld)", (long long)rc);
    unsigned char* base = nullptr;
    int optin = 0;
    int s = setup(dev, &base, &optin);
    if (s != GBO_OK) return s;

    const size_t N = (size_t)Nx * Ny * Nz;
    P.rb = static_cast<FT*>(phi);
    P.cb = reinterpret_cast<Cx<FT>*>(base + L.cb);
    Cx<FT>* tw_xh = reinterpret_cast<Cx<FT>*>(base + L.tw_xh);
    Cx<FT>* tw_x = reinterpret_cast<Cx<FT>*>(base + L.tw_x);
    Cx<FT>* tw_y = reinterpret_cast<Cx<FT>*>(base + L.tw_y);
    Cx<FT>* tw_z = reinterpret_cast<Cx<FT>*>(base + L.tw_z);
    Cx<FT>* tq_z = reinterpret_cast<Cx<FT>*>(base + L.tq_z);
    FT* lx = reinterpret_cast<FT*>(base + L.lx);
    FT* ly = reinterpret_cast<FT*>(base + L.ly);
    FT* lz = reinterpret_cast<FT*>(base + L.lz);
    P.tw_xh = tw_xh; P.tw_x = tw_x; P.tw_y = tw_y; P.tw_z = tw_z; P.tq_z = tq_z;
    P.lx = lx; P.ly = ly; P.lz = lz;
    P.has_z = !flat;
    P.scale = flat ? FT(1.0 / ((double)Nx * Ny)) : FT(1.0 / ((double)Nx * Ny * Nz));

    // shared-memory tiles chosen exactly as the model's solver chooses them
    const size_t lim = GBO_PASS_SMEM_LIMIT;
    int ZT = GBO_DCT_TILE, XL = 8, YT = 16;
    while (ZT > 2 && dct_smem<FT>(ZT, Nz) > lim) ZT /= 2;
    while (XL > 1 && rfft_smem<FT>(XL, Nx) > lim) XL /= 2;
    while (YT > 1 && ffty_smem<FT>(YT, Ny) > lim) YT /= 2;
    const size_t smem_z = dct_smem<FT>(ZT, Nz), smem_x = rfft_smem<FT>(XL, Nx), smem_y = ffty_smem<FT>(YT, Ny);
    if (std::max({smem_z, smem_x, smem_y}) > (size_t)optin)
        return fail(GBO_ERR_INVALID, "grid needs %lld bytes of shared memory per block; the device allows %lld",
                    (long long)std::max({smem_z, smem_x, smem_y}), optin);

    if (phi != rhs) {
        rc = cudaMemcpyAsync(phi, rhs, N * sizeof(FT), cudaMemcpyDeviceToDevice, st);
        if (rc != cudaSuccess) return fail(GBO_ERR_CUDA, "copy of the right-hand side failed (error %lld)", (long long)rc);
    }
    const double Lx = (double)FT(gd->x[1] - gd->x[0]), Ly = (double)FT(gd->y[1] - gd->y[0]);
    const double Lz = flat ? 1.0 : (double)FT(gd->z[1] - gd->z[0]);
    k_static_tables<FT><<<8, 256, 0, st>>>(P, tw_xh, tw_x, tw_y, tw_z, tq_z, lx, ly, lz, Lx, Ly, Lz);
    if (!flat) launch_dct_z<FT>(P, 0, ZT, smem_z, st);
    launch_rfft_x<FT>(P, 0, XL, smem_x, st);
    launch_fft_y<FT>(P, 0, YT, smem_y, st);
    launch_rfft_x<FT>(P, 1, XL, smem_x, st);
    if (!flat) launch_dct_z<FT>(P, 1, ZT, smem_z, st);
    rc = cudaGetLastError();
    if (rc != cudaSuccess) return fail(GBO_ERR_CUDA, "Poisson pass launch failed (error %lld)", (long long)rc);
    return GBO_OK;
}

const char* check_grid(const gbo_grid_desc* g) {
    if (!g) return "null grid descriptor";
    if (g->topology[0] != GBO_PERIODIC || g->topology[1] != GBO_PERIODIC) return "x and y must be Periodic";
    if (g->topology[2] != GBO_BOUNDED && g->topology[2] != GBO_FLAT) return "z must be Bounded or Flat";
    if (g->float_type != GBO_FLOAT32 && g->float_type != GBO_FLOAT64) return "float_type must be GBO_FLOAT32 or GBO_FLOAT64";
    if (g->z_faces) return "FFTBasedPoissonSolver requires a regular grid (z_faces must be NULL)";
    if (g->bottom_height) return "the FFT-based solve takes no immersed boundary (bottom_height must be NULL)";
    const int nz = g->topology[2] == GBO_FLAT ? 1 : g->size[2];
    if (g->size[0] < 8 || g->size[1] < 8 || nz < 1) return "Nx and Ny must be at least 8";
    if (g->size[0] % 2) return "Nx must be even";
    if (g->topology[2] == GBO_BOUNDED && nz < 6) return "Nz must be at least 6 on a Bounded z";
    if (!(g->x[1] > g->x[0]) || !(g->y[1] > g->y[0])) return "x and y extents must be increasing";
    if (g->topology[2] == GBO_BOUNDED && !(g->z[1] > g->z[0])) return "z extent must be increasing";
    return nullptr;
}

}  // namespace

extern "C" int gbo_poisson_solve_fft_static(const gbo_grid_desc* grid, void* phi_device, const void* rhs_device,
                                            void* cuda_stream) {
    if (const char* why = check_grid(grid)) return fail_msg(GBO_ERR_INVALID, why);
    if (!phi_device || !rhs_device) return fail_msg(GBO_ERR_INVALID, "null device buffer");
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
    return grid->float_type == GBO_FLOAT32 ? solve<float>(grid, phi_device, rhs_device, st)
                                           : solve<double>(grid, phi_device, rhs_device, st);
}
