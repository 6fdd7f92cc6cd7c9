// gbo_learned.cu -- kernels and host side of the learned preconditioner correction
// (see gbo_learned.cuh for the network, the layouts and the boundary rules).
#include <cmath>
#include <vector>

#include "gbo_learned.cuh"
#include "gbo_umma.cuh"

namespace learned {

using bf16 = __nv_bfloat16;

struct ConvP {
    const bf16* in;      // [n][cin]
    const bf16* w;       // [cout][kpad(cin)]
    const float* bias;   // [cout]
    bf16* out;           // mode 0: [n][cout]
    void* z;             // mode 1: FT field, z += s (acc + bias) for output channel 0
    const float* scale;  // mode 1: s (the RMS of the incoming z)
    Dims d;
};

GBO_D void cp16(void* smem, const void* src, bool valid) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(src), "r"(valid ? 16 : 0));
}
GBO_D void cp_commit() { asm volatile("cp.async.commit_group;\n" ::); }

// D = A B + D for one 16 × 8 × 16 tile: A row-major 16 × 16, B column-major 16 × 8
// (BF16), D FP32.  Fragments (g = lane / 4, t = lane % 4): a0 = A[g][2t..], a1 =
// A[g+8][2t..], a2 = A[g][2t+8..], a3 = A[g+8][2t+8..]; b0 = B[2t..][g], b1 = B[2t+8..][g];
// d0, d1 = D[g][2t, 2t+1], d2, d3 = D[g+8][2t, 2t+1].
GBO_D void mma16816(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

GBO_D uint32_t pack2(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);  // .x = lo (lower address)
    return *reinterpret_cast<const uint32_t*>(&v);
}

GBO_D void ldsm_x4(uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3, const bf16* p) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3) : "r"(a));
}
GBO_D void ldsm_x2(uint32_t& r0, uint32_t& r1, const bf16* p) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];\n" : "=r"(r0), "=r"(r1) : "r"(a));
}

// Halo-tile convolution: a block computes a TX × TY patch of one z level (128 cells) ×
// cout.  Per 16-channel chunk of the input it stages the (TX+2) × (TY+2) × 3 halo tile
// once in shared memory (each input value then serves all 27 taps) and the chunk's
// weights [cout][27 taps × 16]; each warp then issues, per tap, one ldmatrix for its
// 16 rows of A (rows of the tile shifted by the tap) and cout / 8 MMAs.
namespace halo {
constexpr int TX = 32, TY = 4, HX = TX + 2, HY = TY + 2, HC = HX * HY * 3;  // tile cells
constexpr int CS = 24;             // shared stride of one tile cell (16 channels + pad; conflict-free)
constexpr int BS = 27 * 16 + 8;    // shared stride of one weight row
template <int COUT>
constexpr size_t smem_bytes() { return (size_t)(HC * CS + COUT * BS) * sizeof(bf16); }
}  // namespace halo

template <int CIN, int COUT, int MODE, typename FT>
__global__ void __launch_bounds__(256) k_conv_halo(ConvP p) {
    using namespace halo;
    static_assert((CIN == 8 || CIN % 16 == 0) && COUT % 8 == 0 && COUT <= 64, "channel counts");
    static_assert(CIN != 8 || COUT % 16 == 0, "the 8-channel path pairs n tiles");
    constexpr int NCH = CIN == 8 ? 1 : CIN / 16, CW = CIN == 8 ? 8 : 16;  // chunks, channels per chunk
    constexpr int NT = COUT / 8, KP = kpad(CIN);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    bf16* tile = reinterpret_cast<bf16*>(smem_raw);  // [HC][CS]
    bf16* wsm = tile + HC * CS;                       // [COUT][BS]
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
    const int nx = p.d.nx, ny = p.d.ny, nz = p.d.nz;
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z = blockIdx.z;
    // this warp's 16 output rows: y = y0 + my, x = x0 + mx0 .. mx0 + 15
    const int my = warp >> 1, mx0 = (warp & 1) * 16;
    float acc[NT][4];
#pragma unroll
    for (int q = 0; q < NT; ++q) acc[q][0] = acc[q][1] = acc[q][2] = acc[q][3] = 0.f;
    for (int cc = 0; cc < NCH; ++cc) {
        // halo tile: 16-byte pieces (HC cells × 2 halves)
        for (int e = tid; e < HC * 2; e += 256) {
            const int c = e >> 1, h = e & 1;
            const int tx = c % HX, ty = (c / HX) % HY, tz = c / (HX * HY);
            const int gx = wrapm(x0 + tx - 1, nx), gy = wrapm(y0 + ty - 1, ny), gz = z + tz - 1;
            const bool ok = gz >= 0 && gz < nz && h * 8 < CW;
            const int64_t src = (gx + (int64_t)nx * (gy + (int64_t)ny * gz)) * CIN + cc * 16 + h * 8;
            cp16(tile + c * CS + h * 8, p.in + (ok ? src : 0), ok);
        }
        if constexpr (CIN == 8) {
            // 8 channels: k = tap · 8 + c as stored, two taps per 16-wide MMA step
            for (int e = tid; e < COUT * 28; e += 256) {
                const int n = e / 28, piece = e % 28;
                cp16(wsm + n * BS + piece * 8, p.w + (int64_t)n * KP + piece * 8, true);
            }
        } else {
            // weights of this chunk: row n, tap, 16 channels (two pieces)
            for (int e = tid; e < COUT * 27 * 2; e += 256) {
                const int n = e / 54, rem = e % 54, tap = rem >> 1, h = rem & 1;
                const int64_t src = (int64_t)n * KP + tap * CIN + cc * 16 + h * 8;
                cp16(wsm + n * BS + tap * 16 + h * 8, p.w + src, true);
            }
        }
        cp_commit();
        asm volatile("cp.async.wait_group 0;\n" ::);
        __syncthreads();
        // A rows: lane → row (lane & 15), k half (lane >> 4)
        const int ar = lane & 15, ah = (lane >> 4) * 8;
        if constexpr (CIN == 8) {
            // step s covers taps 2s (k 0-7, lanes 0-15) and 2s + 1 (k 8-15, lanes 16-31); the
            // 28th tap of the last step has zero weights
#pragma unroll 2
            for (int st = 0; st < 14; ++st) {
                const int tap = min(2 * st + (lane >> 4), 26);
                const int dz = tap / 9, dy = (tap / 3) % 3, dx = tap % 3;
                const int tc = (dz * HY + my + dy) * HX + mx0 + ar + dx;
                uint32_t a0, a1, a2, a3;
                ldsm_x4(a0, a1, a2, a3, tile + tc * CS);
#pragma unroll
                for (int q = 0; q < NT; q += 2) {
                    uint32_t b0, b1, b2, b3;
                    const int mi = lane >> 3;
                    ldsm_x4(b0, b1, b2, b3, wsm + ((q + (mi >> 1)) * 8 + (lane & 7)) * BS + st * 16 + (mi & 1) * 8);
                    mma16816(acc[q], a0, a1, a2, a3, b0, b1);
                    mma16816(acc[q + 1], a0, a1, a2, a3, b2, b3);
                }
            }
        } else {
#pragma unroll 3
            for (int tap = 0; tap < 27; ++tap) {
                const int dz = tap / 9, dy = (tap / 3) % 3, dx = tap % 3;  // tile offsets (0..2)
                const int tc = (dz * HY + my + dy) * HX + mx0 + ar + dx;
                uint32_t a0, a1, a2, a3;
                ldsm_x4(a0, a1, a2, a3, tile + tc * CS + ah);
                if constexpr (NT == 1) {
                    uint32_t b0, b1;
                    ldsm_x2(b0, b1, wsm + (lane & 7) * BS + tap * 16 + ((lane >> 3) & 1) * 8);
                    mma16816(acc[0], a0, a1, a2, a3, b0, b1);
                } else {
#pragma unroll
                    for (int q = 0; q < NT; q += 2) {
                        uint32_t b0, b1, b2, b3;
                        const int mi = lane >> 3;
                        ldsm_x4(b0, b1, b2, b3, wsm + ((q + (mi >> 1)) * 8 + (lane & 7)) * BS + tap * 16 + (mi & 1) * 8);
                        mma16816(acc[q], a0, a1, a2, a3, b0, b1);
                        mma16816(acc[q + 1], a0, a1, a2, a3, b2, b3);
                    }
                }
            }
        }
        __syncthreads();
    }
    const int y = y0 + my, xa = x0 + mx0 + g, xb = xa + 8;
    const bool oka = y < ny && xa < nx, okb = y < ny && xb < nx;
    const int64_t ra = xa + (int64_t)nx * (y + (int64_t)ny * z), rb = ra + 8;
    if constexpr (MODE == 0) {
#pragma unroll
        for (int q = 0; q < NT; ++q) {
            const int col = q * 8 + 2 * t;
            const float b0 = p.bias[col], b1 = p.bias[col + 1];
            if (oka)
                *reinterpret_cast<uint32_t*>(p.out + ra * COUT + col) =
                    pack2(fmaxf(acc[q][0] + b0, 0.f), fmaxf(acc[q][1] + b1, 0.f));
            if (okb)
                *reinterpret_cast<uint32_t*>(p.out + rb * COUT + col) =
                    pack2(fmaxf(acc[q][2] + b0, 0.f), fmaxf(acc[q][3] + b1, 0.f));
        }
    } else {
        if (t == 0) {
            FT* zz = static_cast<FT*>(p.z);
            const float s = *p.scale, b0 = p.bias[0];
            if (oka) zz[ra] += FT(s * (acc[0][0] + b0));
            if (okb) zz[rb] += FT(s * (acc[0][2] + b0));
        }
    }
}

// ---------------------------------------------------------------------------
// Convolution on the fifth-generation tensor cores (tcgen05, TMEM accumulators).
//
// Implicit GEMM: M = 128 cells of a level (one MMA, one TMEM lane each), N = 16 output
// channels per block, K = 27 taps × cin.  A block owns BY consecutive rows (y) of one
// z level and stages their halo -- rows y0-1 .. y0+BY, levels z-1 .. z+1, x with one
// periodic halo cell each side -- once in shared memory, channel plane by channel plane
// (8 channels of a cell = 16 bytes): plane cg holds, for every tile position, channels
// 8 cg .. 8 cg + 7.  Tile positions are flattened (dz, row, x + 1) with row stride
// RS = nx + 2, so output cell (row r, x) is M row m = r RS + x and its neighbour
// (dz, dy, dx) sits at tile position m + ((dz (BY + 2) + dy) RS + dx): every tap of the
// 3³ stencil is the same K-major canonical operand (8-row groups 128 bytes apart,
// SBO = 128) started at another 16-byte offset, so the tile is loaded once and each
// tap is one descriptor.  M rows that fall on halo positions or beyond the block's
// rows compute values that are never stored.  K = 16 per MMA: with 16 or more input
// channels one tap and two channel planes (LBO = the plane stride); with 8 input
// channels two consecutive taps (LBO = the distance of their offsets).  Weights are
// the B operand, [k group][16 outputs][8 k] per block.  One thread issues the MMAs,
// tcgen05.commit arrives on an mbarrier, the four warps read their 32 TMEM lanes each
// (tcgen05.ld) and apply bias and ReLU (or the final z update).
// ---------------------------------------------------------------------------
namespace umc {
constexpr int M = 128, NB = 16;
struct Geo {
    int BY, RS, MT, cells;  // rows per block, row stride, M tiles, tile positions per plane
};
GBO_HD Geo geo(int nx) {
    Geo g;
    g.RS = nx + 2;
    g.BY = nx >= M ? 1 : (M - nx) / g.RS + 1;
    g.MT = ((g.BY - 1) * g.RS + nx + M - 1) / M;
    const int tmax = (2 * (g.BY + 2) + 2) * g.RS + 2;  // offset of the last tap
    const int real = 3 * (g.BY + 2) * g.RS;
    g.cells = ((real > M * g.MT + tmax ? real : M * g.MT + tmax) + 7) / 8 * 8;
    return g;
}
GBO_HD constexpr int kgroups(int cin) { return cin == 8 ? 28 : 27 * cin / 8; }
inline size_t smem_bytes(int cin, int nx) {
    const Geo g = geo(nx);
    return (size_t)(cin / 8) * g.cells * 16 + (size_t)kgroups(cin) * NB * 16 + 16;
}
constexpr int WAIT_LIMIT = 1 << 24;  // mbarrier polls before a block reports a timeout
}  // namespace umc

struct UConvP {
    const bf16* in;      // [n][cin]
    const bf16* w;       // [cout / 16][k groups][16][8]
    const float* bias;   // [cout]
    bf16* out;           // mode 0: [n][cout]
    void* z;             // mode 1: FT field, z += s (acc + bias) for output channel 0
    const float* scale;  // mode 1: s
    unsigned* flags;     // GBO_FLAG_TIMEOUT on a wait that gave up (may be null)
    Dims d;
    int cout;
};

template <int CIN, int MODE, typename FT>
__global__ void __launch_bounds__(128) k_conv_umma(UConvP p) {
    using namespace umc;
    constexpr int PL = CIN / 8, KGN = kgroups(CIN);
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const Geo G = geo(p.d.nx);
    bf16* tile = reinterpret_cast<bf16*>(smem_raw);       // [PL][cells][8]
    bf16* wsm = tile + (size_t)PL * G.cells * 8;           // [KGN][NB][8]
    uint64_t* mbar = reinterpret_cast<uint64_t*>(wsm + KGN * NB * 8);
    uint32_t* slot = reinterpret_cast<uint32_t*>(mbar + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nx = p.d.nx, ny = p.d.ny, nz = p.d.nz;
    const int y0 = blockIdx.x * G.BY, z = blockIdx.y, nb = blockIdx.z;
    if (warp == 0) umma::tmem_alloc(slot, 32);
    if (tid == 0) umma::mbar_init(mbar, 1);
    const int real = 3 * (G.BY + 2) * G.RS;
    for (int e = tid; e < PL * G.cells; e += 128) {
        const int cg = e / G.cells, pos = e - cg * G.cells;
        int64_t src = 0;
        bool ok = false;
        if (pos < real) {
            const int xx = pos % G.RS, r = pos / G.RS, ry = r % (G.BY + 2), dz = r / (G.BY + 2);
            const int gz = z + dz - 1;
            if (gz >= 0 && gz < nz) {
                const int gx = wrapm(xx - 1, nx), gy = wrapm(y0 + ry - 1, ny);
                src = (gx + (int64_t)nx * (gy + (int64_t)ny * gz)) * CIN + cg * 8;
                ok = true;
            }
        }
        cp16(tile + ((size_t)cg * G.cells + pos) * 8, p.in + src, ok);
    }
    const bf16* wsrc = p.w + (size_t)nb * KGN * NB * 8;
    for (int e = tid; e < KGN * NB; e += 128) cp16(wsm + e * 8, wsrc + e * 8, true);
    cp_commit();
    asm volatile("cp.async.wait_group 0;\n" ::);
    umma::fence_smem_to_async();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = *slot;
    if (tid == 0) {
        constexpr uint32_t idesc = umma::idesc_bf16_f32(M, NB);
        const uint32_t tb = umma::smem_addr(tile), wb = umma::smem_addr(wsm);
        const uint32_t pstride = (uint32_t)G.cells * 16;
        auto toff = [&](int tap) { return ((tap / 9) * (G.BY + 2) + (tap / 3) % 3) * G.RS + tap % 3; };
        for (int q = 0; q < G.MT; ++q) {
            const uint32_t d = tmem + (uint32_t)(q * NB);
            if constexpr (CIN == 8) {
                for (int st = 0; st < 14; ++st) {
                    const int o0 = toff(2 * st), o1 = 2 * st + 1 <= 26 ? toff(2 * st + 1) : o0 + 1;
                    const uint64_t ad = umma::sdesc(tb + (uint32_t)(M * q + o0) * 16, (uint32_t)(o1 - o0) * 16, 128);
                    const uint64_t bd = umma::sdesc(wb + (uint32_t)(2 * st) * NB * 16, NB * 16, 128);
                    umma::mma_bf16(d, ad, bd, idesc, st > 0);
                }
            } else {
                for (int tap = 0; tap < 27; ++tap) {
                    const uint32_t a0 = tb + (uint32_t)(M * q + toff(tap)) * 16;
#pragma unroll
                    for (int c = 0; c < PL / 2; ++c) {
                        const uint64_t ad = umma::sdesc(a0 + (uint32_t)(2 * c) * pstride, pstride, 128);
                        const uint64_t bd = umma::sdesc(wb + (uint32_t)(tap * PL + 2 * c) * NB * 16, NB * 16, 128);
                        umma::mma_bf16(d, ad, bd, idesc, tap > 0 || c > 0);
                    }
                }
            }
        }
        umma::commit(mbar);
    }
    const bool done = umma::mbar_wait(mbar, 0, WAIT_LIMIT);
    if (!done && tid == 0 && p.flags) atomicOr(p.flags, GBO_FLAG_TIMEOUT);
    umma::fence_after_sync();
    if (done) {
        for (int q = 0; q < G.MT; ++q) {
            float v[16];
            umma::tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(q * NB), v);
            const int m = M * q + 32 * warp + lane;
            const int ry = m / G.RS, x = m - ry * G.RS, y = y0 + ry;
            if (ry < G.BY && x < nx && y < ny) {
                const int64_t cell = x + (int64_t)nx * (y + (int64_t)ny * z);
                if constexpr (MODE == 0) {
                    const float* b = p.bias + nb * NB;
                    uint4 o[2];
                    uint32_t* ow = reinterpret_cast<uint32_t*>(o);
#pragma unroll
                    for (int c = 0; c < 8; ++c) ow[c] = pack2(fmaxf(v[2 * c] + b[2 * c], 0.f), fmaxf(v[2 * c + 1] + b[2 * c + 1], 0.f));
                    uint4* dst = reinterpret_cast<uint4*>(p.out + cell * p.cout + nb * NB);
                    dst[0] = o[0];
                    dst[1] = o[1];
                } else {
                    FT* zz = static_cast<FT*>(p.z);
                    zz[cell] += FT(*p.scale * (v[0] + p.bias[0]));
                }
            }
        }
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_free(tmem, 32);
}

// s = sqrt(mean(r²)) (1 when r = 0): FP64 block sums, the last block finishes
template <typename FT>
__global__ void __launch_bounds__(256) k_rms(const FT* __restrict__ r, int64_t n, double* acc, unsigned* cnt, float* scale) {
    __shared__ double sh[8];
    __shared__ bool last;
    double v = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double x = (double)r[i];
        v += x * x;
    }
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) b += sh[w];
        atomicAdd(acc, b);
        __threadfence();
        last = atomicAdd(cnt, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        const double total = __ldcg(acc);
        const float s = (float)sqrt(total / (double)n);
        *scale = s > 0.f ? s : 1.f;
        *acc = 0.0;
        *cnt = 0u;
    }
}

// The first layer's input: (r / s_r, z / s_z, active, 0 …) in BF16, 8 channels per cell
template <typename FT>
__global__ void k_features(const FT* __restrict__ r, const FT* __restrict__ z, const int* __restrict__ kbot, Dims d,
                           const float* scale_r, const float* scale_z, bf16* __restrict__ out) {
    const int64_t n = d.n(), plane = (int64_t)d.nx * d.ny;
    const float inv = 1.f / *scale_r, invz = 1.f / *scale_z;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
        const int k = (int)(c / plane);
        const float active = (kbot && k < kbot[c % plane]) ? 0.f : 1.f;
        uint4 v;
        v.x = pack2((float)r[c] * inv, (float)z[c] * invz);
        v.y = pack2(active, 0.f);
        v.z = 0u;
        v.w = 0u;
        *reinterpret_cast<uint4*>(out + c * FEAT) = v;
    }
}

// Average pooling 2 × 2 × 2: one thread per coarse cell and 8 channels
template <int C>
__global__ void k_pool(const bf16* __restrict__ in, Dims fine, bf16* __restrict__ out) {
    const Dims cd{fine.nx / 2, fine.ny / 2, fine.nz / 2};
    const int64_t total = cd.n() * (C / 8);
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = e / (C / 8);
        const int ch = (int)(e % (C / 8)) * 8;
        const int i = (int)(c % cd.nx), j = (int)((c / cd.nx) % cd.ny), k = (int)(c / ((int64_t)cd.nx * cd.ny));
        float s[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        for (int o = 0; o < 8; ++o) {
            const int64_t f = (2 * i + (o & 1)) + (int64_t)fine.nx * ((2 * j + ((o >> 1) & 1)) + (int64_t)fine.ny * (2 * k + (o >> 2)));
            const uint4 v = *reinterpret_cast<const uint4*>(in + f * C + ch);
            const bf16* h = reinterpret_cast<const bf16*>(&v);
#pragma unroll
            for (int q = 0; q < 8; ++q) s[q] += __bfloat162float(h[q]);
        }
        uint4 o4;
        o4.x = pack2(s[0] * 0.125f, s[1] * 0.125f);
        o4.y = pack2(s[2] * 0.125f, s[3] * 0.125f);
        o4.z = pack2(s[4] * 0.125f, s[5] * 0.125f);
        o4.w = pack2(s[6] * 0.125f, s[7] * 0.125f);
        *reinterpret_cast<uint4*>(out + c * C + ch) = o4;
    }
}

// Nearest upsampling of the coarse features plus the fine skip: one thread per fine
// cell and 8 channels
template <int C>
__global__ void k_upadd(const bf16* __restrict__ coarse, const bf16* __restrict__ skip, Dims fine, bf16* __restrict__ out) {
    const Dims cd{fine.nx / 2, fine.ny / 2, fine.nz / 2};
    const int64_t total = fine.n() * (C / 8);
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t f = e / (C / 8);
        const int ch = (int)(e % (C / 8)) * 8;
        const int i = (int)(f % fine.nx), j = (int)((f / fine.nx) % fine.ny), k = (int)(f / ((int64_t)fine.nx * fine.ny));
        const int64_t c = (i / 2) + (int64_t)cd.nx * ((j / 2) + (int64_t)cd.ny * (k / 2));
        const uint4 a = *reinterpret_cast<const uint4*>(coarse + c * C + ch);
        const uint4 b = *reinterpret_cast<const uint4*>(skip + f * C + ch);
        const bf16* ha = reinterpret_cast<const bf16*>(&a);
        const bf16* hb = reinterpret_cast<const bf16*>(&b);
        float s[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) s[q] = __bfloat162float(ha[q]) + __bfloat162float(hb[q]);
        uint4 o4;
        o4.x = pack2(s[0], s[1]);
        o4.y = pack2(s[2], s[3]);
        o4.z = pack2(s[4], s[5]);
        o4.w = pack2(s[6], s[7]);
        *reinterpret_cast<uint4*>(out + f * C + ch) = o4;
    }
}

}  // namespace learned

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
using learned::bf16;
using learned::Dims;

struct LearnedNet {
    Dims d[learned::LEVELS];
    bf16* w[learned::NLAYERS] = {};
    bf16* wu[learned::NLAYERS] = {};  // the tcgen05 B operand: [cout / 16][k groups][16][8]
    float* b[learned::NLAYERS] = {};
    // activations: features, encoder outputs, pooled inputs, decoder inputs / outputs
    bf16 *f0 = nullptr, *e0 = nullptr, *d0in = nullptr;
    bf16 *p1 = nullptr, *e1 = nullptr, *d1in = nullptr, *d1 = nullptr;
    bf16 *p2 = nullptr, *e2 = nullptr, *d2in = nullptr, *d2 = nullptr;
    bf16 *p3 = nullptr, *e3 = nullptr, *d3 = nullptr;
    double* acc = nullptr;
    unsigned* cnt = nullptr;
    float* scale = nullptr;  // s_r, s_z
    std::vector<void*> owned;

    template <typename T>
    T* dev(size_t count) {
        void* p = nullptr;
        if (cudaMalloc(&p, std::max<size_t>(1, count) * sizeof(T)) != cudaSuccess) return nullptr;
        cudaMemset(p, 0, std::max<size_t>(1, count) * sizeof(T));
        owned.push_back(p);
        return static_cast<T*>(p);
    }
    ~LearnedNet() {
        for (void* p : owned) cudaFree(p);
    }
};

namespace {
cudaError_t conv_smem_all();
}

LearnedNet* learned_create(int nx, int ny, int nz, const float* weights, int64_t count, std::string* err) {
    using namespace learned;
    if (nx % 8 || ny % 8 || nz % 8 || nx < 8 || ny < 8 || nz < 8) {
        *err = "the learned preconditioner needs Nx, Ny and Nz divisible by 8";
        return nullptr;
    }
    if (!weights || count != file_count()) {
        *err = "learned preconditioner weights: expected " + std::to_string(file_count()) + " FP32 values";
        return nullptr;
    }
    auto* net = new LearnedNet();
    for (int l = 0; l < LEVELS; ++l) net->d[l] = Dims{nx >> l, ny >> l, nz >> l};
    const int64_t n0 = net->d[0].n(), n1 = net->d[1].n(), n2 = net->d[2].n(), n3 = net->d[3].n();
    bool ok = true;
    auto need = [&](auto* p) { ok = ok && p != nullptr; return p; };
    // weights: the file's [cout][cin][kz][ky][kx] then bias, re-laid to [cout][tap·cin + ci]
    const float* at = weights;
    for (int l = 0; l < NLAYERS && ok; ++l) {
        const int cin = LAYER_CIN[l], cout = LAYER_COUT[l], kp = kpad(cin);
        std::vector<bf16> hw((size_t)cout * kp, __float2bfloat16(0.f));
        std::vector<float> hb(cout, 0.f);
        for (int co = 0; co < FILE_COUT[l]; ++co)
            for (int c = 0; c < FILE_CIN[l]; ++c)
                for (int tap = 0; tap < 27; ++tap) hw[(size_t)co * kp + tap * cin + c] = __float2bfloat16(*at++);
        for (int co = 0; co < FILE_COUT[l]; ++co) hb[co] = *at++;
        // the same weights as tcgen05 B operands: block nb of 16 outputs, k group kg (tap kg with
        // 8 input channels, else tap kg / (cin/8) and channels 8 (kg mod cin/8) ..), 8 k each
        const int kgn = umc::kgroups(cin), pl = cin / 8, nbk = (cout + 15) / 16;
        std::vector<bf16> hu((size_t)nbk * kgn * 16 * 8, __float2bfloat16(0.f));
        for (int nb = 0; nb < nbk; ++nb)
            for (int kg = 0; kg < kgn; ++kg)
                for (int n = 0; n < 16; ++n)
                    for (int e = 0; e < 8; ++e) {
                        const int co = nb * 16 + n;
                        const int tap = cin == 8 ? kg : kg / pl, ci = cin == 8 ? e : (kg % pl) * 8 + e;
                        if (tap < 27 && co < cout && ci < cin)
                            hu[(((size_t)nb * kgn + kg) * 16 + n) * 8 + e] = hw[(size_t)co * kp + tap * cin + ci];
                    }
        net->w[l] = need(net->dev<bf16>(hw.size()));
        net->wu[l] = need(net->dev<bf16>(hu.size()));
        net->b[l] = need(net->dev<float>(std::max<size_t>(hb.size(), 16)));
        if (ok) {
            cudaMemcpy(net->w[l], hw.data(), hw.size() * sizeof(bf16), cudaMemcpyHostToDevice);
            cudaMemcpy(net->wu[l], hu.data(), hu.size() * sizeof(bf16), cudaMemcpyHostToDevice);
            cudaMemcpy(net->b[l], hb.data(), hb.size() * sizeof(float), cudaMemcpyHostToDevice);
        }
    }
    net->f0 = need(net->dev<bf16>(n0 * FEAT));
    net->e0 = need(net->dev<bf16>(n0 * C0));
    net->d0in = need(net->dev<bf16>(n0 * C0));
    net->p1 = need(net->dev<bf16>(n1 * C0));
    net->e1 = need(net->dev<bf16>(n1 * C1));
    net->d1in = need(net->dev<bf16>(n1 * C1));
    net->d1 = need(net->dev<bf16>(n1 * C0));
    net->p2 = need(net->dev<bf16>(n2 * C1));
    net->e2 = need(net->dev<bf16>(n2 * C2));
    net->d2in = need(net->dev<bf16>(n2 * C2));
    net->d2 = need(net->dev<bf16>(n2 * C1));
    net->p3 = need(net->dev<bf16>(n3 * C2));
    net->e3 = need(net->dev<bf16>(n3 * C3));
    net->d3 = need(net->dev<bf16>(n3 * C2));
    net->acc = need(net->dev<double>(1));
    net->cnt = need(net->dev<unsigned>(1));
    net->scale = need(net->dev<float>(2));
    if (ok && conv_smem_all() != cudaSuccess) ok = false;
    if (!ok || cudaGetLastError() != cudaSuccess) {
        *err = "learned preconditioner: device allocation or kernel set-up failed";
        delete net;
        return nullptr;
    }
    return net;
}

void learned_destroy(LearnedNet* net) { delete net; }

namespace {

#ifndef GBO_LEARNED_UMMA
#define GBO_LEARNED_UMMA 0
#endif

template <int CIN, int COUT, int MODE, typename FT>
void conv(const LearnedNet* net, int layer, int level, const bf16* in, bf16* out, void* z, cudaStream_t st,
          unsigned* flags) {
    const learned::Dims& d = net->d[level];
    if (GBO_LEARNED_UMMA) {
        const learned::umc::Geo g = learned::umc::geo(d.nx);
        learned::UConvP p{in, net->wu[layer], net->b[layer], out, z, net->scale + 1, flags, d, COUT};
        const dim3 grid((d.ny + g.BY - 1) / g.BY, d.nz, (COUT + 15) / 16);
        learned::k_conv_umma<CIN, MODE, FT><<<grid, 128, learned::umc::smem_bytes(CIN, d.nx), st>>>(p);
        return;
    }
    using namespace learned::halo;
    learned::ConvP p{in, net->w[layer], net->b[layer], out, z, net->scale + 1, net->d[level]};
    const dim3 grid((d.nx + TX - 1) / TX, (d.ny + TY - 1) / TY, d.nz);
    learned::k_conv_halo<CIN, COUT, MODE, FT><<<grid, 256, smem_bytes<COUT>(), st>>>(p);
}

// dynamic shared memory above the default 48 KB for every instance
template <int CIN, int COUT, int MODE, typename FT>
cudaError_t conv_smem() {
    return cudaFuncSetAttribute(learned::k_conv_halo<CIN, COUT, MODE, FT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)learned::halo::smem_bytes<COUT>());
}
template <int CIN, int MODE, typename FT>
cudaError_t uconv_smem() {
    return cudaFuncSetAttribute(learned::k_conv_umma<CIN, MODE, FT>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
}
cudaError_t conv_smem_all() {
    using namespace learned;
    cudaError_t e = cudaSuccess;
    for (cudaError_t r : {uconv_smem<8, 0, float>(), uconv_smem<16, 0, float>(), uconv_smem<32, 0, float>(),
                          uconv_smem<48, 0, float>(), uconv_smem<64, 0, float>(), uconv_smem<16, 1, float>(),
                          uconv_smem<8, 0, double>(), uconv_smem<16, 0, double>(), uconv_smem<32, 0, double>(),
                          uconv_smem<48, 0, double>(), uconv_smem<64, 0, double>(), uconv_smem<16, 1, double>()})
        if (r != cudaSuccess) e = r;
    for (cudaError_t r : {conv_smem<FEAT, C0, 0, float>(), conv_smem<C0, C1, 0, float>(), conv_smem<C1, C2, 0, float>(),
                          conv_smem<C2, C3, 0, float>(), conv_smem<C3, C2, 0, float>(), conv_smem<C2, C1, 0, float>(),
                          conv_smem<C1, C0, 0, float>(), conv_smem<C0, 8, 1, float>(), conv_smem<FEAT, C0, 0, double>(),
                          conv_smem<C0, C1, 0, double>(), conv_smem<C1, C2, 0, double>(), conv_smem<C2, C3, 0, double>(),
                          conv_smem<C3, C2, 0, double>(), conv_smem<C2, C1, 0, double>(), conv_smem<C1, C0, 0, double>(),
                          conv_smem<C0, 8, 1, double>()})
        if (r != cudaSuccess) e = r;
    return e;
}

unsigned grid_for(int64_t work) { return (unsigned)std::min<int64_t>((work + 255) / 256, 152 * 16); }

template <typename FT>
int apply(LearnedNet* net, const FT* r, FT* z, const int* kbot, cudaStream_t st, unsigned* flags) {
    using namespace learned;
    const Dims* d = net->d;
    k_rms<FT><<<grid_for(d[0].n()), 256, 0, st>>>(r, d[0].n(), net->acc, net->cnt, net->scale);
    k_rms<FT><<<grid_for(d[0].n()), 256, 0, st>>>(z, d[0].n(), net->acc, net->cnt, net->scale + 1);
    k_features<FT><<<grid_for(d[0].n()), 256, 0, st>>>(r, z, kbot, d[0], net->scale, net->scale + 1, net->f0);
    conv<FEAT, C0, 0, FT>(net, L_ENC0, 0, net->f0, net->e0, nullptr, st, flags);
    k_pool<C0><<<grid_for(d[1].n() * C0 / 8), 256, 0, st>>>(net->e0, d[0], net->p1);
    conv<C0, C1, 0, FT>(net, L_ENC1, 1, net->p1, net->e1, nullptr, st, flags);
    k_pool<C1><<<grid_for(d[2].n() * C1 / 8), 256, 0, st>>>(net->e1, d[1], net->p2);
    conv<C1, C2, 0, FT>(net, L_ENC2, 2, net->p2, net->e2, nullptr, st, flags);
    k_pool<C2><<<grid_for(d[3].n() * C2 / 8), 256, 0, st>>>(net->e2, d[2], net->p3);
    conv<C2, C3, 0, FT>(net, L_ENC3, 3, net->p3, net->e3, nullptr, st, flags);
    conv<C3, C2, 0, FT>(net, L_DEC3, 3, net->e3, net->d3, nullptr, st, flags);
    k_upadd<C2><<<grid_for(d[2].n() * C2 / 8), 256, 0, st>>>(net->d3, net->e2, d[2], net->d2in);
    conv<C2, C1, 0, FT>(net, L_DEC2, 2, net->d2in, net->d2, nullptr, st, flags);
    k_upadd<C1><<<grid_for(d[1].n() * C1 / 8), 256, 0, st>>>(net->d2, net->e1, d[1], net->d1in);
    conv<C1, C0, 0, FT>(net, L_DEC1, 1, net->d1in, net->d1, nullptr, st, flags);
    k_upadd<C0><<<grid_for(d[0].n() * C0 / 8), 256, 0, st>>>(net->d1, net->e0, d[0], net->d0in);
    conv<C0, 8, 1, FT>(net, L_OUT, 0, net->d0in, nullptr, z, st, flags);
    return 17;
}

}  // namespace

int learned_apply(LearnedNet* net, const void* r, void* z, const int* kbot, int fp64, cudaStream_t stream,
                  unsigned* flags) {
    if (fp64) return apply<double>(net, static_cast<const double*>(r), static_cast<double*>(z), kbot, stream, flags);
    return apply<float>(net, static_cast<const float*>(r), static_cast<float*>(z), kbot, stream, flags);
}
