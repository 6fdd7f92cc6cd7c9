// gbo_learned.cu -- kernels and host side of the learned preconditioner correction
// (see gbo_learned.cuh for the network, the layouts and the boundary rules).
#include <cmath>
#include <vector>

#include "../../include/gbo.h"
#include "gbo_learned.cuh"
#include "gbo_umma.cuh"

void gbo_record_error(const char* msg);  // gbo_model.cu: message for gbo_last_error(NULL)

namespace learned {

using bf16 = __nv_bfloat16;

struct ConvP {
    const bf16* in;      // [n][cin]
    const bf16* w;       // [cout][kpad(cin)]
    const float* bias;   // [cout]
    bf16* out;           // mode 0: [n][cout]
    void* z;             // mode 1: FT field, z += s (acc + bias) for output channel 0; mode 3: FP32 output
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
// Implicit GEMM: M = 128 cells of a level per MMA (one TMEM lane each), N = 16 output
// channels per block, K = 27 taps × cin.  A block owns BY consecutive rows (y) of the
// level and marches upward through KZ levels.  Its shared memory holds a ring of four
// z-slices; a slice is the block's rows with one halo row each side and x with one
// periodic halo cell each side, channel plane by channel plane (plane cg holds
// channels 8 cg .. 8 cg + 7 of every cell, 16 bytes a cell).  Cells of a slice are
// flattened (row, x + 1) with row stride RS = nx + 2, so output cell (row r, x) is M
// row m = r RS + x and its neighbour (dy, dx) in the slice of level z + dz sits at
// position m + dy RS + dx: every tap is the same K-major canonical operand (8-row
// groups 128 bytes apart, SBO = 128) started at another 16-byte offset of one slice,
// and the halo is loaded once per level.  M rows on halo positions or beyond the
// block's rows compute values that are never stored.  K = 16 per MMA: with 16 or more
// input channels one tap and two channel planes (LBO = the plane stride); with 8 input
// channels two taps of the same level (LBO = the distance of their offsets; the ninth
// tap of a level is paired with a zero weight group).  Weights are the B operand,
// [k group][16 outputs][8 k], loaded once per block.
//
// Per level: the threads start the copies of the slice two levels up (into the ring
// slot freed by the previous level), one thread issues the level's MMAs and commits
// them to an mbarrier, every thread waits (bounded), the four warps read their 32 TMEM
// lanes (tcgen05.ld) and store bias + ReLU (or the final z update), then all wait for
// their copies and synchronise.  The copies of the next slice overlap the MMAs and
// the epilogue.
// ---------------------------------------------------------------------------
namespace umc {
constexpr int M = 128, NB = 16, NS = 4;
struct Geo {
    int BY, RS, MT, cells;  // rows per block, row stride, M tiles, positions per slice plane
};
GBO_HD Geo geo(int nx, int BY) {
    Geo g;
    g.BY = BY;
    g.RS = nx + 2;
    g.MT = ((BY - 1) * g.RS + nx + M - 1) / M;
    const int reach = 2 * g.RS + 3;  // the farthest tap offset in a slice (+1 for the zero pair)
    const int real = (BY + 2) * g.RS;
    const int need = M * g.MT + reach;
    g.cells = ((real > need ? real : need) + 7) / 8 * 8;
    return g;
}
// k groups of the B operand: 8 input channels -- per level, 9 taps and one zero group;
// otherwise tap-major, cin / 8 groups per tap
GBO_HD constexpr int kgroups(int cin) { return cin == 8 ? 30 : 27 * cin / 8; }
inline size_t smem_bytes(int cin, int nx, int BY) {
    const Geo g = geo(nx, BY);
    return (size_t)NS * (cin / 8) * g.cells * 16 + (size_t)kgroups(cin) * NB * 16 + 32;
}
// Rows per block (BY) and levels per block (KZ): up to 1 024 cells and 200 KB of shared
// memory per block, then fewer levels and rows until the launch has at least four blocks
// per SM (the coarse levels of the network have few cells).
struct Shape {
    int by, kz;
};
inline Shape block_shape(int cin, int cout, int nx, int ny, int nz) {
    int by = nx >= 1024 ? 1 : 1024 / nx;
    by = by > ny ? ny : by;
    while (by > 1 && (smem_bytes(cin, nx, by) > 200 * 1024 || geo(nx, by).MT > 16)) --by;
    int kz = nz < 16 ? nz : 16;
    auto blocks = [&](int b, int k) { return (long)((ny + b - 1) / b) * ((nz + k - 1) / k) * ((cout + 15) / 16); };
    while (blocks(by, kz) < 4 * 152 && kz > 2) kz = (kz + 1) / 2;
    while (blocks(by, kz) < 4 * 152 && by > 1) by = (by + 1) / 2;
    while (blocks(by, kz) < 4 * 152 && kz > 1) kz = (kz + 1) / 2;
    return {by, kz};
}
constexpr int WAIT_LIMIT = 1 << 24;  // mbarrier polls before a block reports a timeout
}  // namespace umc

struct UConvP {
    const bf16* in;      // [n][cin]
    const bf16* w;       // [cout / 16][k groups][16][8]
    const float* bias;   // [cout]
    bf16* out;           // mode 0: [n][cout]
    void* z;             // mode 1: FT field, z += s (acc + bias) for output channel 0; mode 3: FP32 output
    const float* scale;  // mode 1: s
    unsigned* flags;     // GBO_FLAG_TIMEOUT on a wait that gave up (may be null)
    Dims d;
    int cout, by, kz;    // output channels, rows per block, levels per block
};

template <int CIN, int MODE, typename FT>
__global__ void __launch_bounds__(256) k_conv_umma(UConvP p) {
    using namespace umc;
    constexpr int PL = CIN / 8, KGN = kgroups(CIN);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const Geo G = geo(p.d.nx, p.by);
    const int slot_elems = PL * G.cells * 8;               // bf16 per ring slot
    bf16* ring = reinterpret_cast<bf16*>(smem_raw);       // [NS][PL][cells][8]
    bf16* wsm = ring + (size_t)NS * slot_elems;            // [KGN][NB][8]
    uint64_t* mbar = reinterpret_cast<uint64_t*>(wsm + KGN * NB * 8);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nx = p.d.nx, ny = p.d.ny, nz = p.d.nz;
    const int y0 = blockIdx.x * G.BY, z0 = blockIdx.y * p.kz, nb = blockIdx.z;
    const int kz = min(p.kz, nz - z0);
    const uint32_t ncols = G.MT * NB <= 32 ? 32 : (G.MT * NB <= 64 ? 64 : (G.MT * NB <= 128 ? 128 : 256));
    if (warp == 0) umma::tmem_alloc(tslot, ncols);
    if (tid == 0) umma::mbar_init(mbar, 1);
    const int real = (G.BY + 2) * G.RS;
    // copies of the slice of level zl into ring slot s (zero outside the domain in z)
    auto load_slice = [&](int zl, int s) {
        bf16* dst = ring + (size_t)s * slot_elems;
        const bool zin = zl >= 0 && zl < nz;
        for (int e = tid; e < PL * G.cells; e += 256) {
            const int cg = e / G.cells, pos = e - cg * G.cells;
            int64_t src = 0;
            bool ok = false;
            if (zin && pos < real) {
                const int ry = pos / G.RS, xx = pos - ry * G.RS;
                const int gx = wrapm(xx - 1, nx), gy = wrapm(y0 + ry - 1, ny);
                src = (gx + (int64_t)nx * (gy + (int64_t)ny * zl)) * CIN + cg * 8;
                ok = true;
            }
            cp16(dst + ((size_t)cg * G.cells + pos) * 8, p.in + src, ok);
        }
    };
    for (int q = 0; q < 3; ++q) load_slice(z0 - 1 + q, q);
    const bf16* wsrc = p.w + (size_t)nb * KGN * NB * 8;
    for (int e = tid; e < KGN * NB; e += 256) cp16(wsm + e * 8, wsrc + e * 8, true);
    cp_commit();
    asm volatile("cp.async.wait_group 0;\n" ::);
    umma::fence_smem_to_async();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = *tslot;
    const uint32_t rb = umma::smem_addr(ring), wb = umma::smem_addr(wsm);
    // descriptors are their operand's address plus an offset: the start field (16-byte
    // units, 14 bits) never carries, every operand lies below 256 KB of shared memory
    constexpr uint32_t LBO8 = 16;  // 8 inputs: taps j, j + 1 in the same row
    const uint64_t da_near = umma::sdesc(rb, CIN == 8 ? LBO8 : (uint32_t)G.cells * 16, 128);
    const uint64_t da_row = umma::sdesc(rb, (uint32_t)(G.RS - 2) * 16, 128);  // 8 inputs: taps 2 and 3
    const uint64_t db0 = umma::sdesc(wb, NB * 16, 128);
    const uint32_t pstride = (uint32_t)G.cells * 16, sstride = (uint32_t)PL * pstride;
    constexpr uint32_t idesc = umma::idesc_bf16_f32(M, NB);
    bool alive = true;
    for (int k = 0; k < kz && alive; ++k) {
        // the slice two levels up goes into the slot the level below last used
        if (k + 1 < kz) load_slice(z0 + k + 2, (k + 3) % NS);
        cp_commit();
        if (tid == 0) {
            for (int q = 0; q < G.MT; ++q) {
                const uint32_t d = tmem + (uint32_t)(q * NB);
                int step = 0;
                for (int dz = 0; dz < 3; ++dz) {
                    // offset of this slot's M tile, in 16-byte units
                    const uint64_t so = (uint64_t)(((k + dz) % NS) * sstride + (uint32_t)(M * q) * 16) >> 4;
                    if constexpr (CIN == 8) {
#pragma unroll
                        for (int j = 0; j < 9; j += 2) {
                            const uint64_t o0 = (uint64_t)((j / 3) * G.RS + j % 3);
                            // taps j, j + 1 are one cell apart, except 2 (row 0) and 3 (row 1)
                            const uint64_t ad = (j == 2 ? da_row : da_near) + so + o0;
                            umma::mma_bf16(d, ad, db0 + (uint64_t)(dz * 10 + j) * NB, idesc, step++ > 0);
                        }
                    } else {
#pragma unroll
                        for (int j = 0; j < 9; ++j) {
                            const uint64_t a0 = da_near + so + (uint64_t)((j / 3) * G.RS + j % 3);
                            const int tap = dz * 9 + j;
#pragma unroll
                            for (int c = 0; c < PL / 2; ++c)
                                umma::mma_bf16(d, a0 + (uint64_t)(2 * c) * (pstride >> 4),
                                               db0 + (uint64_t)(tap * PL + 2 * c) * NB, idesc, step++ > 0);
                        }
                    }
                }
            }
            umma::commit(mbar);
        }
        // every thread polls (bounded); the block then agrees, so all leave the march together
        alive = __syncthreads_and(umma::mbar_wait(mbar, (uint32_t)(k & 1), WAIT_LIMIT));
        if (!alive) {
            if (tid == 0 && p.flags) atomicOr(p.flags, GBO_FLAG_TIMEOUT);
            break;
        }
        umma::fence_after_sync();
        const int zl = z0 + k;
        // warp w reads TMEM lanes 32 (w mod 4) ..; warps 0-3 take the even M tiles, 4-7 the odd
        for (int q = warp >> 2; q < G.MT; q += 2) {
            float v[16];
            umma::tmem_ld16(tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)(q * NB), v);
            const int m = M * q + 32 * (warp & 3) + lane;
            const int ry = m / G.RS, x = m - ry * G.RS, y = y0 + ry;
            if (ry < G.BY && x < nx && y < ny) {
                const int64_t cell = x + (int64_t)nx * (y + (int64_t)ny * zl);
                if constexpr (MODE == 0 || MODE == 2) {
                    // 0: bias and ReLU (a layer's activation); 2: the plain sum (a data gradient)
                    uint4 o[2];
                    uint32_t* ow = reinterpret_cast<uint32_t*>(o);
                    if constexpr (MODE == 0) {
                        const float* b = p.bias + nb * NB;
#pragma unroll
                        for (int c = 0; c < 8; ++c)
                            ow[c] = pack2(fmaxf(v[2 * c] + b[2 * c], 0.f), fmaxf(v[2 * c + 1] + b[2 * c + 1], 0.f));
                    } else {
#pragma unroll
                        for (int c = 0; c < 8; ++c) ow[c] = pack2(v[2 * c], v[2 * c + 1]);
                    }
                    uint4* dst = reinterpret_cast<uint4*>(p.out + cell * p.cout + nb * NB);
                    dst[0] = o[0];
                    dst[1] = o[1];
                } else if constexpr (MODE == 1) {
                    FT* zz = static_cast<FT*>(p.z);
                    zz[cell] += FT(*p.scale * (v[0] + p.bias[0]));
                } else {
                    // 3: the network's output channel in FP32 (training)
                    static_cast<float*>(p.z)[cell] = v[0] + p.bias[0];
                }
            }
        }
        asm volatile("cp.async.wait_group 0;\n" ::);
        umma::fence_smem_to_async();
        umma::fence_before_sync();
        __syncthreads();
        umma::fence_after_sync();
    }
    asm volatile("cp.async.wait_group 0;\n" ::);  // no copy of this block outlives it
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_free(tmem, ncols);
}

// ---------------------------------------------------------------------------
// Training kernels.
//
// Weight gradient of one convolution: gW[o][c][tap] = Σ_cells gy[cell][o] x[cell + tap][c]
// (and gb[o] = Σ gy[cell][o]), BF16 tensor-core MMAs (mma.sync.m16n8k16, FP32
// accumulation): M = 16 outputs, N = 8 inputs, K = 16 cells.  A block owns BY rows of
// the level for KZ levels and a group of (tap, 16 outputs, 8 inputs) fragments (8 per
// warp); per level it stages gy of its rows and the three-level halo of x in shared
// memory, and every lane points ldmatrix at the rows (cells) it needs, so the taps are
// per-lane addresses into one tile.  Partial sums go to the FP32 gradient by atomics.
// ---------------------------------------------------------------------------
namespace wg {
constexpr int FPW = 8;             // fragments per warp
constexpr int FPB = 8 * FPW;       // fragments per block
inline int rows_per_block(int nx, int ny) {
    int by = nx >= 256 ? 2 : 512 / nx;
    return by > ny ? ny : by;
}
inline size_t smem_bytes(int cin, int cout, int nx, int by) {
    const int cells = by * nx, kpad = (cells + 15) / 16 * 16;
    return (size_t)kpad * cout * 2 + (size_t)3 * (by + 2) * (nx + 2) * cin * 2 + 64;
}
}  // namespace wg

struct WGradP {
    const bf16* x;     // [n][cin]   the layer's input
    const bf16* gy;    // [n][coutp] the gradient of its (pre-activation) output, cout padded to 16
    float* gw;         // [cout][cin][27]
    float* gb;         // [cout]
    Dims d;
    int cout, cin_file;  // real outputs; real inputs (the gradient's layout; the kernel's CIN may be padded)
    int by, kz;          // rows per block, levels per block
};

template <int CIN, int COUTP>
__global__ void __launch_bounds__(256) k_conv_wgrad(WGradP p) {
    constexpr int NO = COUTP / 16, NC = CIN / 8, F = 27 * NO * NC;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int nx = p.d.nx, ny = p.d.ny, nz = p.d.nz, by = p.by, RS = nx + 2;
    const int cells = by * nx, kpad = (cells + 15) / 16 * 16;
    bf16* gys = reinterpret_cast<bf16*>(smem_raw);        // [kpad][COUTP]
    bf16* xs = gys + (size_t)kpad * COUTP;                 // [3][by + 2][RS][CIN]
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
    const int y0 = blockIdx.x * by, z0 = blockIdx.y * p.kz, f0 = blockIdx.z * wg::FPB;
    const int kz = min(p.kz, nz - z0);
    float acc[wg::FPW][4];
#pragma unroll
    for (int j = 0; j < wg::FPW; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
    float bsum = 0.f;  // threads < COUTP: Σ gy of output channel tid
    for (int k = 0; k < kz; ++k) {
        const int zl = z0 + k;
        // gy of the block's rows at this level (zero past the last row / the padding)
        for (int e = tid; e < kpad * (COUTP / 8); e += 256) {
            const int m = e / (COUTP / 8), h = e % (COUTP / 8);
            const int ry = m / nx, x = m - ry * nx, y = y0 + ry;
            const bool ok = m < cells && y < ny;
            cp16(gys + (size_t)m * COUTP + h * 8, p.gy + (ok ? ((x + (int64_t)nx * (y + (int64_t)ny * zl)) * COUTP + h * 8) : 0), ok);
        }
        // x on levels zl-1 .. zl+1, rows y0-1 .. y0+by, x with one periodic halo cell each side
        for (int e = tid; e < 3 * (by + 2) * RS * NC; e += 256) {
            const int pos = e / NC, h = e % NC;
            const int dz = pos / ((by + 2) * RS), rem = pos % ((by + 2) * RS), ry = rem / RS, xx = rem % RS;
            const int gz = zl + dz - 1;
            const bool ok = gz >= 0 && gz < nz;
            const int gx = wrapm(xx - 1, nx), gy_ = wrapm(y0 + ry - 1, ny);
            cp16(xs + (size_t)pos * CIN + h * 8, p.x + (ok ? ((gx + (int64_t)nx * (gy_ + (int64_t)ny * gz)) * CIN + h * 8) : 0), ok);
        }
        cp_commit();
        asm volatile("cp.async.wait_group 0;\n" ::);
        __syncthreads();
        if (tid < COUTP && blockIdx.z == 0)
            for (int m = 0; m < cells; ++m) bsum += __bfloat162float(gys[(size_t)m * COUTP + tid]);
        for (int m0 = 0; m0 < kpad; m0 += 16) {
#pragma unroll
            for (int j = 0; j < wg::FPW; ++j) {
                const int f = f0 + warp + 8 * j;
                if (f >= F) break;
                const int tap = f / (NO * NC), o16 = (f / NC) % NO, c8 = f % NC;
                const int dz = tap / 9, dy = (tap / 3) % 3, dx = tap % 3;
                // A = gy^T (16 outputs × 16 cells): four 8 × 8 matrices, rows = cells
                const int mi = lane >> 3, r = lane & 7;
                const bf16* arow = gys + (size_t)(m0 + (mi >> 1) * 8 + r) * COUTP + o16 * 16 + (mi & 1) * 8;
                uint32_t a0, a1, a2, a3;
                {
                    const unsigned ad = (unsigned)__cvta_generic_to_shared(arow);
                    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                                 : "=r"(a0), "=r"(a1), "=r"(a2), "=r"(a3) : "r"(ad));
                }
                // B = x at the tap (16 cells × 8 inputs): two 8 × 8 matrices, rows = cells
                int mb = m0 + (lane & 15);
                mb = mb < cells ? mb : cells - 1;  // padding cells have gy = 0
                const int ry = mb / nx, x = mb - ry * nx;
                const bf16* brow = xs + (size_t)((dz * (by + 2) + ry + dy) * RS + x + dx) * CIN + c8 * 8;
                uint32_t b0, b1;
                {
                    const unsigned bd = (unsigned)__cvta_generic_to_shared(brow);
                    asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0,%1}, [%2];\n"
                                 : "=r"(b0), "=r"(b1) : "r"(bd));
                }
                mma16816(acc[j], a0, a1, a2, a3, b0, b1);
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int j = 0; j < wg::FPW; ++j) {
        const int f = f0 + warp + 8 * j;
        if (f >= F) break;
        const int tap = f / (NO * NC), o16 = (f / NC) % NO, c8 = f % NC;
        const int oa = o16 * 16 + g, ob = oa + 8, c = c8 * 8 + 2 * t, cf = p.cin_file;
        auto put = [&](int o, int ci, float v) {
            if (o < p.cout && ci < cf) atomicAdd(p.gw + ((size_t)o * cf + ci) * 27 + tap, v);
        };
        put(oa, c, acc[j][0]);
        put(oa, c + 1, acc[j][1]);
        put(ob, c, acc[j][2]);
        put(ob, c + 1, acc[j][3]);
    }
    if (tid < p.cout && blockIdx.z == 0) atomicAdd(p.gb + tid, bsum);
}

// Backward of an up-sampling + skip pair and of pooling, fused with the ReLU mask of the
// layer whose output the gradient reaches:
//   coarse mode (pool == nullptr, fine_in != nullptr): out[c] = Σ_children fine_in ⊙ (act > 0)
//   fine mode: out[f] = (pool[parent(f)] / 8 + skip[f]) ⊙ (act[f] > 0), pool / skip optional
// (all [cells][C] BF16, one thread per cell and 8 channels, FP32 sums).
template <int C>
__global__ void k_grad_combine(const bf16* __restrict__ fine_in, const bf16* __restrict__ pool,
                               const bf16* __restrict__ skip, const bf16* __restrict__ act, Dims d, int coarse_mode,
                               bf16* __restrict__ out) {
    const Dims cd{d.nx / 2, d.ny / 2, d.nz / 2};
    const Dims od = coarse_mode ? cd : d;
    const int64_t total = od.n() * (C / 8);
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = e / (C / 8);
        const int ch = (int)(e % (C / 8)) * 8;
        const int i = (int)(c % od.nx), j = (int)((c / od.nx) % od.ny), k = (int)(c / ((int64_t)od.nx * od.ny));
        float s[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        auto add = [&](const bf16* src, int64_t cell, float f) {
            const uint4 v = *reinterpret_cast<const uint4*>(src + cell * C + ch);
            const bf16* h = reinterpret_cast<const bf16*>(&v);
#pragma unroll
            for (int q = 0; q < 8; ++q) s[q] += f * __bfloat162float(h[q]);
        };
        if (coarse_mode) {
            for (int o = 0; o < 8; ++o)
                add(fine_in, (2 * i + (o & 1)) + (int64_t)d.nx * ((2 * j + ((o >> 1) & 1)) + (int64_t)d.ny * (2 * k + (o >> 2))), 1.f);
        } else {
            if (pool) add(pool, (i / 2) + (int64_t)cd.nx * ((j / 2) + (int64_t)cd.ny * (k / 2)), 0.125f);
            if (skip) add(skip, c, 1.f);
            if (fine_in) add(fine_in, c, 1.f);
        }
        const uint4 a = *reinterpret_cast<const uint4*>(act + c * C + ch);
        const bf16* ha = reinterpret_cast<const bf16*>(&a);
        uint4 o4;
        uint32_t* ow = reinterpret_cast<uint32_t*>(&o4);
#pragma unroll
        for (int q = 0; q < 4; ++q)
            ow[q] = pack2(__bfloat162float(ha[2 * q]) > 0.f ? s[2 * q] : 0.f, __bfloat162float(ha[2 * q + 1]) > 0.f ? s[2 * q + 1] : 0.f);
        *reinterpret_cast<uint4*>(out + c * C + ch) = o4;
    }
}

// The training loss of one sample (the loss of the offline trainer, restated):
//   t = (e - z) / s_z,  d = (y - t)·a less its active mean,  t_c = t·a less its active mean,
//   loss = Σ d² / Σ t_c²,  ∂loss/∂y = 2 d / Σ t_c² (the mean removal is a projection).
// sums[0..2] = Σ a, Σ (y - t) a, Σ t a; sums[3..4] = Σ d², Σ t_c² (FP64, block partials + atomics).
template <typename FT>
__global__ void k_loss_sums(const float* __restrict__ y, const FT* __restrict__ e, const FT* __restrict__ z,
                            const float* __restrict__ act, const float* sz, int64_t n, int pass, double* sums) {
    __shared__ double sh[3][8];
    double a0 = 0, a1 = 0, a2 = 0;
    const double m_a = pass ? sums[0] : 1.0;
    const double md = pass ? sums[1] / m_a : 0.0, mt = pass ? sums[2] / m_a : 0.0;
    const double rs = 1.0 / (double)*sz;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double a = act[i];
        const double t = ((double)e[i] - (double)z[i]) * rs;
        const double dy = ((double)y[i] - t) * a;
        if (!pass) {
            a0 += a; a1 += dy; a2 += t * a;
        } else {
            const double d = dy - md * a, tc = (t - mt) * a;
            a0 += d * d; a1 += tc * tc;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        a0 += __shfl_down_sync(0xffffffffu, a0, o);
        a1 += __shfl_down_sync(0xffffffffu, a1, o);
        a2 += __shfl_down_sync(0xffffffffu, a2, o);
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) { sh[0][w] = a0; sh[1][w] = a1; sh[2][w] = a2; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double b0 = 0, b1 = 0, b2 = 0;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) { b0 += sh[0][q]; b1 += sh[1][q]; b2 += sh[2][q]; }
        if (!pass) {
            atomicAdd(sums + 0, b0); atomicAdd(sums + 1, b1); atomicAdd(sums + 2, b2);
        } else {
            atomicAdd(sums + 3, b0); atomicAdd(sums + 4, b1);
        }
    }
}
// ∂loss/∂y into channel 0 of the output layer's gradient ([n][16] BF16, other channels zero)
template <typename FT>
__global__ void k_loss_grad(const float* __restrict__ y, const FT* __restrict__ e, const FT* __restrict__ z,
                            const float* __restrict__ act, const float* sz, int64_t n, const double* sums,
                            bf16* __restrict__ gy) {
    const double m_a = sums[0], md = sums[1] / m_a;
    const double den = sums[4] > 1e-30 ? sums[4] : 1e-30;
    const double rs = 1.0 / (double)*sz;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double a = act[i];
        const double t = ((double)e[i] - (double)z[i]) * rs;
        const double d = ((double)y[i] - t) * a - md * a;
        uint4 o[2] = {make_uint4(0u, 0u, 0u, 0u), make_uint4(0u, 0u, 0u, 0u)};
        o[0].x = pack2((float)(2.0 * d / den), 0.f);
        uint4* dst = reinterpret_cast<uint4*>(gy + i * 16);
        dst[0] = o[0];
        dst[1] = o[1];
    }
}

// Adam (β1, β2, ε; bias corrections c1 = 1 / (1 - β1^t), c2 = 1 / (1 - β2^t)) on the FP32
// master weights, then the gradient is cleared for the next step.
__global__ void k_adam(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v, float* __restrict__ g, int64_t n,
                       float lr, float b1, float b2, float eps, float c1, float c2) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        w[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
        g[i] = 0.f;
    }
}

// One layer's FP32 master weights (file layout W[cout][cin][27], then bias) into a
// tcgen05 B operand: forward (k group kg of input channels) or, with transposed set, the
// operand of the data-gradient convolution: input channels = the layer's outputs, outputs
// = its inputs, taps mirrored (26 - tap).
__global__ void k_pack_weights(const float* __restrict__ wl, int fcin, int fcout, int kcin, int nbk, int transposed,
                               bf16* __restrict__ out) {
    const int kgn = umc::kgroups(kcin), pl = kcin / 8;
    const int64_t total = (int64_t)nbk * kgn * 16 * 8;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
        const int e = (int)(q % 8), n = (int)((q / 8) % 16), kg = (int)((q / 128) % kgn), nb = (int)(q / (128 * kgn));
        const int oc = nb * 16 + n;  // the operand's output channel
        const int tap = kcin == 8 ? (kg % 10 < 9 ? 9 * (kg / 10) + kg % 10 : 27) : kg / pl;
        const int ic = kcin == 8 ? e : (kg % pl) * 8 + e;  // the operand's input channel
        float val = 0.f;
        if (tap < 27) {
            if (!transposed) {
                if (oc < fcout && ic < fcin) val = wl[((size_t)oc * fcin + ic) * 27 + tap];
            } else {
                if (ic < fcout && oc < fcin) val = wl[((size_t)ic * fcin + oc) * 27 + (26 - tap)];
            }
        }
        out[q] = __float2bfloat16(val);
    }
}

// Network input for training: (r / s_r, z / s_z, active) with the active mask given as a field.
template <typename FT>
__global__ void k_features_act(const FT* __restrict__ r, const FT* __restrict__ z, const float* __restrict__ act, int64_t n,
                               const float* scale_r, const float* scale_z, bf16* __restrict__ out) {
    const float inv = 1.f / *scale_r, invz = 1.f / *scale_z;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
        uint4 v;
        v.x = pack2((float)r[c] * inv, (float)z[c] * invz);
        v.y = pack2(act[c], 0.f);
        v.z = 0u;
        v.w = 0u;
        *reinterpret_cast<uint4*>(out + c * FEAT) = v;
    }
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
                        // 8 inputs: group kg = 10 dz + j holds tap 9 dz + j (j = 9 is zero)
                        const int tap = cin == 8 ? (kg % 10 < 9 ? 9 * (kg / 10) + kg % 10 : 27) : kg / pl;
                        const int ci = cin == 8 ? e : (kg % pl) * 8 + e;
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

// Which kernel runs a layer of the inference: the tcgen05 convolution for the
// full-resolution input layer (8 input channels; 345 µs against 654 µs for mma.sync at
// 256²×128), the mma.sync halo-tile convolution for the layers where it measured faster
// (the coarse levels, where a tcgen05 block's tile and weight staging is not amortised,
// and the 16 → 1 output layer, which fills one sixteenth of an N = 16 MMA).
template <int CIN, int COUT, int MODE>
constexpr bool use_tcgen05() { return CIN == learned::FEAT && MODE == 0; }

template <int CIN, int COUT, int MODE, typename FT>
void conv(const LearnedNet* net, int layer, int level, const bf16* in, bf16* out, void* z, cudaStream_t st,
          unsigned* flags) {
    const learned::Dims& d = net->d[level];
    if constexpr (use_tcgen05<CIN, COUT, MODE>()) {
        namespace U = learned::umc;
        const U::Shape sh = U::block_shape(CIN, COUT, d.nx, d.ny, d.nz);
        learned::UConvP p{in, net->wu[layer], net->b[layer], out, z, net->scale + 1, flags, d, COUT, sh.by, sh.kz};
        const dim3 grid((d.ny + sh.by - 1) / sh.by, (d.nz + sh.kz - 1) / sh.kz, (COUT + 15) / 16);
        learned::k_conv_umma<CIN, MODE, FT><<<grid, 256, U::smem_bytes(CIN, d.nx, sh.by), st>>>(p);
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

// ---------------------------------------------------------------------------
// Training on the GPU (gbo_learned_trainer_*): forward with the tcgen05 convolutions,
// the loss, backward (data gradients with the same tcgen05 kernel on transposed,
// mirrored weights; weight gradients with k_conv_wgrad), Adam on FP32 master weights.
// ---------------------------------------------------------------------------
namespace {

template <int CIN, int MODE>
void uconv(const learned::Dims& d, const bf16* in, const bf16* w, const float* bias, bf16* out, void* z,
           const float* scale, int cout, unsigned* flags, cudaStream_t st) {
    namespace U = learned::umc;
    const U::Shape sh = U::block_shape(CIN, cout, d.nx, d.ny, d.nz);
    learned::UConvP p{in, w, bias, out, z, scale, flags, d, cout, sh.by, sh.kz};
    const dim3 grid((d.ny + sh.by - 1) / sh.by, (d.nz + sh.kz - 1) / sh.kz, (cout + 15) / 16);
    learned::k_conv_umma<CIN, MODE, float><<<grid, 256, U::smem_bytes(CIN, d.nx, sh.by), st>>>(p);
}

int wgrad_rows(int cin, int coutp, int nx, int ny) {
    int by = learned::wg::rows_per_block(nx, ny);
    while (by > 1 && learned::wg::smem_bytes(cin, coutp, nx, by) > 220 * 1024) --by;
    return by;
}

template <int CIN, int COUTP>
void wgrad(const learned::Dims& d, const bf16* x, const bf16* gy, float* gw, float* gb, int cout, int cin_file,
           cudaStream_t st) {
    const int by = wgrad_rows(CIN, COUTP, d.nx, d.ny), kz = d.nz < 16 ? d.nz : 16;
    constexpr int F = 27 * (COUTP / 16) * (CIN / 8);
    learned::WGradP p{x, gy, gw, gb, d, cout, cin_file, by, kz};
    const dim3 grid((d.ny + by - 1) / by, (d.nz + kz - 1) / kz, (F + learned::wg::FPB - 1) / learned::wg::FPB);
    learned::k_conv_wgrad<CIN, COUTP><<<grid, 256, learned::wg::smem_bytes(CIN, COUTP, d.nx, by), st>>>(p);
}

template <int C>
void combine(const learned::Dims& fine, const bf16* fine_in, const bf16* pool, const bf16* skip, const bf16* act,
             int coarse_mode, bf16* out, cudaStream_t st) {
    const int64_t n = coarse_mode ? fine.n() / 8 : fine.n();
    learned::k_grad_combine<C><<<grid_for(n * C / 8), 256, 0, st>>>(fine_in, pool, skip, act, fine, coarse_mode, out);
}

template <int CIN, int MODE>
cudaError_t umma_attr() {
    return cudaFuncSetAttribute(learned::k_conv_umma<CIN, MODE, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
}
template <int CIN, int COUTP>
cudaError_t wgrad_attr() {
    return cudaFuncSetAttribute(learned::k_conv_wgrad<CIN, COUTP>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
}

}  // namespace

struct gbo_learned_trainer {
    LearnedNet* net = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t join_ev = nullptr;  // orders the stream after the caller's legacy-stream work
    int64_t count = 0, off[learned::NLAYERS] = {};
    float *wm = nullptr, *m = nullptr, *v = nullptr, *g = nullptr, *y = nullptr;
    double* sums = nullptr;
    unsigned* flags = nullptr;
    bf16* wt[learned::NLAYERS] = {};
    bf16 *gyO = nullptr, *gU0 = nullptr, *gE0 = nullptr, *gD1 = nullptr, *gU1 = nullptr, *gE1 = nullptr, *gP1 = nullptr;
    bf16 *gD2 = nullptr, *gU2 = nullptr, *gE2 = nullptr, *gP2 = nullptr, *gD3 = nullptr, *gE3 = nullptr, *gP3 = nullptr;
    int adam_t = 0;
    std::string err;
    std::vector<void*> owned;
    template <typename T>
    T* dev(size_t n) {
        void* p = nullptr;
        if (cudaMalloc(&p, std::max<size_t>(1, n) * sizeof(T)) != cudaSuccess) return nullptr;
        cudaMemset(p, 0, std::max<size_t>(1, n) * sizeof(T));
        owned.push_back(p);
        return static_cast<T*>(p);
    }
    // the samples were just written by the caller: wait (on the device) for the work
    // already issued to the legacy default stream
    void join_caller() {
        cudaEventRecord(join_ev, cudaStreamLegacy);
        cudaStreamWaitEvent(stream, join_ev, 0);
    }
    ~gbo_learned_trainer() {
        if (join_ev) cudaEventDestroy(join_ev);
        for (void* p : owned) cudaFree(p);
        if (net) learned_destroy(net);
        if (stream) cudaStreamDestroy(stream);
    }

    // the BF16 operands (forward, transposed) and the biases from the FP32 master weights
    void pack() {
        using namespace learned;
        for (int l = 0; l < NLAYERS; ++l) {
            const float* wl = wm + off[l];
            const int nbk = (LAYER_COUT[l] + 15) / 16;
            k_pack_weights<<<grid_for((int64_t)nbk * umc::kgroups(LAYER_CIN[l]) * 128), 256, 0, stream>>>(
                wl, FILE_CIN[l], FILE_COUT[l], LAYER_CIN[l], nbk, 0, net->wu[l]);
            cudaMemcpyAsync(net->b[l], wl + (int64_t)FILE_COUT[l] * FILE_CIN[l] * 27, FILE_COUT[l] * sizeof(float),
                            cudaMemcpyDeviceToDevice, stream);
            if (l > 0) {
                const int kcin = l == L_OUT ? 16 : LAYER_COUT[l];
                const int nbt = (LAYER_CIN[l] + 15) / 16;
                k_pack_weights<<<grid_for((int64_t)nbt * umc::kgroups(kcin) * 128), 256, 0, stream>>>(
                    wl, FILE_CIN[l], FILE_COUT[l], kcin, nbt, 1, wt[l]);
            }
        }
    }

    void forward(const float* r, const float* z, const float* act) {
        using namespace learned;
        LearnedNet* n = net;
        const Dims* d = n->d;
        const int64_t n0 = d[0].n();
        k_rms<float><<<grid_for(n0), 256, 0, stream>>>(r, n0, n->acc, n->cnt, n->scale);
        k_rms<float><<<grid_for(n0), 256, 0, stream>>>(z, n0, n->acc, n->cnt, n->scale + 1);
        k_features_act<float><<<grid_for(n0), 256, 0, stream>>>(r, z, act, n0, n->scale, n->scale + 1, n->f0);
        uconv<FEAT, 0>(d[0], n->f0, n->wu[L_ENC0], n->b[L_ENC0], n->e0, nullptr, nullptr, C0, flags, stream);
        k_pool<C0><<<grid_for(d[1].n() * C0 / 8), 256, 0, stream>>>(n->e0, d[0], n->p1);
        uconv<C0, 0>(d[1], n->p1, n->wu[L_ENC1], n->b[L_ENC1], n->e1, nullptr, nullptr, C1, flags, stream);
        k_pool<C1><<<grid_for(d[2].n() * C1 / 8), 256, 0, stream>>>(n->e1, d[1], n->p2);
        uconv<C1, 0>(d[2], n->p2, n->wu[L_ENC2], n->b[L_ENC2], n->e2, nullptr, nullptr, C2, flags, stream);
        k_pool<C2><<<grid_for(d[3].n() * C2 / 8), 256, 0, stream>>>(n->e2, d[2], n->p3);
        uconv<C2, 0>(d[3], n->p3, n->wu[L_ENC3], n->b[L_ENC3], n->e3, nullptr, nullptr, C3, flags, stream);
        uconv<C3, 0>(d[3], n->e3, n->wu[L_DEC3], n->b[L_DEC3], n->d3, nullptr, nullptr, C2, flags, stream);
        k_upadd<C2><<<grid_for(d[2].n() * C2 / 8), 256, 0, stream>>>(n->d3, n->e2, d[2], n->d2in);
        uconv<C2, 0>(d[2], n->d2in, n->wu[L_DEC2], n->b[L_DEC2], n->d2, nullptr, nullptr, C1, flags, stream);
        k_upadd<C1><<<grid_for(d[1].n() * C1 / 8), 256, 0, stream>>>(n->d2, n->e1, d[1], n->d1in);
        uconv<C1, 0>(d[1], n->d1in, n->wu[L_DEC1], n->b[L_DEC1], n->d1, nullptr, nullptr, C0, flags, stream);
        k_upadd<C0><<<grid_for(d[0].n() * C0 / 8), 256, 0, stream>>>(n->d1, n->e0, d[0], n->d0in);
        uconv<C0, 3>(d[0], n->d0in, n->wu[L_OUT], n->b[L_OUT], nullptr, y, nullptr, 8, flags, stream);
    }

    void loss(const float* z, const float* e, const float* act) {
        const int64_t n0 = net->d[0].n();
        cudaMemsetAsync(sums, 0, 8 * sizeof(double), stream);
        learned::k_loss_sums<float><<<grid_for(n0), 256, 0, stream>>>(y, e, z, act, net->scale + 1, n0, 0, sums);
        learned::k_loss_sums<float><<<grid_for(n0), 256, 0, stream>>>(y, e, z, act, net->scale + 1, n0, 1, sums);
        learned::k_loss_grad<float><<<grid_for(n0), 256, 0, stream>>>(y, e, z, act, net->scale + 1, n0, sums, gyO);
    }

    float* gw(int l) { return g + off[l]; }
    float* gb(int l) { return g + off[l] + (int64_t)learned::FILE_COUT[l] * learned::FILE_CIN[l] * 27; }

    void backward() {
        using namespace learned;
        LearnedNet* n = net;
        const Dims* d = n->d;
        cudaStream_t st = stream;
        wgrad<C0, 16>(d[0], n->d0in, gyO, gw(L_OUT), gb(L_OUT), 1, FILE_CIN[L_OUT], st);
        uconv<16, 2>(d[0], gyO, wt[L_OUT], nullptr, gU0, nullptr, nullptr, C0, flags, st);
        combine<C0>(d[0], gU0, nullptr, nullptr, n->d1, 1, gD1, st);
        wgrad<C1, 16>(d[1], n->d1in, gD1, gw(L_DEC1), gb(L_DEC1), C0, FILE_CIN[L_DEC1], st);
        uconv<C0, 2>(d[1], gD1, wt[L_DEC1], nullptr, gU1, nullptr, nullptr, C1, flags, st);
        combine<C1>(d[1], gU1, nullptr, nullptr, n->d2, 1, gD2, st);
        wgrad<C2, 32>(d[2], n->d2in, gD2, gw(L_DEC2), gb(L_DEC2), C1, FILE_CIN[L_DEC2], st);
        uconv<C1, 2>(d[2], gD2, wt[L_DEC2], nullptr, gU2, nullptr, nullptr, C2, flags, st);
        combine<C2>(d[2], gU2, nullptr, nullptr, n->d3, 1, gD3, st);
        wgrad<C3, 48>(d[3], n->e3, gD3, gw(L_DEC3), gb(L_DEC3), C2, FILE_CIN[L_DEC3], st);
        uconv<C2, 2>(d[3], gD3, wt[L_DEC3], nullptr, gE3, nullptr, nullptr, C3, flags, st);
        combine<C3>(d[3], gE3, nullptr, nullptr, n->e3, 0, gE3, st);  // the ReLU mask of e3, in place
        wgrad<C2, 64>(d[3], n->p3, gE3, gw(L_ENC3), gb(L_ENC3), C3, FILE_CIN[L_ENC3], st);
        uconv<C3, 2>(d[3], gE3, wt[L_ENC3], nullptr, gP3, nullptr, nullptr, C2, flags, st);
        combine<C2>(d[2], nullptr, gP3, gU2, n->e2, 0, gE2, st);
        wgrad<C1, 48>(d[2], n->p2, gE2, gw(L_ENC2), gb(L_ENC2), C2, FILE_CIN[L_ENC2], st);
        uconv<C2, 2>(d[2], gE2, wt[L_ENC2], nullptr, gP2, nullptr, nullptr, C1, flags, st);
        combine<C1>(d[1], nullptr, gP2, gU1, n->e1, 0, gE1, st);
        wgrad<C0, 32>(d[1], n->p1, gE1, gw(L_ENC1), gb(L_ENC1), C1, FILE_CIN[L_ENC1], st);
        uconv<C1, 2>(d[1], gE1, wt[L_ENC1], nullptr, gP1, nullptr, nullptr, C0, flags, st);
        combine<C0>(d[0], nullptr, gP1, gU0, n->e0, 0, gE0, st);
        wgrad<FEAT, 16>(d[0], n->f0, gE0, gw(L_ENC0), gb(L_ENC0), C0, FILE_CIN[L_ENC0], st);
    }

    int check() {
        // a launch refused at configuration (shared memory, grid) is reported here, not by the sync
        const cudaError_t launch = cudaGetLastError();
        if (launch != cudaSuccess) {
            err = std::string("a learned-trainer kernel could not be launched: ") + cudaGetErrorString(launch);
            return GBO_ERR_CUDA;
        }
        unsigned h = 0;
        if (cudaMemcpyAsync(&h, flags, sizeof(unsigned), cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
            cudaStreamSynchronize(stream) != cudaSuccess) {
            err = std::string("CUDA error in the learned trainer: ") + cudaGetErrorString(cudaGetLastError());
            return GBO_ERR_CUDA;
        }
        if (h & GBO_FLAG_TIMEOUT) { err = "a tensor-core wait of the learned trainer gave up"; return GBO_ERR_TIMEOUT; }
        return GBO_OK;
    }
};

extern "C" {

int gbo_learned_trainer_create(int32_t nx, int32_t ny, int32_t nz, const float* weights, int64_t count,
                               gbo_learned_trainer** out) {
    using namespace learned;
    if (!out) return GBO_ERR_INVALID;
    *out = nullptr;
    std::string why;
    LearnedNet* net = learned_create(nx, ny, nz, weights, count, &why);
    if (!net) { gbo_record_error(why.c_str()); return GBO_ERR_INVALID; }
    auto* t = new gbo_learned_trainer();
    t->net = net;
    t->count = count;
    bool ok = cudaStreamCreateWithFlags(&t->stream, cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreateWithFlags(&t->join_ev, cudaEventDisableTiming) == cudaSuccess;
    int64_t at = 0;
    for (int l = 0; l < NLAYERS; ++l) {
        t->off[l] = at;
        at += (int64_t)FILE_COUT[l] * FILE_CIN[l] * 27 + FILE_COUT[l];
    }
    auto need = [&](auto* p) { ok = ok && p != nullptr; return p; };
    t->wm = need(t->dev<float>(count));
    t->m = need(t->dev<float>(count));
    t->v = need(t->dev<float>(count));
    t->g = need(t->dev<float>(count));
    const Dims* d = net->d;
    t->y = need(t->dev<float>(d[0].n()));
    t->sums = need(t->dev<double>(8));
    t->flags = need(t->dev<unsigned>(1));
    for (int l = 1; l < NLAYERS; ++l) {
        const int kcin = l == L_OUT ? 16 : LAYER_COUT[l];
        t->wt[l] = need(t->dev<bf16>((size_t)((LAYER_CIN[l] + 15) / 16) * umc::kgroups(kcin) * 128));
    }
    t->gyO = need(t->dev<bf16>(d[0].n() * 16));
    t->gU0 = need(t->dev<bf16>(d[0].n() * C0));
    t->gE0 = need(t->dev<bf16>(d[0].n() * C0));
    t->gD1 = need(t->dev<bf16>(d[1].n() * C0));
    t->gU1 = need(t->dev<bf16>(d[1].n() * C1));
    t->gE1 = need(t->dev<bf16>(d[1].n() * C1));
    t->gP1 = need(t->dev<bf16>(d[1].n() * C0));
    t->gD2 = need(t->dev<bf16>(d[2].n() * C1));
    t->gU2 = need(t->dev<bf16>(d[2].n() * C2));
    t->gE2 = need(t->dev<bf16>(d[2].n() * C2));
    t->gP2 = need(t->dev<bf16>(d[2].n() * C1));
    t->gD3 = need(t->dev<bf16>(d[3].n() * C2));
    t->gE3 = need(t->dev<bf16>(d[3].n() * C3));
    t->gP3 = need(t->dev<bf16>(d[3].n() * C2));
    for (cudaError_t r : {umma_attr<16, 2>(), umma_attr<32, 2>(), umma_attr<48, 2>(), umma_attr<64, 2>(), umma_attr<16, 3>(),
                          umma_attr<8, 0>(), umma_attr<16, 0>(), umma_attr<32, 0>(), umma_attr<48, 0>(), umma_attr<64, 0>(),
                          wgrad_attr<16, 16>(), wgrad_attr<32, 16>(), wgrad_attr<48, 32>(), wgrad_attr<64, 48>(),
                          wgrad_attr<48, 64>(), wgrad_attr<32, 48>(), wgrad_attr<16, 32>(), wgrad_attr<8, 16>()})
        ok = ok && r == cudaSuccess;
    if (ok) ok = cudaMemcpy(t->wm, weights, count * sizeof(float), cudaMemcpyHostToDevice) == cudaSuccess;
    if (ok) {
        t->pack();
        ok = cudaStreamSynchronize(t->stream) == cudaSuccess && cudaGetLastError() == cudaSuccess;
    }
    if (!ok) {
        gbo_record_error("learned trainer: device allocation or set-up failed");
        delete t;
        return GBO_ERR_CUDA;
    }
    *out = t;
    return GBO_OK;
}

void gbo_learned_trainer_destroy(gbo_learned_trainer* t) { delete t; }

int gbo_learned_trainer_gradients(gbo_learned_trainer* t, const float* r, const float* z, const float* e,
                                  const float* active, double* loss, float* grad) {
    if (!t || !r || !z || !e || !active || !loss || !grad) return GBO_ERR_INVALID;
    t->join_caller();
    cudaMemsetAsync(t->g, 0, t->count * sizeof(float), t->stream);
    t->forward(r, z, active);
    t->loss(z, e, active);
    t->backward();
    double s[8];
    cudaMemcpyAsync(s, t->sums, sizeof(s), cudaMemcpyDeviceToHost, t->stream);
    cudaMemcpyAsync(grad, t->g, t->count * sizeof(float), cudaMemcpyDeviceToHost, t->stream);
    const int rc = t->check();
    if (rc != GBO_OK) { gbo_record_error(t->err.c_str()); return rc; }
    *loss = s[3] / (s[4] > 1e-30 ? s[4] : 1e-30);
    return GBO_OK;
}

int gbo_learned_trainer_step(gbo_learned_trainer* t, const float* r, const float* z, const float* e, const float* active,
                             double lr, double* loss) {
    if (!t || !r || !z || !e || !active) return GBO_ERR_INVALID;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    t->join_caller();
    t->forward(r, z, active);
    t->loss(z, e, active);
    t->backward();
    t->adam_t += 1;
    const float c1 = 1.f / (1.f - std::pow(b1, (float)t->adam_t)), c2 = 1.f / (1.f - std::pow(b2, (float)t->adam_t));
    learned::k_adam<<<grid_for(t->count), 256, 0, t->stream>>>(t->wm, t->m, t->v, t->g, t->count, (float)lr, b1, b2, eps, c1, c2);
    t->pack();
    if (loss) {
        double s[8];
        cudaMemcpyAsync(s, t->sums, sizeof(s), cudaMemcpyDeviceToHost, t->stream);
        const int rc = t->check();
        if (rc != GBO_OK) { gbo_record_error(t->err.c_str()); return rc; }
        *loss = s[3] / (s[4] > 1e-30 ? s[4] : 1e-30);
    }
    return GBO_OK;
}

int gbo_learned_trainer_weights(gbo_learned_trainer* t, float* out) {
    if (!t || !out) return GBO_ERR_INVALID;
    cudaMemcpyAsync(out, t->wm, t->count * sizeof(float), cudaMemcpyDeviceToHost, t->stream);
    const int rc = t->check();
    if (rc != GBO_OK) gbo_record_error(t->err.c_str());
    return rc;
}

int gbo_learned_trainer_stream(gbo_learned_trainer* t, void** stream) {
    if (!t || !stream) return GBO_ERR_INVALID;
    *stream = t->stream;
    return GBO_OK;
}

}  // extern "C"
