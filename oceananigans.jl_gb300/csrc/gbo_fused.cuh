// gbo_fused.cuh -- column-marching fused momentum tendency + RK3 predictor kernel.
//
// Same arithmetic as k_momentum (gbo_step.cuh), organised for the GPU:
//   * a 32 x 8 block owns a tile of (i, j) columns and marches upward over a
//     chunk of levels k;
//   * x / y stencils (halo 3) are read from shared-memory planes that the block
//     loads once per level (periodic wrap and the z-halo rules applied at load), in
//     16-byte chunks where the grid allows (x halo widened to 4 for that);
//   * z stencils come from per-thread register windows that slide with k;
//   * every face flux is evaluated once: a thread computes the fluxes through
//     the west, south and top faces of its control volumes, exchanges west and
//     south values with its neighbours through shared memory, and carries the
//     top value to the next level as the bottom value.
// The extra faces on the tile's east column and north row are evaluated by
// warps 0 and 1 after their own work, taking the vertical windows of those columns from
// a small shared-memory ring prefetched two levels ahead; off an immersed grid by a
// separately compiled form of the face code (on an immersed grid one copy serves both).
#pragma once
#include <initializer_list>
#include <type_traits>
#include "gbo_step.cuh"

// Resident blocks per SM the FP32 kernel is compiled for (registers are capped so
// that this many 256-thread blocks fit).
#ifndef GBO_FUSED_MIN_BLOCKS
#define GBO_FUSED_MIN_BLOCKS 3
#endif

namespace fused {

// planes: x halo 4 (a row is 40 values: 16-byte chunks starting on a multiple of four
// columns), y halo 3
constexpr int TX = 32, TY = 8, H = 3, HX = 4;
constexpr int PX = TX + 2 * HX, PY = TY + 2 * H, PS = PX * PY;
constexpr int NT = TX * TY;
constexpr int EPT = (PS + NT - 1) / NT;  // plane elements loaded per thread (4/8-byte copies)
// 16-byte chunks: values per chunk, chunks per row and plane, chunks per thread
template <typename FT> constexpr int VW = 16 / (int)sizeof(FT);
template <typename FT> constexpr int CPR = PX / VW<FT>;
template <typename FT> constexpr int CPT = (CPR<FT> * PY + NT - 1) / NT;
static_assert(PX % 4 == 0 && HX % 4 == 0, "plane rows must split into 16-byte chunks");
// immersed-boundary column table: halo 4 (a centred reconstruction checks cells up to 4 away)
constexpr int KBH = 4, KBX = TX + 2 * KBH, KBY = TY + 2 * KBH, KBS = KBX * KBY;
GBO_D int kbidx(int x, int y) { return (y + KBH) * KBX + (x + KBH); }

GBO_D int pidx(int x, int y) { return (y + H) * PX + (x + HX); }

// exchange quantities (west-face values live in WX[q][ty][tx], tx = 0..TX;
// south-face values in SY[q][ty][tx], ty = 0..TY)
enum { A_UU = 0, A_UV, A_UW, C_11, C_12, C_13, A_CX, Q_CX, NWX };   // west faces
enum { A_VU = 0, A_VV, A_VW, C_22, C_12N, C_23, A_CY, Q_CY, NSY };  // south faces

// Plane rings: a level's plane stays in its slot while it is in use and the
// next level's planes are prefetched asynchronously into the free slots.
template <typename FT>
struct __align__(16) Smem {
    FT U[3][PS], V[3][PS], W[3][PS];  // u, v: levels k-1, k (+k+1 in flight); w: faces k, k+1 (+k+2)
    FT NU[4][PS];                      // νₑ: k-1, k, k+1 (+k+2)
    FT PH[2][PS];                      // pHY′: k (+k+1)
    FT CC[2][PS];                      // tracer: k (+k+1)
    FT WX[NWX][TY][TX + 1];
    FT SY[NSY][TY + 1][TX];
    // vertical windows of the tile-edge columns: u of the east column (warp 0, lane = row)
    // and v of the north row (warp 1, lane = column), level L in slot L & 7; each entry is
    // written and read by one thread only
    FT EU[8][TY], EV[8][TX];
    // last, so that launches without AMD or an immersed boundary omit it (smem_bytes):
    union {
        FT KP[3][PS];                  // AMD κₑ: k, k+1 (+k+2)
        int KB[KBS];                   // immersed cells per column, tile with halo 4
    };
};
// Dynamic shared memory of a launch: the last member only with AMD or an immersed grid.
template <typename FT>
constexpr size_t smem_bytes(bool amd_or_ibg) {
    return amd_or_ibg ? sizeof(Smem<FT>) : sizeof(Smem<FT>) - sizeof(FT) * 3 * PS;
}

// Asynchronous 4/8-byte global -> shared copy; src_bytes = 0 writes zero.
template <typename FT>
GBO_D void cp_async(FT* dst, const FT* src, bool zero) {
    unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    if (sizeof(FT) == 4)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(d), "l"(src), "r"(zero ? 0 : 4));
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(d), "l"(src), "r"(zero ? 0 : 8));
}
// Asynchronous 16-byte copy (both addresses 16-byte aligned); zero = write zeros.
GBO_D void cp_async16(void* dst, const void* src, bool zero) {
    unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(src), "r"(zero ? 0 : 16));
}
GBO_D void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
GBO_D void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::); }

// Per-thread plane-load plan: offsets (within one z-level) of the wrapped (i, j) points
// this thread copies; identical for every level.  With vec, the thread copies 16-byte
// chunks (plane chunk tid + m NT): a chunk starts on a column that is a multiple of the
// chunk width, and with Nx a multiple of it a chunk never straddles the periodic seam,
// so each chunk is one contiguous, aligned run of the row it wraps to.
struct PlanePlan {
    int off[EPT];
    int n;
    int vec;
};
template <typename FT>
GBO_D PlanePlan make_plan(const GridP<FT>& g, int i0, int j0, int tid, int vec) {
    PlanePlan p;
    p.n = 0;
    p.vec = vec;
#pragma unroll
    for (int m = 0; m < EPT; ++m) {
        int e = tid + m * NT;
        p.off[m] = 0;
        if (vec) {
            if (m < CPT<FT> && e < CPR<FT> * PY) {
                const int px = (e % CPR<FT>) * VW<FT>, py = e / CPR<FT>;
                const int gi = wrapm(i0 + px - HX, g.Nx), gj = wrapm(j0 + py - H, g.Ny);
                p.off[m] = gi + g.Nx * gj;
                p.n = m + 1;
            }
        } else if (e < PS) {
            const int px = e % PX, py = e / PX;
            const int gi = wrapm(i0 + px - HX, g.Nx), gj = wrapm(j0 + py - H, g.Ny);
            p.off[m] = gi + g.Nx * gj;
            p.n = m + 1;
        }
    }
    return p;
}
// Level to read for a Center-in-z field at level k (mirror one halo layer; -1 = zero)
GBO_D int zsrc_c(int k, int Nz, int flatz) {
    if (flatz) return 0;
    if (k < -1 || k > Nz) return -1;
    return k < 0 ? 0 : (k >= Nz ? Nz - 1 : k);
}
// Level for w at face k (walls and beyond read zero)
GBO_D int zsrc_w(int k, int Nz) { return (k <= 0 || k >= Nz) ? -1 : k; }

template <typename FT>
GBO_D void issue_plane(FT* dst, const FT* src, int zl, size_t plane, const PlanePlan& pp, int tid) {
    const FT* base = src + (zl < 0 ? 0 : (size_t)zl * plane);
    if (pp.vec) {
#pragma unroll
        for (int m = 0; m < CPT<FT>; ++m)
            if (m < pp.n) cp_async16(dst + (tid + m * NT) * VW<FT>, base + pp.off[m], zl < 0);
    } else {
#pragma unroll
        for (int m = 0; m < EPT; ++m)
            if (m < pp.n) cp_async(dst + tid + m * NT, base + pp.off[m], zl < 0);
    }
}

// Whether a launch can copy its planes in 16-byte chunks: Nx a multiple of the chunk
// width (so is the plane size) and every field the planes come from 16-byte aligned
template <typename FT>
inline int planes_vec(const GridP<FT>& g, std::initializer_list<const void*> fields) {
    if (g.Nx % VW<FT> != 0) return 0;
    for (const void* f : fields)
        if (f && ((size_t)f & 15) != 0) return 0;
    return 1;
}

template <typename FT>
GBO_D FT flux_c4_w5(FT a0, FT a1, FT a2, FT a3, const FT* S) {
    FT ut = cen4<FT>(a0, a1, a2, a3);
    return ut * weno5<FT>(S, bias_left(ut));
}

// whether face code evaluates a cell's own face: a compile-time constant for the
// separately compiled forms, a run-time flag for the shared one
GBO_D constexpr bool own_value(std::true_type) { return true; }
GBO_D constexpr bool own_value(std::false_type) { return false; }
GBO_D bool own_value(bool b) { return b; }

template <typename FT>
struct Col {
    FT uc[7], vc[7], wc[6];
    FT fWu, fWv, fWw;
    FT t13, t23, t33;
    FT cc[7];
    FT fWc, qzc;
};

}  // namespace fused

// Column-marching fused kernel (see the file header).  TR: also advance one tracer
// (P.c -> P.co, P.Gc) in the same march.
template <typename FT, bool TR, int CLK, bool IBG = false>
__global__ void __launch_bounds__(256, sizeof(FT) == 4 ? GBO_FUSED_MIN_BLOCKS : 1) k_momentum_fused(StepP<FT> P, int kchunk, int vec) {
    using namespace fused;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Smem<FT>& s = *reinterpret_cast<Smem<FT>*>(smem_raw);
    const GridP<FT>& g = P.g;
    Met<FT> M(g);
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
    const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
    const int i = i0 + tx, j = j0 + ty;
    const int kb = blockIdx.z * kchunk, ke = min(g.Nz, kb + kchunk);
    constexpr bool closure = CLK != CL_NONE;
    constexpr bool amd = CLK == CL_AMD;
    const bool inside = (i < g.Nx) && (j < g.Ny);
    // the tracer's register window holds field values (reference profile added); its
    // shared-memory planes hold the stored values (departures where a profile exists)
    CFld<FT> Ug = cfld(P.u, g), Vg = cfld(P.v, g), Cg = cfld(P.c, g, P.cref);
    WFld<FT> Wg = wfld(P.w, g);
    const int Nz = g.Nz, fz = g.flatz;
    const FT Az = M.Az();
    const size_t plane = (size_t)g.Nx * g.Ny;
    const PlanePlan pp = make_plan(g, i0, j0, tid, vec);
    const int ii = i % g.Nx, jj = j % g.Ny;
    const size_t ccol = (size_t)ii + (size_t)g.Nx * jj;  // this thread's column (in the domain)

    // ring slots: U/V slot of level k = k mod 3, W slot of face k = k mod 3,
    // NU slot of level k = k mod 4, PH/CC slot = k mod 2, KP slot = k mod 3
    // (m3 only in the prologue; the loop tracks k mod 3 in r3)
    auto m3 = [](int k) { return ((k % 3) + 3) % 3; };
    auto m4 = [](int k) { return k & 3; };
    auto m2 = [](int k) { return k & 1; };

    // ---- immersed boundary (IBG): the rules of gbo_tendency.cuh (ibg_level, imm_periph,
    // cond_zero) evaluated from a shared tile of the column table; (x, y) are tile-local ----
    static_assert(!IBG || CLK == CL_NONE, "the fused immersed-boundary kernel carries no closure");
    if constexpr (IBG) {
        for (int e = tid; e < KBS; e += NT) {
            const int x = e % KBX - KBH, y = e / KBX - KBH;
            s.KB[e] = __ldg(g.kbot + wrapt(i0 + x, g.Nx) + (size_t)g.Nx * wrapt(j0 + y, g.Ny));
        }
    }
    // cell (x, y, k) immersed / inactive (immersed or outside the Bounded z)
    auto imm_t = [&](int x, int y, int kk) { return kk >= 0 && kk < Nz && kk < s.KB[kbidx(x, y)]; };
    auto inact_t = [&](int x, int y, int kk) { return kk < 0 || kk >= Nz || kk < s.KB[kbidx(x, y)]; };
    // immersed_peripheral_node with Face flags
    auto periph_t = [&](int x, int y, int kk, bool fx, bool fy, bool fzz) {
        bool any_imm = false, any_out = false;
        for (int a = 0; a <= (fx ? 1 : 0); ++a)
            for (int b = 0; b <= (fy ? 1 : 0); ++b)
                for (int c2 = 0; c2 <= (fzz ? 1 : 0); ++c2) {
                    const int k2 = kk - c2;
                    const bool out = k2 < 0 || k2 >= Nz;
                    any_out |= out;
                    any_imm |= (!out) && k2 < s.KB[kbidx(x - a, y - b)];
                }
        return any_imm && !any_out;
    };
    // reconstruction level (3 WENO5 / C4, 2 WENO3, 1 second order) in direction d at (x, y, k)
    auto level_t = [&](int d, int x, int y, int kk, bool loc_face) {
        for (int B = 3; B >= 2; --B) {
            const int lo = loc_face ? -B : -B + 1, hi = loc_face ? B - 1 : B;
            bool near = false;
            for (int o = lo; o <= hi; ++o) {
                const int xx = x + (d == 0 ? o : 0), yy = y + (d == 1 ? o : 0), k2 = kk + (d == 2 ? o : 0);
                bool ia = inact_t(xx, yy, k2);
                if (!loc_face) ia = ia && inact_t(xx - (d == 0), yy - (d == 1), k2 - (d == 2));
                near |= ia;
            }
            if (!near) return B;
        }
        return 1;
    };
    auto sym_t = [&](int d, int x, int y, int kk, bool loc_face) { return level_t(d, x, y, kk, loc_face) == 3 ? 3 : 1; };
    // advective momentum flux ũ ψ on the immersed grid: zero on the periphery, symmetric
    // (level sl) and biased (level bl) reconstructions of reduced order near inactive cells
    auto mflux_t = [&](bool zero, auto qs, int sl, auto qb, int bl) -> FT {
        if (zero) return FT(0);
        const FT ut = symm<FT>(qs, sl);
        return ut * biased<FT>(qb, bias_left(ut), bl);
    };

    // the tile-edge column whose faces this thread evaluates after its own (the east column
    // for warp 0, the north row for warp 1), wrapped: on grids narrower than a tile it lies
    // more than one period outside the domain; its vertical window goes to EU / EV
    const size_t fcol = (size_t)wrapm(i0 + (ty == 0 ? TX : tx), g.Nx) + (size_t)g.Nx * wrapm(j0 + (ty == 0 ? tx : TY), g.Ny);
    const bool edgeW = ty == 0 && tx < TY, edgeS = ty == 1;
    auto issue_edge = [&](int kk) {
        const int zl = zsrc_c(kk, Nz, fz);
        const size_t off = fcol + (zl < 0 ? 0 : (size_t)zl * plane);
        if (edgeW) cp_async(&s.EU[kk & 7][tx], P.u + off, zl < 0);
        else if (edgeS) cp_async(&s.EV[kk & 7][tx], P.v + off, zl < 0);
    };

    // ---- prologue: planes for level kb ----
    issue_plane(s.U[m3(kb - 1)], P.u, zsrc_c(kb - 1, Nz, fz), plane, pp, tid);
    issue_plane(s.V[m3(kb - 1)], P.v, zsrc_c(kb - 1, Nz, fz), plane, pp, tid);
    issue_plane(s.U[m3(kb)], P.u, zsrc_c(kb, Nz, fz), plane, pp, tid);
    issue_plane(s.V[m3(kb)], P.v, zsrc_c(kb, Nz, fz), plane, pp, tid);
    if (!fz) {
        issue_plane(s.W[m3(kb)], P.w, zsrc_w(kb, Nz), plane, pp, tid);
        issue_plane(s.W[m3(kb + 1)], P.w, zsrc_w(kb + 1, Nz), plane, pp, tid);
    }
    if (closure) {
        issue_plane(s.NU[m4(kb - 1)], P.nu, zsrc_c(kb - 1, Nz, fz), plane, pp, tid);
        issue_plane(s.NU[m4(kb)], P.nu, zsrc_c(kb, Nz, fz), plane, pp, tid);
        issue_plane(s.NU[m4(kb + 1)], P.nu, zsrc_c(kb + 1, Nz, fz), plane, pp, tid);
    }
    if (P.has_phy) issue_plane(s.PH[m2(kb)], P.phy, zsrc_c(kb, Nz, fz), plane, pp, tid);
    if (TR) issue_plane(s.CC[m2(kb)], P.c, zsrc_c(kb, Nz, fz), plane, pp, tid);
    if (TR && amd) {
        issue_plane(s.KP[m3(kb)], P.kap, zsrc_c(kb, Nz, fz), plane, pp, tid);
        issue_plane(s.KP[m3(kb + 1)], P.kap, zsrc_c(kb + 1, Nz, fz), plane, pp, tid);
    }
    if (!fz)
        for (int o = -2; o <= 1; ++o) issue_edge(kb + o);
    cp_async_commit();
    Col<FT> c;
#pragma unroll
    for (int o = 0; o < 7; ++o) {
        c.uc[o] = Ug.col(ccol, kb - 3 + o);
        c.vc[o] = Vg.col(ccol, kb - 3 + o);
        if (TR) c.cc[o] = Cg.col(ccol, kb - 3 + o);
    }
#pragma unroll
    for (int o = 0; o < 6; ++o) c.wc[o] = Wg.col(ccol, kb - 2 + o);
    const FT wm3 = Wg.col(ccol, kb - 3);
    FT km_amd = FT(0);
    if (TR && amd) km_amd = cfld(P.kap, g).col(ccol, kb - 1);
    cp_async_wait_all();
    __syncthreads();
    // bottom fluxes at level kb (faces kb / centre kb-1)
    {
        const FT* Wk = s.W[m3(kb)];
        if constexpr (IBG) {
            c.fWu = mflux_t(periph_t(tx, ty, kb, true, false, true), [&](int o) { return Az * Wk[pidx(tx + o, ty)]; },
                            sym_t(0, tx, ty, kb, true), [&](int o) { return c.uc[3 + o]; }, level_t(2, tx, ty, kb, true));
            c.fWv = mflux_t(periph_t(tx, ty, kb, false, true, true), [&](int o) { return Az * Wk[pidx(tx, ty + o)]; },
                            sym_t(1, tx, ty, kb, true), [&](int o) { return c.vc[3 + o]; }, level_t(2, tx, ty, kb, true));
            const int kc = kb - 1;
            c.fWw = mflux_t(periph_t(tx, ty, kc, false, false, false), [&](int o) { return Az * (o == -3 ? wm3 : c.wc[2 + o]); },
                            sym_t(2, tx, ty, kc, false), [&](int o) { return o == -3 ? wm3 : c.wc[2 + o]; },
                            level_t(2, tx, ty, kc, false));
        } else {
        {
            FT wt = cen4<FT>(Az * Wk[pidx(tx - 2, ty)], Az * Wk[pidx(tx - 1, ty)], Az * Wk[pidx(tx, ty)], Az * Wk[pidx(tx + 1, ty)]);
            auto q = [&](int o) { return c.uc[3 + o]; };
            c.fWu = wt * biased<FT>(q, bias_left(wt), zlev_biased_face(kb + 1, Nz));
        }
        {
            FT wt = cen4<FT>(Az * Wk[pidx(tx, ty - 2)], Az * Wk[pidx(tx, ty - 1)], Az * Wk[pidx(tx, ty)], Az * Wk[pidx(tx, ty + 1)]);
            auto q = [&](int o) { return c.vc[3 + o]; };
            c.fWv = wt * biased<FT>(q, bias_left(wt), zlev_biased_face(kb + 1, Nz));
        }
        {
            const int kc = kb - 1;
            auto qs = [&](int o) { return Az * (o == -3 ? wm3 : c.wc[2 + o]); };
            FT wt = symm<FT>(qs, zlev_symm_center(kc + 1, Nz));
            auto qb = [&](int o) { return o == -3 ? wm3 : c.wc[2 + o]; };
            c.fWw = wt * biased<FT>(qb, bias_left(wt), zlev_biased_center(kc + 1, Nz));
        }
        }
        c.t13 = c.t23 = c.t33 = FT(0);
        if (closure) {
            const FT* Nm = s.NU[m4(kb - 1)];
            const FT* Nk = s.NU[m4(kb)];
            FT nfcf = FT(0.5) * (FT(0.5) * (Nm[pidx(tx - 1, ty)] + Nm[pidx(tx, ty)]) + FT(0.5) * (Nk[pidx(tx - 1, ty)] + Nk[pidx(tx, ty)]));
            FT dzu = (c.uc[3] - c.uc[2]) * M.rdzf(kb);
            FT dxw = (Wk[pidx(tx, ty)] - Wk[pidx(tx - 1, ty)]) * g.rdx;
            c.t13 = FT(-2) * (nfcf * (FT(0.5) * (dzu + dxw)));
            FT ncff = FT(0.5) * (FT(0.5) * (Nm[pidx(tx, ty - 1)] + Nm[pidx(tx, ty)]) + FT(0.5) * (Nk[pidx(tx, ty - 1)] + Nk[pidx(tx, ty)]));
            FT dzv = (c.vc[3] - c.vc[2]) * M.rdzf(kb);
            FT dyw = (Wk[pidx(tx, ty)] - Wk[pidx(tx, ty - 1)]) * g.rdy;
            c.t23 = FT(-2) * (ncff * (FT(0.5) * (dzv + dyw)));
            c.t33 = FT(-2) * (Nm[pidx(tx, ty)] * ((c.wc[2] - c.wc[1]) * M.rdzc(kb - 1)));
        }
        if (TR) {
            FT wk = c.wc[2];
            auto q = [&](int o) { return c.cc[3 + o]; };
            c.fWc = Az * wk * biased<FT>(q, bias_left(wk), IBG ? level_t(2, tx, ty, kb, true) : zlev_biased_face(kb + 1, Nz));
            c.qzc = FT(0);
            if (closure) {
                FT km = amd ? km_amd : s.NU[m4(kb - 1)][pidx(tx, ty)];
                const FT* Kb = amd ? s.KP[m3(kb)] : s.NU[m4(kb)];  // pick the plane, then load
                FT kk = Kb[pidx(tx, ty)];
                FT kz = amd ? FT(0.5) * (km + kk) : FT(0.5) * (km + kk) / P.Pr;
                c.qzc = -kz * ((c.cc[3] - c.cc[2]) * M.rdzf(kb));
            }
        }
    }

    const FT dt = stage_dt(P);
    int r3 = m3(kb);
    for (int k = kb; k < ke; ++k) {
        // ring slots of levels k-1, k, k+1 (and k+2, which shares the slot of k-1)
        const int s3k = r3, s3p = r3 == 2 ? 0 : r3 + 1, s3m = r3 == 0 ? 2 : r3 - 1;
        // ---- prefetch the planes first needed at level k+1 (free ring slots) ----
        const int kn = k + 1;
        if (kn < ke) {
            issue_plane(s.U[s3p], P.u, zsrc_c(kn, Nz, fz), plane, pp, tid);
            issue_plane(s.V[s3p], P.v, zsrc_c(kn, Nz, fz), plane, pp, tid);
            if (!fz) issue_plane(s.W[s3m], P.w, zsrc_w(kn + 1, Nz), plane, pp, tid);
            if (closure) issue_plane(s.NU[m4(kn + 1)], P.nu, zsrc_c(kn + 1, Nz, fz), plane, pp, tid);
            if (P.has_phy) issue_plane(s.PH[m2(kn)], P.phy, zsrc_c(kn, Nz, fz), plane, pp, tid);
            if (TR) issue_plane(s.CC[m2(kn)], P.c, zsrc_c(kn, Nz, fz), plane, pp, tid);
            if (TR && amd) issue_plane(s.KP[s3m], P.kap, zsrc_c(kn + 1, Nz, fz), plane, pp, tid);
            if (!fz) issue_edge(k + 2);  // read from level k + 1 on
        }
        cp_async_commit();
        // ---- early loads: window tops for the next level, G⁻ of this level ----
        const FT un = Ug.col(ccol, k + 4), vn = Vg.col(ccol, k + 4), wn = Wg.col(ccol, k + 4);
        const FT cnext = TR ? Cg.col(ccol, k + 4) : FT(0);
        const size_t idx = ii + (size_t)g.Nx * jj + plane * k;
        FT Gum = FT(0), Gvm = FT(0), Gwm = FT(0), Gcm = FT(0);
        if (!P.first && inside) {
            Gum = P.Gu[idx];
            Gvm = P.Gv[idx];
            if (!fz && k > 0) Gwm = P.Gw[idx];
            if (TR) Gcm = P.Gc[idx];
        }
        const FT* Uk = s.U[s3k];
        const FT* Um = s.U[s3m];
        const FT* Vk = s.V[s3k];
        const FT* Vm = s.V[s3m];
        const FT* Wk = s.W[s3k];
        const FT* Wp = s.W[s3p];
        const FT* Nm = s.NU[m4(k - 1)];
        const FT* Nk = s.NU[m4(k)];
        const FT* Np = s.NU[m4(k + 1)];
        const FT* PHk = s.PH[m2(k)];
        const FT* CCk = s.CC[m2(k)];
        const FT* Kk = s.KP[s3k];
        const FT* Kp = s.KP[s3p];
        const FT Ax = M.Ax(k), Ay = M.Ay(k);
        // horizontal reconstructions of a departure field: the level's profile value is
        // constant along x and y, and every stencil reproduces constants, so the field's
        // reconstruction is the profile value plus that of the departures (the smoothness
        // indicators see only differences)
        const FT cref_k = (TR && sizeof(FT) == 4 && P.cref && !fz) ? __ldg(P.cref + k) : FT(0);
        auto with_ref = [&](FT x) -> FT {
            if constexpr (sizeof(FT) == 4) return cref_k + x;
            else return x;
        };

        // ---- west / south face quantities of this thread (and the tile edges) ----
        auto west = [&](int x, int y, auto own_t) {
            const bool own = own_value(own_t);  // a constant for std::true_type / std::false_type
            FT S[6];
            if constexpr (IBG) {
#pragma unroll
                for (int o = 0; o < 6; ++o) S[o] = Uk[pidx(x - 3 + o, y)];
                s.WX[A_UU][y][x] = mflux_t(periph_t(x - 1, y, k, false, false, false), [&](int o) { return Ax * S[o + 3]; },
                                           sym_t(0, x - 1, y, k, false), [&](int o) { return S[o + 3]; }, level_t(0, x - 1, y, k, false));
#pragma unroll
                for (int o = 0; o < 6; ++o) S[o] = Vk[pidx(x - 3 + o, y)];
                s.WX[A_UV][y][x] = mflux_t(periph_t(x, y, k, true, true, false), [&](int o) { return Ax * Uk[pidx(x, y + o)]; },
                                           sym_t(1, x, y, k, true), [&](int o) { return S[o + 3]; }, level_t(0, x, y, k, true));
            } else {
                // u and v through this x face: both WENO5 reconstructions at once
                FT T[6];
#pragma unroll
                for (int o = 0; o < 6; ++o) {
                    S[o] = Uk[pidx(x - 3 + o, y)];
                    T[o] = Vk[pidx(x - 3 + o, y)];
                }
                const FT uu = cen4<FT>(Ax * S[1], Ax * S[2], Ax * S[3], Ax * S[4]);
                const FT uv = cen4<FT>(Ax * Uk[pidx(x, y - 2)], Ax * Uk[pidx(x, y - 1)], Ax * Uk[pidx(x, y)], Ax * Uk[pidx(x, y + 1)]);
                FT ru, rv;
                weno5_2<FT>(S, bias_left(uu), T, bias_left(uv), ru, rv);
                s.WX[A_UU][y][x] = uu * ru;
                s.WX[A_UV][y][x] = uv * rv;
            }
            // w and the tracer through this x face, paired where both exist
            bool paired = false;
            if constexpr (!IBG && TR) {
                if (!fz) {
                    paired = true;
                    FT uz[4];
                    if (own) {
#pragma unroll
                        for (int o = 0; o < 4; ++o) uz[o] = c.uc[1 + o];
                    } else {
#pragma unroll
                        for (int o = 0; o < 4; ++o) uz[o] = s.EU[(k - 2 + o) & 7][y];
                    }
                    auto qs = [&](int o) { return M.Ax(k + o) * uz[o + 2]; };
                    const FT uw = symm<FT>(qs, zlev_symm_face(k + 1, Nz));
                    const FT uc = Uk[pidx(x, y)];
                    FT T[6];
#pragma unroll
                    for (int o = 0; o < 6; ++o) {
                        S[o] = Wk[pidx(x - 3 + o, y)];
                        T[o] = CCk[pidx(x - 3 + o, y)];
                    }
                    FT rw, rc;
                    weno5_2<FT>(S, bias_left(uw), T, bias_left(uc), rw, rc);
                    s.WX[A_UW][y][x] = uw * rw;
                    s.WX[A_CX][y][x] = Ax * uc * with_ref(rc);
                }
            }
            if (!fz && !paired) {
                FT uz[4];
                if (own) {
#pragma unroll
                    for (int o = 0; o < 4; ++o) uz[o] = c.uc[1 + o];
                } else {
#pragma unroll
                    for (int o = 0; o < 4; ++o) uz[o] = s.EU[(k - 2 + o) & 7][y];
                }
                auto qs = [&](int o) { return M.Ax(k + o) * uz[o + 2]; };
#pragma unroll
                for (int o = 0; o < 6; ++o) S[o] = Wk[pidx(x - 3 + o, y)];
                if constexpr (IBG) {
                    s.WX[A_UW][y][x] = mflux_t(periph_t(x, y, k, true, false, true), qs, sym_t(2, x, y, k, true),
                                               [&](int o) { return S[o + 3]; }, level_t(0, x, y, k, true));
                } else {
                    FT ut = symm<FT>(qs, zlev_symm_face(k + 1, Nz));
                    s.WX[A_UW][y][x] = ut * weno5<FT>(S, bias_left(ut));
                }
            }
            if (closure) {
                FT s11 = (Uk[pidx(x, y)] - Uk[pidx(x - 1, y)]) * g.rdx;
                s.WX[C_11][y][x] = FT(-2) * (Nk[pidx(x - 1, y)] * s11);
                FT nffc = FT(0.5) * (FT(0.5) * (Nk[pidx(x - 1, y - 1)] + Nk[pidx(x, y - 1)]) + FT(0.5) * (Nk[pidx(x - 1, y)] + Nk[pidx(x, y)]));
                FT dyu = (Uk[pidx(x, y)] - Uk[pidx(x, y - 1)]) * g.rdy;
                FT dxv = (Vk[pidx(x, y)] - Vk[pidx(x - 1, y)]) * g.rdx;
                s.WX[C_12][y][x] = FT(-2) * (nffc * (FT(0.5) * (dyu + dxv)));
                if (own) {
                    s.WX[C_13][y][x] = c.t13;
                } else if (!fz) {
                    FT nfcf = FT(0.5) * (FT(0.5) * (Nm[pidx(x - 1, y)] + Nm[pidx(x, y)]) + FT(0.5) * (Nk[pidx(x - 1, y)] + Nk[pidx(x, y)]));
                    FT dzu = (Uk[pidx(x, y)] - Um[pidx(x, y)]) * M.rdzf(k);
                    FT dxw = (Wk[pidx(x, y)] - Wk[pidx(x - 1, y)]) * g.rdx;
                    s.WX[C_13][y][x] = FT(-2) * (nfcf * (FT(0.5) * (dzu + dxw)));
                }
            }
            if (TR) {
                if (!paired) {
                    FT ut = Uk[pidx(x, y)];
#pragma unroll
                    for (int o = 0; o < 6; ++o) S[o] = CCk[pidx(x - 3 + o, y)];
                    if constexpr (IBG)
                        s.WX[A_CX][y][x] = Ax * ut * with_ref(biased<FT>([&](int o) { return S[o + 3]; }, bias_left(ut), level_t(0, x, y, k, true)));
                    else
                        s.WX[A_CX][y][x] = Ax * ut * with_ref(weno5<FT>(S, bias_left(ut)));
                }
                if (closure) {
                    const FT* K = amd ? Kk : Nk;
                    FT kx = amd ? FT(0.5) * (K[pidx(x - 1, y)] + K[pidx(x, y)]) : FT(0.5) * (K[pidx(x - 1, y)] + K[pidx(x, y)]) / P.Pr;
                    s.WX[Q_CX][y][x] = -kx * ((CCk[pidx(x, y)] - CCk[pidx(x - 1, y)]) * g.rdx);
                }
            }
        };
        auto south = [&](int x, int y, auto own_t) {
            const bool own = own_value(own_t);  // a constant for std::true_type / std::false_type
            FT S[6];
            if constexpr (IBG) {
#pragma unroll
                for (int o = 0; o < 6; ++o) S[o] = Uk[pidx(x, y - 3 + o)];
                s.SY[A_VU][y][x] = mflux_t(periph_t(x, y, k, true, true, false), [&](int o) { return Ay * Vk[pidx(x + o, y)]; },
                                           sym_t(0, x, y, k, true), [&](int o) { return S[o + 3]; }, level_t(1, x, y, k, true));
#pragma unroll
                for (int o = 0; o < 6; ++o) S[o] = Vk[pidx(x, y - 3 + o)];
                s.SY[A_VV][y][x] = mflux_t(periph_t(x, y - 1, k, false, false, false), [&](int o) { return Ay * S[o + 3]; },
                                           sym_t(1, x, y - 1, k, false), [&](int o) { return S[o + 3]; }, level_t(1, x, y - 1, k, false));
            } else {
                // u and v through this y face: both WENO5 reconstructions at once
                FT T[6];
#pragma unroll
                for (int o = 0; o < 6; ++o) {
                    S[o] = Uk[pidx(x, y - 3 + o)];
                    T[o] = Vk[pidx(x, y - 3 + o)];
                }
                const FT vu = cen4<FT>(Ay * Vk[pidx(x - 2, y)], Ay * Vk[pidx(x - 1, y)], Ay * Vk[pidx(x, y)], Ay * Vk[pidx(x + 1, y)]);
                const FT vv = cen4<FT>(Ay * T[1], Ay * T[2], Ay * T[3], Ay * T[4]);
                FT ru, rv;
                weno5_2<FT>(S, bias_left(vu), T, bias_left(vv), ru, rv);
                s.SY[A_VU][y][x] = vu * ru;
                s.SY[A_VV][y][x] = vv * rv;
            }
            // w and the tracer through this y face, paired where both exist
            bool paired = false;
            if constexpr (!IBG && TR) {
                if (!fz) {
                    paired = true;
                    FT vz[4];
                    if (own) {
#pragma unroll
                        for (int o = 0; o < 4; ++o) vz[o] = c.vc[1 + o];
                    } else {
#pragma unroll
                        for (int o = 0; o < 4; ++o) vz[o] = s.EV[(k - 2 + o) & 7][x];
                    }
                    auto qs = [&](int o) { return M.Ay(k + o) * vz[o + 2]; };
                    const FT vw = symm<FT>(qs, zlev_symm_face(k + 1, Nz));
                    const FT vc = Vk[pidx(x, y)];
                    FT T[6];
#pragma unroll
                    for (int o = 0; o < 6; ++o) {
                        S[o] = Wk[pidx(x, y - 3 + o)];
                        T[o] = CCk[pidx(x, y - 3 + o)];
                    }
                    FT rw, rc;
                    weno5_2<FT>(S, bias_left(vw), T, bias_left(vc), rw, rc);
                    s.SY[A_VW][y][x] = vw * rw;
                    s.SY[A_CY][y][x] = Ay * vc * with_ref(rc);
                }
            }
            if (!fz && !paired) {
                FT vz[4];
                if (own) {
#pragma unroll
                    for (int o = 0; o < 4; ++o) vz[o] = c.vc[1 + o];
                } else {
#pragma unroll
                    for (int o = 0; o < 4; ++o) vz[o] = s.EV[(k - 2 + o) & 7][x];
                }
                auto qs = [&](int o) { return M.Ay(k + o) * vz[o + 2]; };
#pragma unroll
                for (int o = 0; o < 6; ++o) S[o] = Wk[pidx(x, y - 3 + o)];
                if constexpr (IBG) {
                    s.SY[A_VW][y][x] = mflux_t(periph_t(x, y, k, false, true, true), qs, sym_t(2, x, y, k, true),
                                               [&](int o) { return S[o + 3]; }, level_t(1, x, y, k, true));
                } else {
                    FT vt = symm<FT>(qs, zlev_symm_face(k + 1, Nz));
                    s.SY[A_VW][y][x] = vt * weno5<FT>(S, bias_left(vt));
                }
            }
            if (closure) {
                FT s22 = (Vk[pidx(x, y)] - Vk[pidx(x, y - 1)]) * g.rdy;
                s.SY[C_22][y][x] = FT(-2) * (Nk[pidx(x, y - 1)] * s22);
                FT nffc = FT(0.5) * (FT(0.5) * (Nk[pidx(x - 1, y - 1)] + Nk[pidx(x, y - 1)]) + FT(0.5) * (Nk[pidx(x - 1, y)] + Nk[pidx(x, y)]));
                FT dyu = (Uk[pidx(x, y)] - Uk[pidx(x, y - 1)]) * g.rdy;
                FT dxv = (Vk[pidx(x, y)] - Vk[pidx(x - 1, y)]) * g.rdx;
                s.SY[C_12N][y][x] = FT(-2) * (nffc * (FT(0.5) * (dyu + dxv)));
                if (own) {
                    s.SY[C_23][y][x] = c.t23;
                } else if (!fz) {
                    FT ncff = FT(0.5) * (FT(0.5) * (Nm[pidx(x, y - 1)] + Nm[pidx(x, y)]) + FT(0.5) * (Nk[pidx(x, y - 1)] + Nk[pidx(x, y)]));
                    FT dzv = (Vk[pidx(x, y)] - Vm[pidx(x, y)]) * M.rdzf(k);
                    FT dyw = (Wk[pidx(x, y)] - Wk[pidx(x, y - 1)]) * g.rdy;
                    s.SY[C_23][y][x] = FT(-2) * (ncff * (FT(0.5) * (dzv + dyw)));
                }
            }
            if (TR) {
                if (!paired) {
                    FT vt = Vk[pidx(x, y)];
#pragma unroll
                    for (int o = 0; o < 6; ++o) S[o] = CCk[pidx(x, y - 3 + o)];
                    if constexpr (IBG)
                        s.SY[A_CY][y][x] = Ay * vt * with_ref(biased<FT>([&](int o) { return S[o + 3]; }, bias_left(vt), level_t(1, x, y, k, true)));
                    else
                        s.SY[A_CY][y][x] = Ay * vt * with_ref(weno5<FT>(S, bias_left(vt)));
                }
                if (closure) {
                    const FT* K = amd ? Kk : Nk;
                    FT ky = amd ? FT(0.5) * (K[pidx(x, y - 1)] + K[pidx(x, y)]) : FT(0.5) * (K[pidx(x, y - 1)] + K[pidx(x, y)]) / P.Pr;
                    s.SY[Q_CY][y][x] = -ky * ((CCk[pidx(x, y)] - CCk[pidx(x, y - 1)]) * g.rdy);
                }
            }
        };
        // the faces of this thread's cells (windows in registers), then the tile's east
        // column (warp 0, lanes < TY) and north row (warp 1) from the edge columns.  Each
        // form is compiled separately (own a compile-time constant in each), except on an
        // immersed grid, whose much larger face code keeps one copy for both (a second
        // copy measured slower there)
        if constexpr (IBG) {
#pragma unroll 1
            for (int pass = 0; pass < 2; ++pass) {
                const bool own = pass == 0;
                if (own || (ty == 0 && tx < TY)) west(own ? tx : TX, own ? ty : tx, own);
                if (own || ty == 1) south(tx, own ? ty : TY, own);
            }
        } else {
            west(tx, ty, std::true_type{});
            south(tx, ty, std::true_type{});
            if (ty == 0 && tx < TY) west(TX, tx, std::false_type{});
            if (ty == 1) south(tx, TY, std::false_type{});
        }

        // ---- top-face quantities (carried to the next level) ----
        FT fWu_t = FT(0), fWv_t = FT(0), fWw_t = FT(0), t13_t = FT(0), t23_t = FT(0), t33_t = FT(0);
        FT fWc_t = FT(0), qzc_t = FT(0);
        if (!fz) {
            if constexpr (IBG) {
                fWu_t = mflux_t(periph_t(tx, ty, k + 1, true, false, true), [&](int o) { return Az * Wp[pidx(tx + o, ty)]; },
                                sym_t(0, tx, ty, k + 1, true), [&](int o) { return c.uc[4 + o]; }, level_t(2, tx, ty, k + 1, true));
                fWv_t = mflux_t(periph_t(tx, ty, k + 1, false, true, true), [&](int o) { return Az * Wp[pidx(tx, ty + o)]; },
                                sym_t(1, tx, ty, k + 1, true), [&](int o) { return c.vc[4 + o]; }, level_t(2, tx, ty, k + 1, true));
                fWw_t = mflux_t(periph_t(tx, ty, k, false, false, false), [&](int o) { return Az * c.wc[3 + o]; },
                                sym_t(2, tx, ty, k, false), [&](int o) { return c.wc[3 + o]; }, level_t(2, tx, ty, k, false));
            } else {
                // u and v through the top face (the same reconstruction level): paired
                // WENO5 away from the walls
                const int lf = zlev_biased_face(k + 2, Nz);
                const FT wu = cen4<FT>(Az * Wp[pidx(tx - 2, ty)], Az * Wp[pidx(tx - 1, ty)], Az * Wp[pidx(tx, ty)], Az * Wp[pidx(tx + 1, ty)]);
                const FT wv = cen4<FT>(Az * Wp[pidx(tx, ty - 2)], Az * Wp[pidx(tx, ty - 1)], Az * Wp[pidx(tx, ty)], Az * Wp[pidx(tx, ty + 1)]);
                if (lf == 3) {
                    FT ru, rv;
                    weno5_2<FT>(&c.uc[1], bias_left(wu), &c.vc[1], bias_left(wv), ru, rv);
                    fWu_t = wu * ru;
                    fWv_t = wv * rv;
                } else {
                    fWu_t = wu * biased<FT>([&](int o) { return c.uc[4 + o]; }, bias_left(wu), lf);
                    fWv_t = wv * biased<FT>([&](int o) { return c.vc[4 + o]; }, bias_left(wv), lf);
                }
                // w (and the tracer, paired when both take WENO5) through the centre above
                const int lc = zlev_biased_center(k + 1, Nz);
                const FT ww = symm<FT>([&](int o) { return Az * c.wc[3 + o]; }, zlev_symm_center(k + 1, Nz));
                if (TR && lc == 3 && lf == 3) {
                    const FT wc = c.wc[3];
                    FT rw, rc;
                    weno5_2<FT>(&c.wc[0], bias_left(ww), &c.cc[1], bias_left(wc), rw, rc);
                    fWw_t = ww * rw;
                    fWc_t = Az * wc * rc;
                } else {
                    fWw_t = ww * biased<FT>([&](int o) { return c.wc[3 + o]; }, bias_left(ww), lc);
                    if (TR) {
                        const FT wc = c.wc[3];
                        fWc_t = Az * wc * biased<FT>([&](int o) { return c.cc[4 + o]; }, bias_left(wc), lf);
                    }
                }
            }
            if (closure) {
                FT nfcf = FT(0.5) * (FT(0.5) * (Nk[pidx(tx - 1, ty)] + Nk[pidx(tx, ty)]) + FT(0.5) * (Np[pidx(tx - 1, ty)] + Np[pidx(tx, ty)]));
                FT dzu = (c.uc[4] - c.uc[3]) * M.rdzf(k + 1);
                FT dxw = (Wp[pidx(tx, ty)] - Wp[pidx(tx - 1, ty)]) * g.rdx;
                t13_t = FT(-2) * (nfcf * (FT(0.5) * (dzu + dxw)));
                FT ncff = FT(0.5) * (FT(0.5) * (Nk[pidx(tx, ty - 1)] + Nk[pidx(tx, ty)]) + FT(0.5) * (Np[pidx(tx, ty - 1)] + Np[pidx(tx, ty)]));
                FT dzv = (c.vc[4] - c.vc[3]) * M.rdzf(k + 1);
                FT dyw = (Wp[pidx(tx, ty)] - Wp[pidx(tx, ty - 1)]) * g.rdy;
                t23_t = FT(-2) * (ncff * (FT(0.5) * (dzv + dyw)));
                t33_t = FT(-2) * (Nk[pidx(tx, ty)] * ((c.wc[3] - c.wc[2]) * M.rdzc(k)));
            }
            if (TR) {
                if constexpr (IBG) {
                    const FT wt = c.wc[3];
                    fWc_t = Az * wt * biased<FT>([&](int o) { return c.cc[4 + o]; }, bias_left(wt), level_t(2, tx, ty, k + 1, true));
                }
                if (closure) {
                    const FT* K0 = amd ? Kk : Nk;
                    const FT* K1 = amd ? Kp : Np;
                    FT kk = K0[pidx(tx, ty)];
                    FT kp = K1[pidx(tx, ty)];
                    FT kz = amd ? FT(0.5) * (kk + kp) : FT(0.5) * (kk + kp) / P.Pr;
                    qzc_t = -kz * ((c.cc[4] - c.cc[3]) * M.rdzf(k + 1));
                }
            }
        }
        __syncthreads();

        // ---- tendencies and predictor ----
        if (inside) {
            const FT rVc = M.rVc(k);
            {
                FT dx_ = s.WX[A_UU][ty][tx + 1] - s.WX[A_UU][ty][tx];
                FT dy_ = s.SY[A_VU][ty + 1][tx] - s.SY[A_VU][ty][tx];
                FT dz_ = fz ? FT(0) : (fWu_t - c.fWu);
                FT G = -(rVc * (dx_ + dy_ + dz_));
                if (P.has_cor) {
                    // masked_Ay_qᶜᶠᶜ on an immersed grid (coriolis_schemes.jl:55-58)
                    auto AyV = [&](int x, int y) { return (IBG && periph_t(x, y, k, false, true, false)) ? FT(0) : Ay * Vk[pidx(x, y)]; };
                    FT ixy = FT(0.5) * (FT(0.5) * (AyV(tx - 1, ty) + AyV(tx, ty)) + FT(0.5) * (AyV(tx - 1, ty + 1) + AyV(tx, ty + 1)));
                    FT xfu = -P.f * ixy * (FT(1) / Ay);
                    G = G - xfu;
                }
                if (P.has_phy)
                    G = G - ((IBG && (imm_t(tx - 1, ty, k) || imm_t(tx, ty, k))) ? FT(0) : (PHk[pidx(tx, ty)] - PHk[pidx(tx - 1, ty)])) * g.rdx;
                if (closure) {
                    FT cdx = Ax * s.WX[C_11][ty][tx + 1] - Ax * s.WX[C_11][ty][tx];
                    FT cdy = Ay * s.SY[C_12N][ty + 1][tx] - Ay * s.SY[C_12N][ty][tx];
                    FT cdz = fz ? FT(0) : (Az * t13_t - Az * c.t13);
                    G = G - rVc * (cdx + cdy + cdz);
                }
                P.Gu[idx] = G;
                P.uo[idx] = rk3_update(Uk[pidx(tx, ty)], G, Gum, P, dt);
            }
            {
                FT dx_ = s.WX[A_UV][ty][tx + 1] - s.WX[A_UV][ty][tx];
                FT dy_ = s.SY[A_VV][ty + 1][tx] - s.SY[A_VV][ty][tx];
                FT dz_ = fz ? FT(0) : (fWv_t - c.fWv);
                FT G = -(rVc * (dx_ + dy_ + dz_));
                if (P.has_cor) {
                    auto AxU = [&](int x, int y) { return (IBG && periph_t(x, y, k, true, false, false)) ? FT(0) : Ax * Uk[pidx(x, y)]; };
                    FT ixy = FT(0.5) * (FT(0.5) * (AxU(tx, ty - 1) + AxU(tx + 1, ty - 1)) + FT(0.5) * (AxU(tx, ty) + AxU(tx + 1, ty)));
                    FT yfu = P.f * ixy * (FT(1) / Ax);
                    G = G - yfu;
                }
                if (P.has_phy)
                    G = G - ((IBG && (imm_t(tx, ty - 1, k) || imm_t(tx, ty, k))) ? FT(0) : (PHk[pidx(tx, ty)] - PHk[pidx(tx, ty - 1)])) * g.rdy;
                if (closure) {
                    FT cdx = Ax * s.WX[C_12][ty][tx + 1] - Ax * s.WX[C_12][ty][tx];
                    FT cdy = Ay * s.SY[C_22][ty + 1][tx] - Ay * s.SY[C_22][ty][tx];
                    FT cdz = fz ? FT(0) : (Az * t23_t - Az * c.t23);
                    G = G - rVc * (cdx + cdy + cdz);
                }
                P.Gv[idx] = G;
                P.vo[idx] = rk3_update(Vk[pidx(tx, ty)], G, Gvm, P, dt);
            }
            if (!fz) {
                if (k == 0) {
                    P.wo[idx] = FT(0);
                } else {
                    FT dx_ = s.WX[A_UW][ty][tx + 1] - s.WX[A_UW][ty][tx];
                    FT dy_ = s.SY[A_VW][ty + 1][tx] - s.SY[A_VW][ty][tx];
                    FT dz_ = fWw_t - c.fWw;
                    FT rVf = M.rVf(k);
                    FT G = -(rVf * (dx_ + dy_ + dz_));
                    if (closure) {
                        FT Axf = M.Axf(k), Ayf = M.Ayf(k);
                        FT cdx = Axf * s.WX[C_13][ty][tx + 1] - Axf * s.WX[C_13][ty][tx];
                        FT cdy = Ayf * s.SY[C_23][ty + 1][tx] - Ayf * s.SY[C_23][ty][tx];
                        FT cdz = Az * t33_t - Az * c.t33;
                        G = G - rVf * (cdx + cdy + cdz);
                    }
                    P.Gw[idx] = G;
                    P.wo[idx] = rk3_update(Wk[pidx(tx, ty)], G, Gwm, P, dt);
                }
            }
            if (TR) {
                FT dx_ = s.WX[A_CX][ty][tx + 1] - s.WX[A_CX][ty][tx];
                FT dy_ = s.SY[A_CY][ty + 1][tx] - s.SY[A_CY][ty][tx];
                FT dz_ = fz ? FT(0) : (fWc_t - c.fWc);
                FT G = -(rVc * (dx_ + dy_ + dz_));
                if (closure) {
                    FT cdx = Ax * s.WX[Q_CX][ty][tx + 1] - Ax * s.WX[Q_CX][ty][tx];
                    FT cdy = Ay * s.SY[Q_CY][ty + 1][tx] - Ay * s.SY[Q_CY][ty][tx];
                    FT cdz = fz ? FT(0) : (Az * qzc_t - Az * c.qzc);
                    G = G - rVc * (cdx + cdy + cdz);
                }
                if (!fz) {
                    if (k == Nz - 1 && P.flux_top != FT(0)) G -= P.flux_top * Az / (Az * M.dzc(k));
                    if (k == 0 && P.flux_bot != FT(0)) G += P.flux_bot * Az / (Az * M.dzc(k));
                }
                P.Gc[idx] = G;
                P.co[idx] = rk3_update(CCk[pidx(tx, ty)], G, Gcm, P, dt);  // the stored value (departure)
            }
        }

        // ---- advance: carry top -> bottom, slide the windows ----
        c.fWu = fWu_t; c.fWv = fWv_t; c.fWw = fWw_t;
        c.t13 = t13_t; c.t23 = t23_t; c.t33 = t33_t;
        c.fWc = fWc_t; c.qzc = qzc_t;
#pragma unroll
        for (int o = 0; o < 6; ++o) { c.uc[o] = c.uc[o + 1]; c.vc[o] = c.vc[o + 1]; }
        c.uc[6] = un;
        c.vc[6] = vn;
#pragma unroll
        for (int o = 0; o < 5; ++o) c.wc[o] = c.wc[o + 1];
        c.wc[5] = wn;
        if (TR) {
#pragma unroll
            for (int o = 0; o < 6; ++o) c.cc[o] = c.cc[o + 1];
            c.cc[6] = cnext;
        }
        cp_async_wait_all();
        __syncthreads();
        r3 = s3p;
    }
}

// ---------------------------------------------------------------------------
// Smagorinsky-Lilly νₑ on a shared-memory tile: the block stages u, v, w, b on a
// (32+8) x (8+2) x (KT+2) box once (halo synthesis at load, 16-byte chunks where the
// grid allows; the stencils reach one point beyond the tile) and every thread
// evaluates the closure for KT levels of its column from shared memory.
// Arithmetic identical to k_smagorinsky (gbo_kernels.cuh), its three coefficients
// included: Lilly's, the level's c² of DynamicSmagorinsky averaged over x-y, and the
// cell's max(𝒥ᴸᴹ, minimum_numerator) / 𝒥ᴹᴹ of Lagrangian averaging (b is not staged then).
// ---------------------------------------------------------------------------
namespace smag {
// box: x from -4 (rows of 16-byte chunks that start on a multiple of four columns) to
// TX + 3, y and z from -1 to TY and KT
constexpr int TX = 32, TY = 8, KT = 4, BHX = 4;
constexpr int BX = TX + 2 * BHX, BY = TY + 2, BZ = KT + 2, BS = BX * BY * BZ;
constexpr int NT = TX * TY;
GBO_D int bidx(int x, int y, int z) { return ((z + 1) * BY + (y + 1)) * BX + (x + BHX); }
// squared edge strains of the tile: Σ₁₂² at (x ∈ 0..TX, y ∈ 0..TY, z < KT),
// Σ₁₃² at (x ∈ 0..TX, y < TY, z ∈ 0..KT), Σ₂₃² at (x < TX, y ∈ 0..TY, z ∈ 0..KT)
constexpr int E12 = (TX + 1) * (TY + 1) * KT, E13 = (TX + 1) * TY * (KT + 1), E23 = TX * (TY + 1) * (KT + 1);
GBO_D int i12(int x, int y, int z) { return (z * (TY + 1) + y) * (TX + 1) + x; }
GBO_D int i13(int x, int y, int z) { return (z * TY + y) * (TX + 1) + x; }
GBO_D int i23(int x, int y, int z) { return (z * (TY + 1) + y) * TX + x; }
template <typename FT>
struct __align__(16) Smem {
    FT u[BS], v[BS], w[BS], b[BS];
};

// Stage u, v, w and c (b when c is null: zeros) over the box of the block at (i0, j0, k0):
// periodic wrap in x and y; for centre fields one mirrored layer below and above the
// domain and zero beyond, for w zero at and beyond the walls (the CFld / WFld rules);
// cref (c stored as departures) is added to c.  With Nx a multiple of the chunk width
// and the fields 16-byte aligned, a box row is copied as 16-byte chunks (a chunk starts
// on a multiple of its width, so it never straddles the periodic seam); otherwise one
// value per copy.  Ends with the block's copies complete and visible (__syncthreads).
template <typename FT>
GBO_D void fill_box(Smem<FT>& s, const GridP<FT>& g, const FT* u, const FT* v, const FT* w, const FT* c,
                    const FT* cref, int i0, int j0, int k0, int tid) {
    constexpr int V = fused::VW<FT>, CR = BX / V;
    const int Nz = g.Nz, fz = g.flatz;
    const size_t plane = (size_t)g.Nx * g.Ny;
    const bool vec = g.Nx % V == 0 && ((((size_t)u | (size_t)v | (size_t)w | (size_t)c) & 15) == 0);
    const int n = vec ? CR * BY * BZ : BS, step = vec ? V : 1;
    for (int e = tid; e < n; e += NT) {
        const int cx = vec ? e % CR : e % BX, y = (vec ? e / CR : e / BX) % BY - 1, z = (vec ? e / (CR * BY) : e / (BX * BY)) - 1;
        const int x = vec ? cx * V - BHX : cx - BHX;
        const size_t col = wrapt(i0 + x, g.Nx) + (size_t)g.Nx * wrapt(j0 + y, g.Ny);
        const int zc = fused::zsrc_c(k0 + z, Nz, fz), zw = fz ? -1 : fused::zsrc_w(k0 + z, Nz);
        const size_t oc = col + (zc < 0 ? 0 : (size_t)zc * plane), ow = col + (zw < 0 ? 0 : (size_t)zw * plane);
        const int d = e * step;
        if (vec) {
            fused::cp_async16(&s.u[d], u + oc, zc < 0);
            fused::cp_async16(&s.v[d], v + oc, zc < 0);
            fused::cp_async16(&s.w[d], w + ow, zw < 0);
            if (c) fused::cp_async16(&s.b[d], c + oc, zc < 0);
            else
                for (int q = 0; q < V; ++q) s.b[d + q] = FT(0);
        } else {
            fused::cp_async(&s.u[d], u + oc, zc < 0);
            fused::cp_async(&s.v[d], v + oc, zc < 0);
            fused::cp_async(&s.w[d], w + ow, zw < 0);
            if (c) fused::cp_async(&s.b[d], c + oc, zc < 0);
            else s.b[d] = FT(0);
        }
    }
    fused::cp_async_commit();
    fused::cp_async_wait_all();
    if (c && cref) {
        // each thread adds the reference profile to the values it copied (its own copies
        // are complete after the wait); zero-filled layers stay zero
        for (int e = tid; e < n; e += NT) {
            const int z = (vec ? e / (CR * BY) : e / (BX * BY)) - 1;
            const int zc = fused::zsrc_c(k0 + z, Nz, fz);
            if (zc < 0) continue;
            const FT r = __ldg(cref + zc);
            for (int q = 0; q < step; ++q) s.b[e * step + q] += r;
        }
    }
    __syncthreads();
}
template <typename FT>
struct SmemS : Smem<FT> {
    FT s12[E12], s13[E13], s23[E23];
    FT df2[KT];  // Δᶠ² = (∛(Δx Δy Δz))² of the tile's levels, one cbrt per level
};
}  // namespace smag

template <typename FT>
__global__ void __launch_bounds__(256) k_smagorinsky_tiled(StepP<FT> P, FT* __restrict__ nu_out) {
    using namespace smag;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SmemS<FT>& s = *reinterpret_cast<SmemS<FT>*>(smem_raw);
    const GridP<FT>& g = P.g;
    Met<FT> M(g);
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
    const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY, k0 = blockIdx.z * KT;
    const bool buoy = P.buoyancy && !g.flatz && !P.jlm && !P.cs2;
    const int Nz = g.Nz, fz = g.flatz;
    // w is null on a flat grid: the zero-filled copies never read it
    fill_box<FT>(s, g, P.u, P.v, fz ? P.u : P.w, buoy ? P.b : nullptr, P.bref, i0, j0, k0, tid);
    auto U = [&](int x, int y, int zz) { return s.u[bidx(x, y, zz)]; };
    auto V = [&](int x, int y, int zz) { return s.v[bidx(x, y, zz)]; };
    auto W = [&](int x, int y, int zz) { return s.w[bidx(x, y, zz)]; };
    // strain components at the staggered points around the cells (velocity_tracer_gradients.jl),
    // each evaluated once for the tile
    for (int e = tid; e < E12; e += TX * TY) {
        const int x = e % (TX + 1), y = (e / (TX + 1)) % (TY + 1), z = e / ((TX + 1) * (TY + 1));
        FT dyu = (U(x, y, z) - U(x, y - 1, z)) * g.rdy;
        FT dxv = (V(x, y, z) - V(x - 1, y, z)) * g.rdx;
        FT v12 = FT(0.5) * (dyu + dxv);
        s.s12[e] = v12 * v12;
    }
    for (int e = tid; e < E13; e += TX * TY) {
        const int x = e % (TX + 1), y = (e / (TX + 1)) % TY, z = e / ((TX + 1) * TY);
        FT v13 = FT(0);
        if (!fz) {
            FT dzu = (U(x, y, z) - U(x, y, z - 1)) * M.rdzf(k0 + z);
            FT dxw = (W(x, y, z) - W(x - 1, y, z)) * g.rdx;
            v13 = FT(0.5) * (dzu + dxw);
        }
        s.s13[e] = v13 * v13;
    }
    for (int e = tid; e < E23; e += TX * TY) {
        const int x = e % TX, y = (e / TX) % (TY + 1), z = e / (TX * (TY + 1));
        FT v23 = FT(0);
        if (!fz) {
            FT dzv = (V(x, y, z) - V(x, y, z - 1)) * M.rdzf(k0 + z);
            FT dyw = (W(x, y, z) - W(x, y - 1, z)) * g.rdy;
            v23 = FT(0.5) * (dzv + dyw);
        }
        s.s23[e] = v23 * v23;
    }
    if (tid < KT) {
        const FT Df = cbrt(g.dx * g.dy * M.dzc(k0 + tid));
        s.df2[tid] = Df * Df;
    }
    __syncthreads();
    const int i = i0 + tx, j = j0 + ty;
    if (i >= g.Nx || j >= g.Ny) return;
    for (int z = 0; z < KT; ++z) {
        const int k = k0 + z;
        if (k >= Nz) break;
        FT s11 = (U(tx + 1, ty, z) - U(tx, ty, z)) * g.rdx;
        FT s22 = (V(tx, ty + 1, z) - V(tx, ty, z)) * g.rdy;
        FT s33 = fz ? FT(0) : (W(tx, ty, z + 1) - W(tx, ty, z)) * M.rdzc(k);
        FT tr = s11 * s11 + s22 * s22 + s33 * s33;
        FT ixy = FT(0.5) * (FT(0.5) * (s.s12[i12(tx, ty, z)] + s.s12[i12(tx + 1, ty, z)]) +
                            FT(0.5) * (s.s12[i12(tx, ty + 1, z)] + s.s12[i12(tx + 1, ty + 1, z)]));
        FT ixz, iyz;
        if (fz) {
            ixz = FT(0);
            iyz = FT(0);
        } else {
            ixz = FT(0.5) * (FT(0.5) * (s.s13[i13(tx, ty, z)] + s.s13[i13(tx + 1, ty, z)]) +
                             FT(0.5) * (s.s13[i13(tx, ty, z + 1)] + s.s13[i13(tx + 1, ty, z + 1)]));
            iyz = FT(0.5) * (FT(0.5) * (s.s23[i23(tx, ty, z)] + s.s23[i23(tx, ty + 1, z)]) +
                             FT(0.5) * (s.s23[i23(tx, ty, z + 1)] + s.s23[i23(tx, ty + 1, z + 1)]));
        }
        FT Sig2 = tr + FT(2) * ixy + FT(2) * ixz + FT(2) * iyz;
        const size_t q = i + (size_t)g.Nx * (j + (size_t)g.Ny * k);
        FT cs2;
        if (P.jlm) {
            FT lm = P.jlm[q];
            lm = isnan(lm) ? lm : (lm > P.lm_min ? lm : P.lm_min);
            const FT mm = P.jmm[q];
            cs2 = mm > FT(0) ? lm / mm : FT(0);
        } else if (P.cs2) {
            cs2 = P.cs2[k];
        } else {
            FT N2 = FT(0);
            if (buoy) {
                FT b1 = (s.b[bidx(tx, ty, z)] - s.b[bidx(tx, ty, z - 1)]) * M.rdzf(k);
                FT b2 = (s.b[bidx(tx, ty, z + 1)] - s.b[bidx(tx, ty, z)]) * M.rdzf(k + 1);
                N2 = FT(0.5) * (b1 + b2);
            }
            FT N2p = fmax(FT(0), N2);
            FT r = P.Cb * N2p / Sig2;
            FT mn = isnan(r) ? r : fmin(FT(1), r);
            FT vs2 = FT(1) - mn;
            FT vs = (Sig2 == FT(0)) ? FT(0) : sqrt(vs2);
            cs2 = vs * (P.C * P.C);
        }
        nu_out[q] = cs2 * s.df2[z] * sqrt(FT(2) * Sig2);
    }
}

// ---------------------------------------------------------------------------
// Anisotropic minimum dissipation νₑ (and κₑ of one tracer) on the same shared-
// memory tile as k_smagorinsky_tiled: u, v, w and the tracer are staged once on a
// (32+2) x (8+2) x (KT+2) box (halo synthesis at load) and amd_point (the
// arithmetic of k_amd) reads them through tile accessors with global indices.
// ---------------------------------------------------------------------------
namespace smag {
template <typename FT>
struct TileFld {  // global (i, j, k) -> tile cell of the block at (i0, j0, k0)
    const FT* a;
    int i0, j0, k0;
    GBO_D FT operator()(int i, int j, int k) const { return a[bidx(i - i0, j - j0, k - k0)]; }
};
template <typename FT>
struct TileFields {
    TileFld<FT> u, v, nu, phy, w;
};
}  // namespace smag

// AMD on an immersed grid: the tile in shared memory, every cell evaluated by amd_point
// through the strain code with the immersed grid's conditional derivatives
// (conditional_differences.jl:15-43)
template <typename FT>
__global__ void __launch_bounds__(256) k_amd_tiled_ibg(StepP<FT> P, FT* __restrict__ nu_out, FT* __restrict__ kap_out) {
    using namespace smag;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Smem<FT>& s = *reinterpret_cast<Smem<FT>*>(smem_raw);
    const GridP<FT>& g = P.g;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
    const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY, k0 = blockIdx.z * KT;
    const bool has_c = P.c != nullptr;
    fill_box<FT>(s, g, P.u, P.v, g.flatz ? P.u : P.w, has_c ? P.c : nullptr, P.cref, i0, j0, k0, tid);
    const int i = i0 + tx, j = j0 + ty;
    if (i >= g.Nx || j >= g.Ny) return;
    const TileFld<FT> tu{s.u, i0, j0, k0}, tv{s.v, i0, j0, k0}, tw{s.w, i0, j0, k0}, tc{s.b, i0, j0, k0};
    const TileFields<FT> F{tu, tv, tu, tu, tw};
    const StrainT<FT, TileFields<FT>> S(g, F);
    for (int z = 0; z < KT; ++z) {
        const int k = k0 + z;
        if (k >= g.Nz) break;
        amd_point<FT>(P, g, S, tc, has_c, i, j, k, i + (size_t)g.Nx * (j + (size_t)g.Ny * k), nu_out, kap_out);
    }
}

namespace smag {
// AMD: the tile plus the six normalised off-diagonal velocity gradients at their edges
// (x·y edges at every level, x·z and y·z edges at every face of the tile).  ∂y w is kept
// one column wider: the tracer term interpolates it over x and z (ℑxzᶜᵃᶜ, as the
// reference does, anisotropic_minimum_dissipation.jl:344)
constexpr int E23X = (TX + 1) * (TY + 1) * (KT + 1);
GBO_D int i23x(int x, int y, int z) { return (z * (TY + 1) + y) * (TX + 1) + x; }
template <typename FT>
struct SmemA : Smem<FT> {
    FT dxv[E12], dyu[E12], dxw[E13], dzu[E13], dyw[E23X], dzv[E23];
    FT d2[KT];  // δ² = 3 / (Δ̃x⁻² + Δ̃y⁻² + Δ̃z⁻²) of the tile's levels
};
}  // namespace smag

// Anisotropic minimum dissipation νₑ (and κₑ of one tracer) on a 32×8×4 tile
// (anisotropic_minimum_dissipation.jl:161-204,243-358; velocity_tracer_gradients.jl:
// 120-250).  The normalised gradients Δ̃ᵢ/Δ̃ⱼ ∂ⱼuᵢ of the cross terms live on edges and
// each cell interpolates products of them from four edges; every edge value is shared by
// four cells, so the block evaluates each once into shared memory (the filter-width
// ratios once per level), then every cell combines its 24 edge values with the same
// arithmetic, in the same order, as the per-point amd_point.  Rectilinear grids only (an
// immersed grid takes k_amd_tiled_ibg).
template <typename FT>
__global__ void __launch_bounds__(256) k_amd_tiled(StepP<FT> P, FT* __restrict__ nu_out, FT* __restrict__ kap_out) {
    using namespace smag;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SmemA<FT>& s = *reinterpret_cast<SmemA<FT>*>(smem_raw);
    const GridP<FT>& g = P.g;
    Met<FT> M(g);
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
    const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY, k0 = blockIdx.z * KT;
    const bool has_c = P.c != nullptr;
    const int fz = g.flatz;
    fill_box<FT>(s, g, P.u, P.v, fz ? P.u : P.w, has_c ? P.c : nullptr, P.cref, i0, j0, k0, tid);
    auto U = [&](int x, int y, int z) { return s.u[bidx(x, y, z)]; };
    auto V = [&](int x, int y, int z) { return s.v[bidx(x, y, z)]; };
    auto W = [&](int x, int y, int z) { return s.w[bidx(x, y, z)]; };
    auto C = [&](int x, int y, int z) { return s.b[bidx(x, y, z)]; };
    // filter widths 2Δ (the reference's Δᶠ at the evaluation index) and their ratios
    const FT Dx = FT(2) * g.dx, Dy = FT(2) * g.dy;
    const FT rxy = Dx / Dy, ryx = Dy / Dx;
    for (int e = tid; e < E12; e += TX * TY) {
        const int x = e % (TX + 1), y = (e / (TX + 1)) % (TY + 1), z = e / ((TX + 1) * (TY + 1));
        s.dyu[e] = ryx * ((U(x, y, z) - U(x, y - 1, z)) * g.rdy);
        s.dxv[e] = rxy * ((V(x, y, z) - V(x - 1, y, z)) * g.rdx);
    }
    for (int e = tid; e < E13; e += TX * TY) {
        const int x = e % (TX + 1), y = (e / (TX + 1)) % TY, z = e / ((TX + 1) * TY), k = k0 + z;
        const FT Dz = FT(2) * M.dzc(k);
        s.dxw[e] = (Dx / Dz) * (fz ? FT(0) : (W(x, y, z) - W(x - 1, y, z)) * g.rdx);
        s.dzu[e] = (Dz / Dx) * (fz ? FT(0) : (U(x, y, z) - U(x, y, z - 1)) * M.rdzf(k));
    }
    for (int e = tid; e < E23; e += TX * TY) {
        const int x = e % TX, y = (e / TX) % (TY + 1), z = e / (TX * (TY + 1)), k = k0 + z;
        const FT Dz = FT(2) * M.dzc(k);
        s.dzv[e] = (Dz / Dy) * (fz ? FT(0) : (V(x, y, z) - V(x, y, z - 1)) * M.rdzf(k));
    }
    for (int e = tid; e < E23X; e += TX * TY) {
        const int x = e % (TX + 1), y = (e / (TX + 1)) % (TY + 1), z = e / ((TX + 1) * (TY + 1)), k = k0 + z;
        const FT Dz = FT(2) * M.dzc(k);
        s.dyw[e] = (Dy / Dz) * (fz ? FT(0) : (W(x, y, z) - W(x, y - 1, z)) * g.rdy);
    }
    auto sq = [](FT a) { return a * a; };
    if (tid < KT) {
        const FT Dz = FT(2) * M.dzc(k0 + tid);
        s.d2[tid] = FT(3) / (FT(1) / sq(Dx) + FT(1) / sq(Dy) + FT(1) / sq(Dz));
    }
    __syncthreads();
    const int i = i0 + tx, j = j0 + ty;
    if (i >= g.Nx || j >= g.Ny) return;
    // ℑ over the four edges around the cell, in the reference's order (a₀₀ + a₁₀, a₀₁ + a₁₁)
    auto I4 = [](FT a, FT b, FT c, FT d) { return FT(0.5) * (FT(0.5) * (a + b) + FT(0.5) * (c + d)); };
    for (int z = 0; z < KT; ++z) {
        const int k = k0 + z;
        if (k >= g.Nz) break;
        const FT Dz = FT(2) * M.dzc(k);
        const FT S11 = (U(tx + 1, ty, z) - U(tx, ty, z)) * g.rdx;
        const FT S22 = (V(tx, ty + 1, z) - V(tx, ty, z)) * g.rdy;
        const FT S33 = fz ? FT(0) : (W(tx, ty, z + 1) - W(tx, ty, z)) * M.rdzc(k);
        // edge values: x·y edges (i, j), (i+1, j), (i, j+1), (i+1, j+1) at level k; x·z edges
        // (i, k), (i+1, k), (i, k+1), (i+1, k+1); y·z edges (j, k), (j+1, k), (j, k+1), (j+1, k+1)
        const int a0 = i12(tx, ty, z), a1 = i12(tx + 1, ty, z), a2 = i12(tx, ty + 1, z), a3 = i12(tx + 1, ty + 1, z);
        const int b0 = i13(tx, ty, z), b1 = i13(tx + 1, ty, z), b2 = i13(tx, ty, z + 1), b3 = i13(tx + 1, ty, z + 1);
        const int c0 = i23(tx, ty, z), c1 = i23(tx, ty + 1, z), c2 = i23(tx, ty, z + 1), c3 = i23(tx, ty + 1, z + 1);
        const FT xv[4] = {s.dxv[a0], s.dxv[a1], s.dxv[a2], s.dxv[a3]};
        const FT yu[4] = {s.dyu[a0], s.dyu[a1], s.dyu[a2], s.dyu[a3]};
        const FT xw[4] = {s.dxw[b0], s.dxw[b1], s.dxw[b2], s.dxw[b3]};
        const FT zu[4] = {s.dzu[b0], s.dzu[b1], s.dzu[b2], s.dzu[b3]};
        const FT yw[4] = {s.dyw[i23x(tx, ty, z)], s.dyw[i23x(tx, ty + 1, z)], s.dyw[i23x(tx, ty, z + 1)],
                          s.dyw[i23x(tx, ty + 1, z + 1)]};
        const FT zv[4] = {s.dzv[c0], s.dzv[c1], s.dzv[c2], s.dzv[c3]};
        FT s12[4], s13[4], s23[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            s12[q] = FT(0.5) * (yu[q] + xv[q]);
            s13[q] = FT(0.5) * (zu[q] + xw[q]);
            s23[q] = FT(0.5) * (zv[q] + yw[q]);
        }
        auto IP = [&](const FT* a, const FT* b) { return I4(a[0] * b[0], a[1] * b[1], a[2] * b[2], a[3] * b[3]); };
        auto I = [&](const FT* a) { return I4(a[0], a[1], a[2], a[3]); };
        const FT xv2 = IP(xv, xv), yu2 = IP(yu, yu), xw2 = IP(xw, xw), zu2 = IP(zu, zu), yw2 = IP(yw, yw), zv2 = IP(zv, zv);
        const FT q = sq(S11) + sq(S22) + sq(S33) + xv2 + yu2 + xw2 + zu2 + yw2 + zv2;
        const FT d2 = s.d2[z];
        FT nsgs = FT(0);
        if (q != FT(0)) {
            const FT r1 = S11 * sq(S11) + S22 * xv2 + S33 * xw2 + FT(2) * S11 * IP(xv, s12) + FT(2) * S11 * IP(xw, s13) +
                          FT(2) * I(xv) * I(xw) * I(s23);
            const FT r2 = S11 * yu2 + S22 * sq(S22) + S33 * yw2 + FT(2) * S22 * IP(yu, s12) + FT(2) * I(yu) * I(yw) * I(s13) +
                          FT(2) * S22 * IP(yw, s23);
            const FT r3 = S11 * zu2 + S22 * zv2 + S33 * sq(S33) + FT(2) * I(zu) * I(zv) * I(s12) + FT(2) * S33 * IP(zu, s13) +
                          FT(2) * S33 * IP(zv, s23);
            const FT r = r1 + r2 + r3;
            nsgs = -P.C * d2 * (r - FT(0)) / q;
        }
        const size_t idx = i + (size_t)g.Nx * (j + (size_t)g.Ny * k);
        nu_out[idx] = fmax(FT(0), nsgs);
        if (kap_out && has_c) {
            // tracer gradients at the six faces, Δ̃-weighted
            const FT Dz1 = FT(2) * M.dzc(k + 1);
            const FT cx0 = Dx * ((C(tx, ty, z) - C(tx - 1, ty, z)) * g.rdx);
            const FT cx1 = Dx * ((C(tx + 1, ty, z) - C(tx, ty, z)) * g.rdx);
            const FT cy0 = Dy * ((C(tx, ty, z) - C(tx, ty - 1, z)) * g.rdy);
            const FT cy1 = Dy * ((C(tx, ty + 1, z) - C(tx, ty, z)) * g.rdy);
            const FT cz0 = Dz * ((C(tx, ty, z) - C(tx, ty, z - 1)) * M.rdzf(k));
            const FT cz1 = Dz1 * ((C(tx, ty, z + 1) - C(tx, ty, z)) * M.rdzf(k + 1));
            const FT dxc2 = FT(0.5) * (sq(cx0) + sq(cx1)), dyc2 = FT(0.5) * (sq(cy0) + sq(cy1));
            const FT dzc2 = FT(0.5) * (sq(cz0) + sq(cz1));
            const FT sigma = dxc2 + dyc2 + dzc2;
            FT ksgs = FT(0);
            if (sigma != FT(0)) {
                const FT ix = FT(0.5) * (cx0 + cx1), iy = FT(0.5) * (cy0 + cy1), iz = FT(0.5) * (cz0 + cz1);
                const FT cx_ux = S11 * dxc2 + I(xv) * ix * iy + I(xw) * ix * iz;
                // ∂y w interpolated over x and z, as the reference does (see SmemA)
                const FT ywx = I4(s.dyw[i23x(tx, ty, z)], s.dyw[i23x(tx + 1, ty, z)], s.dyw[i23x(tx, ty, z + 1)],
                                  s.dyw[i23x(tx + 1, ty, z + 1)]);
                const FT cy_uy = I(yu) * iy * ix + S22 * dyc2 + ywx * iy * iz;
                const FT cz_uz = I(zu) * iz * ix + I(zv) * iz * iy + S33 * dzc2;
                const FT theta = cx_ux + cy_uy + cz_uz;
                ksgs = -P.C * d2 * theta / sigma;
            }
            kap_out[idx] = fmax(FT(0), ksgs);
        }
    }
}
