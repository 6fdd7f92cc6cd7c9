// gbo_fft.cuh -- shared-memory batched FFT engine and the Poisson pass kernels.
//
// The reference solves ∇²ϕ = b by eigenfunction expansion
// (src/Solvers/fft_based_poisson_solver.jl:94-124): DCT-II in Bounded
// directions (REDFT10 on the CPU, a permuted complex FFT + twiddles on the GPU,
// discrete_transforms.jl:108-182, index_permutations.jl:18-90), FFTs in Periodic
// ones, ϕ̂ = -b̂/(λx+λy+λz) with the zero mode set to zero, then the inverse
// transforms.  That is a C2C transform over a complex copy of the whole field
// with ~8 separate permute / twiddle / copy launches.  Here the field stays real
// until the x pass, which produces the Hermitian half spectrum directly:
//   Z pass   real -> real   DCT-II along z (Makhoul reordering, two columns per complex line)
//   X pass   real -> complex  R2C along x (half-length complex FFT + split)
//   Y pass   complex in place: FFT along y, divide by the eigenvalues, inverse FFT
//   X⁻¹, Z⁻¹ the inverses.
// All 1-D transforms run in shared memory (Stockham autosort, radix 4/2/3/5),
// one block per batch of lines with coalesced loads along the contiguous axis.
// Forward transforms are unnormalised; the whole normalisation is applied once
// in the Y pass (or in the Thomas kernel for the Fourier-tridiagonal solver).
#pragma once
#include "gbo_common.cuh"

#define GBO_MAX_RADICES 16

struct FFTPlan1D {
    int n;
    int nrad;
    int rad[GBO_MAX_RADICES];
};

// y = DFT over each of L lines of length n held in A (scratch B); returns the buffer
// holding the result.  sign = -1 forward, +1 inverse (unnormalised).
// tw[m] = exp(-2πi m / n), m = 0..n-1.
template <typename FT>
__device__ Cx<FT>* block_fft(Cx<FT>* A, Cx<FT>* B, int L, const FFTPlan1D& pl, int sign, const Cx<FT>* __restrict__ tw,
                             bool il = false) {
    const int n = pl.n;
    int Ns = 1;
    for (int s = 0; s < pl.nrad; ++s) {
        const int R = pl.rad[s];
        const int nR = n / R;
        const int twstep = n / (Ns * R);
        // element (line, m) lives at line*n + m, or at m*L + line when interleaved
        const int es = il ? L : 1;
        for (int t = threadIdx.x; t < L * nR; t += blockDim.x) {
            const int line = il ? t % L : t / nR;
            const int jj = il ? t / L : t - line * nR;
            const int kk = jj % Ns;
            const Cx<FT>* x = A + (il ? line : line * n);
            Cx<FT>* y = B + (il ? line : line * n);
            Cx<FT> v[5];
            for (int r = 0; r < R; ++r) {
                Cx<FT> a = x[(jj + r * nR) * es];
                if (r > 0 && kk > 0) {
                    Cx<FT> wv = tw[(kk * r * twstep) % n];
                    if (sign > 0) wv.im = -wv.im;
                    a = a * wv;
                }
                v[r] = a;
            }
            Cx<FT> V[5];
            if (R == 2) {
                V[0] = v[0] + v[1];
                V[1] = v[0] - v[1];
            } else if (R == 4) {
                Cx<FT> s02 = v[0] + v[2], d02 = v[0] - v[2], s13 = v[1] + v[3], d13 = v[1] - v[3];
                // multiply d13 by -i (forward) or +i (inverse)
                Cx<FT> jd13 = sign < 0 ? cx(d13.im, -d13.re) : cx(-d13.im, d13.re);
                V[0] = s02 + s13;
                V[1] = d02 + jd13;
                V[2] = s02 - s13;
                V[3] = d02 - jd13;
            } else {
                // generic small DFT with roots of unity taken from the table
                for (int q = 0; q < R; ++q) {
                    Cx<FT> acc = v[0];
                    for (int r = 1; r < R; ++r) {
                        Cx<FT> wv = tw[((q * r) % R) * nR];
                        if (sign > 0) wv.im = -wv.im;
                        acc = acc + v[r] * wv;
                    }
                    V[q] = acc;
                }
            }
            const int idxD = (jj / Ns) * Ns * R + kk;
            for (int q = 0; q < R; ++q) y[(idxD + q * Ns) * es] = V[q];
        }
        __syncthreads();
        Cx<FT>* tmp = A;
        A = B;
        B = tmp;
        Ns *= R;
    }
    return A;
}


// Compile-time-length variant of block_fft: the radix sequence, spans and
// twiddle strides are constants, so the index arithmetic reduces to shifts,
// multiplies and masks and the stage loop unrolls.
struct CPlan {
    int nrad;
    int rad[GBO_MAX_RADICES];
};
// maxr: the largest radix a stage may use (each pass kernel picks it: the register
// butterflies of radix 8 and 16 pay off on some lengths and cost on others, measured)
__host__ __device__ constexpr CPlan cplan(int n, int maxr = 4) {
    CPlan p{0, {}};
    int m = n;
    if (maxr >= 16)
        while (m % 16 == 0) { p.rad[p.nrad++] = 16; m /= 16; }
    if (maxr >= 8)
        while (m % 8 == 0) { p.rad[p.nrad++] = 8; m /= 8; }
    while (m % 4 == 0) { p.rad[p.nrad++] = 4; m /= 4; }
    while (m % 2 == 0) { p.rad[p.nrad++] = 2; m /= 2; }
    while (m % 3 == 0) { p.rad[p.nrad++] = 3; m /= 3; }
    while (m % 5 == 0) { p.rad[p.nrad++] = 5; m /= 5; }
    return p;
}

// Small DFTs held in registers, built from radix-4 and radix-2 layers (the Cooley-Tukey
// factorisation; internal twiddles are the constants of the eighth and sixteenth roots of
// unity).  sign = -1 forward, +1 inverse.
template <typename FT>
GBO_D void dft4r(Cx<FT>& a0, Cx<FT>& a1, Cx<FT>& a2, Cx<FT>& a3, int sign) {
    const Cx<FT> s02 = a0 + a2, d02 = a0 - a2, s13 = a1 + a3, d13 = a1 - a3;
    const Cx<FT> jd13 = sign < 0 ? cx(d13.im, -d13.re) : cx(-d13.im, d13.re);  // ∓i (a1 - a3)
    a0 = s02 + s13;
    a1 = d02 + jd13;
    a2 = s02 - s13;
    a3 = d02 - jd13;
}
// x · exp(sign 2πi m / 16) for the m that occur in the 16- and 8-point transforms
template <typename FT>
GBO_D Cx<FT> rot16(Cx<FT> x, int m, int sign) {
    const FT c1 = FT(0.92387953251128675613), s1 = FT(0.38268343236508977173), h = FT(0.70710678118654752440);
    Cx<FT> w;
    switch (m) {
        case 0: return x;
        case 1: w = cx(c1, s1); break;
        case 2: w = cx(h, h); break;
        case 3: w = cx(s1, c1); break;
        case 4: w = cx(FT(0), FT(1)); break;
        case 6: w = cx(-h, h); break;
        case 9: w = cx(-c1, -s1); break;
        default: w = cx(FT(1), FT(0));
    }
    if (sign < 0) w.im = -w.im;
    return x * w;
}
// X[q] = Σ_r v[r] exp(sign 2πi q r / 8)
template <typename FT>
GBO_D void dft8r(Cx<FT> (&v)[8], int sign) {
    Cx<FT> e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6], o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
    dft4r(e0, e1, e2, e3, sign);
    dft4r(o0, o1, o2, o3, sign);
    o1 = rot16(o1, 2, sign);  // ω₈ = ω₁₆²
    o2 = rot16(o2, 4, sign);
    o3 = rot16(o3, 6, sign);
    v[0] = e0 + o0; v[4] = e0 - o0;
    v[1] = e1 + o1; v[5] = e1 - o1;
    v[2] = e2 + o2; v[6] = e2 - o2;
    v[3] = e3 + o3; v[7] = e3 - o3;
}
// X[q] = Σ_r v[r] exp(sign 2πi q r / 16): four 4-point transforms over r = 4 n₁ + n₂,
// the twiddles ω₁₆^(n₂ q₁), four 4-point transforms over n₂
template <typename FT>
GBO_D void dft16r(Cx<FT> (&v)[16], int sign) {
#pragma unroll
    for (int n2 = 0; n2 < 4; ++n2) dft4r(v[n2], v[4 + n2], v[8 + n2], v[12 + n2], sign);
    // v[4 q1 + n2] now holds A[n2][q1]
#pragma unroll
    for (int n2 = 1; n2 < 4; ++n2)
#pragma unroll
        for (int q1 = 1; q1 < 4; ++q1) v[4 * q1 + n2] = rot16(v[4 * q1 + n2], n2 * q1, sign);
    Cx<FT> X[16];
#pragma unroll
    for (int q1 = 0; q1 < 4; ++q1) {
        Cx<FT> a0 = v[4 * q1], a1 = v[4 * q1 + 1], a2 = v[4 * q1 + 2], a3 = v[4 * q1 + 3];
        dft4r(a0, a1, a2, a3, sign);
        X[q1] = a0; X[q1 + 4] = a1; X[q1 + 8] = a2; X[q1 + 12] = a3;
    }
#pragma unroll
    for (int q = 0; q < 16; ++q) v[q] = X[q];
}

template <typename FT, int N, int R, int NS, bool IL>
__device__ __forceinline__ void fft_stage(const Cx<FT>* __restrict__ A, Cx<FT>* __restrict__ B, int L, int lg, int sign,
                                          const Cx<FT>* __restrict__ tw) {
    constexpr int NR = N / R;
    constexpr int TWS = N / (NS * R);
    const int es = IL ? L : 1;
    for (int t = threadIdx.x; t < L * NR; t += blockDim.x) {
        // interleaved: L is a power of two (lg = log2 L), so the split is a mask and a shift
        const int line = IL ? (t & (L - 1)) : t / NR;
        const int jj = IL ? (t >> lg) : t - line * NR;
        const int kk = jj % NS;
        const Cx<FT>* x = A + (IL ? line : line * N);
        Cx<FT>* y = B + (IL ? line : line * N);
        Cx<FT> v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            Cx<FT> a = x[(jj + r * NR) * es];
            if (r > 0) {
                Cx<FT> wv = tw[kk * r * TWS];
                if (sign > 0) wv.im = -wv.im;
                a = a * wv;
            }
            v[r] = a;
        }
        Cx<FT> V[R];
        if constexpr (R == 16) {
            dft16r<FT>(v, sign);
#pragma unroll
            for (int q = 0; q < R; ++q) V[q] = v[q];
        } else if constexpr (R == 8) {
            dft8r<FT>(v, sign);
#pragma unroll
            for (int q = 0; q < R; ++q) V[q] = v[q];
        } else if (R == 2) {
            V[0] = v[0] + v[1];
            V[1] = v[0] - v[1];
        } else if (R == 4) {
            Cx<FT> s02 = v[0] + v[2], d02 = v[0] - v[2], s13 = v[1] + v[3], d13 = v[1] - v[3];
            Cx<FT> jd13 = sign < 0 ? cx(d13.im, -d13.re) : cx(-d13.im, d13.re);
            V[0] = s02 + s13;
            V[1] = d02 + jd13;
            V[2] = s02 - s13;
            V[3] = d02 - jd13;
        } else {
#pragma unroll
            for (int q = 0; q < R; ++q) {
                Cx<FT> acc = v[0];
#pragma unroll
                for (int r = 1; r < R; ++r) {
                    Cx<FT> wv = tw[((q * r) % R) * NR];
                    if (sign > 0) wv.im = -wv.im;
                    acc = acc + v[r] * wv;
                }
                V[q] = acc;
            }
        }
        const int idxD = (jj / NS) * NS * R + kk;
#pragma unroll
        for (int q = 0; q < R; ++q) y[(idxD + q * NS) * es] = V[q];
    }
    __syncthreads();
}

template <typename FT, int N, int S, int NS, bool IL, int MAXR>
struct FFTStages {
    static __device__ __forceinline__ Cx<FT>* run(Cx<FT>* A, Cx<FT>* B, int L, int lg, int sign, const Cx<FT>* tw) {
        constexpr CPlan p = cplan(N, MAXR);
        if constexpr (S >= p.nrad) {
            return A;
        } else {
            constexpr int R = p.rad[S];
            fft_stage<FT, N, R, NS, IL>(A, B, L, lg, sign, tw);
            return FFTStages<FT, N, S + 1, NS * R, IL, MAXR>::run(B, A, L, lg, sign, tw);
        }
    }
};

template <typename FT, int N, bool IL, int MAXR>
__device__ __forceinline__ Cx<FT>* block_fft_n(Cx<FT>* A, Cx<FT>* B, int L, int sign, const Cx<FT>* tw) {
    return FFTStages<FT, N, 0, 1, IL, MAXR>::run(A, B, L, __ffs(L) - 1, sign, tw);
}

// Dispatch helper: a kernel template parameter NC (0 = runtime length) selects
// the compile-time engine when the length matches.  IL: interleaved line layout
// (element (line, m) at m*L + line), used where a block's lines are columns of a
// strided axis so that loads, scatters and butterflies are bank-conflict free; L is
// then a power of two.  tw is the block's shared-memory copy of the twiddles.
template <typename FT, int NC, bool IL, int MAXR = 4>
__device__ __forceinline__ Cx<FT>* fft_any(Cx<FT>* A, Cx<FT>* B, int L, const FFTPlan1D& pl, int sign, const Cx<FT>* tw) {
    if constexpr (NC > 0) return block_fft_n<FT, NC, IL, MAXR>(A, B, L, sign, tw);
    else return block_fft<FT>(A, B, L, pl, sign, tw, IL);
}

// Makhoul reordering: the element x(k) of a length-N real sequence goes to v[dest(k)]
// (index_permutations.jl:18-20 restated: even samples first, odd samples reversed).
GBO_D int makhoul_dest(int k, int N) { return (k & 1) ? N - 1 - (k >> 1) : (k >> 1); }

// Asynchronous global -> shared copy of 4, 8 or 16 bytes (zero-filled when zero is
// set; src must still be a valid address).  The pass kernels issue their whole tile
// this way and wait once, instead of one dependent load per element.
template <int BYTES>
GBO_D void cp_async_n(void* dst, const void* src, bool zero) {
    static_assert(BYTES == 4 || BYTES == 8 || BYTES == 16, "cp.async copies 4, 8 or 16 bytes");
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;\n" ::"r"(d), "l"(src), "n"(BYTES), "r"(zero ? 0 : BYTES));
}
GBO_D void cp_async_wait() {
    asm volatile("cp.async.commit_group;\n" ::);
    asm volatile("cp.async.wait_group 0;\n" ::);
}

struct PoissonTables;  // host side

// Tile shapes of the pass kernels: columns per DCT block and the shared-memory budget
// per block within which the tiles are chosen (both solvers choose them the same way).
#ifndef GBO_DCT_TILE
#define GBO_DCT_TILE 32
#endif
#ifndef GBO_PASS_SMEM_LIMIT
#define GBO_PASS_SMEM_LIMIT (100 * 1024)
#endif

// Shared memory of the pass kernels: the two work buffers of the block's lines, then the
// twiddles of its transforms staged once per block (the butterflies read them from
// shared memory instead of global memory)
template <typename FT>
inline size_t dct_smem(int ZT, int Nz) { return ((size_t)ZT * Nz + 2 * (size_t)Nz) * sizeof(Cx<FT>); }
template <typename FT>
inline size_t rfft_smem(int XL, int Nx) { return ((size_t)XL * (Nx + 1) + (size_t)Nx) * sizeof(Cx<FT>); }
template <typename FT>
inline size_t ffty_smem(int YT, int Ny) { return (2 * (size_t)YT * Ny + (size_t)Ny) * sizeof(Cx<FT>); }
// the launch shapes the kernels accept: interleaved line counts are powers of two
GBO_HD constexpr bool pow2(int v) { return v > 0 && (v & (v - 1)) == 0; }

// stage n complex values (twiddles) asynchronously; waited for with the tile
template <typename FT>
GBO_D void stage_table(Cx<FT>* dst, const Cx<FT>* __restrict__ src, int n) {
    for (int t = threadIdx.x; t < n; t += blockDim.x) cp_async_n<sizeof(Cx<FT>)>(&dst[t], src + t, false);
}

template <typename FT>
struct PassP {
    int Nx, Ny, Nz, Nh;        // Nh = Nx/2 + 1
    FT* rb;                    // real buffer Nx*Ny*Nz
    Cx<FT>* cb;                // complex buffer Nh*Ny*Nz
    FFTPlan1D px_half, py, pz; // plans for lengths Nx/2, Ny, Nz
    const Cx<FT>* tw_xh;       // n = Nx/2
    const Cx<FT>* tw_x;        // n = Nx (real-FFT split twiddles)
    const Cx<FT>* tw_y;        // n = Ny
    const Cx<FT>* tw_z;        // n = Nz
    const Cx<FT>* tq_z;        // exp(-iπk/(2Nz)), k = 0..Nz-1
    const FT* lx;              // eigenvalues λx (Nh entries used)
    const FT* ly;
    const FT* lz;
    FT scale;                  // 1/(Nx Ny Nz) or 1/(Nx Ny)
    int has_z;                 // Bounded z with a DCT pass
};

// ---------------------------------------------------------------------------
// Z pass: DCT-II (forward) / its inverse along z, in place on the real buffer.
// Block: ZT consecutive x columns at one y, all Nz levels.
// ---------------------------------------------------------------------------
template <typename FT, int NC>
__global__ void k_dct_z(PassP<FT> P, int inverse, int ZT) {
    extern __shared__ __align__(16) unsigned char fft_smem[];
    const int N = P.Nz;
    const int L = ZT / 2;  // a power of two
    const int lz = __ffs(ZT) - 1, ll = lz - 1;
    Cx<FT>* A = reinterpret_cast<Cx<FT>*>(fft_smem);
    Cx<FT>* B = A + L * N;
    Cx<FT>* T = B + L * N;  // twiddles of the length-N FFT
    Cx<FT>* Q = T + N;      // ω^k = exp(-iπk/(2N)) of the DCT post-processing
    const int j = blockIdx.y;
    const int i0 = blockIdx.x * ZT;
    const size_t plane = (size_t)P.Nx * P.Ny;
    FT* col0 = P.rb + i0 + (size_t)P.Nx * j;
    stage_table(T, P.tw_z, N);
    stage_table(Q, P.tq_z, N);
    // 16-byte vectors of VW columns where the rows allow them: VW consecutive reals of one
    // level are VW / 2 consecutive complex slots of the block's layout
    constexpr int VW = 16 / sizeof(FT);
    const bool vec = P.Nx % VW == 0 && ZT % VW == 0 && (reinterpret_cast<uintptr_t>(P.rb) & 15) == 0;
    const int lv = lz - (VW == 4 ? 2 : 1);  // log2(ZT / VW)
    if (!inverse) {
        if (vec) {
            for (int t = threadIdx.x; t < ZT * N / VW; t += blockDim.x) {
                const int c = (t & (ZT / VW - 1)) * VW, k = t >> lv;
                const bool in = i0 + c < P.Nx;
                cp_async_n<16>(&A[makhoul_dest(k, N) * L + (c >> 1)], in ? col0 + c + plane * k : col0, !in);
            }
        } else {
            for (int t = threadIdx.x; t < ZT * N; t += blockDim.x) {
                int c = t & (ZT - 1), k = t >> lz;
                const bool in = i0 + c < P.Nx;
                Cx<FT>& d = A[makhoul_dest(k, N) * L + (c >> 1)];
                cp_async_n<sizeof(FT)>((c & 1) ? &d.im : &d.re, in ? col0 + c + plane * k : col0, !in);
            }
        }
        cp_async_wait();
        __syncthreads();
        Cx<FT>* R = fft_any<FT, NC, true>(A, B, L, P.pz, -1, T);
        Cx<FT>* O = (R == A) ? B : A;
        FT* out = reinterpret_cast<FT*>(O);  // ZT x N reals staged for coalesced stores
        for (int t = threadIdx.x; t < L * N; t += blockDim.x) {
            int l = t & (L - 1), k = t >> ll;
            Cx<FT> Zk = R[k * L + l], Zn = R[(k == 0 ? 0 : N - k) * L + l];
            Cx<FT> w = Q[k];
            Cx<FT> s = Zk + conj(Zn), d = Zk - conj(Zn);
            Cx<FT> ws = w * s, wd = w * d;
            out[(2 * l) + ZT * k] = ws.re;       // X_a[k] = Re(ω^k (Z_k + Z*_{N-k}))
            out[(2 * l + 1) + ZT * k] = wd.im;   // X_b[k] = Im(ω^k (Z_k - Z*_{N-k}))
        }
        __syncthreads();
        if (vec) {
            for (int t = threadIdx.x; t < ZT * N / VW; t += blockDim.x) {
                const int c = (t & (ZT / VW - 1)) * VW, k = t >> lv;
                if (i0 + c < P.Nx)
                    *reinterpret_cast<uint4*>(col0 + c + plane * k) = *reinterpret_cast<const uint4*>(out + c + ZT * k);
            }
        } else {
            for (int t = threadIdx.x; t < ZT * N; t += blockDim.x) {
                int c = t & (ZT - 1), k = t >> lz;
                if (i0 + c < P.Nx) col0[c + plane * k] = out[c + ZT * k];
            }
        }
    } else {
        FT* in = reinterpret_cast<FT*>(B);
        if (vec) {
            for (int t = threadIdx.x; t < ZT * N / VW; t += blockDim.x) {
                const int c = (t & (ZT / VW - 1)) * VW, k = t >> lv;
                const bool ok = i0 + c < P.Nx;
                cp_async_n<16>(&in[c + ZT * k], ok ? col0 + c + plane * k : col0, !ok);
            }
        } else {
            for (int t = threadIdx.x; t < ZT * N; t += blockDim.x) {
                int c = t & (ZT - 1), k = t >> lz;
                const bool ok = i0 + c < P.Nx;
                cp_async_n<sizeof(FT)>(&in[c + ZT * k], ok ? col0 + c + plane * k : col0, !ok);
            }
        }
        cp_async_wait();
        __syncthreads();
        for (int t = threadIdx.x; t < L * N; t += blockDim.x) {
            int l = t & (L - 1), k = t >> ll;
            FT Xa = in[2 * l + ZT * k], Xb = in[2 * l + 1 + ZT * k];
            FT Xan = k == 0 ? FT(0) : in[2 * l + ZT * (N - k)];
            FT Xbn = k == 0 ? FT(0) : in[2 * l + 1 + ZT * (N - k)];
            Cx<FT> w = conj(Q[k]);
            // V_a = ω^{-k}(X_a[k] - i X_a[N-k]) / 2 ; V_b likewise ; Z = V_a + i V_b
            Cx<FT> Va = FT(0.5) * (w * cx(Xa, -Xan));
            Cx<FT> Vb = FT(0.5) * (w * cx(Xb, -Xbn));
            A[k * L + l] = cx(Va.re - Vb.im, Va.im + Vb.re);
        }
        __syncthreads();
        Cx<FT>* R = fft_any<FT, NC, true>(A, B, L, P.pz, +1, T);
        if (vec) {
            for (int t = threadIdx.x; t < ZT * N / VW; t += blockDim.x) {
                const int c = (t & (ZT / VW - 1)) * VW, k = t >> lv;
                if (i0 + c < P.Nx)
                    *reinterpret_cast<uint4*>(col0 + c + plane * k) =
                        *reinterpret_cast<const uint4*>(&R[makhoul_dest(k, N) * L + (c >> 1)]);
            }
        } else {
            for (int t = threadIdx.x; t < ZT * N; t += blockDim.x) {
                int c = t & (ZT - 1), k = t >> lz;
                Cx<FT> z = R[makhoul_dest(k, N) * L + (c >> 1)];
                if (i0 + c < P.Nx) col0[c + plane * k] = (c & 1) ? z.im : z.re;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// X pass: real FFT along x through a half-length complex FFT.
// Forward: rb (Nx reals per line) -> cb (Nh = Nx/2+1 complex per line).
// Inverse: cb -> rb.  Block: XL lines (consecutive (j, k) pairs).
// ---------------------------------------------------------------------------
template <typename FT, int NC>
__global__ void k_rfft_x(PassP<FT> P, int inverse, int XL) {
    extern __shared__ __align__(16) unsigned char fft_smem[];
    // compile-time lengths when the kernel is instantiated for this size (constant divisors)
    const int M = NC > 0 ? NC : P.Nx / 2, Nh = NC > 0 ? NC + 1 : P.Nh;
    const int Nx = 2 * M;
    constexpr int VW = 16 / sizeof(FT);
    // whole 16-byte vectors per line, 16-byte aligned lines (the real buffer may be a caller's)
    const bool vec = Nx % (2 * VW) == 0 && (reinterpret_cast<uintptr_t>(P.rb) & 15) == 0;
    Cx<FT>* A = reinterpret_cast<Cx<FT>*>(fft_smem);
    Cx<FT>* B = A + XL * M;
    Cx<FT>* T = A + XL * (Nx + 1);    // twiddles of the half-length FFT
    Cx<FT>* X = T + M;                // the real-FFT split twiddles
    const int nlines = P.Ny * P.Nz;
    const int line0 = blockIdx.x * XL;
    const int L = min(XL, nlines - line0);
    stage_table(T, P.tw_xh, M);
    stage_table(X, P.tw_x, M);
    if (!inverse) {
        const FT* src = P.rb + (size_t)line0 * Nx;
        FT* As = reinterpret_cast<FT*>(A);  // interleaving x[2m], x[2m+1] is exactly re, im
        if (vec) {
            for (int t = threadIdx.x; t < L * Nx / VW; t += blockDim.x) cp_async_n<16>(&As[t * VW], src + t * VW, false);
        } else {
            for (int t = threadIdx.x; t < L * Nx; t += blockDim.x) cp_async_n<sizeof(FT)>(&As[t], src + t, false);
        }
        cp_async_wait();
        __syncthreads();
        Cx<FT>* R = fft_any<FT, NC, false>(A, B, L, P.px_half, -1, T);
        Cx<FT>* dst = P.cb + (size_t)line0 * Nh;
        for (int t = threadIdx.x; t < L * Nh; t += blockDim.x) {
            int l = t / Nh, k = t - l * Nh;
            Cx<FT> Zk = R[l * M + (k == M ? 0 : k)];
            Cx<FT> Zn = R[l * M + (k == 0 ? 0 : M - k)];
            Cx<FT> e = FT(0.5) * (Zk + conj(Zn));
            Cx<FT> d = FT(0.5) * (Zk - conj(Zn));
            Cx<FT> o = cx(d.im, -d.re);  // (Z_k - Z*_{M-k}) / (2i)
            Cx<FT> w = X[k == M ? 0 : k];
            if (k == M) w = cx(FT(-1), FT(0));
            dst[t] = e + w * o;
        }
    } else {
        const Cx<FT>* src = P.cb + (size_t)line0 * Nh;
        Cx<FT>* S = B;  // the block's L lines of Nh coefficients, staged asynchronously
        for (int t = threadIdx.x; t < L * Nh; t += blockDim.x) cp_async_n<sizeof(Cx<FT>)>(&S[t], src + t, false);
        cp_async_wait();
        __syncthreads();
        for (int t = threadIdx.x; t < L * M; t += blockDim.x) {
            int l = t / M, k = t - l * M;
            Cx<FT> Xk = S[l * Nh + k], Xn = S[l * Nh + (M - k)];
            Cx<FT> e = Xk + conj(Xn);
            Cx<FT> w = conj(X[k]);
            Cx<FT> o = w * (Xk - conj(Xn));
            A[l * M + k] = cx(e.re - o.im, e.im + o.re);  // e + i o
        }
        __syncthreads();
        Cx<FT>* R = fft_any<FT, NC, false>(A, B, L, P.px_half, +1, T);
        FT* dst = P.rb + (size_t)line0 * Nx;
        const FT* Rs = reinterpret_cast<const FT*>(R);
        if (vec) {
            for (int t = threadIdx.x; t < L * Nx / VW; t += blockDim.x)
                reinterpret_cast<uint4*>(dst)[t] = reinterpret_cast<const uint4*>(Rs)[t];
        } else {
            for (int t = threadIdx.x; t < L * Nx; t += blockDim.x) dst[t] = Rs[t];
        }
    }
}

// ---------------------------------------------------------------------------
// Y pass for the FFT solver: FFT along y, ϕ̂ = -b̂ / (λx + λy + λz) (zero mode 0),
// inverse FFT along y.  Block: YT consecutive kx at one kz, all Ny.
// mode: 0 = forward+divide+inverse, 1 = forward only, 2 = inverse only.
// ---------------------------------------------------------------------------
template <typename FT, int NC>
__global__ void k_fft_y(PassP<FT> P, int mode, int YT) {
    extern __shared__ __align__(16) unsigned char fft_smem[];
    const int N = P.Ny, Nh = P.Nh;
    const int ly = __ffs(YT) - 1;  // YT is a power of two
    Cx<FT>* A = reinterpret_cast<Cx<FT>*>(fft_smem);
    Cx<FT>* B = A + YT * N;
    Cx<FT>* T = B + YT * N;  // twiddles of the length-N FFT
    const int kz = blockIdx.y;
    const int kx0 = blockIdx.x * YT;
    Cx<FT>* base = P.cb + kx0 + (size_t)Nh * N * kz;
    stage_table(T, P.tw_y, N);
    for (int t = threadIdx.x; t < YT * N; t += blockDim.x) {
        int c = t & (YT - 1), ky = t >> ly;
        const bool ok = kx0 + c < Nh;
        cp_async_n<sizeof(Cx<FT>)>(&A[ky * YT + c], ok ? base + c + (size_t)Nh * ky : base, !ok);
    }
    cp_async_wait();
    __syncthreads();
    Cx<FT>* R = A;
    // radix-16 register butterflies in single precision (fewer shared-memory stages; measured
    // faster on this pass, slower on the x and z passes)
    constexpr int YR = sizeof(FT) == 4 ? 16 : 4;
    if (mode != 2) R = fft_any<FT, NC, true, YR>(A, B, YT, P.py, -1, T);
    if (mode == 0) {
        for (int t = threadIdx.x; t < YT * N; t += blockDim.x) {
            int c = t & (YT - 1), ky = t >> ly;
            int kx = kx0 + c;
            if (kx < Nh) {
                FT lam = (P.lx[kx] + P.ly[ky]) + (P.has_z ? P.lz[kz] : FT(0));
                Cx<FT> b = R[t];
                Cx<FT> phi = (kx == 0 && ky == 0 && kz == 0) ? cx(FT(0), FT(0))
                                                             : cx(-b.re / lam, -b.im / lam);
                R[t] = P.scale * phi;
            }
        }
        __syncthreads();
    }
    if (mode != 1) {
        Cx<FT>* O = (R == A) ? B : A;
        R = fft_any<FT, NC, true, YR>(R, O, YT, P.py, +1, T);
    }
    for (int t = threadIdx.x; t < YT * N; t += blockDim.x) {
        int c = t & (YT - 1), ky = t >> ly;
        if (kx0 + c < Nh) base[c + (size_t)Nh * ky] = R[ky * YT + c];
    }
}

// ---------------------------------------------------------------------------
// Batched Thomas sweep along z in FP64 for the Fourier-tridiagonal solver
// (fourier_tridiagonal_poisson_solver.jl:199-229; batched_tridiagonal_solver.jl:217-243):
//   D_k ϕ_k + ϕ_{k-1}/Δzᶠ_k + ϕ_{k+1}/Δzᶠ_{k+1} = Δzᶜ_k b̂_k,
//   D_1 = -1/Δzᶠ_2 - Δzᶜ_1 (λx+λy), D_N = -1/Δzᶠ_N - Δzᶜ_N (λx+λy),
//   D_k = -(1/Δzᶠ_{k+1} + 1/Δzᶠ_k) - Δzᶜ_k (λx+λy).
// The forward update is elided where |β| ≤ 10 eps (the singular (0,0) mode);
// the (0,0) column then has its vertical mean removed, which is the reference's
// `ϕ .- mean(ϕ)` applied in spectral space.
//
// One thread per (kx, ky) column; a plane of the half spectrum is Nh·Ny
// consecutive columns, so thread c of a level reads and writes column c of that
// plane and every access is coalesced.  The pivots 1/β_k and ratios t_k are
// tabulated once per model (k_thomas_tables, laid out [level][column]); the forward
// sweep keeps the eliminated right-hand side in a global FP64 scratch of the same
// layout, which the backward sweep reads in reverse: the sweep streams at HBM speed
// with full occupancy instead of holding whole columns in shared memory.
// ---------------------------------------------------------------------------
struct ThomasP {
    int Nh, Ny, Nz;
    const double* rdzf;   // 1/Δzᶠ(kr), indexed kr + zoff
    const double* dzc;    // Δzᶜ(kr)
    int zoff;
    const double* lx;     // λx, λy in FP64
    const double* ly;
    double scale;         // 1/(Nx Ny)
    double* ws;           // scratch: 2 arrays of Nz * Nh * Ny doubles (re, im of the forward sweep)
    double* tab_s;        // pivots: 1/β of level kr, or 0 where the elimination is elided (Nz * Nh * Ny)
    double* tab_t;        // elimination factors t of level kr (Nz * Nh * Ny; kr = 1 unused)
};

// The tridiagonal system of column (kx, ky) (fourier_tridiagonal_poisson_solver.jl:199-212,
// 225-260): diagonal D(kr) = -(1/Δzᶠ(kr+1) + 1/Δzᶠ(kr)) - Δzᶜ(kr) λ with the Neumann rows at the
// ends, off-diagonals 1/Δzᶠ, λ = λx + λy.
struct ThomasColumn {
    const ThomasP& T;
    double lam;
    GBO_D double D(int kr) const {
        if (kr == 1) return -T.rdzf[2 + T.zoff] - T.dzc[1 + T.zoff] * lam;
        if (kr == T.Nz) return -T.rdzf[T.Nz + T.zoff] - T.dzc[T.Nz + T.zoff] * lam;
        return -(T.rdzf[kr + 1 + T.zoff] + T.rdzf[kr + T.zoff]) - T.dzc[kr + T.zoff] * lam;
    }
    GBO_D double off(int q) const { return T.rdzf[q + 1 + T.zoff]; }
};

// Pivots of the Thomas sweep (batched_tridiagonal_solver.jl:217-243): β, t = c/β and the
// elision of the forward update where |β| <= 10 eps depend on the grid and the column's
// wavenumbers only, never on the right-hand side, so they are computed once per model and
// the sweep itself has no FP64 division (the costly operation of the sweep on this GPU).
static __global__ void __launch_bounds__(128) k_thomas_tables(ThomasP T) {
    const size_t ncol = (size_t)T.Nh * T.Ny;
    const size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (c >= ncol) return;
    const ThomasColumn C{T, T.lx[c % T.Nh] + T.ly[c / T.Nh]};
    const double tiny = 10 * 2.220446049250313e-16;
    double beta = C.D(1);
    double rbeta = 1.0 / beta;
    T.tab_s[c] = rbeta;
    T.tab_t[c] = 0.0;
    for (int kr = 2; kr <= T.Nz; ++kr) {
        const double a = C.off(kr - 1);
        const double t = a * rbeta;
        const size_t at = c + ncol * (kr - 1);
        T.tab_t[at] = t;
        beta = C.D(kr) - a * t;
        rbeta = 1.0 / beta;
        T.tab_s[at] = fabs(beta) > tiny ? rbeta : 0.0;
    }
}

// The sweep with tabulated pivots: forward elimination (ϕ = (f - a ϕ⁻) / β, elided where
// the table holds 0) into the FP64 scratch, backward substitution into the spectrum.
// Multiplying by 1/β differs from dividing by β in the last bit only.
template <typename FT>
__global__ void __launch_bounds__(128) k_thomas_z(PassP<FT> P, ThomasP T) {
    const size_t ncol = (size_t)T.Nh * T.Ny;
    const size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (c >= ncol) return;
    const int kx = (int)(c % T.Nh), ky = (int)(c / T.Nh);
    const int Nz = T.Nz;
    double* wre = T.ws;
    double* wim = T.ws + ncol * Nz;
    const double* ts = T.tab_s;
    const double* tt = T.tab_t;
    const ThomasColumn C{T, 0.0};
    Cx<FT>* col = P.cb + c;
    const double s1 = __ldg(ts + c);
    Cx<FT> f1 = col[0];
    double pre = (double)f1.re * s1, pim = (double)f1.im * s1;
    wre[c] = pre;
    wim[c] = pim;
    // forward elimination of level kr (1-based) with right-hand side fk and pivot s
    auto forward = [&](int kr, Cx<FT> fk, double s) {
        const double a = C.off(kr - 1);
        const size_t at = c + ncol * (kr - 1);
        const double sre = ((double)fk.re - a * pre) * s;
        const double sim = ((double)fk.im - a * pim) * s;
        pre = s != 0.0 ? sre : 0.0;
        pim = s != 0.0 ? sim : 0.0;
        wre[at] = pre;
        wim[at] = pim;
    };
    // the loads of four levels are issued together (they do not depend on the recurrence)
    int kr = 2;
    for (; kr + 3 <= Nz; kr += 4) {
        Cx<FT> f[4];
        double sv[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            f[q] = col[ncol * (kr - 1 + q)];
            sv[q] = __ldg(ts + c + ncol * (kr - 1 + q));
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) forward(kr + q, f[q], sv[q]);
    }
    for (; kr <= Nz; ++kr) forward(kr, col[ncol * (kr - 1)], __ldg(ts + c + ncol * (kr - 1)));
    // backward substitution; the (0,0) column keeps its solution for the mean
    const bool mean_col = kx == 0 && ky == 0;
    col[ncol * (Nz - 1)] = cx((FT)(pre * T.scale), (FT)(pim * T.scale));
    auto backward = [&](int kq, double r, double i, double t) {
        pre = r - t * pre;
        pim = i - t * pim;
        const size_t at = c + ncol * (kq - 1);
        if (mean_col) { wre[at] = pre; wim[at] = pim; }
        col[ncol * (kq - 1)] = cx((FT)(pre * T.scale), (FT)(pim * T.scale));
    };
    kr = Nz - 1;
    for (; kr - 3 >= 1; kr -= 4) {
        double r[4], i[4], t[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            r[q] = wre[c + ncol * (kr - q - 1)];
            i[q] = wim[c + ncol * (kr - q - 1)];
            t[q] = __ldg(tt + c + ncol * (kr - q));
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) backward(kr - q, r[q], i[q], t[q]);
    }
    for (; kr >= 1; --kr) backward(kr, wre[c + ncol * (kr - 1)], wim[c + ncol * (kr - 1)], __ldg(tt + c + ncol * kr));
    if (mean_col) {
        double mre = 0, mim = 0;
        for (int k = 0; k < Nz; ++k) { mre += wre[c + ncol * k]; mim += wim[c + ncol * k]; }
        mre /= Nz;
        mim /= Nz;
        for (int k = 0; k < Nz; ++k)
            col[ncol * k] = cx((FT)((wre[c + ncol * k] - mre) * T.scale), (FT)((wim[c + ncol * k] - mim) * T.scale));
    }
}

// ---------------------------------------------------------------------------
// Host-side launchers (instantiated in gbo_fft.cu): pick the compile-time
// engine for the common lengths and the runtime engine otherwise.
// ---------------------------------------------------------------------------
template <typename FT> void launch_dct_z(const PassP<FT>& P, int inverse, int ZT, size_t smem, cudaStream_t st);
template <typename FT> void launch_rfft_x(const PassP<FT>& P, int inverse, int XL, size_t smem, cudaStream_t st);
template <typename FT> void launch_fft_y(const PassP<FT>& P, int mode, int YT, size_t smem, cudaStream_t st);
template <typename FT> void launch_thomas_z(const PassP<FT>& P, const ThomasP& T, cudaStream_t st);
void launch_thomas_tables(const ThomasP& T, cudaStream_t st);
template <typename FT> cudaError_t fft_set_smem(size_t smem_z, size_t smem_x, size_t smem_y);
