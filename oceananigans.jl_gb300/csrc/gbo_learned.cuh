// gbo_learned.cuh -- the learned correction of the conjugate-gradient preconditioner.
//
// The FFT preconditioner of the underlying grid (conjugate_gradient_poisson_solver.jl:
// 141-211) is exact away from the immersed boundary.  The learned part adds a
// correction where it is not: z = z_fft + s_z · net(r/s_r, z_fft/s_z, active), s_r and
// s_z the RMS of the residual and of z_fft, with a small 3-D U-Net of four levels (16, 32, 48, 64 channels, 3³
// kernels, ReLU, average pooling, nearest upsampling with additive skips).  The
// preconditioner is then nonlinear, so the CG that uses it is the flexible
// (Polak-Ribière) variant.  There is no reference counterpart: the reference offers
// FFT-based, diagonal and no preconditioning only.
//
// Data layout: activations are BF16, channels last ([cell][channel], cell = i + nx (j +
// ny k) on the level's grid), so the 8 or 16 channels of one neighbour are one or two
// 16-byte copies.  Weights are BF16 [cout][27 · cin] (k = tap · cin + ci, tap = 9 (dz+1)
// + 3 (dy+1) + (dx+1)), zero padded to whole 64-wide k stages; biases FP32.  Boundaries:
// periodic in x and y, zero padding in z.
//
// Convolutions are implicit GEMMs on the warp-level tensor-core instruction
// mma.sync.m16n8k16 (BF16 in, FP32 accumulate): a block computes a 32 × 4 patch of one
// level (128 cells) × cout.  Per 16-channel chunk of the input it stages the patch's
// halo tile (34 × 6 × 3 cells) and the chunk's weights in shared memory with
// asynchronous copies; every input value then serves all 27 taps, and each of the
// eight warps loads its A fragments per tap with one ldmatrix from the shifted tile.
#pragma once
#include <cuda_bf16.h>

#include <cstdint>
#include <string>

#include "gbo_common.cuh"

namespace learned {

constexpr int LEVELS = 4;
constexpr int C0 = 16, C1 = 32, C2 = 48, C3 = 64;
constexpr int FEAT = 8;  // input channels of the first convolution (3 used)
constexpr int KS = 64;   // weight rows are padded to a multiple of KS

// The layers in order; cin / cout as above, out = final layer (one channel into z)
enum { L_ENC0 = 0, L_ENC1, L_ENC2, L_ENC3, L_DEC3, L_DEC2, L_DEC1, L_OUT, NLAYERS };
constexpr int LAYER_CIN[NLAYERS] = {FEAT, C0, C1, C2, C3, C2, C1, C0};
constexpr int LAYER_COUT[NLAYERS] = {C0, C1, C2, C3, C2, C1, C0, 8};  // out: channel 0 used
// in the weight file (FP32, the training layout [cout][cin][3][3][3] then bias[cout]):
// the real input channels of the first layer and the real outputs of the last
constexpr int FILE_CIN[NLAYERS] = {3, C0, C1, C2, C3, C2, C1, C0};
constexpr int FILE_COUT[NLAYERS] = {C0, C1, C2, C3, C2, C1, C0, 1};

GBO_HD constexpr int kpad(int cin) { return ((27 * cin + KS - 1) / KS) * KS; }

// Number of FP32 values in a weight file (all layers, weights then biases per layer).
inline int64_t file_count() {
    int64_t n = 0;
    for (int l = 0; l < NLAYERS; ++l) n += (int64_t)FILE_COUT[l] * FILE_CIN[l] * 27 + FILE_COUT[l];
    return n;
}

struct Dims {
    int nx, ny, nz;
    GBO_HD int64_t n() const { return (int64_t)nx * ny * nz; }
};

}  // namespace learned

// Opaque network state owned by a model (learned_create / learned_destroy).
struct LearnedNet;

// Build the network for an Nx × Ny × Nz grid from an FP32 weight file of
// learned::file_count() values; returns nullptr and sets *err on failure.
LearnedNet* learned_create(int nx, int ny, int nz, const float* weights, int64_t count, std::string* err);
void learned_destroy(LearnedNet* net);
// z += s_z · net(r / s_r, z / s_z, active) on `stream` (capturable: no allocation, no host
// synchronisation).  r, z are FT (float or double, `fp64` selects) interior fields;
// kbot the immersed-bottom table (nullptr: every cell active).  Returns the kernels
// launched.
// flags: the model's device flag word (GBO_FLAG_TIMEOUT when a tensor-core wait gave up).
int learned_apply(LearnedNet* net, const void* r, void* z, const int* kbot, int fp64, cudaStream_t stream,
                  unsigned* flags);
