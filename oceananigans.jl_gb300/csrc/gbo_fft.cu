#include <algorithm>
// gbo_fft.cu -- instantiations and launchers of the spectral Poisson pass kernels.
#include "gbo_fft.cuh"

#define GBO_FFT_SIZES(X) X(16) X(32) X(48) X(64) X(96) X(128) X(256) X(512)

template <typename FT>
void launch_dct_z(const PassP<FT>& P, int inverse, int ZT, size_t smem, cudaStream_t st) {
    dim3 grid((P.Nx + ZT - 1) / ZT, P.Ny);
    switch (P.Nz) {
#define CASE(n) case n: k_dct_z<FT, n><<<grid, 256, smem, st>>>(P, inverse, ZT); return;
        GBO_FFT_SIZES(CASE)
#undef CASE
        default: k_dct_z<FT, 0><<<grid, 256, smem, st>>>(P, inverse, ZT);
    }
}

template <typename FT>
void launch_rfft_x(const PassP<FT>& P, int inverse, int XL, size_t smem, cudaStream_t st) {
    dim3 grid((P.Ny * P.Nz + XL - 1) / XL);
    switch (P.Nx / 2) {
#define CASE(n) case n: k_rfft_x<FT, n><<<grid, 256, smem, st>>>(P, inverse, XL); return;
        GBO_FFT_SIZES(CASE)
#undef CASE
        default: k_rfft_x<FT, 0><<<grid, 256, smem, st>>>(P, inverse, XL);
    }
}

template <typename FT>
void launch_fft_y(const PassP<FT>& P, int mode, int YT, size_t smem, cudaStream_t st) {
    dim3 grid((P.Nh + YT - 1) / YT, P.Nz);
    switch (P.Ny) {
#define CASE(n) case n: k_fft_y<FT, n><<<grid, 256, smem, st>>>(P, mode, YT); return;
        GBO_FFT_SIZES(CASE)
#undef CASE
        default: k_fft_y<FT, 0><<<grid, 256, smem, st>>>(P, mode, YT);
    }
}

template <typename FT>
void launch_thomas_z(const PassP<FT>& P, const ThomasP& T, cudaStream_t st) {
    const size_t ncol = (size_t)T.Nh * T.Ny;
    k_thomas_z<FT><<<(unsigned)((ncol + 127) / 128), 128, 0, st>>>(P, T);
}

void launch_thomas_tables(const ThomasP& T, cudaStream_t st) {
    const size_t ncol = (size_t)T.Nh * T.Ny;
    k_thomas_tables<<<(unsigned)((ncol + 127) / 128), 128, 0, st>>>(T);
}

template <typename FT>
cudaError_t fft_set_smem(size_t sz, size_t sx, size_t sy) {
    cudaError_t e = cudaSuccess;
    auto set = [&](const void* f, size_t b) {
        cudaError_t r = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)std::max<size_t>(b, 1));
        if (r != cudaSuccess) e = r;
    };
#define CASE(n) set((const void*)k_dct_z<FT, n>, sz); set((const void*)k_rfft_x<FT, n>, sx); set((const void*)k_fft_y<FT, n>, sy);
    GBO_FFT_SIZES(CASE)
#undef CASE
    set((const void*)k_dct_z<FT, 0>, sz);
    set((const void*)k_rfft_x<FT, 0>, sx);
    set((const void*)k_fft_y<FT, 0>, sy);
    return e;
}

#define INST(FT)                                                                                  \
    template void launch_dct_z<FT>(const PassP<FT>&, int, int, size_t, cudaStream_t);             \
    template void launch_rfft_x<FT>(const PassP<FT>&, int, int, size_t, cudaStream_t);            \
    template void launch_fft_y<FT>(const PassP<FT>&, int, int, size_t, cudaStream_t);             \
    template void launch_thomas_z<FT>(const PassP<FT>&, const ThomasP&, cudaStream_t);                  \
    template cudaError_t fft_set_smem<FT>(size_t, size_t, size_t);
INST(float)
INST(double)
