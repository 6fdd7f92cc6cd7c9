// gbo_dynamic_inst.cuh -- launchers of the DynamicSmagorinsky stencil kernels (Σ, Σ̄, LM
// and MM), instantiated per float type in gbo_dynamic_f32.cu / gbo_dynamic_f64.cu, which
// compile beside the model's translation unit; see gbo_dynamic.cuh.
#pragma once
#include "gbo_dynamic.cuh"

// grid of the tiled kernels
template <typename FT>
dim3 dtile_grid(const GridP<FT>& g) {
    using namespace dtile;
    return dim3((g.Nx + TX - 1) / TX, (g.Ny + TY - 1) / TY, (g.Nz + KT - 1) / KT);
}

template <typename FT, class V>
void dtile_sigma(cudaStream_t st, const GridP<FT>& g, const V& vel, FT* sig, FT* sigb) {
    k_dyn_sigma_tiled<FT, V><<<dtile_grid(g), dim3(dtile::TX, dtile::TY, dtile::KT), sizeof(dtile::SmemS<FT>), st>>>(
        g, vel, sig, sigb);
}
template <typename FT, class V>
void dtile_lm(cudaStream_t st, const GridP<FT>& g, const V& vel, const FT* sig, const FT* sigb, FT* lm, FT* mm) {
    k_lm_mm_tiled<FT, V><<<dtile_grid(g), dim3(dtile::TX, dtile::TY, dtile::KT), sizeof(dtile::SmemL<FT>), st>>>(
        g, vel, sig, sigb, lm, mm);
}

// shared memory above the default 48 KB for every instance (model creation, any context)
template <typename FT>
cudaError_t dyn_set_smem() {
    cudaError_t e = cudaSuccess;
    auto set = [&](const void* f, size_t b) {
        const cudaError_t r = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b);
        if (r != cudaSuccess) e = r;
    };
    set((const void*)k_dyn_sigma_tiled<FT, PlainVel<FT>>, sizeof(dtile::SmemS<FT>));
    set((const void*)k_dyn_sigma_tiled<FT, LagVel<FT>>, sizeof(dtile::SmemS<FT>));
    set((const void*)k_lm_mm_tiled<FT, PlainVel<FT>>, sizeof(dtile::SmemL<FT>));
    set((const void*)k_lm_mm_tiled<FT, LagVel<FT>>, sizeof(dtile::SmemL<FT>));
    return e;
}

template <typename FT>
void dyn_launch_sigma(cudaStream_t st, const GridP<FT>& g, const PlainVel<FT>& vel, FT* sig, FT* sigb) {
    dtile_sigma<FT>(st, g, vel, sig, sigb);
}
template <typename FT>
void dyn_launch_sigma(cudaStream_t st, const GridP<FT>& g, const LagVel<FT>& vel, FT* sig, FT* sigb) {
    dtile_sigma<FT>(st, g, vel, sig, sigb);
}
template <typename FT>
void dyn_launch_lm(cudaStream_t st, const GridP<FT>& g, const PlainVel<FT>& vel, const FT* sig, const FT* sigb, FT* lm,
                   FT* mm) {
    dtile_lm<FT>(st, g, vel, sig, sigb, lm, mm);
}
template <typename FT>
void dyn_launch_lm(cudaStream_t st, const GridP<FT>& g, const LagVel<FT>& vel, const FT* sig, const FT* sigb, FT* lm,
                   FT* mm) {
    dtile_lm<FT>(st, g, vel, sig, sigb, lm, mm);
}

#define GBO_DYN_INSTANCES(FT)                                                                                     \
    template void dyn_launch_sigma<FT>(cudaStream_t, const GridP<FT>&, const PlainVel<FT>&, FT*, FT*);            \
    template void dyn_launch_sigma<FT>(cudaStream_t, const GridP<FT>&, const LagVel<FT>&, FT*, FT*);              \
    template void dyn_launch_lm<FT>(cudaStream_t, const GridP<FT>&, const PlainVel<FT>&, const FT*, const FT*, FT*, \
                                    FT*);                                                                         \
    template void dyn_launch_lm<FT>(cudaStream_t, const GridP<FT>&, const LagVel<FT>&, const FT*, const FT*, FT*, FT*); \
    template cudaError_t dyn_set_smem<FT>();
