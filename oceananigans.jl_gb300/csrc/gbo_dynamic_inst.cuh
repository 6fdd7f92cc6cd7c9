// gbo_dynamic_inst.cuh -- launchers of the DynamicSmagorinsky stencil kernels (Σ, Σ̄, LM
// and MM), instantiated per float type in gbo_dynamic_f32.cu / gbo_dynamic_f64.cu, which
// compile beside the model's translation unit; see gbo_dynamic.cuh.
#pragma once
#include "gbo_dynamic.cuh"

template <typename FT>
void dyn_launch_sigma(dim3 grid, dim3 block, cudaStream_t st, const GridP<FT>& g, const PlainVel<FT>& vel, FT* sig,
                      FT* sigb) {
    k_dyn_sigma<FT, PlainVel<FT>><<<grid, block, 0, st>>>(g, vel, sig, sigb);
}
template <typename FT>
void dyn_launch_sigma(dim3 grid, dim3 block, cudaStream_t st, const GridP<FT>& g, const LagVel<FT>& vel, FT* sig,
                      FT* sigb) {
    k_dyn_sigma<FT, LagVel<FT>><<<grid, block, 0, st>>>(g, vel, sig, sigb);
}
template <typename FT>
void dyn_launch_lm_sums(dim3 grid, dim3 block, cudaStream_t st, const GridP<FT>& g, const PlainVel<FT>& vel,
                        const FT* sig, const FT* sigb, double* part) {
    k_dyn_lm<FT, PlainVel<FT>><<<grid, block, 0, st>>>(g, vel, sig, sigb, part);
}
template <typename FT>
void dyn_launch_lag_lm(dim3 grid, dim3 block, cudaStream_t st, const GridP<FT>& g, const LagVel<FT>& vel,
                       const FT* sig, const FT* sigb, FT* lm, FT* mm) {
    k_lag_lm<FT, LagVel<FT>><<<grid, block, 0, st>>>(g, vel, sig, sigb, lm, mm);
}

#define GBO_DYN_INSTANCES(FT)                                                                                      \
    template void dyn_launch_sigma<FT>(dim3, dim3, cudaStream_t, const GridP<FT>&, const PlainVel<FT>&, FT*, FT*); \
    template void dyn_launch_sigma<FT>(dim3, dim3, cudaStream_t, const GridP<FT>&, const LagVel<FT>&, FT*, FT*);   \
    template void dyn_launch_lm_sums<FT>(dim3, dim3, cudaStream_t, const GridP<FT>&, const PlainVel<FT>&,          \
                                         const FT*, const FT*, double*);                                           \
    template void dyn_launch_lag_lm<FT>(dim3, dim3, cudaStream_t, const GridP<FT>&, const LagVel<FT>&, const FT*,  \
                                        const FT*, FT*, FT*);
