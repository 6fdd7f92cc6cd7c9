// gbo_fused_inst.cuh -- the instances of the fused momentum kernel for one float type
// and tracer flag (GBO_FUSED_FT, GBO_FUSED_TR), each in its own translation unit so
// that the four compile in parallel: the launch by closure kind and the shared-memory
// attribute of each instance.
#include "gbo_fused.cuh"

template <typename FT, bool TR>
void launch_fused(int closure, bool ibg, dim3 grid, dim3 block, cudaStream_t st, const StepP<FT>& P, int kchunk) {
    const size_t smem = fused::smem_bytes<FT>(closure == CL_AMD || ibg);
    // the fields whose planes the kernel copies
    const int vec = fused::planes_vec<FT>(P.g, {P.u, P.v, P.w, closure != CL_NONE ? P.nu : nullptr,
                                                P.has_phy ? P.phy : nullptr, TR ? P.c : nullptr,
                                                closure == CL_AMD ? P.kap : nullptr});
    if (ibg) k_momentum_fused<FT, TR, CL_NONE, true><<<grid, block, smem, st>>>(P, kchunk, vec);
    else if (closure == CL_SMAG) k_momentum_fused<FT, TR, CL_SMAG><<<grid, block, smem, st>>>(P, kchunk, vec);
    else if (closure == CL_AMD) k_momentum_fused<FT, TR, CL_AMD><<<grid, block, smem, st>>>(P, kchunk, vec);
    else k_momentum_fused<FT, TR, CL_NONE><<<grid, block, smem, st>>>(P, kchunk, vec);
}

template <typename FT, bool TR>
cudaError_t fused_set_smem_tr() {
    const int b = (int)sizeof(fused::Smem<FT>);
    cudaError_t e = cudaSuccess;
    for (const void* f : {(const void*)k_momentum_fused<FT, TR, CL_NONE>, (const void*)k_momentum_fused<FT, TR, CL_SMAG>,
                          (const void*)k_momentum_fused<FT, TR, CL_AMD>, (const void*)k_momentum_fused<FT, TR, CL_NONE, true>}) {
        cudaError_t r = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
        if (r != cudaSuccess) e = r;
    }
    return e;
}

template void launch_fused<GBO_FUSED_FT, GBO_FUSED_TR>(int, bool, dim3, dim3, cudaStream_t, const StepP<GBO_FUSED_FT>&, int);
template cudaError_t fused_set_smem_tr<GBO_FUSED_FT, GBO_FUSED_TR>();
