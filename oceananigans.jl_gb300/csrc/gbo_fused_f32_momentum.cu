// gbo_fused_f32_momentum.cu -- fused momentum kernel instances: float, momentum only.
#define GBO_FUSED_FT float
#define GBO_FUSED_TR false
#include "gbo_fused_inst.cuh"
