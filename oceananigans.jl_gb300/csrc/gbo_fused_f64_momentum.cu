// gbo_fused_f64_momentum.cu -- fused momentum kernel instances: double, momentum only.
#define GBO_FUSED_FT double
#define GBO_FUSED_TR false
#include "gbo_fused_inst.cuh"
