// gbo_fused_f32_tracer.cu -- fused momentum kernel instances: float, with tracer 0 in the same march.
#define GBO_FUSED_FT float
#define GBO_FUSED_TR true
#include "gbo_fused_inst.cuh"
