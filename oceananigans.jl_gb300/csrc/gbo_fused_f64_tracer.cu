// gbo_fused_f64_tracer.cu -- fused momentum kernel instances: double, with tracer 0 in the same march.
#define GBO_FUSED_FT double
#define GBO_FUSED_TR true
#include "gbo_fused_inst.cuh"
