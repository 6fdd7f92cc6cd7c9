// gbo_dynamic_f64.cu -- DynamicSmagorinsky stencil kernels, double precision.
#include "gbo_dynamic_inst.cuh"
GBO_DYN_INSTANCES(double)
