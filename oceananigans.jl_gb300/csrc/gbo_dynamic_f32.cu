// gbo_dynamic_f32.cu -- DynamicSmagorinsky stencil kernels, single precision.
#include "gbo_dynamic_inst.cuh"
GBO_DYN_INSTANCES(float)
