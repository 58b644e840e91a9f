// fv3g_substep_h5.cu -- advection substep kernels for hord 5: fourth-order PPM with the 2-dx filter.
#include "fv3g_substep.cuh"

FV3G_SUBSTEP_INSTANTIATE(5)
