// fv3g_substep_h8.cu -- advection substep kernels for hord 8: PPM with the Lin (2004) monotonicity constraint.
#include "fv3g_substep.cuh"

FV3G_SUBSTEP_INSTANTIATE(8)
