// fv3g_substep_h1.cu -- advection substep kernels for hord 1: the linear scheme with the lim_fac 2-dx filter.
#include "fv3g_substep.cuh"

FV3G_SUBSTEP_INSTANTIATE(1)
