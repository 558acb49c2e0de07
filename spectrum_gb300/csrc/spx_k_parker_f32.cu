// spx_k_parker_f32.cu -- the parker stepping kernels in float arithmetic (analytic field derivatives),
// one per background.
#include "spx_k_family.cuh"

SPX_FAMILY_TU(parker, f32, kParker, float, 1, false)
