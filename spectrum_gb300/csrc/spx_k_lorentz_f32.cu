// spx_k_lorentz_f32.cu -- the lorentz stepping kernels in float arithmetic (analytic field derivatives),
// one per background.
#include "spx_k_family.cuh"

SPX_FAMILY_TU(lorentz, f32, kLorentz, float, 1, false)
