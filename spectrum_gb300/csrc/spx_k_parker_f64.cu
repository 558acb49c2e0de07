// spx_k_parker_f64.cu -- the parker stepping kernels in double arithmetic with analytic field
// derivatives, one per background.
#include "spx_k_family.cuh"

SPX_FAMILY_TU(parker, f64, kParker, double, 1, false)
