// spx_k_parker_f64rk.cu -- the parker stepping kernels in double arithmetic with analytic field
// derivatives and any Butcher table (coefficients from constant memory), one per background.
#include "spx_k_family.cuh"

SPX_FAMILY_TU(parker, f64rk, kParker, double, 1, true)
