// spx_k_guiding_f64rk.cu -- the guiding stepping kernels in double arithmetic with analytic field
// derivatives and any Butcher table (coefficients from constant memory), one per background.
#include "spx_k_family.cuh"

SPX_FAMILY_TU(guiding, f64rk, kGuiding, double, 1, true)
