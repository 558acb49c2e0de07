// spx_k_lorentz_f64rk.cu -- the lorentz stepping kernels in double arithmetic with analytic field
// derivatives and any Butcher table (coefficients from constant memory), one per background.
#include "spx_k_family.cuh"

SPX_FAMILY_TU(lorentz, f64rk, kLorentz, double, 1, true)
