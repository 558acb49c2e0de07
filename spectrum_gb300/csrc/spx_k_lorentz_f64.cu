// spx_k_lorentz_f64.cu -- the lorentz stepping kernels in double arithmetic with analytic field
// derivatives, one per background.
#include "spx_k_family.cuh"

SPX_FAMILY_TU(lorentz, f64, kLorentz, double, 1, false)
