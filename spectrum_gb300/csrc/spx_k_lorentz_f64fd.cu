// spx_k_lorentz_f64fd.cu -- the lorentz stepping kernels in double arithmetic with the reference's
// compiled-in numerical field derivatives, one per background.
#include "spx_k_family.cuh"

SPX_FAMILY_TU(lorentz, f64fd, kLorentz, double, 0, false)
