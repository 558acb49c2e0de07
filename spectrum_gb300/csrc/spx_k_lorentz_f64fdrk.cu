// spx_k_lorentz_f64fdrk.cu -- the lorentz stepping kernels in double arithmetic with the reference's
// compiled-in numerical field derivatives and any Butcher table (coefficients from constant memory),
// one per background.
#include "spx_k_family.cuh"

SPX_FAMILY_TU(lorentz, f64fdrk, kLorentz, double, 0, true)
