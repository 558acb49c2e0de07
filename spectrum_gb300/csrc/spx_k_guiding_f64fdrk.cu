// spx_k_guiding_f64fdrk.cu -- the guiding stepping kernels in double arithmetic with the reference's
// compiled-in numerical field derivatives and any Butcher table (coefficients from constant memory),
// one per background.
#include "spx_k_family.cuh"

SPX_FAMILY_TU(guiding, f64fdrk, kGuiding, double, 0, true)
