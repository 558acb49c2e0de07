// spx_k_parker_f64fdrk.cu -- the parker stepping kernels in double arithmetic with the reference's
// compiled-in numerical field derivatives and any Butcher table (coefficients from constant memory),
// one per background.
#include "spx_k_family.cuh"

SPX_FAMILY_TU(parker, f64fdrk, kParker, double, 0, true)
