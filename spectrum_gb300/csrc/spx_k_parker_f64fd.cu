// spx_k_parker_f64fd.cu -- the parker stepping kernels in double arithmetic with the reference's
// compiled-in numerical field derivatives, one per background.
#include "spx_k_family.cuh"

SPX_FAMILY_TU(parker, f64fd, kParker, double, 0, false)
