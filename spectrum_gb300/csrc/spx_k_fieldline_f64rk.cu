// spx_k_fieldline_f64rk.cu -- the field-line tracer's stepping kernels in double arithmetic with any
// Butcher table (coefficients from constant memory), one per background, with the reference's field
// evaluation (as spx_k_fieldline_f64.cu).
#include "spx_k_family.cuh"

SPX_FAMILY_TU(fieldline, f64rk, kFieldline, double, 0, true)
