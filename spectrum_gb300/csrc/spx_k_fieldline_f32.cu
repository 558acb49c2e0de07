// spx_k_fieldline_f32.cu -- the field-line tracer's stepping kernels in float arithmetic, one per
// background.
#include "spx_k_family.cuh"

SPX_FAMILY_TU(fieldline, f32, kFieldline, float, 1, false)
