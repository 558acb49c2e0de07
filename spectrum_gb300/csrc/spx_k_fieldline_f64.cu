// spx_k_fieldline_f64.cu -- the field-line tracer's stepping kernels in double arithmetic, Euler or the
// classic RK4, one per background. A field line evaluates B alone, never a derivative, so one unit serves
// both derivative options; it is compiled with the reference's field evaluation (derivative method 0),
// whose arithmetic the oracle repeats (the analytic method's closed-form solar wind rounds differently).
#include "spx_k_family.cuh"

SPX_FAMILY_TU(fieldline, f64, kFieldline, double, 0, false)
