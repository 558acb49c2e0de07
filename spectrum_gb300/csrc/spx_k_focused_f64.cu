// spx_k_focused_f64.cu -- the focused stepping kernels in double arithmetic with analytic field
// derivatives, one per background.
#include "spx_k_family.cuh"

SPX_FAMILY_TU(focused, f64, kFocused, double, 1, false)
