// spx_k_focused_f64fd.cu -- the focused stepping kernels in double arithmetic with the reference's
// compiled-in numerical field derivatives, one per background.
#include "spx_k_family.cuh"

SPX_FAMILY_TU(focused, f64fd, kFocused, double, 0, false)
