// spx_k_focused_f32.cu -- the focused stepping kernels in float arithmetic (analytic field derivatives),
// one per background.
#include "spx_k_family.cuh"

SPX_FAMILY_TU(focused, f32, kFocused, float, 1, false)
