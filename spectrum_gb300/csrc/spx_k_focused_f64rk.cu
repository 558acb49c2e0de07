// spx_k_focused_f64rk.cu -- the focused stepping kernels in double arithmetic with analytic field
// derivatives and any Butcher table (coefficients from constant memory), one per background.
#include "spx_k_family.cuh"

SPX_FAMILY_TU(focused, f64rk, kFocused, double, 1, true)
