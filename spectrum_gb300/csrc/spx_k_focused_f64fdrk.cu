// spx_k_focused_f64fdrk.cu -- the focused stepping kernels in double arithmetic with the reference's
// compiled-in numerical field derivatives and any Butcher table (coefficients from constant memory),
// one per background.
#include "spx_k_family.cuh"

SPX_FAMILY_TU(focused, f64fdrk, kFocused, double, 0, true)
