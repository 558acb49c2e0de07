// spx_k_guiding_f64.cu -- the guiding-centre stepping kernels (TrajectoryGuiding and
// TrajectoryGuidingScatt) in double arithmetic (analytic field derivatives), one per static background.
#include "spx_k_family.cuh"

SPX_FAMILY_TU(guiding, f64, kGuiding, double, 1, false)
