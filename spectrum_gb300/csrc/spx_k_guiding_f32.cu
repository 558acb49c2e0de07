// spx_k_guiding_f32.cu -- the guiding-centre stepping kernels (TrajectoryGuiding and
// TrajectoryGuidingScatt) in float arithmetic (analytic field derivatives), one per static background.
#include "spx_k_family.cuh"

SPX_FAMILY_TU(guiding, f32, kGuiding, float, 1, false)
