// spx_k_guiding_f64fd.cu -- the guiding-centre stepping kernels (TrajectoryGuiding and
// TrajectoryGuidingScatt) in double arithmetic with the reference's numerical field derivatives, one per static background.
#include "spx_k_family.cuh"

SPX_FAMILY_TU(guiding, f64fd, kGuiding, double, 0, false)
