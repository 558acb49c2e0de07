// spx_k_guiding_f32p.cu -- the guiding-centre stepping kernels in float arithmetic for TrajectoryGuiding
// proper: no pitch-angle scattering and no perpendicular diffusion compiled in, so the kernel holds only
// the drift step (the family's shared kernel carries all four types' code).
#include "spx_k_family.cuh"

SPX_FAMILY_TU_DK(guiding, f32p, kGuiding, kDkNoDiffusion, kLayoutAny)
