// spx_k_parker_f32fcs.cu -- the parker stepping kernels in float arithmetic with analytic field
// derivatives, specialised for DiffusionFullConstant and the boundary layout of one time boundary,
// two spheres and no momentum boundary.
#include "spx_k_family.cuh"

SPX_FAMILY_TU_DK(parker, f32fcs, kParker, kDfFull, kLayoutSpheres)
