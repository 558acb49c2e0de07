// spx_k_parker_f32rb.cu -- the parker stepping kernels in float arithmetic with analytic field
// derivatives, specialised for DiffusionRigidityMagneticFieldPowerLaw (the modulation workloads):
// no dispatch over the other diffusion classes and no difference-quotient gradients.
#include "spx_k_family.cuh"

SPX_FAMILY_TU_DK(parker, f32rb, kParker, kDfRigidityB, kLayoutAny)
