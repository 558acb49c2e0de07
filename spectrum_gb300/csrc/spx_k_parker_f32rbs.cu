// spx_k_parker_f32rbs.cu -- the parker stepping kernels in float arithmetic with analytic field
// derivatives, specialised for DiffusionRigidityMagneticFieldPowerLaw and the boundary layout of the
// heliospheric modulation runs (one time boundary, two spheres, no momentum boundary): the boundary
// loops unroll and evaluate no other kinds.
#include "spx_k_family.cuh"

SPX_FAMILY_TU_DK(parker, f32rbs, kParker, kDfRigidityB, kLayoutSpheres)
