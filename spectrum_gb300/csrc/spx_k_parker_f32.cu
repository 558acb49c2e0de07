// spx_k_parker_f32.cu -- the parker stepping kernels in float arithmetic, one per background.
#include "spx_launch.hh"
#include "spx_traj.cuh"

namespace spx {

template <int BG>
static cudaError_t go(const LaunchArgs& a)
{
   const auto* P = static_cast<const ProblemDescT<float>*>(a.problems_r);
   step_kernel<kParker, BG, float><<<a.grid, a.block, 0, a.stream>>>(P, a.problems_d, a.cfg, a.ctr, a.counts, a.sums,
                                                                  a.n_events, a.records, a.queue);
   return cudaGetLastError();
}

cudaError_t launch_parker_f32(int bg, const LaunchArgs& a)
{
   switch (bg) {
   case kBgUniform: return go<kBgUniform>(a);
   case kBgShock: return go<kBgShock>(a);
   case kBgSmoothShock: return go<kBgSmoothShock>(a);
   case kBgDipole: return go<kBgDipole>(a);
   case kBgSolarWind: return go<kBgSolarWind>(a);
   default: return cudaErrorInvalidValue;
   }
}

template <int BG>
static int occ(int block)
{
   int n = 0;
   if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, step_kernel<kParker, BG, float>, block, 0) != cudaSuccess) n = 0;
   return n;
}

int occupancy_parker_f32(int bg, int block)
{
   switch (bg) {
   case kBgUniform: return occ<kBgUniform>(block);
   case kBgShock: return occ<kBgShock>(block);
   case kBgSmoothShock: return occ<kBgSmoothShock>(block);
   case kBgDipole: return occ<kBgDipole>(block);
   case kBgSolarWind: return occ<kBgSolarWind>(block);
   default: return 0;
   }
}

}  // namespace spx
