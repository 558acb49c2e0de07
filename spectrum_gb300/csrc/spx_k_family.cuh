// spx_k_family.cuh -- launch and occupancy entry points of the stepping kernel for one
// trajectory family in one arithmetic, switching over the background classes. Each spx_k_*.cu
// instantiates it once, so the six families compile in parallel.
#pragma once

#include "spx_launch.hh"
#include "spx_traj.cuh"

namespace spx {

template <int TT, class R>
struct FamilyTU {
   // dynamic shared memory: the boundary states of every lane of a block
   static size_t smem(int slots, int block) { return (size_t)(slots > 0 ? slots : 1) * block * sizeof(BndState<R>); }

   template <int BG, int DM>
   static cudaError_t go_dm(const LaunchArgs& a)
   {
      const auto* P = static_cast<const ProblemDescT<R>*>(a.problems_r);
      step_kernel<TT, BG, R, DM><<<a.grid, a.block, smem(a.bnd_slots, a.block.x), a.stream>>>(
          P, a.problems_d, a.cfg, a.ctr, a.counts, a.sums, a.n_events, a.records, a.queue);
      return cudaGetLastError();
   }

   // FP64 kernels exist for both derivative methods; the FP32 kernels are analytic only.
   template <int BG>
   static cudaError_t go(const LaunchArgs& a)
   {
      if constexpr (sizeof(R) == sizeof(double)) {
         if (a.cfg.deriv_mode == 0) return go_dm<BG, 0>(a);
      }
      return go_dm<BG, 1>(a);
   }

   template <int BG, int DM>
   static int occ_dm(int block, int slots)
   {
      int n = 0;
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, step_kernel<TT, BG, R, DM>, block, smem(slots, block)) !=
          cudaSuccess)
         n = 0;
      return n;
   }

   template <int BG>
   static int occ(int block, int slots, int deriv_mode)
   {
      if constexpr (sizeof(R) == sizeof(double)) {
         if (deriv_mode == 0) return occ_dm<BG, 0>(block, slots);
      }
      return occ_dm<BG, 1>(block, slots);
   }

   static cudaError_t launch(int bg, const LaunchArgs& a)
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

   static int occupancy(int bg, int block, int slots, int deriv_mode)
   {
      switch (bg) {
      case kBgUniform: return occ<kBgUniform>(block, slots, deriv_mode);
      case kBgShock: return occ<kBgShock>(block, slots, deriv_mode);
      case kBgSmoothShock: return occ<kBgSmoothShock>(block, slots, deriv_mode);
      case kBgDipole: return occ<kBgDipole>(block, slots, deriv_mode);
      case kBgSolarWind: return occ<kBgSolarWind>(block, slots, deriv_mode);
      default: return 0;
      }
   }
};

}  // namespace spx

#define SPX_FAMILY_TU(fam, prec, TT, R)                                                                    \
   namespace spx {                                                                                          \
   cudaError_t launch_##fam##_##prec(int bg, const LaunchArgs& a) { return FamilyTU<TT, R>::launch(bg, a); } \
   int occupancy_##fam##_##prec(int bg, int block, int slots, int deriv_mode)                               \
   {                                                                                                        \
      return FamilyTU<TT, R>::occupancy(bg, block, slots, deriv_mode);                                      \
   }                                                                                                        \
   }
