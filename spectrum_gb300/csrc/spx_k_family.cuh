// spx_k_family.cuh -- launch and occupancy entry points of the stepping kernel for one
// trajectory family, arithmetic, field-derivative method and table kind (Euler and the classic RK4
// with unrolled constants, or any Butcher table from constant memory), and for the FP32 Parker kernels
// a diffusion class and boundary layout fixed at compile time, switching over the background classes.
// Each spx_k_*.cu instantiates it once, so the 24 kernel sets compile in parallel.
#pragma once

#include "spx_launch.hh"
#include "spx_traj.cuh"

namespace spx {

template <int TT, class R, int DM, bool GT, int DK = -1, int BL = kLayoutAny>
struct FamilyTU {
   // dynamic shared memory: the boundary states of every lane of a block
   static size_t smem(int slots, int block) { return (size_t)(slots > 0 ? slots : 1) * block * sizeof(BndState<R>); }

   // the guiding-centre family runs on static backgrounds only (no kernels for the moving shocks)
   template <int BG>
   static constexpr bool kBuilt = !(TT == kGuiding && (BG == kBgShock || BG == kBgSmoothShock));

   template <int BG>
   static cudaError_t go(const LaunchArgs& a)
   {
      if constexpr (kBuilt<BG>) {
         const auto* P = static_cast<const ProblemDescT<R>*>(a.problems_r);
         step_kernel<TT, BG, R, DM, GT, DK, BL><<<a.grid, a.block, smem(a.bnd_slots, a.block.x), a.stream>>>(
             P, a.problems_d, a.cfg, a.ctr, a.counts, a.sums, a.n_events, a.records, a.queue);
         return cudaGetLastError();
      }
      else return cudaErrorInvalidValue;
   }

   template <int BG>
   static int occ(int block, int slots)
   {
      int n = 0;
      if constexpr (kBuilt<BG>) {
         if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, step_kernel<TT, BG, R, DM, GT, DK, BL>, block, smem(slots, block)) !=
             cudaSuccess)
            n = 0;
      }
      return n;
   }

   static cudaError_t launch(int bg, const LaunchArgs& a)
   {
      switch (bg) {
      case kBgUniform: return go<kBgUniform>(a);
      case kBgShock: return go<kBgShock>(a);
      case kBgSmoothShock: return go<kBgSmoothShock>(a);
      case kBgDipole: return go<kBgDipole>(a);
      case kBgSolarWind: return go<kBgSolarWind>(a);
      case kBgGrid: return go<kBgGrid>(a);
      default: return cudaErrorInvalidValue;
      }
   }

   static int occupancy(int bg, int block, int slots)
   {
      switch (bg) {
      case kBgUniform: return occ<kBgUniform>(block, slots);
      case kBgShock: return occ<kBgShock>(block, slots);
      case kBgSmoothShock: return occ<kBgSmoothShock>(block, slots);
      case kBgDipole: return occ<kBgDipole>(block, slots);
      case kBgSolarWind: return occ<kBgSolarWind>(block, slots);
      case kBgGrid: return occ<kBgGrid>(block, slots);
      default: return 0;
      }
   }
};

}  // namespace spx

// One translation unit: the kernels of one family, arithmetic, derivative method (DM 1: analytic
// field derivatives; DM 0: the reference's compiled-in numerical ones, FP64 only) and table kind
// (GT 1: any Butcher table, FP64 only).
// SPX_FAMILY_TU_DK: the FP32 analytic kernels with the diffusion class fixed at compile time (DK), and
// with it the boundary layout (BL, a BndLayout).
#define SPX_FAMILY_TU_DK(fam, prec, TT, DK, BL)                                                                    \
   namespace spx {                                                                                                  \
   cudaError_t launch_##fam##_##prec(int bg, const LaunchArgs& a) { return FamilyTU<TT, float, 1, false, DK, BL>::launch(bg, a); } \
   int occupancy_##fam##_##prec(int bg, int block, int slots) { return FamilyTU<TT, float, 1, false, DK, BL>::occupancy(bg, block, slots); } \
   }

#define SPX_FAMILY_TU(fam, prec, TT, R, DM, GT)                                                                    \
   namespace spx {                                                                                                  \
   cudaError_t launch_##fam##_##prec(int bg, const LaunchArgs& a) { return FamilyTU<TT, R, DM, GT>::launch(bg, a); } \
   int occupancy_##fam##_##prec(int bg, int block, int slots) { return FamilyTU<TT, R, DM, GT>::occupancy(bg, block, slots); } \
   }
