// spx_launch.hh -- host entry points of the stepping kernels, one translation unit per trajectory
// family, arithmetic, (FP64) field-derivative method and table kind so they compile in parallel.
// The *_f64rk and *_f64fdrk kernels take any Butcher table; the others Euler and the classic RK4.
#pragma once

#include <cuda_runtime.h>

#include "spx_params.hh"

namespace spx {

struct LaunchArgs {
   dim3 grid, block;
   cudaStream_t stream;
   const void* problems_r;          // ProblemDescT<R>* for the launch arithmetic
   const ProblemDesc* problems_d;   // FP64 descriptors (set-up and events)
   RunConfig cfg;
   RunCounters* ctr;
   int32_t* counts;
   double* sums;
   unsigned long long* n_events;
   TrajRecord* records;
   int queue;                       // 1: persistent work-queue schedule
   int bnd_slots;                   // boundary states per lane (the largest problem's count)
};

#define SPX_DECLARE_FAMILY(fam)                                        \
   cudaError_t launch_##fam##_f64(int bg, const LaunchArgs& a);        \
   cudaError_t launch_##fam##_f64fd(int bg, const LaunchArgs& a);      \
   cudaError_t launch_##fam##_f32(int bg, const LaunchArgs& a);        \
   cudaError_t launch_##fam##_f64rk(int bg, const LaunchArgs& a);      \
   cudaError_t launch_##fam##_f64fdrk(int bg, const LaunchArgs& a);    \
   int occupancy_##fam##_f64(int bg, int block, int slots);            \
   int occupancy_##fam##_f64fd(int bg, int block, int slots);          \
   int occupancy_##fam##_f32(int bg, int block, int slots);            \
   int occupancy_##fam##_f64rk(int bg, int block, int slots);          \
   int occupancy_##fam##_f64fdrk(int bg, int block, int slots);
SPX_DECLARE_FAMILY(parker)
// the FP32 Parker kernels specialised for one diffusion class, and for it and the layout of one time
// boundary and two spheres (kLayoutSpheres)
cudaError_t launch_parker_f32rb(int bg, const LaunchArgs& a);
cudaError_t launch_parker_f32fc(int bg, const LaunchArgs& a);
cudaError_t launch_parker_f32rbs(int bg, const LaunchArgs& a);
cudaError_t launch_parker_f32fcs(int bg, const LaunchArgs& a);
int occupancy_parker_f32rb(int bg, int block, int slots);
int occupancy_parker_f32fc(int bg, int block, int slots);
int occupancy_parker_f32rbs(int bg, int block, int slots);
int occupancy_parker_f32fcs(int bg, int block, int slots);
// the FP32 guiding-centre kernels for TrajectoryGuiding proper (kDkNoDiffusion)
cudaError_t launch_guiding_f32p(int bg, const LaunchArgs& a);
int occupancy_guiding_f32p(int bg, int block, int slots);
SPX_DECLARE_FAMILY(lorentz)
SPX_DECLARE_FAMILY(focused)
SPX_DECLARE_FAMILY(guiding)
#undef SPX_DECLARE_FAMILY
// the field-line tracer (B only: no field derivatives, so no *_f64fd units)
cudaError_t launch_fieldline_f64(int bg, const LaunchArgs& a);
cudaError_t launch_fieldline_f64rk(int bg, const LaunchArgs& a);
cudaError_t launch_fieldline_f32(int bg, const LaunchArgs& a);
int occupancy_fieldline_f64(int bg, int block, int slots);
int occupancy_fieldline_f64rk(int bg, int block, int slots);
int occupancy_fieldline_f32(int bg, int block, int slots);

}  // namespace spx
