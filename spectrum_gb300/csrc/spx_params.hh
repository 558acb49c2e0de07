// spx_params.hh -- plain-old-data plugin descriptors, filled on the host from the reference's
// DataContainer blobs and read by the stepping kernels from device memory.
//
// One ProblemDescT<R> holds everything a trajectory of one problem needs: background, diffusion,
// source, boundaries, initial conditions and distribution layouts. The descriptors are templates
// over the real type R: the host parses into ProblemDescT<double> and derives a
// ProblemDescT<float> copy, so the FP32 kernel reads no FP64 data in its step loop (on GB300 the
// FP64 pipe, which also converts double to float, runs at a small fraction of the FP32 rate).
// Kinds are the numbers of include/spx.h; lengths are code units of the reference
// (common/specie.hh:30-82).
#pragma once

#include <cstdint>

namespace spx {

constexpr int kMaxBnd = 4;     // boundaries per class (time, space, momentum)
constexpr int kMaxDistro = 4;  // distributions per problem

// kGuiding is the kernel family of all four guiding-centre types: TrajectoryGuiding (201), with
// RunConfig::pa_scattering TrajectoryGuidingScatt (202), and with RunConfig::traj_kind 203/204 the
// perpendicular-diffusion types TrajectoryGuidingDiff and TrajectoryGuidingDiffScatt, as the reference
// derives the last three from the first. kFieldline is the field-line tracer TrajectoryFieldline.
enum TrajKind : int {
   kFieldline = 199, kLorentz = 200, kGuiding = 201, kGuidingScatt = 202, kGuidingDiff = 203, kGuidingDiffScatt = 204, kFocused = 205,
   kParker = 206, kParkerSource = 207
};

enum BgKind : int { kBgUniform = 1, kBgShock = 2, kBgSmoothShock = 3, kBgDipole = 4, kBgSolarWind = 5, kBgGrid = 6 };
// BackgroundDiscontinuity and BackgroundSmoothDiscontinuity: plugin kinds only. The parser turns them into
// kBgShock and kBgSmoothShock descriptors with the downstream state given instead of derived from the
// jump conditions (and the smooth one's own transition steepness), so they run on the shock kernels.
enum BgPluginKind : int { kBgDiscontinuity = 7, kBgSmoothDiscontinuity = 8 };

enum DiffKind : int {
   kDfIsotropic = 1, kDfQLT, kDfPara, kDfPerp, kDfFull, kDfFlowMomentum, kDfKinEnergyRadial, kDfRigidityB,
   kDfStrauss2013, kDfPotgieter2015, kDfEmpiricalSOQLT, kDfWNLT, kDfWNLTRamp
};

enum BndKind : int {
   kBtTimeExpire = 1, kBtTimePass, kBtTimeRecurrent,
   kBtPlaneAbsorb = 10, kBtPlaneReflect, kBtPlanePass, kBtBoxReflect, kBtSphereAbsorb, kBtSphereReflect,
   kBtRankineAbsorb, kBtCylinderAbsorb, kBtRegionAbsorb, kBtSpherePass,
   kBtMomentumInject = 30, kBtMomentumPass, kBtMomentumSlab, kBtMomentumShell, kBtMirror
};

// Boundary layouts a kernel can be compiled for. kLayoutAny: counts and kinds from the descriptor.
// kLayoutSpheres: exactly one time boundary (expiry or pass), two spheres (absorbing, reflecting or
// passing) and no momentum boundary, the set-up of the heliospheric modulation runs.
enum BndLayout : int { kLayoutAny = 0, kLayoutSpheres = 1 };

enum IniKind : int {
   kItFixed = 1, kItInterval,
   kIsFixed = 10, kIsLine, kIsCircle, kIsBox, kIsSphere, kIsSphereSector, kIsRankine, kIsCylinder, kIsCylinderSector,
   kImFixed = 30, kImBeam, kImRing, kImShell, kImThickShell, kImMaxwell,
   kImLogEnergyPitchBand = 40, kIsEquatorialBand = 41
};

enum DistKind : int {
   kDsTimeUniform = 1, kDsPositionUniform, kDsMomentumUniform, kDsPositionMomentumUniform, kDsSpectrumPowerLaw,
   kDsSpectrumBentPowerLaw, kDsCumulative1, kDsCumulative2, kDsDivergenceFlow, kDsLossCone, kDsAnisotropyLISM,
   kDsTimeMu = 20
};

template <class R>
struct BgParamsT {
   int kind;
   R t0, dmax0;
   R r0[3], u0[3], B0[3];
   R n_shock[3], u1[3], B1[3], E0[3], E1[3];
   R v_shock, compression, width, dmax_fraction;
   R tanh_k;                  // the smooth transition's tanh_width_factor: 8 (shock), 4 (discontinuity)
   R M[3];                    // dipole moment B0 r_ref^3
   R eprime[3][3];            // solar wind rotation frame (rows)
   R w0, r_ref, ur0, A;       // A = Br0 r_ref^2
   // uniform Cartesian grid (BackgroundServerCartesian): node (i, j, k) sits at
   // cent_min + (i, j, k) * zone; kGridStride values per node, x fastest
   R cent_min[3], zone[3], zone_min;
   int grid_n[3];
   const R* grid;             // device address of the node values (set when the context uploads)
   // block mode (grid_nb[0] > 0): the reference's Cartesian data server over its reader's blocks of
   // kGridBlockZones^3 zones, grid_nb[k] blocks per axis over [dom_min, dom_max] (file units, au),
   // grid_ghost ghost cells per block side; node values in fluid units, and the ratios
   // {length, velocity, magnetic field} Fluid/Particle and Fluid::c_code in gunits
   int grid_nb[3], grid_ghost;
   int grid_order;            // SERVER_INTERP_ORDER of the block mode: 1 the stencil, 0 the zone's values,
                              // -1 the reader's interpolation with numerical gradients (FP64)
   R dom_min[3], dom_max[3], blk_len[3], gunits[4];
};

// The DK of the guiding-centre kernels compiled for TrajectoryGuiding proper: no pitch-angle scattering and
// no perpendicular diffusion, so neither step is in the kernel.
constexpr int kDkNoDiffusion = -2;

// Zones per block edge of the reference's Cartesian blocks (block_size_cartesian, src/reader_cartesian.hh:17)
constexpr int kGridBlockZones = 4;

// Values per grid node: U (3), B (3), |B| (the magnitude at the node), one pad (32 B per node in FP32)
constexpr int kGridStride = 8;

template <class R>
struct DiffParamsT {
   int kind, i0, i1;
   R a[10];
};

template <class R>
struct SrcParamsT {
   int kind;                  // 0 none, 1 constant, 2 momentum injection, 3 momentum injection in a spherical shell
   R p_inj, rate;
   R r0[3], r_sh, w_sh;       // the shell of kind 3
};

template <class R>
struct BndParamsT {
   int kind, cls;             // cls: 0 time, 1 space, 2 momentum
   int reflect, recurrent;
   int max_crossings, n_actions;
   int actions[kMaxDistro];
   int region_ind;
   R timemark, timemark_lo;   // timemark_lo: the part of the double timemark a float cannot hold
   R momentum, radius, z_nose, r1, r2, region_val;
   R origin[3], norm[3], corner0[3], corner1[3], normals[3][3], axis[3], fa[3][3];
   R slab_r0[3], slab_r1[3], slab_n[3];
};

template <class R>
struct IniParamsT {
   int kind, n_int, flag;
   R a[8];
   R v0[3], v1[3], v2[3];
};

template <class R>
struct DistParamsT {
   int kind, width, dims, n_actions;
   int n_bins[3], log_bins[3], bin_outside[3];
   R limits0[3], bin_size[3];
   R val_hot, val_cold;
   int val_time, val_coord, pos_idx, mom_idx;
   R J0, T0, pow_law, T_b, pow_law_comb, bend, A0;
   // DistributionAnisotropyLISM: the binning frame (rows), the LISM flow velocity, the density gradient
   // across the LISM field (pow_law holds its momentum power-law slope)
   R rot[3][3], u_lism[3], grad_perp[3];
   int64_t offset_counts;     // into the context's counts array
   int64_t offset_sums;       // into the context's sums array (doubles)
   // DistributionBase::AddRecord (keep_records): the value and weight of every processed event are
   // appended at rec_vals[3k], rec_wts[width k] for slot k = atomicAdd(rec_n, 1) below rec_cap (set in the
   // FP64 descriptors only; null when records are not kept)
   int keep_records;
   double* rec_vals;
   double* rec_wts;
   unsigned long long* rec_n;
   int64_t rec_cap;
};

template <class R>
struct ProblemDescT {
   BgParamsT<R> bg;
   DiffParamsT<R> df;
   SrcParamsT<R> src;
   IniParamsT<R> it, is, im;
   BndParamsT<R> bt[kMaxBnd], bs[kMaxBnd], bm[kMaxBnd];
   DistParamsT<R> d[kMaxDistro];
   int nbt, nbs, nbm, nd;
   int has_diff;
   uint32_t problem_id;
   uint64_t seed;
   int64_t n_traj;            // trajectories of this problem in one run
   int64_t first;             // index of its first trajectory in the launch's global order
   int64_t id_base;           // trajectory id of its first trajectory in this run (ids continue across runs)
};

using ProblemDesc = ProblemDescT<double>;
using BgParams = BgParamsT<double>;
using DiffParams = DiffParamsT<double>;
using BndParams = BndParamsT<double>;
using IniParams = IniParamsT<double>;
using DistParams = DistParamsT<double>;

// Per-trajectory final state, the same fields as the reference harness writes.
struct TrajRecord {
   uint32_t attempts, status;
   uint64_t steps;
   double t, pos[3], mom[3];
   double t0, pos0[3], mom0[3];
   double amp, logwgt;
};

// Kernel-wide settings (one per launch).
struct RunConfig {
   int traj_kind, time_flow, rk, deriv_mode, pa_scattering, max_attempts;
   double steps_per_orbit;
   float steps_per_orbit_f;
   int record_final;
   int n_problems;
   int steps_per_sync;
   uint32_t step_cap;         // 0, or the steps after which a trajectory is dropped (autotuning samples)
   int mu_method;             // guiding-centre pitch-angle step: 0 Euler, 1 Milstein, 2 RK2 (STOCHASTIC_METHOD_MU)
   int perp_method;           // guiding-centre perpendicular step: 0 Euler, 1 Milstein, 2 RK2 (STOCHASTIC_METHOD_PERP)
   int64_t total_traj;
   int64_t run_index;         // trajectory ids of run r are r * n_traj + local (new streams per run)
   // the Butcher table of the general-table kernels: stages, order, adaptive, and the offset of its
   // coefficients in the shared table (spx_rk_tables.h)
   int rk_stages, rk_order, rk_adaptive, rk_offset;
   // 1 when a problem has a DistributionLossCone: the |B| extrema along each trajectory are tracked
   // (the reference's RECORD_BMAG_EXTREMA build, src/trajectory_base.cc:581-592)
   int track_bmag;
};

// Device-side counters of one run (scratch memory, zeroed before each launch).
struct RunCounters {
   unsigned long long next_traj;     // work-queue head
   unsigned long long finished;
   unsigned long long steps;
   unsigned long long retries;
   unsigned long long given_up;
   unsigned long long events;
   unsigned int error;               // first device-side error code (0 = none)
   unsigned int pad;
};

// Host-side conversion of the double descriptors to another real type.
template <class R>
void convert_problem(const ProblemDesc& s, ProblemDescT<R>& d);

}  // namespace spx
