// spx_traj.cuh -- the per-trajectory stepping loop on the device: SetStart, the Parker
// Euler-Maruyama advance, the Runge-Kutta advance of Lorentz and focused trajectories (with the
// Euler pitch-angle scattering step), boundary handling, distribution events, and the kernel
// that schedules trajectories onto lanes.
//
// One lane integrates one trajectory. The state a lane carries from step to step is only time,
// position, momentum, weights, the time-step memory and the boundary deltas; the fields are
// evaluated at the start of every step (the reference evaluates them at the end of the previous
// step, src/trajectory_parker.cc:300, which gives the same values). The plain schedule gives
// lane k the trajectories k, k + stride, ...; the queue schedule refills finished lanes from a
// global work-queue counter, one atomic per warp and refill, lanes ranked with __ballot_sync/__popc.
#pragma once

#include "spx_physics.cuh"
#include "spx_rk_tables.h"

namespace spx {

constexpr uint32_t TRAJ_FINISH = 0x0010u, TRAJ_TIME_CROSSED = 0x0020u, TRAJ_SPATIAL_CROSSED = 0x0040u,
                   TRAJ_MOMENTUM_CROSSED = 0x0080u, TRAJ_DISCARD = 0x0100u, TRAJ_GAVE_UP = 0x10000u;
constexpr uint32_t kMaxTrajSteps = 10000000u;  // src/trajectory_base.hh:38
constexpr int kMaxBndTotal = 3 * kMaxBnd;

constexpr unsigned kErrAction = 1u;  // RunCounters::error: an action beyond the ActionTable

// Lane state carried across steps.
template <class R, class A>
struct Lane {
   int prob;
   uint32_t traj_id, attempt, steps, status;
   uint32_t nrm;     // GuidingScatt: normals drawn so far (the k-th is the first of step block k); Parker with
                     // a general Butcher table: step blocks drawn so far (rejected steps draw too)
   uint32_t n_adapt; // general Butcher tables: consecutive rejected steps
   A t;
   AV3<A> pos, mom;  // mom: Parker (p,-,-), Focused (p, mu, -), Lorentz (px, py, pz), Guiding (p_perp, -, p_para),
                     // Fieldline (-, -, p_para)
   R amp, wgt, dt, dt_adapt, src_del_old;
};

// Initial point of the trajectory (needed only by events and records).
struct Start {
   double t0;
   V3<double> pos0, mom0, bhat0;
   // |B| at the first point and its extrema along the trajectory (DistributionLossCone; tracked only
   // with RunConfig::track_bmag)
   double bmag0, bmag_min, bmag_max;
   uint32_t nuni;  // guiding types: uniforms drawn so far, set-up included (the perpendicular Milstein and RK2
                   // schemes draw one a step); kept here, with the lane's other memory-resident state
};

struct Sinks {
   int32_t* counts;
   double* sums;
   unsigned long long* n_events;  // [problem * kMaxDistro + distro]
   RunCounters* ctr;
};

template <class R, class A>
__device__ __forceinline__ V3<R> lane_mom(const Lane<R, A>& L) { return val3<R>(L.mom); }

__device__ __forceinline__ double neg(double a) { return -a; }
__device__ __forceinline__ FF neg(FF a) { return {-a.hi, -a.lo}; }

template <int TT>
__device__ __forceinline__ constexpr unsigned traj_mask()
{
   return TT == kLorentz ? (kE | kB)                                 // src/trajectory_lorentz.cc:36
        : TT == kFieldline ? kB  // which_field_to_follow, src/trajectory_fieldline.hh:30 and .cc:37-38
        : TT == kFocused ? (kAll | kGradB | kGradU | kDUdt)           // src/trajectory_focused.cc:40
        : TT == kGuiding ? (kAll | kGradB)  // src/trajectory_guiding.cc:51-52; dB/dt is zero for the static backgrounds
                         : (kU | kB | kGradU | kGradB);               // src/trajectory_parker.cc:204
}

// Momentum magnitude passed to the field evaluators (ConvertMomentum()[0]; Fieldline |p_para|,
// src/trajectory_fieldline.hh:80-83).
template <int TT, class R>
__device__ __forceinline__ R field_p(V3<R> mom)
{
   return (TT == kLorentz || TT == kGuiding) ? norm(mom) : (TT == kFieldline ? m_abs(mom.z) : mom.x);
}

// ---- random numbers for set-up -----------------------------------------------------------
struct InitRng {
   uint64_t seed;
   uint32_t traj, problem, attempt, n_uniform, n_normal;
   __device__ double uniform()
   {
      uint32_t k = n_uniform++;
      uint4 b = rng_block(seed, k >> 2, traj, problem, kRngInit, attempt);
      uint32_t x = (k & 3) == 0 ? b.x : ((k & 3) == 1 ? b.y : ((k & 3) == 2 ? b.z : b.w));
      return u01d(x);
   }
   __device__ double normal()
   {
      uint32_t j = n_normal++;
      double n[4];
      normals4<double>(rng_block(seed, j >> 2, traj, problem, kRngInitNormal, attempt), n);
      return n[j & 3];
   }
};

// ---- initial conditions (src/initial_*.cc), sampled in FP64 once per trajectory ------------
static __device__ __noinline__ double sample_time(InitRng& rng, const ProblemDesc& P, int64_t local)
{
   const IniParams& q = P.it;
   if (q.kind == kItInterval) {
      if (q.n_int <= 0) return q.a[0] + (q.a[1] - q.a[0]) * rng.uniform();
      // trajectory k takes the k-th element of the sequence (the reference steps a per-process counter)
      return q.a[0] + ((double)local + 0.5) * ((q.a[1] - q.a[0]) / (double)q.n_int);
   }
   return q.a[0];
}

static __device__ __noinline__ V3<double> sample_pos(InitRng& rng, const ProblemDesc& P, int64_t local)
{
   const IniParams& q = P.is;
   const double two_pi = 6.283185307179586476925286766559;
   V3<double> v0 = ld3(q.v0), v1 = ld3(q.v1), v2 = ld3(q.v2);
   switch (q.kind) {
   case kIsLine:
      if (q.n_int <= 0) return v0 + rng.uniform() * (v1 - v0);
      return v0 + ((double)local + 0.5) * ((v1 - v0) / (double)q.n_int);
   case kIsBox: {
      double x = q.v0[0] + (q.v1[0] - q.v0[0]) * rng.uniform();
      double y = q.v0[1] + (q.v1[1] - q.v0[1]) * rng.uniform();
      double z = q.v0[2] + (q.v1[2] - q.v0[2]) * rng.uniform();
      return mk(x, y, z);
   }
   case kIsCircle: {
      double phi = two_pi * rng.uniform();
      return (v0 + cos(phi) * v1) + sin(phi) * v2;
   }
   case kIsSphere:
   case kIsSphereSector: {
      double ct, st, phi;
      if (q.kind == kIsSphere) {
         ct = -1.0 + 2.0 * rng.uniform();
         st = sqrt(1.0 - ct * ct);
         phi = two_pi * rng.uniform();
      }
      else {
         ct = q.a[5] + (q.a[6] - q.a[5]) * rng.uniform();
         st = sqrt(1.0 - ct * ct);
         phi = q.a[3] + (q.a[4] - q.a[3]) * rng.uniform();
      }
      return v0 + mk(q.a[0] * st * cos(phi), q.a[0] * st * sin(phi), q.a[0] * ct);
   }
   case kIsRankine: {
      double ct = q.a[2] + (1.0 - q.a[2]) * rng.uniform();
      double r = q.a[0] * sqrt(2.0 / (1.0 + ct)), z = r * ct, s = sqrt(r * r - z * z);
      double phi = two_pi * rng.uniform();
      return v0 + mk(s * cos(phi), s * sin(phi), z);
   }
   case kIsCylinder: case kIsCylinderSector: {  // src/initial_space.cc:576-583, 638-645
      double z = rng.uniform(), phi;
      V3<double> ry = mk(q.a[0], q.a[1], q.a[2]);
      if (q.kind == kIsCylinder) phi = two_pi * rng.uniform();
      else phi = q.a[3] + (q.a[4] - q.a[3]) * rng.uniform();
      return ((v0 + cos(phi) * v2) + sin(phi) * ry) + z * v1;
   }
   case kIsEquatorialBand: {
      double Lv = q.a[1] + (q.a[2] - q.a[1]) * rng.uniform();
      double phi = two_pi * rng.uniform();
      return v0 + mk(Lv * q.a[0] * cos(phi), Lv * q.a[0] * sin(phi), 0.0);
   }
   default: return v0;
   }
}

// GetMomSample(axis) (src/initial_base.cc:133-143) with the samplers of
// src/initial_momentum.cc; the result is in the trajectory's native momentum coordinates.
static __device__ __noinline__ V3<double> sample_mom(InitRng& rng, const ProblemDesc& P, int traj, V3<double> axis_in)
{
   const IniParams& q = P.im;
   V3<double> axis = unit(axis_in);
   const double two_pi = 6.283185307179586476925286766559;
   switch (q.kind) {
   case kImFixed: return ld3(q.v0);  // Lorentz and Fieldline
   case kImBeam:
      if (traj == kLorentz) return q.a[0] * axis;
      if (traj == kGuiding) return mk(0.0, 0.0, q.a[0]);
      return mk(q.a[0], 0.0, 0.0);
   case kImRing:
      if (traj == kLorentz) {
         double phi = two_pi * rng.uniform();
         V3<double> e1 = second_unit(axis), e2 = cross(axis, e1);
         return (q.a[0] * q.a[2]) * axis + (q.a[0] * q.a[3]) * (cos(phi) * e1 + sin(phi) * e2);
      }
      if (traj == kGuiding) return mk(q.a[0] * q.a[3], 0.0, q.a[0] * q.a[2]);
      return mk(q.a[0], q.a[2], 0.0);
   case kImShell:
   case kImThickShell: {
      double p = q.a[0];
      if (q.kind == kImThickShell) {
         if (q.flag) p = pow(10.0, q.a[0] + (q.a[1] - q.a[0]) * rng.uniform());
         else p = q.a[0] + (q.a[1] - q.a[0]) * rng.uniform();
      }
      if (traj == kParker || traj == kParkerSource) return mk(p, 0.0, 0.0);
      if (traj == kFieldline) return mk(0.0, 0.0, p);  // src/initial_momentum.cc:290-291, 390-391
      if (traj == kFocused) { double mu = -1.0 + 2.0 * rng.uniform(); return mk(p, mu, 0.0); }
      if (traj == kGuiding) { double mu = -1.0 + 2.0 * rng.uniform(), st = sqrt(1.0 - mu * mu); return mk(p * st, 0.0, p * mu); }
      double mu = -1.0 + 2.0 * rng.uniform(), st = sqrt(1.0 - mu * mu), phi = two_pi * rng.uniform();
      return mk(p * st * cos(phi), p * st * sin(phi), p * mu);
   }
   case kImMaxwell: {
      if (traj == kFieldline) return mk(0.0, 0.0, q.a[0]);  // the mean only, no draws (src/initial_momentum.cc:522-525)
      double p_para = q.a[0] + q.a[1] * rng.normal();
      double p_perp = q.a[2] * sqrt(-2.0 * log(rng.uniform()));
      if (traj == kLorentz) {
         double phi = two_pi * rng.uniform();
         V3<double> e1 = second_unit(axis), e2 = cross(axis, e1);
         return p_para * axis + p_perp * (cos(phi) * e1 + sin(phi) * e2);
      }
      if (traj == kGuiding) return mk(p_perp, 0.0, p_para);
      double p = sqrt(p_para * p_para + p_perp * p_perp);
      if (traj == kFocused) return mk(p, p_para / p, 0.0);
      return mk(p, 0.0, 0.0);
   }
   case kImLogEnergyPitchBand: {
      double le1 = log(q.a[0]), le2 = log(q.a[1]);
      double e = exp(le1 + (le2 - le1) * rng.uniform());
      double mu = q.a[2] + (q.a[3] - q.a[2]) * rng.uniform();
      double p = mom_of<double>(e);
      if (traj == kLorentz) {
         double psi = two_pi * rng.uniform(), st = sqrt(1.0 - mu * mu);
         V3<double> e1 = second_unit(axis), e2 = cross(axis, e1);
         return (p * mu) * axis + (p * st) * (cos(psi) * e1 + sin(psi) * e2);
      }
      if (traj == kFocused) return mk(p, mu, 0.0);
      if (traj == kGuiding) return mk(p * sqrt(1.0 - mu * mu), 0.0, p * mu);
      return mk(p, 0.0, 0.0);
   }
   }
   return mk(0.0, 0.0, 0.0);
}

// ---- distribution events (DistributionBase::ProcessTrajectory, src/distribution_base.cc:174-194;
// DistributionTemplated::AddEvent, src/distribution_templated.cc:145-181), in FP64 ----------
// The event's "second point" is the current state; its spatial data are the fields of the
// step's start point, as in the reference (HandleBoundaries runs before CommonFields).
struct EventPoint {
   double t;
   V3<double> pos, mom, bhat;
   double divU, amp, wgt, bmag;
};

static __device__ __noinline__ void process_event(int traj, const EventPoint& e, const Start& s0, const ProblemDesc& P,
                                           int prob, int di, int action, const Sinks& S)
{
   const DistParams& d = P.d[di];
   if (action >= d.n_actions) {
      atomicCAS(&S.ctr->error, 0u, kErrAction);
      return;
   }
   V3<double> value = mk(0.0, 0.0, 0.0);
   double w[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
   switch (d.kind) {
   case kDsTimeUniform: value.x = d.val_time == 0 ? s0.t0 : e.t; break;
   case kDsPositionUniform: case kDsLossCone:
      value = d.val_time == 0 ? s0.pos0 : e.pos;
      if (d.val_coord == 1) {  // Metric<SphericalRTP>::PosToCurv, common/coordinates.hh:124-135
         double r = norm(value), phi = atan2(value.y, value.x);
         if (phi < 0.0) phi += 6.283185307179586476925286766559;
         value = mk(r, acos(value.z / r), phi);
      }
      break;
   case kDsMomentumUniform: {
      V3<double> m = d.val_time == 0 ? s0.mom0 : e.mom;
      V3<double> bh = d.val_time == 0 ? s0.bhat0 : e.bhat;
      if (d.val_coord == 0 || (traj != kLorentz && traj != kGuiding && traj != kFieldline)) value = m;
      else if (traj == kFieldline) value = mk(m.z, 0.0, 0.0);  // src/distribution_other.cc:276-279
      else if (traj == kLorentz) { double mm = norm(m); value = mk(mm, dot(m, bh) / mm, 0.0); }
      else { double mm = norm(m); value = mk(mm, m.z / mm, 0.0); }
      break;
   }
   case kDsPositionMomentumUniform: {
      V3<double> p = d.val_time == 0 ? s0.pos0 : e.pos, m = d.val_time == 0 ? s0.mom0 : e.mom;
      value.x = d.pos_idx == 3 ? norm(p) : p[d.pos_idx];
      value.y = m[d.mom_idx];
      break;
   }
   case kDsSpectrumPowerLaw: case kDsSpectrumBentPowerLaw:
      // the parallel component for Fieldline (src/distribution_other.cc:557)
      value.x = enr_kin<double>((traj == kLorentz || traj == kGuiding) ? norm(s0.mom0)
                                : (traj == kFieldline ? s0.mom0.z : s0.mom0.x));
      break;
   case kDsCumulative1: case kDsCumulative2: value.x = e.t; break;
   case kDsDivergenceFlow: value = s0.mom0; break;
   case kDsTimeMu:
      value.x = e.t;
      value.y = traj == kLorentz ? dot(e.mom, e.bhat) / norm(e.mom) : traj == kGuiding ? e.mom.z / norm(e.mom) : e.mom.y;
      break;
   case kDsAnisotropyLISM: {  // EvaluateValue, src/distribution_other.cc:416-426
      // the first point's momentum in the binning frame, as (theta, phi) of its direction; the
      // reference leaves the third value unset although its set-up bins the first and the third
      // (dims 5): here it is 0
      const V3<double> m = s0.mom0;
      V3<double> q = mk(m.x * d.rot[0][0] + m.y * d.rot[0][1] + m.z * d.rot[0][2],
                        m.x * d.rot[1][0] + m.y * d.rot[1][1] + m.z * d.rot[1][2],
                        m.x * d.rot[2][0] + m.y * d.rot[2][1] + m.z * d.rot[2][2]);
      double r = norm(q), phi = atan2(q.y, q.x);
      if (phi < 0.0) phi += 6.283185307179586476925286766559;
      value = mk(acos(q.z / r), phi, 0.0);
      break;
   }
   }
   switch (d.kind) {
   case kDsTimeUniform: case kDsPositionUniform: case kDsMomentumUniform: case kDsPositionMomentumUniform: case kDsTimeMu:
      w[0] = action == 0 ? d.val_hot : d.val_cold;
      break;
   case kDsSpectrumPowerLaw: case kDsSpectrumBentPowerLaw:
      if (action == 0) {  // DISTRO_KINETIC_ENERGY_POWER_LAW_TYPE 0, src/distribution_other.cc:567-591
         double m2 = (traj == kLorentz || traj == kGuiding) ? norm(e.mom) : (traj == kFieldline ? e.mom.z : e.mom.x);
         double ke = enr_kin<double>(m2), v = vel_of<double>(m2);
         w[0] = d.J0 * v * pow(ke / d.T0, d.pow_law) / (m2 * m2);
         if (d.kind == kDsSpectrumBentPowerLaw) w[0] /= pow(1.0 + pow(ke / d.T_b, d.pow_law_comb), d.bend);
      }
      else w[0] = d.val_cold;
      break;
   case kDsCumulative1: { V3<double> dp = e.pos - s0.pos0; w[0] = dp.x; w[1] = dp.y; w[2] = dp.z; break; }
   case kDsCumulative2: {
      V3<double> dp = e.pos - s0.pos0;
      for (int i = 0; i < 3; i++)
         for (int j = 0; j < 3; j++) w[3 * i + j] = dp[i] * dp[j];
      break;
   }
   case kDsDivergenceFlow: w[0] = action == 0 ? d.A0 * pow(fabs(e.divU), d.pow_law) : d.val_cold; break;
   case kDsLossCone:  // DistributionLossCone::RecordLossCone, src/distribution_other.cc:858-862
      w[0] = s0.bmag_min;
      w[1] = s0.bmag_max;
      w[2] = asin(sqrt((d.val_time == 0 ? s0.bmag0 : e.bmag) / s0.bmag_max));
      break;
   case kDsAnisotropyLISM: {  // the five anisotropy weights, src/distribution_other.cc:433-483
      const V3<double> ul = mk(d.u_lism[0], d.u_lism[1], d.u_lism[2]);
      const double m1 = norm(s0.mom0), m2 = norm(e.mom);
      // the second point's momentum in the LISM frame: p - gamma m U (RelFactor1, common/physics.hh:260-263)
      const double rf = sqrt(1.0 + (m2 / 1.0 / c_code<double>()) * (m2 / 1.0 / c_code<double>()));
      const V3<double> rel = e.mom - (rf * 1.0) * ul;
      const double rn = norm(rel);
      const V3<double> ru = mk(rel.x / rn, rel.y / rn, rel.z / rn);
      if (action == 0) {  // Compton-Getting factor
         const V3<double> mh = mk(s0.mom0.x / m1, s0.mom0.y / m1, s0.mom0.z / m1);
         w[0] = 1.0 - dot(d.pow_law * ul, mh) / vel_of<double>(m1);
      }
      else if (action == 1) w[0] = pow(rn / m1, d.pow_law);
      else if (action == 2) w[0] = dot(ru, e.bhat);
      else if (action == 3) { const double c = dot(ru, e.bhat); w[0] = 0.5 * (3.0 * (c * c) - 1.0); }
      else {  // b x gradient: the guiding centre dotted with the density gradient
         const V3<double> gp = mk(d.grad_perp[0], d.grad_perp[1], d.grad_perp[2]);
         const double rl = rn * c_code<double>() / (fabs(1.0) * e.bmag);
         w[0] = dot(gp, e.pos + rl * cross(ru, e.bhat));
      }
      break;
   }
   }
   // AddRecord follows AddEvent for every processed event, outliers included (src/distribution_base.cc:192-193)
   if (d.rec_n) {
      const unsigned long long k = atomicAdd(d.rec_n, 1ull);
      if (k < (unsigned long long)d.rec_cap) {
         for (int i = 0; i < 3; i++) d.rec_vals[3 * k + i] = value[i];
         for (int j = 0; j < d.width; j++) d.rec_wts[(int64_t)d.width * k + j] = w[j];
      }
   }
   int bin[3] = {0, 0, 0};
   for (int k = 0; k < 3; k++) {
      if (!(d.dims & (1 << k))) continue;
      double val = (d.log_bins[k] ? log10(value[k]) : value[k]) - d.limits0[k];
      if (val != val) return;
      // a "left" outlier is dropped unless bin_outside; the bin is then still val / bin_size, which
      // is how a negative bin width (max < min, e.g. backward exit times) bins correctly
      if (val < 0.0 && !d.bin_outside[k]) return;
      double q = val / d.bin_size[k];
      if (q >= (double)d.n_bins[k]) {
         if (d.bin_outside[k]) { bin[k] = d.n_bins[k] - 1; continue; }
         return;
      }
      // the reference indexes before the array for q <= -1 (bin_outside set); bin 0 here
      bin[k] = q <= -1.0 ? 0 : (int)q;
   }
   int64_t lin = (int64_t)d.n_bins[2] * ((int64_t)d.n_bins[1] * bin[0] + bin[1]) + bin[2];
   double ew = exp(e.wgt);
   for (int k = 0; k < d.width; k++) atomicAdd(&S.sums[d.offset_sums + lin * d.width + k], w[k] * ew + e.amp);
   atomicAdd(&S.counts[d.offset_counts + lin], 1);
   atomicAdd(&S.n_events[(int64_t)prob * kMaxDistro + di], 1ull);
   atomicAdd(&S.ctr->events, 1ull);  // the run's total, for spx_stats
}

template <class R, class A>
__device__ __forceinline__ EventPoint event_point(const Lane<R, A>& L, const SD<R>& sp)
{
   EventPoint e;
   e.t = acc_dbl(L.t);
   e.pos = mk(acc_dbl(L.pos.x), acc_dbl(L.pos.y), acc_dbl(L.pos.z));
   e.mom = mk(acc_dbl(L.mom.x), acc_dbl(L.mom.y), acc_dbl(L.mom.z));
   e.bhat = mk((double)sp.bhat.x, (double)sp.bhat.y, (double)sp.bhat.z);
   e.divU = (double)sd_divU(sp);
   e.bmag = (double)sp.Bmag;
   e.amp = (double)L.amp;
   e.wgt = (double)L.wgt;
   return e;
}

// Boundaries are held compactly: j < nbt time, then nbs spatial, then nbm momentum boundaries.
template <class R>
__device__ __forceinline__ const BndParamsT<R>& bnd_param(const ProblemDescT<R>& P, int j)
{
   return j < P.nbt ? P.bt[j] : (j < P.nbt + P.nbs ? P.bs[j - P.nbt] : P.bm[j - P.nbt - P.nbs]);
}

template <int TT, class R, class A>
__device__ __forceinline__ void distro_events(const Lane<R, A>& L, const SD<R>& sp, const Start& s0,
                                              const ProblemDesc& Pd, int j, const Sinks& S)
{
   const BndParams& b = bnd_param(Pd, j);
   EventPoint e = event_point(L, sp);
   for (int di = 0; di < Pd.nd; di++) {
      int action = di < b.n_actions ? b.actions[di] : -1;
      if (action >= 0) process_event(TT, e, s0, Pd, L.prob, di, action, S);
   }
}

// The crossed part of HandleBoundaries: momentum, then spatial, then time boundaries, each class
// with the distribution events of its last crossed boundary, then RecordBoundary of the crossed.
template <int TT, class R, class A>
__device__ __forceinline__ void handle_crossings(Lane<R, A>& L, BndView<R> bv, const SD<R>& sp, const Start& s0,
                                                 const ProblemDescT<R>& P, const ProblemDesc& Pd, const Sinks& S,
                                                 unsigned crossed)
{
   V3<R> pos = val3<R>(L.pos), mom = lane_mom(L);
   const int s_lo = P.nbt, m_lo = P.nbt + P.nbs;
   // momentum boundaries
   int active = -1;
   for (int i = 0; i < P.nbm; i++) {
      const int j = m_lo + i;
      if (!(crossed & (1u << j))) continue;
      active = j;
      if (!P.bm[i].reflect && bv.ld(j).crossings_left == 1) L.status |= TRAJ_MOMENTUM_CROSSED | TRAJ_FINISH;
   }
   if (active >= 0) distro_events<TT>(L, sp, s0, Pd, active, S);
   // spatial boundaries
   active = -1;
   for (int i = 0; i < P.nbs; i++) {
      const int j = s_lo + i;
      if (!(crossed & (1u << j))) continue;
      active = j;
      const BndParamsT<R>& b = P.bs[i];
      BndState<R> st = bv.ld(j);
      if (b.reflect) {
         // src/trajectory_base.cc:462-483: mirror the position, reverse the momentum
         V3<R> shift = (R(2) * st.delta) * bnd_normal(b, pos);
         add3(L.pos, R(-1) * shift);
         // ReverseMomentum: the base negates the vector (src/trajectory_base.cc:139-142; Lorentz and
         // Fieldline), Focused its mu (src/trajectory_focused.hh:141-144), Guiding its parallel component
         // (src/trajectory_guiding.hh:123-126), Parker nothing
         if (TT == kLorentz || TT == kFieldline) { L.mom.x = neg(L.mom.x); L.mom.y = neg(L.mom.y); L.mom.z = neg(L.mom.z); }
         else if (TT == kFocused) L.mom.y = neg(L.mom.y);
         else if (TT == kGuiding) L.mom.z = neg(L.mom.z);
         pos = val3<R>(L.pos);
         mom = lane_mom(L);
         compute_bnd<1>(b, st, L.t, pos, mom, sp.bhat, sp.region, TT);
         st.crossings_left--;
         bv.st(j, st);
      }
      else if (st.crossings_left == 1) L.status |= TRAJ_SPATIAL_CROSSED | TRAJ_FINISH;
   }
   if (active >= 0) distro_events<TT>(L, sp, s0, Pd, active, S);
   // time boundaries
   active = -1;
   for (int j = 0; j < s_lo; j++) {
      if (!(crossed & (1u << j))) continue;
      active = j;
      if (bv.ld(j).crossings_left == 1) L.status |= TRAJ_TIME_CROSSED | TRAJ_FINISH;
   }
   if (active >= 0) distro_events<TT>(L, sp, s0, Pd, active, S);
   // RecordBoundary of the crossed ones, in slot order
   for (int j = 0; j < s_lo; j++)
      if (crossed & (1u << j)) {
         BndState<R> st = bv.ld(j);
         record_bnd<0>(P.bt[j], st, L.t, pos, mom, sp.bhat, sp.region, TT);
         bv.st(j, st);
      }
   for (int i = 0; i < P.nbs; i++)
      if (crossed & (1u << (s_lo + i))) {
         BndState<R> st = bv.ld(s_lo + i);
         record_bnd<1>(P.bs[i], st, L.t, pos, mom, sp.bhat, sp.region, TT);
         bv.st(s_lo + i, st);
      }
   for (int i = 0; i < P.nbm; i++)
      if (crossed & (1u << (m_lo + i))) {
         BndState<R> st = bv.ld(m_lo + i);
         record_bnd<2>(P.bm[i], st, L.t, pos, mom, sp.bhat, sp.region, TT);
         bv.st(m_lo + i, st);
      }
}

// ---- HandleBoundaries (src/trajectory_base.cc:413-535) ---------------------------------------
// ComputeAllBoundaries, the momentum/space/time handlers with their distribution events, and
// UpdateAllBoundaries. A boundary that was not crossed is recorded right after it is computed
// (RecordBoundary only copies delta to delta_old for it); crossed ones after their events.
// Boundary counts per class: from the descriptor, or constants of the layout the kernel is compiled for
// (the loops below then unroll).
template <int BL, class R> __device__ __forceinline__ int n_time_bnd(const ProblemDescT<R>& P) { return BL == kLayoutSpheres ? 1 : P.nbt; }
template <int BL, class R> __device__ __forceinline__ int n_space_bnd(const ProblemDescT<R>& P) { return BL == kLayoutSpheres ? 2 : P.nbs; }
template <int BL, class R> __device__ __forceinline__ int n_mom_bnd(const ProblemDescT<R>& P) { return BL == kLayoutSpheres ? 0 : P.nbm; }

template <int TT, int BL, class R, class A>
__device__ __forceinline__ void handle_boundaries(Lane<R, A>& L, BndView<R> bv, const SD<R>& sp, const Start& s0,
                                                  const ProblemDescT<R>& P, const ProblemDesc& Pd, const Sinks& S)
{
   V3<R> pos = val3<R>(L.pos), mom = lane_mom(L);
   unsigned crossed = 0;
   const int nbt = n_time_bnd<BL>(P), nbs = n_space_bnd<BL>(P), nbm = n_mom_bnd<BL>(P);
   // one loop per class, each evaluating its own kinds: time, spatial, momentum slots in order
   for (int j = 0; j < nbt; j++) {
      BndState<R> b = bv.ld(j);
      compute_bnd<0, BL>(P.bt[j], b, L.t, pos, mom, sp.bhat, sp.region, TT);
      if (b.crossed) crossed |= 1u << j;
      else b.delta_old = b.delta;
      bv.st(j, b);
   }
   for (int i = 0; i < nbs; i++) {
      const int j = nbt + i;
      BndState<R> b = bv.ld(j);
      compute_bnd<1, BL>(P.bs[i], b, L.t, pos, mom, sp.bhat, sp.region, TT);
      if (b.crossed) crossed |= 1u << j;
      else b.delta_old = b.delta;
      bv.st(j, b);
   }
   for (int i = 0; i < nbm; i++) {
      const int j = nbt + nbs + i;
      BndState<R> b = bv.ld(j);
      compute_bnd<2, BL>(P.bm[i], b, L.t, pos, mom, sp.bhat, sp.region, TT);
      if (b.crossed) crossed |= 1u << j;
      else b.delta_old = b.delta;
      bv.st(j, b);
   }
   // a crossing is rare: keep its handling off the straight-line path
   if (__builtin_expect(crossed == 0u, 1)) return;
   handle_crossings<TT>(L, bv, sp, s0, P, Pd, S, crossed);
}

// SpaceTerminateCheck (src/trajectory_base.cc:188-237); true if the trajectory ended mid-step
template <int TT, class R, class A>
__device__ __forceinline__ bool space_terminate(Lane<R, A>& L, BndView<R> bv, const SD<R>& sp, const Start& s0,
                                                const ProblemDescT<R>& P, const ProblemDesc& Pd, const Sinks& S)
{
   V3<R> pos = val3<R>(L.pos), mom = lane_mom(L);
   for (int i = 0; i < P.nbs; i++) {
      const int j = P.nbt + i;
      BndState<R> b = bv.ld(j);
      compute_bnd<1>(P.bs[i], b, L.t, pos, mom, sp.bhat, sp.region, TT);
      bv.st(j, b);
      if (b.crossed && b.crossings_left == 1) {
         L.status |= TRAJ_SPATIAL_CROSSED | TRAJ_FINISH;
         distro_events<TT>(L, sp, s0, Pd, j, S);
         L.steps++;
         return true;
      }
   }
   return false;
}

// TimeBoundaryProximityCheck (src/trajectory_base.cc:151-179)
template <class R>
__device__ __forceinline__ R time_proximity(R dt, R dmax, BndView<R> bv, int nbt, bool fwd)
{
   R c = c_code<R>();
   R dn = fwd ? -Lim<R>::large * dmax / c : Lim<R>::large * dmax / c;
   for (int b = 0; b < nbt; b++) {
      R delta = bv.ld(b).delta;
      if (fwd) { if (delta <= R(0) && delta > dn) dn = delta; }
      else { if (delta >= R(0) && delta < dn) dn = delta; }
   }
   if (fwd) { if (dt >= -dn) dt = m_max(-(R(1) + Lim<R>::little) * dn, Lim<R>::small * dmax / c); }
   else { if (dt >= dn) dt = m_max((R(1) + Lim<R>::little) * dn, Lim<R>::small * dmax / c); }
   return dt;
}

// UpdateBmagExtrema (src/trajectory_base.cc:586-592) of the previous step: the reference folds in the
// fields each advanced step ends with, which are this step's start fields; a retried step's start was
// folded in already. Out of line behind a branch on the run configuration: inlined, the compiler
// predicates the double comparisons and conversion into every step of every kernel.
static __device__ __noinline__ void fold_bmag(Start& s0, double bmag)
{
   s0.bmag_min = fmin(s0.bmag_min, bmag);
   s0.bmag_max = fmax(s0.bmag_max, bmag);
}

template <class R>
__device__ __forceinline__ void track_bmag(Start& s0, const RunConfig& cfg, const SD<R>& sp)
{
   if (cfg.track_bmag) fold_bmag(s0, (double)sp.Bmag);
}

// Integrate's time-step check (src/trajectory_base.cc:979-983) of the previous step: dt against the
// dmax of the point where that step ended. That point is where this step starts, so the dmax of
// this step's field evaluation is the same number the reference compares with; a failed check
// discards the attempt before anything else of this step happens.
template <class R, class A>
__device__ __forceinline__ bool prev_step_ok(Lane<R, A>& L, R dmax)
{
   if (L.steps > 0 && !(L.dt >= Lim<R>::tiny * dmax / c_code<R>())) {
      L.status |= TRAJ_DISCARD;
      return false;
   }
   return true;
}

// ---- Parker (src/trajectory_parker.cc:83-306) ----------------------------------------------
template <int BG, class R>
__device__ __noinline__ bool parker_divk_fd(const ProblemDescT<R>& P, int deriv_mode, R t, V3<R> pos, R p, R vmag,
                                            const SD<R>& sp, V3<R>& divK)
{
   // TRAJ_PARKER_DIVK_METHOD 0 (src/trajectory_parker.cc:87-119): central differences of the tensor
   R delta = m_min(larmor(p, sp.Bmag), sp.dmax);
   R dk[3] = {R(0), R(0), R(0)};
#pragma unroll 1
   for (int j = 0; j < 3; j++) {
      SD<R> sf, sb;
      R pt[3] = {pos.x, pos.y, pos.z};
      pt[j] = pt[j] + delta;
      if (!get_fields<BG>(P.bg, deriv_mode, t, mk(pt[0], pt[1], pt[2]), p, kU | kB, sf)) return false;
      Kap<R> kf = kappa_pp(P.df, mk(pt[0], pt[1], pt[2]), p, vmag, kap_in(sf));
      pt[j] -= R(2) * delta;
      if (!get_fields<BG>(P.bg, deriv_mode, t, mk(pt[0], pt[1], pt[2]), p, kU | kB, sb)) return false;
      Kap<R> kb = kappa_pp(P.df, mk(pt[0], pt[1], pt[2]), p, vmag, kap_in(sb));
      for (int i = 0; i < 3; i++) {
         R f = kf.perp * (i == j ? R(1) : R(0)) + (kf.para - kf.perp) * sf.bhat[j] * sf.bhat[i];
         R b = kb.perp * (i == j ? R(1) : R(0)) + (kb.para - kb.perp) * sb.bhat[j] * sb.bhat[i];
         dk[i] += R(0.5) * (f - b) / delta;
      }
   }
   divK = mk(dk[0], dk[1], dk[2]);
   return true;
}

template <int BG, int DK, int BL, class R, class A>
__device__ __forceinline__ void parker_advance(Lane<R, A>& L, BndView<R> bv, Start& s0,
                                               const ProblemDescT<R>& P, const ProblemDesc& Pd, const RunConfig& cfg,
                                               const Sinks& S)
{
   constexpr bool kFP64 = sizeof(R) == sizeof(double);
   const bool fwd = cfg.time_flow == 0;
   const int deriv_mode = kFP64 ? cfg.deriv_mode : 1;
   V3<R> pos = val3<R>(L.pos);
   R p = (R)acc_val(L.mom.x);
   R t = (R)acc_val(L.t);
   SD<R> sp;
   const unsigned mask = traj_mask<kParker>() | (kappa_grad_is_analytic(P.df, DK) ? kDerivedOnly : 0u);
   if (!get_fields<BG>(P.bg, deriv_mode, t, pos, p, mask, sp)) { L.status |= TRAJ_DISCARD; return; }
   if (!prev_step_ok(L, sp.dmax)) return;
   track_bmag(s0, cfg, sp);
   R vmag = vel_of(p);
   // DiffusionCoeff (src/trajectory_parker.cc:83-153)
   Kap<R> K = kappa_pp<R, DK>(P.df, pos, p, vmag, kap_in(sp));
   V3<R> divK;
   if (kFP64 && deriv_mode == 0) {
      if (!parker_divk_fd<BG>(P, deriv_mode, t, pos, p, vmag, sp, divK)) { L.status |= TRAJ_DISCARD; return; }
   }
   else {
      // TRAJ_PARKER_DIVK_METHOD 1 (src/trajectory_parker.cc:120-140)
      V3<R> gpe, gpa;
      kappa_grad<R, false, DK>(P.df, pos, p, vmag, sp, K, gpe, gpa);
      V3<R> t1 = gpa - gpe;
      divK = (gpe + dot(sp.bhat, t1) * sp.bhat) + (K.para - K.perp) * (sd_divbhat(sp) * sp.bhat + sd_b_gradbhat(sp));
   }
   V3<R> slope = fwd ? sp.U + divK : sp.U - divK;
   R divU = sd_divU(sp);
   R slope_p = -p * divU / R(3);
   R sa = R(0);
   if (P.src.kind == 1) sa = P.src.rate;  // SourceConstant: S0 every step (src/source_other.cc:41-59)
   else if (P.src.kind >= 2) {
      // TrajectoryParkerSource::Slopes / SourceMomentumInjection::EvaluateSource
      // (src/trajectory_parker_source.cc:58-66, src/source_other.cc:113-119); dt is the previous step's.
      // SourceSphericalShockInjection (:166-177) injects only inside the shell r_sh <= |r - r0| <= r_sh + w_sh.
      R del = p - P.src.p_inj;
      if (del * L.src_del_old < R(0)) {
         if (P.src.kind == 2) sa = P.src.rate / L.dt;
         else {
            R r = norm(pos - ld3(P.src.r0));
            if (P.src.r_sh <= r && r <= P.src.r_sh + P.src.w_sh) sa = P.src.rate / L.dt;
         }
      }
      L.src_del_old = del;
   }
   // PhysicalStep (src/trajectory_parker.cc:212-221)
   R dtp = R(0.5) * sp.dmax / norm(slope);
   dtp = m_min(dtp, R(0.5) * (sp.dmax * sp.dmax) / m_max(K.perp, K.para));
   dtp = m_min(dtp, R(0.5) * R(3) * R(0.01) / m_abs(divU));
   L.dt = time_proximity(m_min(dtp, L.dt_adapt), sp.dmax, bv, n_time_bnd<BL>(P), fwd);
   // EulerDiffSlopes (src/trajectory_parker.cc:159-180)
   R n[4];
   normals4<R>(rng_block(P.seed, L.steps, L.traj_id, P.problem_id, kRngStep, L.attempt), n);
   R sdt = m_sqrt(L.dt);
   R sperp = m_sqrt(R(2) * K.perp), spara = m_sqrt(R(2) * K.para);
   // the reference's field-aligned basis (GetSecondUnitVec): n0, n1 across, n2 along the field
   V3<R> fa[3];
   fa[2] = sp.bhat;
   fa[0] = second_unit(sp.bhat);
   fa[1] = cross(fa[2], fa[0]);
   R dWx = sdt * n[0], dWy = sdt * n[1], dWz = sdt * n[2];
   V3<R> dr = from_basis(mk(sperp * dWx, sperp * dWy, spara * dWz), fa);
   // RKStep with the Euler table, then the stochastic displacement
   R dts = L.dt * R(1);
   if (fwd) {
      acc_add(L.t, L.dt);
      if constexpr (kFP64) {
         acc_add(L.pos.x, dts * slope.x); acc_add(L.pos.y, dts * slope.y); acc_add(L.pos.z, dts * slope.z);
         acc_add(L.mom.x, dts * slope_p);
         acc_add(L.pos.x, dr.x); acc_add(L.pos.y, dr.y); acc_add(L.pos.z, dr.z);
      }
      else {
         add3(L.pos, dts * slope + dr);
         acc_add(L.mom.x, dts * slope_p);
      }
   }
   else {
      acc_add(L.t, -L.dt);
      if constexpr (kFP64) {
         acc_add(L.pos.x, -(dts * slope.x)); acc_add(L.pos.y, -(dts * slope.y)); acc_add(L.pos.z, -(dts * slope.z));
         acc_add(L.mom.x, -(dts * slope_p));
         acc_add(L.pos.x, dr.x); acc_add(L.pos.y, dr.y); acc_add(L.pos.z, dr.z);
      }
      else {
         add3(L.pos, dr - dts * slope);
         acc_add(L.mom.x, -(dts * slope_p));
      }
   }
   if (sa != R(0)) L.amp += dts * sa * m_exp(L.wgt);
   handle_boundaries<kParker, BL>(L, bv, sp, s0, P, Pd, S);
   L.steps++;
}

// ---- Runge-Kutta advance for Lorentz and Focused (src/trajectory_base.cc:315-406, 545-579) ----
// Butcher tables. FixedRk: Euler (S = 1) and the classic fourth-order table (S = 4), with their
// coefficients as constants so that every stage unrolls into registers. TableRk: any table of
// spx_rk_tables.h (the general-table FP64 kernels), read from constant memory; its slopes live in
// local memory and its adaptive tables estimate the error and reject steps (RKStep,
// src/trajectory_base.cc:366-406).
template <int S>
struct FixedRk {
   static constexpr int kMax = S;
   static constexpr bool kGeneral = false;
   __host__ __device__ static constexpr int stages() { return S; }
   template <class R> __device__ __forceinline__ R a(int s) const { return s == 0 ? R(0) : (s == 3 ? R(1) : R(0.5)); }
   template <class R> __device__ __forceinline__ R b(int s, int l) const
   {
      return (s == 1 && l == 0) ? R(0.5) : ((s == 2 && l == 1) ? R(0.5) : ((s == 3 && l == 2) ? R(1) : R(0)));
   }
   template <class R> __device__ __forceinline__ R v(int l) const
   {
      return S == 1 ? R(1) : ((l == 0 || l == 3) ? R(1.0 / 6.0) : R(1.0 / 3.0));
   }
};

static __constant__ double c_rk_coeffs[] = SPX_RK_COEFFS_INIT;

struct TableRk {
   static constexpr int kMax = SPX_RK_MAX_STAGES;
   static constexpr bool kGeneral = true;
   int s, order, adaptive, off;
   __device__ __forceinline__ int stages() const { return s; }
   template <class R> __device__ __forceinline__ R a(int i) const { return (R)c_rk_coeffs[off + i]; }
   template <class R> __device__ __forceinline__ R b(int i, int j) const { return (R)c_rk_coeffs[off + s + i * (i - 1) / 2 + j]; }
   template <class R> __device__ __forceinline__ R v(int j) const { return (R)c_rk_coeffs[off + s + s * (s - 1) / 2 + j]; }
   template <class R> __device__ __forceinline__ R w(int j) const { return (R)c_rk_coeffs[off + 2 * s + s * (s - 1) / 2 + j]; }
};

// RKStep's adaptive control (common/rk_config.hh:25-34, src/trajectory_base.cc:391-404): the error
// of the step's position against its lower-order estimate, the next dt_adaptive, and whether the
// step is rejected. Consecutive rejections beyond max_time_adaptations (src/trajectory_base.hh:41)
// discard the attempt.
template <class R, class A>
__device__ __forceinline__ bool rk_rejects(Lane<R, A>& L, V3<R> pos, V3<R> pos_lo, int order)
{
   R e = R(1e-9) + R(1e-9) * (norm(pos) + norm(pos_lo));
   e = m_sqrt(norm2(pos - pos_lo) / (e * e));
   L.dt_adapt = L.dt * R(0.995) * m_pow(e, R(-1) / R(order));
   L.dt_adapt = m_min(L.dt * R(2), L.dt_adapt);
   L.dt_adapt = m_max(L.dt / R(2), L.dt_adapt);
   if (e > R(1) + Lim<R>::tiny) {
      L.status &= ~TRAJ_FINISH;
      if (++L.n_adapt > 100u) L.status |= TRAJ_DISCARD;
      return true;
   }
   L.n_adapt = 0;
   return false;
}

// ---- Parker with any Butcher table (src/trajectory_parker.cc:255-306) ---------------------------
// TrajectoryParker::Slopes at one point (src/trajectory_parker.cc:229-245): DriftCoeff, DiffusionCoeff
// (the divergence of the diffusion tensor by central differences in the reference's derivative
// method, else from the analytic gradients), the position slope U +- div K and the momentum slope
// -p div U / 3.
template <int BG, class R>
__device__ __forceinline__ bool parker_slopes(const ProblemDescT<R>& P, int deriv_mode, R t, V3<R> pos, R p,
                                              const SD<R>& sp, bool fwd, Kap<R>& K, V3<R>& slope, R& slope_p)
{
   const R vmag = vel_of(p);
   K = kappa_pp(P.df, pos, p, vmag, kap_in(sp));
   V3<R> divK;
   if (sizeof(R) == sizeof(double) && deriv_mode == 0) {
      if (!parker_divk_fd<BG>(P, deriv_mode, t, pos, p, vmag, sp, divK)) return false;
   }
   else {
      V3<R> gpe, gpa;
      kappa_grad(P.df, pos, p, vmag, sp, K, gpe, gpa);
      V3<R> t1 = gpa - gpe;
      divK = (gpe + dot(sp.bhat, t1) * sp.bhat) + (K.para - K.perp) * (sd_divbhat(sp) * sp.bhat + sd_b_gradbhat(sp));
   }
   slope = fwd ? sp.U + divK : sp.U - divK;
   slope_p = -p * sd_divU(sp) / R(3);
   return true;
}

// The amplitude slope of TrajectoryParkerSource at one point (src/trajectory_parker_source.cc:58-66,
// src/source_other.cc:41-59, 113-119, 166-177): the source's rate with the lane's dt; the injection
// sources remember the momentum of their last evaluation, the stage points' included.
template <class R, class A>
__device__ __forceinline__ R parker_source(Lane<R, A>& L, const ProblemDescT<R>& P, R p, V3<R> pos)
{
   R sa = R(0);
   if (P.src.kind == 1) sa = P.src.rate;
   else if (P.src.kind >= 2) {
      const R del = p - P.src.p_inj;
      if (del * L.src_del_old < R(0)) {
         if (P.src.kind == 2) sa = P.src.rate / L.dt;
         else {
            const R r = norm(pos - ld3(P.src.r0));
            if (P.src.r_sh <= r && r <= P.src.r_sh + P.src.w_sh) sa = P.src.rate / L.dt;
         }
      }
      L.src_del_old = del;
   }
   return sa;
}

// The slopes of the step's start, PhysicalStep, the stochastic displacement (EulerDiffSlopes, with
// the trajectory's next step block: a rejected step draws one too, as the reference draws its next
// three normals), RKSlopes with the Parker slopes at every stage point, RKStep (an adaptive table may
// reject the step), then the displacement and the boundaries. FP64 only.
template <int BG, class R, class A>
__device__ __forceinline__ void parker_advance_gt(Lane<R, A>& L, BndView<R> bv, Start& s0, const ProblemDescT<R>& P,
                                                  const ProblemDesc& Pd, const RunConfig& cfg, const Sinks& S,
                                                  const TableRk tab)
{
   const bool fwd = cfg.time_flow == 0;
   const int deriv_mode = cfg.deriv_mode;
   const unsigned mask = traj_mask<kParker>() | (kappa_grad_is_analytic(P.df) ? kDerivedOnly : 0u);
   const A t_loc = L.t;
   const AV3<A> pos_loc = L.pos, mom_loc = L.mom;
   const V3<R> pos = val3<R>(L.pos);
   const R p = (R)acc_val(L.mom.x);
   SD<R> sp;
   if (!get_fields<BG>(P.bg, deriv_mode, (R)acc_val(L.t), pos, p, mask, sp)) { L.status |= TRAJ_DISCARD; return; }
   if (!prev_step_ok(L, sp.dmax)) return;
   track_bmag(s0, cfg, sp);
   V3<R> slp[SPX_RK_MAX_STAGES];
   R slm[SPX_RK_MAX_STAGES], sla[SPX_RK_MAX_STAGES];
   Kap<R> K;
   if (!parker_slopes<BG>(P, deriv_mode, (R)acc_val(L.t), pos, p, sp, fwd, K, slp[0], slm[0])) {
      L.status |= TRAJ_DISCARD;
      return;
   }
   sla[0] = parker_source(L, P, p, pos);  // with the previous step's dt, as the reference has it
   // PhysicalStep (src/trajectory_parker.cc:212-221)
   R dtp = R(0.5) * sp.dmax / norm(slp[0]);
   dtp = m_min(dtp, R(0.5) * (sp.dmax * sp.dmax) / m_max(K.perp, K.para));
   dtp = m_min(dtp, R(0.5) * R(3) * R(0.01) / m_abs(sd_divU(sp)));
   L.dt = time_proximity(m_min(dtp, L.dt_adapt), sp.dmax, bv, P.nbt, fwd);
   // EulerDiffSlopes (src/trajectory_parker.cc:159-180)
   R n[4];
   normals4<R>(rng_block(P.seed, L.nrm++, L.traj_id, P.problem_id, kRngStep, L.attempt), n);
   const R sdt = m_sqrt(L.dt);
   const R sperp = m_sqrt(R(2) * K.perp), spara = m_sqrt(R(2) * K.para);
   V3<R> fa[3];
   fa[2] = sp.bhat;
   fa[0] = second_unit(sp.bhat);
   fa[1] = cross(fa[2], fa[0]);
   const V3<R> dr = from_basis(mk(sperp * (sdt * n[0]), sperp * (sdt * n[1]), spara * (sdt * n[2])), fa);
   // RKSlopes; sp holds the latest stage's fields, which the events of a crossing read
#pragma unroll 1
   for (int is = 1; is < tab.s; is++) {
#pragma unroll 1
      for (int il = 0; il < is; il++) {
         const R ds = L.dt * tab.template b<R>(is, il);
         const R dta = tab.template a<R>(is) * L.dt;
         if (fwd) { acc_add(L.t, dta); add3(L.pos, ds * slp[il]); acc_add(L.mom.x, ds * slm[il]); }
         else { acc_add(L.t, -dta); add3(L.pos, R(-1) * (ds * slp[il])); acc_add(L.mom.x, -(ds * slm[il])); }
      }
      if (space_terminate<kParker>(L, bv, sp, s0, P, Pd, S)) return;
      const V3<R> ps = val3<R>(L.pos);
      const R pst = (R)acc_val(L.mom.x), ts = (R)acc_val(L.t);
      Kap<R> Ks;
      if (!get_fields<BG>(P.bg, deriv_mode, ts, ps, pst, mask, sp) ||
          !parker_slopes<BG>(P, deriv_mode, ts, ps, pst, sp, fwd, Ks, slp[is], slm[is])) {
         L.status |= TRAJ_DISCARD;
         return;
      }
      sla[is] = parker_source(L, P, pst, ps);
      L.t = t_loc;
      L.pos = pos_loc;
      L.mom = mom_loc;
   }
   // RKStep
   if (fwd) acc_add(L.t, L.dt); else acc_add(L.t, -L.dt);
   V3<R> pos_lo = val3<R>(L.pos);
#pragma unroll 1
   for (int il = 0; il < tab.s; il++) {
      const R w = L.dt * tab.template v<R>(il);
      if (fwd) { add3(L.pos, w * slp[il]); acc_add(L.mom.x, w * slm[il]); }
      else { add3(L.pos, R(-1) * (w * slp[il])); acc_add(L.mom.x, -(w * slm[il])); }
      if (tab.adaptive) {
         const R wl = L.dt * tab.template w<R>(il);
         pos_lo = fwd ? pos_lo + wl * slp[il] : pos_lo - wl * slp[il];
      }
      if (sla[il] != R(0)) L.amp += L.dt * tab.template v<R>(il) * sla[il] * m_exp(L.wgt);
   }
   if (tab.adaptive && rk_rejects(L, val3<R>(L.pos), pos_lo, tab.order)) {
      // back to the stored point; the amplitude keeps the rejected increment, as in the reference
      L.t = t_loc;
      L.pos = pos_loc;
      L.mom = mom_loc;
      return;
   }
   acc_add(L.pos.x, dr.x); acc_add(L.pos.y, dr.y); acc_add(L.pos.z, dr.z);
   handle_boundaries<kParker, kLayoutAny>(L, bv, sp, s0, P, Pd, S);
   L.steps++;
}

template <int TT, class R>
__device__ __forceinline__ V3<R> vel_load(V3<R> mom)
{
   if (TT == kFocused) { R v = vel_of(mom.x); return (v / mom.x) * mom; }  // Vel<SphericalRMP>
   return vel_cart(mom);
}

// TrajectoryFocused::DriftCoeff (src/trajectory_focused.cc:62-80)
template <class R>
__device__ __forceinline__ V3<R> focused_drift(const SD<R>& s, V3<R> mom, V3<R> vel)
{
   // the operations in the reference's order: ((0.5 st2) (b x grad B)) / B and ((0.5 st2) b) (B . curl B)
   R ct2 = mom.y * mom.y, st2 = R(1) - ct2;
   V3<R> dv = ((R(0.5) * st2) * cross(s.bhat, s.gradBmag)) / s.Bmag;
   V3<R> cur = dot(s.B, sd_curlB(s)) * ((R(0.5) * st2) * s.bhat) + ct2 * cross(s.bhat, vm(s.B, s.gradB));
   dv = dv + cur / (s.Bmag * s.Bmag);
   dv = (larmor(mom.x, s.Bmag) * vel.x) * dv;
   return dv + (s.U + (vel.x * mom.y) * s.bhat);
}

// TrajectoryGuiding::ModifiedFields and DriftCoeff (src/trajectory_guiding.cc:60-96) and the momentum
// slopes of Slopes with PPERP_METHOD 1 (:104-117). The backgrounds are static, so dB/dt and dBmag/dt are
// zero; dbhat/dt = (dB/dt - dBmag/dt bhat) / Bmag is still formed from those zeros so that signed zeros
// propagate as in the reference.
template <class R>
__device__ __forceinline__ V3<R> guiding_drift(const SD<R>& s, V3<R> mom, V3<R> vel, R& dp_perp, R& dp_para)
{
   const R c = c_code<R>();
   const R rL = larmor(mom.x, s.Bmag), rR = larmor(mom.z, s.Bmag);
   const V3<R> zero3 = mk(R(0), R(0), R(0));
   V3<R> dbhatdt = (zero3 - R(0) * s.bhat) / s.Bmag;
   V3<R> curlbhat = (sd_curlB(s) - cross(s.gradBmag, s.bhat)) / s.Bmag;
   V3<R> e_star = (s.E - ((rR * s.Bmag) * dbhatdt) / c) - ((rL * vel.x) * s.gradBmag) / (R(2) * c);
   V3<R> b_star = s.B + (rR * s.Bmag) * curlbhat;
   R bsb = dot(b_star, s.bhat);
   V3<R> drift = (vel.z * b_star + c * cross(e_star, s.bhat)) / bsb;
   dp_perp = R(0.5) * mom.x / s.Bmag * (R(0) + dot(drift, s.gradBmag));
   dp_para = dot(e_star, b_star) / bsb;  // the proton's charge is 1 in code units
   return drift;
}

// TrajectoryGuidingDiff::DiffusionCoeff (src/trajectory_guiding_diff.cc:61-86): the field-aligned frame,
// D_perp (diffusion component 0) and the perpendicular part of its gradient, V_perp.
template <class R>
__device__ __forceinline__ V3<R> guiding_vperp(const DiffParamsT<R>& df, const SD<R>& s, V3<R> pos, V3<R> mom, R& d_perp,
                                               V3<R> (&fa)[3])
{
   const R p = m_sqrt(mom.x * mom.x + mom.z * mom.z);  // ConvertMomentum()[0]
   const R vmag = vel_of(p);
   const R mu = mom.z / norm(mom), Omega = cyclotron(vmag, s.Bmag);  // ConvertMomentum()[1], CyclotronFrequency
   Kap<R> K = kappa_pp(df, pos, p, vmag, kap_in(s), mu, Omega);
   V3<R> gpe, gpa;
   kappa_grad<R, true>(df, pos, p, vmag, s, K, gpe, gpa, mu, Omega);
   fa[2] = s.bhat;
   fa[0] = second_unit(s.bhat);
   fa[1] = cross(fa[2], fa[0]);
   d_perp = K.perp;
   return from_basis(mk(dot(gpe, fa[0]), dot(gpe, fa[1]), R(0)), fa);
}

// sqrt(2 D_perp) at a displaced point (src/trajectory_guiding_diff.cc:152-155): the fields there, then diffusion
// component 0 with the step's momentum. "dmax" receives that evaluation's dmax, which the background's
// GetSafeIncr reads for the next increment (src/background_base.cc:409-413). The reference evaluates these
// points into a record whose field mask is uninitialised; here it is the trajectory's mask.
template <int BG, class R>
__device__ __noinline__ R perp_slope_at(const ProblemDescT<R>& P, int deriv_mode, R t, V3<R> pos, V3<R> mom, R& dmax, bool& ok)
{
   SD<R> s;
   if (!get_fields<BG>(P.bg, deriv_mode, t, pos, norm(mom), traj_mask<kGuiding>(), s)) {
      ok = false;
      return R(0);
   }
   dmax = s.dmax;
   const R p = m_sqrt(mom.x * mom.x + mom.z * mom.z);
   const R vmag = vel_of(p);
   const Kap<R> K = kappa_pp(P.df, pos, p, vmag, kap_in(s), mom.z / norm(mom), cyclotron(vmag, s.Bmag));
   return m_sqrt(R(2) * K.perp);
}

// The trajectory's next uniform deviate: component k % 4 of set-up block k / 4, the count continuing from the
// initial conditions (the reference draws every uniform from one generator, common/random.hh:99-122).
template <class R, class A>
__device__ __forceinline__ double lane_uniform(const Lane<R, A>& L, Start& s0, uint64_t seed, uint32_t problem_id)
{
   const uint32_t k = s0.nuni++;
   const uint4 b = rng_block(seed, k >> 2, L.traj_id, problem_id, kRngInit, L.attempt);
   return u01d((k & 3) == 0 ? b.x : ((k & 3) == 1 ? b.y : ((k & 3) == 2 ? b.z : b.w)));
}

template <int TT, class R>
__device__ __forceinline__ void rk_slopes(const SD<R>& s, V3<R> mom, V3<R> vel, V3<R>& sp, V3<R>& sm, V3<R>& drift)
{
   if (TT == kLorentz) {  // src/trajectory_lorentz.cc:67-71
      sp = vel;
      sm = s.E + cross(vel, s.B) / c_code<R>();
   }
   else if (TT == kFieldline) {  // src/trajectory_fieldline.cc:58-66: along b at the parallel speed
      sp = vel.z * s.bhat;
      sm = mk(R(0), R(0), R(0));
   }
   else if (TT == kGuiding) {
      R dpp, dpl;
      drift = guiding_drift(s, mom, vel, dpp, dpl);
      sp = drift;
      sm = mk(dpp, R(0), dpl);
   }
   else {  // src/trajectory_focused.cc:100-128
      drift = focused_drift(s, mom, vel);
      sp = drift;
      // bb : grad U as GeoMatrix::operator% sums it, row by row (common/matrix.hh:556-561)
      R st2 = R(1) - mom.y * mom.y, bbgu = R(0);
#pragma unroll
      for (int i = 0; i < 3; i++)
         bbgu += (s.bhat[i] * s.bhat[0] * s.gradU.m[i][0] + s.bhat[i] * s.bhat[1] * s.gradU.m[i][1]) +
                 s.bhat[i] * s.bhat[2] * s.gradU.m[i][2];
      V3<R> cd = s.dUdt + vm(s.U, s.gradU);
      R bcd = R(2) * dot(s.bhat, cd) / vel.x;
      R divU = sd_divU(s);
      sm.x = R(0.5) * mom.x * ((R(3) * st2 - R(2)) * bbgu - st2 * divU - mom.y * bcd);
      sm.y = R(0.5) * st2 * (vel.x * sd_divbhat(s) - bcd + mom.y * (divU - R(3) * bbgu));
      sm.z = R(0);
   }
}

template <class A, class R>
__device__ __forceinline__ void clamp_mu(AV3<A>& mom)
{
   // TrajectoryFocused::MomentumCorrection (src/trajectory_focused.cc:146-156)
   R mu = (R)acc_val(mom.y);
   if (mu > R(1)) acc_setf(mom.y, R(1));
   else if (mu < R(-1)) acc_setf(mom.y, R(-1));
}

// NODIFF: compiled for a type without pitch-angle scattering and perpendicular diffusion (TrajectoryGuiding
// proper), so neither step is in the kernel.
template <int TT, int BG, class R, class A, class TAB, bool NODIFF = false>
__device__ __forceinline__ void rk_advance(Lane<R, A>& L, BndView<R> bv, Start& s0, const ProblemDescT<R>& P,
                                           const ProblemDesc& Pd, const RunConfig& cfg, const Sinks& S, const TAB tab)
{
   constexpr bool kFP64 = sizeof(R) == sizeof(double);
   const bool fwd = cfg.time_flow == 0;
   const int deriv_mode = kFP64 ? cfg.deriv_mode : 1;
   const bool scatt = !NODIFF && (TT == kFocused || TT == kGuiding) && cfg.pa_scattering;
   // TrajectoryGuidingDiff / GuidingDiffScatt: perpendicular diffusion on top of the guiding-centre step
   const bool gc_perp = !NODIFF && TT == kGuiding && (cfg.traj_kind == kGuidingDiff || cfg.traj_kind == kGuidingDiffScatt);
   SD<R> sp;
   V3<R> mom = lane_mom(L);
   // the last stored point's momentum (the pitch-angle step below changes it before the stages): a
   // rejected step returns to it, as the reference's Load() does
   [[maybe_unused]] const AV3<A> mom_stored = L.mom;
   if (!get_fields<BG>(P.bg, deriv_mode, (R)acc_val(L.t), val3<R>(L.pos), field_p<TT>(mom), traj_mask<TT>(), sp)) {
      L.status |= TRAJ_DISCARD;
      return;
   }
   // the guiding-centre mask has no grad U, which the diffusion models then see as zero, as in the reference
   if (gc_perp) zero(sp.gradU);
   R d_perp = R(0);
   V3<R> fa[3];
   if (!prev_step_ok(L, sp.dmax)) return;
   track_bmag(s0, cfg, sp);
   V3<R> vel = vel_load<TT>(mom);
   V3<R> drift = mk(R(0), R(0), R(0));
   if (scatt) {
      // TrajectoryGuidingScatt::Advance (src/trajectory_guiding_scatt.cc:277-310): coefficients, the
      // mu-CFL, then the Euler pitch-angle step (:61-84); Focused composes the same step
      R pmag, mu;
      if (TT == kGuiding) { pmag = m_sqrt(mom.x * mom.x + mom.z * mom.z); mu = mom.z / norm(mom); }  // ConvertMomentum
      else { pmag = mom.x; mu = mom.y; }
      R vmag = vel_of(pmag);
      R Omega = cyclotron(vmag, sp.Bmag);
      const V3<R> pos0 = val3<R>(L.pos);
      R Dmumu = kappa_mumu(P.df, pos0, vmag, Omega, mu);
      R Vmu = kappa_mumu_dmu(P.df, pos0, vmag, Omega, mu, Dmumu);
      R dtp;
      if (TT == kGuiding) {
         R d1, d2;
         drift = guiding_drift(sp, mom, vel, d1, d2);
         if (gc_perp) {
            // TrajectoryGuidingDiffScatt::Advance: DiffusionCoeff, DriftCoeff, then GuidingDiff::PhysicalStep
            // (src/trajectory_guiding_diff.cc:343-351) before the pitch-angle limits
            V3<R> vp = guiding_vperp(P.df, sp, val3<R>(L.pos), mom, d_perp, fa);
            V3<R> dv = fwd ? drift + vp : drift - vp;
            dtp = R(0.5) * sp.dmax / (norm(dv) + R(0.5) * norm(vel));
            dtp = m_min(dtp, R(0.5) * (sp.dmax * sp.dmax) / d_perp);
         }
         else dtp = R(0.5) * sp.dmax / (norm(drift) + R(0.5) * norm(vel));
      }
      else {
         drift = focused_drift(sp, mom, vel);
         dtp = R(0.5) * sp.dmax / (norm(drift) + R(0.5) * vel.x);
      }
      const R dth = R(2.0 * 3.141592653589793238462643383279502884 / 180.0);
      R amu = m_abs(mu);
      R dmumax = m_sqrt(R(1) - amu) * dth + R(0.5) * amu * (dth * dth);
      dtp = m_min(dtp, R(0.5) * (dmumax * dmumax) / Dmumu);
      dtp = m_min(dtp, R(0.5) * dmumax / m_abs(Vmu));
      L.dt = time_proximity(m_min(dtp, L.dt_adapt), sp.dmax, bv, P.nbt, fwd);
      R n[4];
      R sq = m_sqrt(R(2) * Dmumu * L.dt);
      R mu_new;
      if (TT == kGuiding) {
         // the k-th normal of the trajectory, redraws included, is the first of step block k; the
         // schemes of src/trajectory_guiding_scatt.cc:61-247 redraw while |mu| > 1 (here at most 256 times).
         // Their finite differences in mu shift by sp_small = 1e-8, below float resolution, so the FP32
         // kernels shift by 1e-3.
         const R ds = sizeof(R) == sizeof(double) ? Lim<R>::small : R(1e-3);
         int tries = 0;
         if (cfg.mu_method == 1) {  // MilsteinPitchAngleScatt (:91-130)
            const R b = m_sqrt(R(2) * Dmumu);
            const R dmu = ds * (mu + ds < R(1) ? R(1) : R(-1));
            const R b1 = (m_sqrt(R(2) * kappa_mumu(P.df, pos0, vmag, Omega, mu + dmu)) - b) / dmu;
            do {
               normals4<R>(rng_block(P.seed, L.nrm++, L.traj_id, P.problem_id, kRngStep, L.attempt), n);
               const R dw = m_sqrt(L.dt) * n[0];
               mu_new = mu + Vmu * L.dt + b * dw + R(0.5) * b * b1 * (dw * dw - L.dt);
            } while (m_abs(mu_new) > R(1) && ++tries < 256);
         }
         else if (cfg.mu_method == 2) {  // RK2PitchAngleScatt (:137-247)
            const R g = R(1) / m_sqrt(R(3));
            const R sv0 = Vmu, sd0 = m_sqrt(R(2) * Dmumu);
            R sv1 = R(0), sd1 = R(0), sd2 = R(0);
            do {
               normals4<R>(rng_block(P.seed, L.nrm++, L.traj_id, P.problem_id, kRngStep, L.attempt), n);
               const R dw = m_sqrt(L.dt) * n[0];
               mu_new = mu + sd0 * dw;
               mu_new += sv0 * L.dt;
               if (m_abs(mu_new) > R(1)) continue;
               const R d = kappa_mumu(P.df, pos0, vmag, Omega, mu_new);
               R dmu = ds * (mu_new + ds < R(1) ? R(1) : R(-1));
               sv1 = (kappa_mumu(P.df, pos0, vmag, Omega, mu_new + dmu) - d) / dmu;
               mu_new = mu + g * sd0 * dw;
               mu_new += sv0 * L.dt;
               if (m_abs(mu_new) > R(1)) continue;
               sd1 = m_sqrt(R(2) * kappa_mumu(P.df, pos0, vmag, Omega, mu_new));
               mu_new = mu - sd0 / (R(3) * g) * dw;
               mu_new += sv0 * L.dt;
               if (m_abs(mu_new) > R(1)) continue;
               sd2 = m_sqrt(R(2) * kappa_mumu(P.df, pos0, vmag, Omega, mu_new));
               dmu = ds * (mu + ds < R(1) ? R(1) : R(-1));
               const R dfit = (m_sqrt(R(2) * kappa_mumu(P.df, pos0, vmag, Omega, mu + dmu)) - sd0) / dmu;
               mu_new = mu + (R(0.5) * sd0 + (sd1 + R(3) * (g * g) * sd2) / (R(2) + R(6) * (g * g))) * dw;
               mu_new += R(0.5) * L.dt * (sv0 + sv1);
               mu_new += R(0.5) * sd0 * dfit * (dw * dw - L.dt);
            } while (m_abs(mu_new) > R(1) && ++tries < 256);
         }
         else {  // EulerPitchAngleScatt (:61-84)
            do {
               normals4<R>(rng_block(P.seed, L.nrm++, L.traj_id, P.problem_id, kRngStep, L.attempt), n);
               mu_new = mu + Vmu * L.dt + sq * n[0];
            } while (m_abs(mu_new) > R(1) && ++tries < 256);
         }
      }
      else {
         normals4<R>(rng_block(P.seed, L.steps, L.traj_id, P.problem_id, kRngStep, L.attempt), n);
         mu_new = mu + Vmu * L.dt + sq * n[0];
         int k = 1, blk = 0;
         while (m_abs(mu_new) > R(1) && blk < 64) {
            if (k == 4) {
               normals4<R>(rng_block(P.seed, L.steps * 64u + (uint32_t)blk, L.traj_id, P.problem_id, kRngExtra, L.attempt), n);
               blk++;
               k = 0;
            }
            mu_new = mu + Vmu * L.dt + sq * n[k++];
         }
      }
      if (m_abs(mu_new) > R(1)) mu_new = mu_new > R(0) ? R(1) : R(-1);
      if (TT == kGuiding) {
         acc_setf(L.mom.x, pmag * m_sqrt(R(1) - mu_new * mu_new));
         acc_setf(L.mom.z, pmag * mu_new);
      }
      else acc_setf(L.mom.y, mu_new);
      mom = lane_mom(L);
      vel = vel_load<TT>(mom);
   }
   const A t_loc = L.t;
   const AV3<A> pos_loc = L.pos, mom_loc = L.mom;
   V3<R> slp[TAB::kMax], slm[TAB::kMax];
   rk_slopes<TT>(sp, mom, vel, slp[0], slm[0], drift);
   V3<R> vperp = mk(R(0), R(0), R(0));
   if (gc_perp) {  // TrajectoryGuidingDiff::Slopes (src/trajectory_guiding_diff.cc:327-336)
      vperp = guiding_vperp(P.df, sp, val3<R>(L.pos), mom, d_perp, fa);
      slp[0] = fwd ? slp[0] + vperp : slp[0] - vperp;
   }
   if (!scatt) {
      R dtp;
      if (TT == kLorentz) {  // src/trajectory_lorentz.cc:51-59
         R vn = norm(vel);
         R Om = m_max(cyclotron(vn, sp.Bmag), Lim<R>::tiny);
         R spo = kFP64 ? (R)cfg.steps_per_orbit : (R)cfg.steps_per_orbit_f;
         dtp = R(6.283185307179586476925286766559005768) / Om / spo;
         dtp = m_min(dtp, R(0.1) * sp.dmax / vn);
      }
      else if (TT == kFieldline) {  // src/trajectory_fieldline.cc:47-50, cfl_adv_tf = 0.5
         dtp = R(0.5) * sp.dmax / m_abs(vel.z);
      }
      else if (TT == kGuiding && gc_perp) {  // src/trajectory_guiding_diff.cc:343-351
         V3<R> dv = fwd ? drift + vperp : drift - vperp;
         dtp = R(0.5) * sp.dmax / (norm(dv) + R(0.5) * norm(vel));
         dtp = m_min(dtp, R(0.5) * (sp.dmax * sp.dmax) / d_perp);
      }
      else if (TT == kGuiding) {  // src/trajectory_guiding.cc:81-86
         dtp = R(0.5) * sp.dmax / (norm(drift) + R(0.5) * norm(vel));
      }
      else {  // src/trajectory_focused.cc:87-91
         dtp = R(0.5) * sp.dmax / (norm(drift) + R(0.5) * vel.x);
      }
      L.dt = time_proximity(m_min(dtp, L.dt_adapt), sp.dmax, bv, P.nbt, fwd);
   }
   V3<R> dr_perp = mk(R(0), R(0), R(0));
   if (gc_perp) {
      // EulerPerpDiffSlopes (src/trajectory_guiding_diff.cc:92-107): the next two normals of the trajectory
      R n[4];
      normals4<R>(rng_block(P.seed, L.nrm++, L.traj_id, P.problem_id, kRngStep, L.attempt), n);
      const R dwx = m_sqrt(L.dt) * n[0];
      normals4<R>(rng_block(P.seed, L.nrm++, L.traj_id, P.problem_id, kRngStep, L.attempt), n);
      const R dwy = m_sqrt(L.dt) * n[0];
      const R b0 = m_sqrt(R(2) * d_perp);
      R drx = b0 * dwx, dry = b0 * dwy;
      if (cfg.perp_method == 1 || cfg.perp_method == 2) {
         // MilsteinPerpDiffSlopes (src/trajectory_guiding_diff.cc:129-176) and RK2PerpDiffSlopes (:182-300):
         // one-sided differences of sqrt(2 D_perp) across the field with GetSafeIncr's 1e-4 dmax steps (1e-2
         // in the FP32 kernels, where 1e-4 is below the resolution of the quotients), and one uniform for the
         // sign of the Levy-area stand-in
         const R incr = kFP64 ? R(1e-4) : R(1e-2);
         const R t0 = (R)acc_val(L.t), dt = L.dt;
         const V3<R> x0 = val3<R>(pos_loc);
         const V3<R> xhat = from_basis(mk(R(1), R(0), R(0)), fa), yhat = from_basis(mk(R(0), R(1), R(0)), fa);
         R dmax = sp.dmax, dx, dy, bx, by, dbdx, dbdy;
         bool ok = true;
         if (cfg.perp_method == 1) {
            dx = incr * dmax;
            bx = perp_slope_at<BG>(P, deriv_mode, t0, x0 + dx * xhat, mom, dmax, ok);
            dbdx = (bx - b0) / dx;
            dy = incr * dmax;
            by = perp_slope_at<BG>(P, deriv_mode, t0, x0 + dy * yhat, mom, dmax, ok);
            dbdy = (by - b0) / dy;
            const R vxy = lane_uniform(L, s0, P.seed, P.problem_id) < 0.5 ? dt : -dt;
            drx = b0 * dwx + R(0.5) * b0 * (dbdx * (dwx * dwx - dt) + dbdy * (dwx * dwy - vxy));
            dry = b0 * dwy + R(0.5) * b0 * (dbdy * (dwy * dwy - dt) + dbdx * (dwx * dwy + vxy));
         }
         else {
            const R g = R(1) / m_sqrt(R(3));
            const V3<R> dpos = from_basis(mk(b0 * dwx, b0 * dwy, R(0)), fa);
            // the two trial points; a terminal crossing at either ends the trajectory there (:204-205, :213-214)
            add3(L.pos, g * dpos);
            if (space_terminate<TT>(L, bv, sp, s0, P, Pd, S)) return;
            const R b1 = perp_slope_at<BG>(P, deriv_mode, t0 + dt, val3<R>(L.pos), mom, dmax, ok);
            L.pos = pos_loc;
            add3(L.pos, R(-1) * mk(dpos.x / (R(3) * g), dpos.y / (R(3) * g), dpos.z / (R(3) * g)));
            if (space_terminate<TT>(L, bv, sp, s0, P, Pd, S)) return;
            const R b2 = perp_slope_at<BG>(P, deriv_mode, t0 + dt, val3<R>(L.pos), mom, dmax, ok);
            L.pos = pos_loc;
            dx = incr * dmax;
            const R bxx = perp_slope_at<BG>(P, deriv_mode, t0, x0 + dx * xhat, mom, dmax, ok);
            dx *= R(0.5);
            bx = perp_slope_at<BG>(P, deriv_mode, t0, x0 + dx * xhat, mom, dmax, ok);
            dbdx = (bx - b0) / dx;
            const R d2x = (bxx - R(2) * bx + b0) / (dx * dx);
            dy = incr * dmax;
            const R byy = perp_slope_at<BG>(P, deriv_mode, t0, x0 + dy * yhat, mom, dmax, ok);
            dy *= R(0.5);
            by = perp_slope_at<BG>(P, deriv_mode, t0, x0 + dy * yhat, mom, dmax, ok);
            dbdy = (by - b0) / dy;
            const R d2y = (byy - R(2) * by + b0) / (dy * dy);
            const R bxy = perp_slope_at<BG>(P, deriv_mode, t0, (x0 + dx * xhat) + dy * yhat, mom, dmax, ok);
            const R d2xy = (bxy - bx - by + b0) / (dx * dy);
            const R vxy = lane_uniform(L, s0, P.seed, P.problem_id) < 0.5 ? dt : -dt;
            const R rx = R(0.5) * b0 * (dbdx * (dwx * dwx - dt) + dbdy * (dwx * dwy - vxy)) +
                         dt * (b0 * b0) * (d2y * dwx - d2xy * dwy) / R(6);
            const R ry = R(0.5) * b0 * (dbdy * (dwy * dwy - dt) + dbdx * (dwx * dwy + vxy)) +
                         dt * (b0 * b0) * (d2x * dwy - d2xy * dwx) / R(6);
            const R bmid = R(0.5) * (b0 + (b1 + R(3) * (g * g) * b2) / (R(1) + R(3) * (g * g)));
            drx = bmid * dwx + rx;
            dry = bmid * dwy + ry;
         }
         if (!ok) {
            L.status |= TRAJ_DISCARD;
            return;
         }
      }
      dr_perp = from_basis(mk(drx, dry, R(0)), fa);
   }
   // RKSlopes: stage "is" (false: the trajectory ended or was discarded in it)
   auto stage = [&](int is) -> bool {
#pragma unroll
      for (int il = 0; il < is; il++) {
         R ds = L.dt * tab.template b<R>(is, il);
         R dta = tab.template a<R>(is) * L.dt;
         if (fwd) { acc_add(L.t, dta); add3(L.pos, ds * slp[il]); add3(L.mom, ds * slm[il]); }
         else { acc_add(L.t, -dta); add3(L.pos, R(-1) * (ds * slp[il])); add3(L.mom, R(-1) * (ds * slm[il])); }
      }
      if (space_terminate<TT>(L, bv, sp, s0, P, Pd, S)) return false;
      V3<R> ms = lane_mom(L);
      if (!get_fields<BG>(P.bg, deriv_mode, (R)acc_val(L.t), val3<R>(L.pos), field_p<TT>(ms), traj_mask<TT>(), sp)) {
         L.status |= TRAJ_DISCARD;
         return false;
      }
      if (TT == kFocused) { clamp_mu<A, R>(L.mom); ms = lane_mom(L); }
      V3<R> vs = vel_cart(ms);  // src/trajectory_base.cc:344 uses the Cartesian velocity for every type
      V3<R> dummy;
      rk_slopes<TT>(sp, ms, vs, slp[is], slm[is], dummy);
      if (gc_perp) {
         zero(sp.gradU);
         R dstage;
         V3<R> fstage[3];
         V3<R> vp = guiding_vperp(P.df, sp, val3<R>(L.pos), ms, dstage, fstage);
         slp[is] = fwd ? slp[is] + vp : slp[is] - vp;
      }
      L.t = t_loc;
      L.pos = pos_loc;
      L.mom = mom_loc;
      return true;
   };
   constexpr int kStages = TAB::kGeneral ? 0 : TAB::kMax;
   const int n_stages = TAB::kGeneral ? tab.stages() : kStages;
   if constexpr (TT == kGuiding || (sizeof(R) == sizeof(float) && TT == kLorentz)) {
      // the guiding-centre stages and the FP32 Lorentz ones stay a loop: unrolled, their field and drift
      // evaluations make the step's code large enough that instruction fetch stalls the warps (steady-state
      // steps/s rolled: guiding centre +22%, Lorentz in the dipole +10%; focused transport ran 3.5% slower rolled)
#pragma unroll 1
      for (int is = 1; is < n_stages; is++)
         if (!stage(is)) return;
   }
   else {
#pragma unroll
      for (int is = 1; is < (TAB::kGeneral ? tab.stages() : TAB::kMax); is++)
         if (!stage(is)) return;
   }
   // RKStep
   if (fwd) acc_add(L.t, L.dt); else acc_add(L.t, -L.dt);
   if constexpr (kFP64) {
      [[maybe_unused]] V3<R> pos_lo = val3<R>(L.pos);
#pragma unroll
      for (int il = 0; il < (TAB::kGeneral ? tab.stages() : TAB::kMax); il++) {
         R w = L.dt * tab.template v<R>(il);
         if (fwd) { add3(L.pos, w * slp[il]); add3(L.mom, w * slm[il]); }
         else { add3(L.pos, R(-1) * (w * slp[il])); add3(L.mom, R(-1) * (w * slm[il])); }
         if constexpr (TAB::kGeneral) {
            if (tab.adaptive) {
               R wl = L.dt * tab.template w<R>(il);
               pos_lo = fwd ? pos_lo + wl * slp[il] : pos_lo - wl * slp[il];
            }
         }
      }
      if constexpr (TAB::kGeneral) {
         // an adaptive table may reject the step: back to the stored point, nothing recorded
         if (tab.adaptive && rk_rejects(L, val3<R>(L.pos), pos_lo, tab.order)) {
            L.t = t_loc;
            L.pos = pos_loc;
            L.mom = mom_stored;
            return;
         }
      }
   }
   else {
      V3<R> dp = mk(R(0), R(0), R(0)), dm = mk(R(0), R(0), R(0));
#pragma unroll
      for (int il = 0; il < (TAB::kGeneral ? tab.stages() : TAB::kMax); il++) {
         R w = tab.template v<R>(il);
         dp = dp + w * slp[il];
         dm = dm + w * slm[il];
      }
      R sdt = fwd ? L.dt : -L.dt;
      add3(L.pos, sdt * dp);
      add3(L.mom, sdt * dm);
   }
   if (gc_perp) {  // Advance: _pos += dr_perp after RKStep (src/trajectory_guiding_diff.cc:373)
      if constexpr (kFP64) { acc_add(L.pos.x, dr_perp.x); acc_add(L.pos.y, dr_perp.y); acc_add(L.pos.z, dr_perp.z); }
      else add3(L.pos, dr_perp);
   }
   handle_boundaries<TT, kLayoutAny>(L, bv, sp, s0, P, Pd, S);
   if (!(L.status & TRAJ_FINISH) && TT == kFocused) clamp_mu<A, R>(L.mom);
   L.steps++;
}

// ---- SetStart (src/trajectory_base.cc:867-939 and overrides) -------------------------------
// Works on a lane record of its own (see start_lane) and writes the boundary states of the lane.
template <int TT, int BG, class R, class A>
__device__ __noinline__ void set_start(Lane<R, A>& L, BndView<R> bv, Start& s0, const ProblemDescT<R>& P,
                                       const ProblemDesc& Pd, const RunConfig& cfg, int64_t local)
{
   constexpr bool kFP64 = sizeof(R) == sizeof(double);
   const int deriv_mode = kFP64 ? cfg.deriv_mode : 1;
   L.status = 0;
   L.steps = 0;
   L.nrm = 0;
   L.n_adapt = 0;
   L.amp = R(0);
   L.wgt = R(0);
   L.dt = R(0);
   L.dt_adapt = R(0);
   L.src_del_old = R(0);
   InitRng rng{Pd.seed, L.traj_id, Pd.problem_id, L.attempt, 0u, 0u};
   double t = sample_time(rng, Pd, local);
   V3<double> pos = sample_pos(rng, Pd, local);
   V3<double> mom = sample_mom(rng, Pd, TT, mk(1.0, 1.0, 1.0));
   acc_set(L.t, t);
   acc_set(L.pos.x, pos.x); acc_set(L.pos.y, pos.y); acc_set(L.pos.z, pos.z);
   acc_set(L.mom.x, mom.x); acc_set(L.mom.y, mom.y); acc_set(L.mom.z, mom.z);
   SD<R> sp;
   V3<R> pr = val3<R>(L.pos);
   R pm = (TT == kLorentz || TT == kGuiding) ? (R)norm(mom) : (TT == kFieldline ? (R)fabs(mom.z) : (R)mom.x);
   if (!get_fields<BG>(P.bg, deriv_mode, (R)t, pr, pm, traj_mask<TT>(), sp)) { L.status |= TRAJ_DISCARD; return; }
   V3<double> bh = mk((double)sp.bhat.x, (double)sp.bhat.y, (double)sp.bhat.z);
   mom = sample_mom(rng, Pd, TT, bh);
   if constexpr (TT == kGuiding) s0.nuni = rng.n_uniform;
   acc_set(L.mom.x, mom.x); acc_set(L.mom.y, mom.y); acc_set(L.mom.z, mom.z);
   s0.t0 = t;
   s0.pos0 = pos;
   s0.mom0 = mom;
   s0.bhat0 = bh;
   s0.bmag0 = s0.bmag_min = s0.bmag_max = (double)sp.Bmag;
   R c = c_code<R>();
   L.dt_adapt = Lim<R>::large * sp.dmax / c;
   V3<R> mr = lane_mom(L);
   for (int j = 0; j < P.nbt + P.nbs + P.nbm; j++) {
      R scale = j < P.nbt ? sp.dmax / c : (j < P.nbt + P.nbs ? sp.dmax : norm(mr));
      BndState<R> st;
      reset_bnd(bnd_param(P, j), st, scale, L.t, pr, mr, sp.bhat, sp.region, TT);
      bv.st(j, st);
   }
   // TrajectoryParkerSource::SetStart (src/trajectory_parker_source.cc:43-50)
   if (P.src.kind >= 2) L.src_del_old = mr.x - P.src.p_inj;
}

// ---- the kernel --------------------------------------------------------------------------------
template <class R>
__device__ __forceinline__ int find_problem(const ProblemDescT<R>* P, int n, int64_t g)
{
   int lo = 0, hi = n - 1;
   while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (P[mid].first <= g) lo = mid;
      else hi = mid - 1;
   }
   return lo;
}

// Takes the lane state by value so that the caller's copy stays in registers.
template <class R, class A>
__device__ __noinline__ void write_record(const Lane<R, A> L, const Start& s0, TrajRecord* rec, int64_t g)
{
   TrajRecord r;
   r.attempts = L.attempt + 1;
   r.status = L.status;
   r.steps = L.steps;
   r.t = acc_dbl(L.t);
   r.pos[0] = acc_dbl(L.pos.x); r.pos[1] = acc_dbl(L.pos.y); r.pos[2] = acc_dbl(L.pos.z);
   r.mom[0] = acc_dbl(L.mom.x); r.mom[1] = acc_dbl(L.mom.y); r.mom[2] = acc_dbl(L.mom.z);
   r.t0 = s0.t0;
   r.pos0[0] = s0.pos0.x; r.pos0[1] = s0.pos0.y; r.pos0[2] = s0.pos0.z;
   r.mom0[0] = s0.mom0.x; r.mom0[1] = s0.mom0.y; r.mom0[2] = s0.mom0.z;
   r.amp = (double)L.amp;
   r.logwgt = (double)L.wgt;
   rec[g] = r;
}

// Start (or restart, with a new attempt number) trajectory g on the lane. SetStart fills a
// separate record that is then copied member by member: the lane state proper is never passed by
// address to an out-of-line call, so it lives in registers for the whole kernel.
template <int TT, int BG, class R, class A>
__device__ __forceinline__ void start_lane(Lane<R, A>& L, BndView<R> bv, Start& s0, const ProblemDescT<R>* P,
                                           const ProblemDesc* Pd, const RunConfig& cfg, int64_t g, uint32_t attempt)
{
   Lane<R, A> n;
   n.prob = find_problem(P, cfg.n_problems, g);
   int64_t local = g - P[n.prob].first;
   n.traj_id = (uint32_t)(cfg.run_index * P[n.prob].n_traj + local);
   n.attempt = attempt;
   set_start<TT, BG>(n, bv, s0, P[n.prob], Pd[n.prob], cfg, local);
   L.prob = n.prob; L.traj_id = n.traj_id; L.attempt = n.attempt; L.steps = n.steps; L.status = n.status; L.nrm = n.nrm;
   L.n_adapt = n.n_adapt;
   L.t = n.t;
   L.pos.x = n.pos.x; L.pos.y = n.pos.y; L.pos.z = n.pos.z;
   L.mom.x = n.mom.x; L.mom.y = n.mom.y; L.mom.z = n.mom.z;
   L.amp = n.amp; L.wgt = n.wgt; L.dt = n.dt; L.dt_adapt = n.dt_adapt; L.src_del_old = n.src_del_old;
}

// Resident blocks of 128 threads per SM the register allocation is sized for. For the FP32
// kernels five blocks (20 warps, at most 102 registers) measured 2-5% faster than four blocks
// without spills: the extra warps hide more dependent-instruction latency than the spilled
// values cost.
#ifndef SPX_MIN_BLOCKS_F32
#define SPX_MIN_BLOCKS_F32 5
#endif
#ifndef SPX_MIN_BLOCKS_F64
#define SPX_MIN_BLOCKS_F64 1
#endif

// One lane per thread. Dynamic shared memory holds the lanes' boundary states
// (boundaries per lane x blockDim.x x sizeof(BndState<R>)).
// DM is the field-derivative method (SPX_OPT_DERIV_MODE) fixed per instantiation, so the analytic
// kernels carry no finite-difference code (whose out-of-line calls would pin the field record to
// the stack).
// DK >= 0: a kernel specialised for one diffusion class (the Parker types); -1 dispatches at run time;
// kDkNoDiffusion: the guiding-centre kernels for TrajectoryGuiding proper (no scattering, no perpendicular step).
// BL: the boundary layout (BndLayout) the Parker step is compiled for; kLayoutAny reads it from the
// descriptor.
template <int TT, int BG, class R, int DM, bool GT, int DK, int BL>
__global__ void __launch_bounds__(128, sizeof(R) == 4 ? SPX_MIN_BLOCKS_F32 : SPX_MIN_BLOCKS_F64)
step_kernel(const ProblemDescT<R>* __restrict__ P, const ProblemDesc* __restrict__ Pd, RunConfig cfg,
            RunCounters* ctr, int32_t* counts, double* sums, unsigned long long* n_events, TrajRecord* rec, int queue)
{
   using A = typename AccOf<R>::type;
   cfg.deriv_mode = DM;
   extern __shared__ __align__(16) unsigned char spx_smem[];
   const BndView<R> bv{reinterpret_cast<BndState<R>*>(spx_smem) + threadIdx.x, (int)blockDim.x};
   Sinks S{counts, sums, n_events, ctr};
   Lane<R, A> L;
   Start s0;
   int64_t g = -1;
   bool active = false;  // the lane holds trajectory g
   bool fresh = false;   // trajectory g is to be (re)started with attempt number "attempt"
   uint32_t attempt = 0;
   unsigned long long my_steps = 0;
   unsigned my_retries = 0, my_given_up = 0, my_done = 0;
   const int64_t total = cfg.total_traj;
   const int64_t stride = (int64_t)gridDim.x * blockDim.x;
   if (!queue) {
      g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
      if (g < total) { active = true; fresh = true; }
   }
   const int K = cfg.steps_per_sync > 0 ? cfg.steps_per_sync : 1;
   while (true) {
      if (queue) {
         // refill idle lanes from the work queue: one atomic per warp
         unsigned idle = __ballot_sync(0xffffffffu, !active);
         if (idle) {
            int lane = threadIdx.x & 31;
            int leader = __ffs(idle) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(&ctr->next_traj, (unsigned long long)__popc(idle));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (!active) {
               int64_t mine = (int64_t)base + __popc(idle & ((1u << lane) - 1u));
               if (mine < total) { g = mine; active = true; fresh = true; attempt = 0; }
            }
         }
         if (!__any_sync(0xffffffffu, active)) break;
      }
      else if (!active) break;
      for (int k = 0; k < K && active; k++) {
         if (fresh) {
            start_lane<TT, BG>(L, bv, s0, P, Pd, cfg, g, attempt);
            fresh = false;
            continue;
         }
         bool done = false;
         if (L.status & TRAJ_DISCARD) {
            // discarded attempt: redo the trajectory with a fresh random stream (src/simulation.cc:262-288)
            if (L.attempt + 1 >= (uint32_t)cfg.max_attempts) {
               L.status |= TRAJ_GAVE_UP;
               my_given_up++;
               done = true;
            }
            else {
               my_retries++;
               attempt = L.attempt + 1;
               fresh = true;
               continue;
            }
         }
         else {
            const ProblemDescT<R>& Pp = P[L.prob];
            if constexpr (GT) {
               // any Butcher table (FP64): the table of the context, from constant memory
               const TableRk tab{cfg.rk_stages, cfg.rk_order, cfg.rk_adaptive, cfg.rk_offset};
               if (TT == kParker) parker_advance_gt<BG>(L, bv, s0, Pp, Pd[L.prob], cfg, S, tab);
               else rk_advance<TT, BG, R, A>(L, bv, s0, Pp, Pd[L.prob], cfg, S, tab);
            }
            else if (TT == kParker) parker_advance<BG, DK, BL>(L, bv, s0, Pp, Pd[L.prob], cfg, S);
            else if (cfg.rk == 25)
               rk_advance<TT, BG, R, A, FixedRk<4>, DK == kDkNoDiffusion>(L, bv, s0, Pp, Pd[L.prob], cfg, S, FixedRk<4>{});
            else rk_advance<TT, BG, R, A, FixedRk<1>, DK == kDkNoDiffusion>(L, bv, s0, Pp, Pd[L.prob], cfg, S, FixedRk<1>{});
            // Integrate's safety limits (src/trajectory_base.cc:964-992)
            if (L.steps > kMaxTrajSteps || !isfinite(L.dt) || L.dt == R(0)) L.status |= TRAJ_DISCARD;
            done = (L.status & TRAJ_FINISH) && !(L.status & TRAJ_DISCARD);
            // timing samples of the autotuner stop every trajectory after a fixed number of steps
            if (cfg.step_cap && L.steps >= cfg.step_cap && !done) {
               my_steps += L.steps;
               active = false;
               if (!queue) {
                  g += stride;
                  if (g < total) { active = true; fresh = true; attempt = 0; }
               }
               continue;
            }
         }
         if (done) {
            my_steps += L.steps;
            my_done++;
            if (cfg.record_final) write_record(L, s0, rec, g);
            active = false;
            if (!queue) {
               g += stride;
               if (g < total) { active = true; fresh = true; attempt = 0; }
            }
         }
      }
   }
   // warp-aggregated counters
   for (int o = 16; o > 0; o >>= 1) {
      my_steps += __shfl_down_sync(0xffffffffu, my_steps, o);
      my_retries += __shfl_down_sync(0xffffffffu, my_retries, o);
      my_given_up += __shfl_down_sync(0xffffffffu, my_given_up, o);
      my_done += __shfl_down_sync(0xffffffffu, my_done, o);
   }
   if ((threadIdx.x & 31) == 0) {
      atomicAdd(&ctr->steps, my_steps);
      if (my_retries) atomicAdd(&ctr->retries, (unsigned long long)my_retries);
      if (my_given_up) atomicAdd(&ctr->given_up, (unsigned long long)my_given_up);
      atomicAdd(&ctr->finished, (unsigned long long)my_done);
   }
}

}  // namespace spx
