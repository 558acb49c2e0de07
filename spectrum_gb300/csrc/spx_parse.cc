// spx_parse.cc -- turns the reference's DataContainer blobs into the POD descriptors of
// spx_params.hh. Each parser reads the records in the order of the reference class's Setup*()
// (cited per class) and precomputes what the reference precomputes there.
#include "spx_parse.hh"

#include <cmath>
#include <cstring>

#include "../../include/spx.h"

namespace spx {
namespace {

struct Reader {
   const uint8_t* p;
   size_t n, pos = 0;
   bool bad = false;

   // One record: a size byte then the payload (common/data_container.cc:205-224).
   size_t rec(void* dst, size_t want)
   {
      if (pos >= n) { bad = true; return 0; }
      size_t len = p[pos];
      if (pos + 1 + len > n || (want && len != want)) { bad = true; pos = n; return 0; }
      if (dst && len) std::memcpy(dst, p + pos + 1, len);
      pos += 1 + len;
      return len;
   }
   double d() { double v = 0.0; rec(&v, 8); return v; }
   int i() { int32_t v = 0; rec(&v, 4); return v; }
   bool b() { uint8_t v = 0; rec(&v, 1); return v != 0; }
   void v3(double* o) { rec(o, 24); }
   void mi(int* o) { int32_t v[3] = {0, 0, 0}; rec(v, 12); o[0] = v[0]; o[1] = v[1]; o[2] = v[2]; }
   int ints(int* o, int max)
   {
      int32_t tmp[64];
      if (pos >= n) { bad = true; return 0; }
      size_t len = p[pos];
      if (len % 4 || len / 4 > 64) { bad = true; return 0; }
      rec(tmp, 0);
      int k = (int)(len / 4);
      if (k > max) { bad = true; return 0; }
      for (int j = 0; j < k; j++) o[j] = tmp[j];
      return k;
   }
   void skip() { rec(nullptr, 0); }
};

// Unit system of the reference (common/specie.hh:30-82): c in code units is c / (0.1 c).
inline double c_code() { return 2.99792458e+10 / (0.1 * 2.99792458e+10); }

inline double dot(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
inline double norm(const double* a) { return std::sqrt(dot(a, a)); }
inline void cross(const double* a, const double* b, double* o)
{
   double r0 = a[1] * b[2] - a[2] * b[1], r1 = a[2] * b[0] - a[0] * b[2], r2 = a[0] * b[1] - a[1] * b[0];
   o[0] = r0; o[1] = r1; o[2] = r2;
}
inline void normalize(double* a)
{
   double n = norm(a);
   a[0] /= n; a[1] /= n; a[2] /= n;
}
// GetSecondUnitVec (common/vectors.cc:453-468)
inline void second_unit(const double* f, double* o)
{
   int m;
   if (std::fabs(f[0]) < std::fabs(f[1])) m = (std::fabs(f[0]) < std::fabs(f[2])) ? 0 : 2;
   else m = (std::fabs(f[1]) < std::fabs(f[2])) ? 1 : 2;
   double e[3] = {0.0, 0.0, 0.0};
   e[m] = 1.0;
   cross(f, e, o);
   normalize(o);
}
inline void induced_e(const double* u, const double* b, double* e)
{
   double x[3];
   cross(u, b, x);
   for (int k = 0; k < 3; k++) e[k] = -(x[k] / c_code());
}

int parse_background(Reader& r, int kind, BgParams& g)
{
   std::memset(&g, 0, sizeof g);
   g.kind = kind;
   // BackgroundBase::SetupBackground, src/background_base.cc:342-346
   g.t0 = r.d();
   r.v3(g.r0);
   r.v3(g.u0);
   r.v3(g.B0);
   g.dmax0 = r.d();
   switch (kind) {
   case kBgUniform:  // src/background_uniform.cc:49-56
      induced_e(g.u0, g.B0, g.E0);
      break;
   case kBgShock:
   case kBgSmoothShock: {  // src/background_shock.cc:56-80
      r.v3(g.n_shock);
      g.v_shock = r.d();
      g.compression = r.d();
      normalize(g.n_shock);
      double un = dot(g.u0, g.n_shock), bn = dot(g.B0, g.n_shock);
      for (int k = 0; k < 3; k++) {
         double u0n = (un - g.v_shock) * g.n_shock[k];
         double u0t = g.u0[k] - un * g.n_shock[k];
         double b0n = bn * g.n_shock[k];
         double b0t = g.B0[k] - b0n;
         g.u1[k] = u0n / g.compression + g.v_shock * g.n_shock[k] + u0t;
         g.B1[k] = b0n + b0t * g.compression;
      }
      induced_e(g.u0, g.B0, g.E0);
      induced_e(g.u1, g.B1, g.E1);
      if (kind == kBgSmoothShock) {  // src/background_smooth_shock.cc:110-117
         g.width = r.d();
         g.dmax_fraction = r.d();
      }
      g.tanh_k = 8.0;  // src/background_smooth_shock.hh:23
      break;
   }
   case kBgDiscontinuity:
   case kBgSmoothDiscontinuity:
      // BackgroundDiscontinuity::SetupBackground (src/background_discontinuity.cc:51-63): the normal, its
      // speed and the state behind it, given; the smooth one adds its width and dmax fraction
      // (src/background_smooth_discontinuity.cc:109-116) and steepness 4 (its .hh:49). Evaluated by the
      // shock kernels: the same piecewise and tanh forms (:75-92 and :121-170 of the two files)
      r.v3(g.n_shock);
      g.v_shock = r.d();
      r.v3(g.u1);
      r.v3(g.B1);
      normalize(g.n_shock);
      induced_e(g.u0, g.B0, g.E0);
      induced_e(g.u1, g.B1, g.E1);
      g.tanh_k = 4.0;
      if (kind == kBgSmoothDiscontinuity) {
         g.width = r.d();
         g.dmax_fraction = r.d();
      }
      g.kind = kind == kBgDiscontinuity ? kBgShock : kBgSmoothShock;
      break;
   case kBgDipole:  // src/background_dipole.cc:48-58
      g.r_ref = r.d();
      g.dmax_fraction = r.d();
      for (int k = 0; k < 3; k++) g.M[k] = g.B0[k] * (g.r_ref * g.r_ref * g.r_ref);
      break;
   case kBgSolarWind: {  // src/background_solarwind.cc:58-84
      double omega[3];
      r.v3(omega);
      g.r_ref = r.d();
      g.dmax_fraction = r.d();
      g.w0 = norm(omega);
      double e2[3] = {0.0, 0.0, 1.0};
      if (g.w0 >= 1.0e-15) { e2[0] = omega[0] / g.w0; e2[1] = omega[1] / g.w0; e2[2] = omega[2] / g.w0; }
      double e0[3], e1[3];
      second_unit(e2, e0);
      cross(e2, e0, e1);
      for (int k = 0; k < 3; k++) { g.eprime[0][k] = e0[k]; g.eprime[1][k] = e1[k]; g.eprime[2][k] = e2[k]; }
      g.ur0 = std::fabs(g.u0[0]);
      g.A = g.B0[0] * g.r_ref * g.r_ref;
      break;
   }
   case kBgGrid:  // BackgroundServerCartesian: the base parameters only; the grid comes separately
      break;
   default:
      return SPX_ERR_UNKNOWN_PLUGIN;
   }
   return r.bad ? SPX_ERR_BAD_BLOB : SPX_OK;
}

int parse_diffusion(Reader& r, int kind, int traj, DiffParams& d)
{
   std::memset(&d, 0, sizeof d);
   d.kind = kind;
   bool parker = (traj == kParker || traj == kParkerSource);
   switch (kind) {
   case kDfIsotropic:  // src/diffusion_other.cc:53-58 (not compiled for Parker, src/diffusion_other.hh:17)
      if (parker) return SPX_ERR_UNKNOWN_PLUGIN;
      d.a[0] = r.d();
      break;
   case kDfQLT:  // src/diffusion_other.cc:130-139
      if (parker) return SPX_ERR_UNKNOWN_PLUGIN;
      d.a[0] = r.d(); d.a[1] = r.d(); d.a[2] = r.d();
      d.a[3] = 6.283185307179586476925286766559005768 / d.a[1];
      d.a[4] = d.a[2] - 1.0;
      break;
   case kDfWNLT: case kDfWNLTRamp:
      // src/diffusion_other.cc:202-208: the QLT parameters, then A2T, A2L; the ramp adds l_max_HP, z_nose,
      // z_sheath (:281-295). Neither class is compiled for Parker (src/diffusion_other.hh:126).
      if (parker) return SPX_ERR_UNKNOWN_PLUGIN;
      d.a[0] = r.d(); d.a[1] = r.d(); d.a[2] = r.d();
      d.a[3] = 6.283185307179586476925286766559005768 / d.a[1];
      d.a[4] = d.a[2] - 1.0;
      d.a[5] = r.d(); d.a[6] = r.d();
      if (kind == kDfWNLTRamp) { d.a[7] = r.d(); d.a[8] = r.d(); d.a[9] = r.d(); }
      break;
   case kDfPara: case kDfPerp: d.a[0] = r.d(); break;
   case kDfFull: d.a[0] = r.d(); d.a[1] = r.d(); break;
   case kDfFlowMomentum: for (int k = 0; k < 6; k++) d.a[k] = r.d(); break;
   case kDfKinEnergyRadial:  // src/diffusion_other.cc:690-706
      for (int k = 0; k < 6; k++) d.a[k] = r.d();
      d.i0 = r.i();
      d.a[6] = r.d(); d.a[7] = r.d(); d.a[8] = r.d();
      d.a[9] = (1.0 / d.a[8]) * (1.0 / d.a[8]);
      break;
   case kDfRigidityB: for (int k = 0; k < 6; k++) d.a[k] = r.d(); break;
   case kDfStrauss2013: case kDfPotgieter2015:
      d.i0 = r.i();
      for (int k = 0; k < 6; k++) d.a[k] = r.d();
      break;
   case kDfEmpiricalSOQLT:  // src/diffusion_other.cc:1030-1043
      d.a[0] = r.d(); d.a[1] = r.d(); d.a[2] = r.d(); d.a[3] = r.d();
      d.i0 = r.i(); d.a[4] = r.d(); d.a[5] = r.d(); d.i1 = r.i(); d.a[6] = r.d();
      break;
   default:
      return SPX_ERR_UNKNOWN_PLUGIN;
   }
   return r.bad ? SPX_ERR_BAD_BLOB : SPX_OK;
}

int parse_boundary(Reader& r, int kind, int traj, BndParams& b)
{
   std::memset(&b, 0, sizeof b);
   b.kind = kind;
   // BoundaryBase::SetupBoundary, src/boundary_base.cc:138-141
   b.max_crossings = r.i();
   b.n_actions = r.ints(b.actions, kMaxDistro);
   switch (kind) {
   case kBtTimeExpire: case kBtTimePass: case kBtTimeRecurrent:  // src/boundary_time.cc
      b.cls = 0;
      b.timemark = r.d();
      if (kind == kBtTimeExpire) b.max_crossings = 1;
      if (kind == kBtTimePass) b.max_crossings = -1;
      if (kind == kBtTimeRecurrent) b.recurrent = 1;
      break;
   case kBtPlaneAbsorb: case kBtPlaneReflect: case kBtPlanePass:  // src/boundary_space.cc:58-203
      b.cls = 1;
      r.v3(b.origin);
      r.v3(b.norm);
      normalize(b.norm);
      if (kind == kBtPlaneAbsorb) b.max_crossings = 1;
      if (kind == kBtPlaneReflect) b.reflect = 1;
      break;
   case kBtBoxReflect: {  // src/boundary_space.cc:249-265
      b.cls = 1;
      b.reflect = 1;
      r.v3(b.corner0);
      for (int s = 0; s < 3; s++) r.v3(b.normals[s]);
      for (int k = 0; k < 3; k++) b.corner1[k] = b.corner0[k] + b.normals[0][k] + b.normals[1][k] + b.normals[2][k];
      for (int s = 0; s < 3; s++) normalize(b.normals[s]);
      break;
   }
   case kBtSphereAbsorb: case kBtSphereReflect: case kBtSpherePass:  // src/boundary_space.cc:383-493
      b.cls = 1;
      r.v3(b.origin);
      b.radius = r.d();
      if (kind == kBtSphereAbsorb) b.max_crossings = 1;
      if (kind == kBtSphereReflect) b.reflect = 1;
      break;
   case kBtRankineAbsorb:  // src/boundary_space.cc:539-601
      b.cls = 1;
      r.v3(b.origin);
      r.v3(b.axis);
      b.z_nose = r.d();
      b.max_crossings = 1;
      break;
   case kBtCylinderAbsorb:  // src/boundary_space.cc:647-729
      b.cls = 1;
      r.v3(b.origin);
      r.v3(b.fa[2]);
      b.radius = r.d();
      normalize(b.fa[2]);
      second_unit(b.fa[2], b.fa[0]);
      cross(b.fa[2], b.fa[0], b.fa[1]);
      b.max_crossings = 1;
      break;
   case kBtRegionAbsorb:  // src/boundary_space.cc:775-848
      b.cls = 1;
      b.region_ind = r.i();
      b.region_val = r.d();
      b.max_crossings = 1;
      if (b.region_ind < 0 || b.region_ind > 2) return SPX_ERR_BAD_BLOB;
      break;
   case kBtMomentumInject: case kBtMomentumPass: case kBtMomentumSlab: case kBtMomentumShell:  // src/boundary_momentum.cc
      // BoundaryMomentum::EvaluateBoundary sets no delta for field lines (src/boundary_momentum.cc:69-75)
      if (traj == kFieldline) return SPX_ERR_UNKNOWN_PLUGIN;
      b.cls = 2;
      b.momentum = r.d();
      if (kind != kBtMomentumPass) b.max_crossings = 1;
      if (kind == kBtMomentumSlab) { r.v3(b.slab_r0); r.v3(b.slab_r1); r.v3(b.slab_n); }
      if (kind == kBtMomentumShell) { r.v3(b.slab_r0); b.r1 = r.d(); b.r2 = r.d(); }
      break;
   case kBtMirror:  // src/boundary_momentum.cc:317-339 (not compiled for Parker or Fieldline, src/boundary_momentum.hh:225)
      if (traj == kParker || traj == kParkerSource || traj == kFieldline) return SPX_ERR_UNKNOWN_PLUGIN;
      b.cls = 2;
      b.reflect = 1;
      break;
   default:
      return SPX_ERR_UNKNOWN_PLUGIN;
   }
   return r.bad ? SPX_ERR_BAD_BLOB : SPX_OK;
}

int parse_initial(Reader& r, int kind, int traj, IniParams& q)
{
   std::memset(&q, 0, sizeof q);
   q.kind = kind;
   bool parker = (traj == kParker || traj == kParkerSource);
   switch (kind) {
   case kItFixed: q.a[0] = r.d(); break;                                       // src/initial_time.cc:48-56
   case kItInterval: q.a[0] = r.d(); q.a[1] = r.d(); q.n_int = r.i(); break;   // src/initial_time.cc:114-130
   case kIsFixed: r.v3(q.v0); break;                                           // src/initial_space.cc:49-57
   case kIsLine: case kIsBox: r.v3(q.v0); r.v3(q.v1); q.n_int = r.i(); break;  // src/initial_space.cc:115-131
   case kIsCircle: {                                                           // src/initial_space.cc:190-202
      double normal[3], radius, su[3];
      r.v3(q.v0);
      r.v3(normal);
      radius = r.d();
      normalize(normal);
      second_unit(normal, su);
      for (int k = 0; k < 3; k++) q.v1[k] = radius * su[k];
      cross(normal, q.v1, q.v2);
      break;
   }
   case kIsSphere: r.v3(q.v0); q.a[0] = r.d(); break;
   case kIsSphereSector:  // src/initial_space.cc:357-377
      r.v3(q.v0);
      q.a[0] = r.d();
      q.a[1] = r.d(); if (q.a[1] < 0.0) q.a[1] = 0.0;
      q.a[2] = r.d(); if (q.a[2] > M_PI) q.a[2] = M_PI; if (q.a[2] < q.a[1]) q.a[2] = q.a[1];
      q.a[3] = r.d();
      q.a[4] = r.d(); if (q.a[4] > 2.0 * M_PI) q.a[4] = 2.0 * M_PI; if (q.a[4] < q.a[3]) q.a[4] = q.a[3];
      q.a[5] = std::cos(q.a[1]);
      q.a[6] = std::cos(q.a[2]);
      break;
   case kIsRankine:  // src/initial_space.cc:432-444
      r.v3(q.v0); q.a[0] = r.d(); q.a[1] = r.d();
      q.a[2] = (2.0 * q.a[0] * q.a[0] - q.a[1] * q.a[1]) / (q.a[1] * q.a[1]);
      break;
   case kIsEquatorialBand: r.v3(q.v0); q.a[0] = r.d(); q.a[1] = r.d(); q.a[2] = r.d(); break;
   case kIsCylinder: case kIsCylinderSector: {
      // InitialSpaceCylinder(Sector)::SetupInitial (src/initial_space.cc:561-570, 621-631): origin, height
      // vector, radius vector x; radius vector y = unit(height) x radius x; the sector's azimuth range
      // clamped to [phi1, min(phi2, 2 pi)]
      r.v3(q.v0); r.v3(q.v1); r.v3(q.v2);
      double h[3] = {q.v1[0], q.v1[1], q.v1[2]}, ry[3];
      normalize(h);
      cross(h, q.v2, ry);
      q.a[0] = ry[0]; q.a[1] = ry[1]; q.a[2] = ry[2];
      if (kind == kIsCylinderSector) {
         q.a[3] = r.d();
         q.a[4] = r.d();
         if (q.a[4] > 6.283185307179586476925286766559) q.a[4] = 6.283185307179586476925286766559;
         if (q.a[4] < q.a[3]) q.a[4] = q.a[3];
      }
      break;
   }
   case kImFixed:  // only compiled for Lorentz and Fieldline (src/initial_momentum.hh:21)
      if (traj != kLorentz && traj != kFieldline) return SPX_ERR_UNKNOWN_PLUGIN;
      r.v3(q.v0);
      break;
   case kImBeam: case kImRing:  // not compiled for Parker or Fieldline (src/initial_momentum.hh:86,131)
      if (parker || traj == kFieldline) return SPX_ERR_UNKNOWN_PLUGIN;
      q.a[0] = r.d();
      if (kind == kImRing) { q.a[1] = r.d(); q.a[2] = std::cos(q.a[1]); q.a[3] = std::sin(q.a[1]); }
      break;
   case kImShell: q.a[0] = r.d(); break;
   case kImThickShell:  // src/initial_momentum.cc:363-375
      q.a[0] = r.d(); q.a[1] = r.d(); q.flag = r.b() ? 1 : 0;
      if (q.flag) { q.a[0] = std::log10(q.a[0]); q.a[1] = std::log10(q.a[1]); }
      break;
   case kImMaxwell:  // src/initial_momentum.cc:503-514
      q.a[0] = r.d(); q.a[1] = r.d() / std::sqrt(2.0); q.a[2] = r.d() / std::sqrt(2.0);
      break;
   case kImLogEnergyPitchBand:  // a pitch-angle band: no meaning along a field line
      if (traj == kFieldline) return SPX_ERR_UNKNOWN_PLUGIN;
      q.a[0] = r.d(); q.a[1] = r.d(); q.a[2] = r.d(); q.a[3] = r.d();
      break;
   default:
      return SPX_ERR_UNKNOWN_PLUGIN;
   }
   return r.bad ? SPX_ERR_BAD_BLOB : SPX_OK;
}

int parse_distribution(Reader& r, int kind, DistParams& d)
{
   std::memset(&d, 0, sizeof d);
   d.kind = kind;
   d.width = (kind == kDsCumulative1 || kind == kDsLossCone) ? 3 : (kind == kDsCumulative2 ? 9 : 1);
   double mn[3], mx[3];
   // DistributionTemplated::SetupDistribution, src/distribution_templated.cc:92-137
   r.mi(d.n_bins);
   r.v3(mn);
   r.v3(mx);
   r.mi(d.log_bins);
   r.mi(d.bin_outside);
   r.skip();  // unit_distro
   r.skip();  // unit_val
   d.keep_records = r.b() ? 1 : 0;
   d.dims = 0;
   for (int k = 0; k < 3; k++) {
      if (d.n_bins[k] > 0) d.dims |= 1 << k;
      if (d.n_bins[k] < 1) d.n_bins[k] = 1;
      double lo = d.log_bins[k] ? std::log10(mn[k]) : mn[k];
      double hi = d.log_bins[k] ? std::log10(mx[k]) : mx[k];
      d.limits0[k] = lo;
      d.bin_size[k] = (hi - lo) / d.n_bins[k];
   }
   switch (kind) {
   case kDsTimeUniform: case kDsPositionUniform: case kDsMomentumUniform: case kDsPositionMomentumUniform:
   case kDsTimeMu:  // DistributionUniform, src/distribution_other.cc:40-60
      d.val_hot = r.d();
      d.val_cold = r.d();
      d.n_actions = 2;
      if (kind == kDsTimeUniform) d.val_time = r.i();
      if (kind == kDsPositionUniform || kind == kDsMomentumUniform) { d.val_time = r.i(); d.val_coord = r.i(); }
      if (kind == kDsPositionMomentumUniform) {
         d.val_time = r.i(); d.pos_idx = r.i(); d.mom_idx = r.i();
         if (d.pos_idx < 0 || d.pos_idx > 3 || d.mom_idx < 0 || d.mom_idx > 2) return SPX_ERR_BAD_BLOB;
      }
      break;
   case kDsSpectrumPowerLaw: case kDsSpectrumBentPowerLaw:  // src/distribution_other.cc:520-560
      d.J0 = r.d(); d.T0 = r.d(); d.pow_law = r.d(); d.val_cold = r.d();
      d.n_actions = 2;
      if (kind == kDsSpectrumBentPowerLaw) {
         d.T_b = r.d();
         double plb = r.d();
         d.bend = r.d();
         d.pow_law_comb = (d.pow_law - plb) / d.bend;
      }
      break;
   case kDsCumulative1: case kDsCumulative2: d.n_actions = 1; break;
   case kDsDivergenceFlow: d.A0 = r.d(); d.pow_law = r.d(); d.val_cold = r.d(); d.n_actions = 2; break;
   case kDsLossCone:  // src/distribution_other.cc:826-840: one action, all three dimensions active
      d.val_time = r.i();
      d.val_coord = r.i();
      d.n_actions = 1;
      if (d.dims != 7) return SPX_ERR_BAD_BLOB;
      break;
   case kDsAnisotropyLISM:  // src/distribution_other.cc:388-409: five actions; its set-up accepts dims 5 only
      for (int k = 0; k < 3; k++) r.v3(d.rot[k]);
      r.v3(d.u_lism);
      d.pow_law = r.d();
      r.v3(d.grad_perp);
      d.n_actions = 5;
      if (d.dims != 5) return SPX_ERR_BAD_BLOB;
      break;
   default:
      return SPX_ERR_UNKNOWN_PLUGIN;
   }
   return r.bad ? SPX_ERR_BAD_BLOB : SPX_OK;
}

}  // namespace

int parse_plugin(ProblemDesc& pd, int traj, int role, int kind, const uint8_t* blob, size_t len, int slot)
{
   Reader r{blob, len};
   switch (role) {
   case SPX_ROLE_BACKGROUND: return parse_background(r, kind, pd.bg);
   case SPX_ROLE_DIFFUSION: {
      int rc = parse_diffusion(r, kind, traj, pd.df);
      if (rc == SPX_OK) pd.has_diff = 1;
      return rc;
   }
   case SPX_ROLE_SOURCE:
      // SourceConstant::SetupSource (src/source_other.cc:41-50): S0; SourceMomentumInjection (:98-107):
      // the injection momentum and the rate
      // SourceSphericalShockInjection (:150-160): p_inj, the shell's centre, radius and width, the rate
      if (kind < 1 || kind > 3) return SPX_ERR_UNKNOWN_PLUGIN;
      pd.src.kind = kind;
      if (kind >= 2) pd.src.p_inj = r.d();
      if (kind == 3) { r.v3(pd.src.r0); pd.src.r_sh = r.d(); pd.src.w_sh = r.d(); }
      pd.src.rate = r.d();
      return r.bad ? SPX_ERR_BAD_BLOB : SPX_OK;
   case SPX_ROLE_BOUNDARY: {
      BndParams b;
      int rc = parse_boundary(r, kind, traj, b);
      if (rc != SPX_OK) return rc;
      BndParams* arr = b.cls == 0 ? pd.bt : (b.cls == 1 ? pd.bs : pd.bm);
      int& cnt = b.cls == 0 ? pd.nbt : (b.cls == 1 ? pd.nbs : pd.nbm);
      if (slot >= 0) {
         if (slot >= cnt) return SPX_ERR_INVALID_ARG;
         arr[slot] = b;
         return SPX_OK;
      }
      if (cnt >= kMaxBnd) return SPX_ERR_LIMIT;
      arr[cnt++] = b;
      return SPX_OK;
   }
   case SPX_ROLE_INITIAL: {
      IniParams q;
      int rc = parse_initial(r, kind, traj, q);
      if (rc != SPX_OK) return rc;
      if (kind < 10) pd.it = q;
      else if (kind < 30 || kind == kIsEquatorialBand) pd.is = q;
      else pd.im = q;
      return SPX_OK;
   }
   case SPX_ROLE_DISTRIBUTION: {
      // DistributionAnisotropyLISM is compiled for Lorentz trajectories only (src/distribution_other.hh:245)
      if (kind == kDsAnisotropyLISM && traj != kLorentz) return SPX_ERR_UNKNOWN_PLUGIN;
      // the divergence-flow weight reads grad U, which a field line's mask (B only) never evaluates
      if (kind == kDsDivergenceFlow && traj == kFieldline) return SPX_ERR_UNKNOWN_PLUGIN;
      DistParams d;
      int rc = parse_distribution(r, kind, d);
      if (rc != SPX_OK) return rc;
      if (slot >= 0) {
         if (slot >= pd.nd) return SPX_ERR_INVALID_ARG;
         pd.d[slot] = d;
         return SPX_OK;
      }
      if (pd.nd >= kMaxDistro) return SPX_ERR_LIMIT;
      pd.d[pd.nd++] = d;
      return SPX_OK;
   }
   default:
      return SPX_ERR_INVALID_ARG;
   }
}

bool background_allowed(int traj, int bg_kind)
{
   // the guiding-centre drift needs dB/dt, which the moving shocks have and the device does not evaluate
   if (traj >= kGuiding && traj <= kGuidingDiffScatt && (bg_kind == kBgShock || bg_kind == kBgSmoothShock)) return false;
   return true;
}

int check_ready(const ProblemDesc& pd, int traj)
{
   // TrajectoryBase::IsSimmulationReady (src/trajectory_base.cc:608-632) and the Parker override
   // requiring a diffusion model (src/trajectory_parker.cc:184-192).
   if (pd.bg.kind == 0 || pd.it.kind == 0 || pd.is.kind == 0 || pd.im.kind == 0 || pd.nbt == 0)
      return SPX_ERR_INCOMPLETE;
   if ((traj == kParker || traj == kParkerSource) && !pd.has_diff) return SPX_ERR_INCOMPLETE;
   // TrajectoryGuidingScatt / GuidingDiff::IsSimmulationReady (src/trajectory_guiding_scatt.cc:43-52,
   // src/trajectory_guiding_diff.cc:43-52)
   if ((traj == kGuidingScatt || traj == kGuidingDiff || traj == kGuidingDiffScatt) && !pd.has_diff) return SPX_ERR_INCOMPLETE;
   if (!background_allowed(traj, pd.bg.kind)) return SPX_ERR_UNKNOWN_PLUGIN;
   if (traj == kParkerSource && pd.src.kind == 0) return SPX_ERR_INCOMPLETE;
   for (int k = 0; k < pd.nbt; k++)
      for (int a = 0; a < pd.bt[k].n_actions && a < pd.nd; a++)
         if (pd.bt[k].actions[a] >= pd.d[a].n_actions) return SPX_ERR_BAD_BLOB;
   for (int k = 0; k < pd.nbs; k++)
      for (int a = 0; a < pd.bs[k].n_actions && a < pd.nd; a++)
         if (pd.bs[k].actions[a] >= pd.d[a].n_actions) return SPX_ERR_BAD_BLOB;
   for (int k = 0; k < pd.nbm; k++)
      for (int a = 0; a < pd.bm[k].n_actions && a < pd.nd; a++)
         if (pd.bm[k].actions[a] >= pd.d[a].n_actions) return SPX_ERR_BAD_BLOB;
   return SPX_OK;
}

namespace {

template <class R, int N>
void cp(const double (&s)[N], R (&d)[N])
{
   for (int k = 0; k < N; k++) d[k] = (R)s[k];
}
template <class R, int N, int M>
void cp(const double (&s)[N][M], R (&d)[N][M])
{
   for (int k = 0; k < N; k++)
      for (int j = 0; j < M; j++) d[k][j] = (R)s[k][j];
}

}  // namespace

template <class R>
void convert_problem(const ProblemDesc& s, ProblemDescT<R>& d)
{
   const BgParams& a = s.bg;
   BgParamsT<R>& b = d.bg;
   b.kind = a.kind; b.t0 = (R)a.t0; b.dmax0 = (R)a.dmax0;
   cp(a.r0, b.r0); cp(a.u0, b.u0); cp(a.B0, b.B0); cp(a.n_shock, b.n_shock); cp(a.u1, b.u1); cp(a.B1, b.B1);
   cp(a.E0, b.E0); cp(a.E1, b.E1);
   b.v_shock = (R)a.v_shock; b.compression = (R)a.compression; b.width = (R)a.width;
   b.dmax_fraction = (R)a.dmax_fraction; b.tanh_k = (R)a.tanh_k;
   cp(a.M, b.M); cp(a.eprime, b.eprime);
   b.w0 = (R)a.w0; b.r_ref = (R)a.r_ref; b.ur0 = (R)a.ur0; b.A = (R)a.A;
   cp(a.cent_min, b.cent_min); cp(a.zone, b.zone); b.zone_min = (R)a.zone_min;
   for (int k = 0; k < 3; k++) b.grid_n[k] = a.grid_n[k];
   b.grid = nullptr;  // the context points it at its own copy of the grid in this arithmetic
   for (int k = 0; k < 3; k++) b.grid_nb[k] = a.grid_nb[k];
   b.grid_ghost = a.grid_ghost;
   b.grid_order = a.grid_order;
   cp(a.dom_min, b.dom_min); cp(a.dom_max, b.dom_max); cp(a.blk_len, b.blk_len); cp(a.gunits, b.gunits);

   d.df.kind = s.df.kind; d.df.i0 = s.df.i0; d.df.i1 = s.df.i1; cp(s.df.a, d.df.a);
   d.src.kind = s.src.kind; d.src.p_inj = (R)s.src.p_inj; d.src.rate = (R)s.src.rate;
   cp(s.src.r0, d.src.r0); d.src.r_sh = (R)s.src.r_sh; d.src.w_sh = (R)s.src.w_sh;

   auto ini = [](const IniParams& x, IniParamsT<R>& y) {
      y.kind = x.kind; y.n_int = x.n_int; y.flag = x.flag;
      cp(x.a, y.a); cp(x.v0, y.v0); cp(x.v1, y.v1); cp(x.v2, y.v2);
   };
   ini(s.it, d.it); ini(s.is, d.is); ini(s.im, d.im);

   auto bnd = [](const BndParams& x, BndParamsT<R>& y) {
      y.kind = x.kind; y.cls = x.cls; y.reflect = x.reflect; y.recurrent = x.recurrent;
      y.max_crossings = x.max_crossings; y.n_actions = x.n_actions;
      for (int k = 0; k < kMaxDistro; k++) y.actions[k] = x.actions[k];
      y.region_ind = x.region_ind;
      y.timemark = (R)x.timemark;
      y.timemark_lo = (R)(x.timemark - (double)y.timemark);
      y.momentum = (R)x.momentum; y.radius = (R)x.radius; y.z_nose = (R)x.z_nose; y.r1 = (R)x.r1; y.r2 = (R)x.r2;
      y.region_val = (R)x.region_val;
      cp(x.origin, y.origin); cp(x.norm, y.norm); cp(x.corner0, y.corner0); cp(x.corner1, y.corner1);
      cp(x.normals, y.normals); cp(x.axis, y.axis); cp(x.fa, y.fa);
      cp(x.slab_r0, y.slab_r0); cp(x.slab_r1, y.slab_r1); cp(x.slab_n, y.slab_n);
   };
   for (int k = 0; k < kMaxBnd; k++) { bnd(s.bt[k], d.bt[k]); bnd(s.bs[k], d.bs[k]); bnd(s.bm[k], d.bm[k]); }

   for (int k = 0; k < kMaxDistro; k++) {
      const DistParams& x = s.d[k];
      DistParamsT<R>& y = d.d[k];
      y.kind = x.kind; y.width = x.width; y.dims = x.dims; y.n_actions = x.n_actions;
      for (int j = 0; j < 3; j++) {
         y.n_bins[j] = x.n_bins[j]; y.log_bins[j] = x.log_bins[j]; y.bin_outside[j] = x.bin_outside[j];
      }
      cp(x.limits0, y.limits0); cp(x.bin_size, y.bin_size);
      y.val_hot = (R)x.val_hot; y.val_cold = (R)x.val_cold;
      y.val_time = x.val_time; y.val_coord = x.val_coord; y.pos_idx = x.pos_idx; y.mom_idx = x.mom_idx;
      y.J0 = (R)x.J0; y.T0 = (R)x.T0; y.pow_law = (R)x.pow_law; y.T_b = (R)x.T_b;
      y.pow_law_comb = (R)x.pow_law_comb; y.bend = (R)x.bend; y.A0 = (R)x.A0;
      cp(x.rot, y.rot); cp(x.u_lism, y.u_lism); cp(x.grad_perp, y.grad_perp);
      y.offset_counts = x.offset_counts; y.offset_sums = x.offset_sums;
   }
   d.nbt = s.nbt; d.nbs = s.nbs; d.nbm = s.nbm; d.nd = s.nd; d.has_diff = s.has_diff;
   d.problem_id = s.problem_id; d.seed = s.seed; d.n_traj = s.n_traj; d.first = s.first; d.id_base = s.id_base;
}

template void convert_problem<float>(const ProblemDesc&, ProblemDescT<float>&);
template void convert_problem<double>(const ProblemDesc&, ProblemDescT<double>&);

}  // namespace spx
