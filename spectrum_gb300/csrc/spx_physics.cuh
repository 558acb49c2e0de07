// spx_physics.cuh -- field evaluators, diffusion models and boundary tests, as device functions
// over the real type R. Each function names the reference code whose arithmetic it carries out.
#pragma once

#include "spx_device.cuh"
#include "spx_params.hh"

namespace spx {

// ---- unit system and proton kinematics (common/specie.hh:30-82, common/physics.hh:246-510) --
template <class R> struct Units;
template <> struct Units<double> {
   static constexpr double c = 2.99792458e+10 / (0.1 * 2.99792458e+10);
};
template <> struct Units<float> {
   static constexpr float c = (float)(2.99792458e+10 / (0.1 * 2.99792458e+10));
};
template <class R> __device__ __forceinline__ R c_code() { return Units<R>::c; }
template <class R> __device__ __forceinline__ R enr_tot(R p) { R c = c_code<R>(); return m_sqrt(p * p + c * c) * c; }
template <class R> __device__ __forceinline__ R enr_kin(R p) { R c = c_code<R>(); return enr_tot(p) - c * c; }
template <class R> __device__ __forceinline__ R vel_of(R p) { R c = c_code<R>(); return p * (c * c) / enr_tot(p); }
template <class R> __device__ __forceinline__ R mom_of(R e) { R c = c_code<R>(); return m_sqrt(e * (e + R(2) * (c * c))) / c; }
template <class R> __device__ __forceinline__ R rigidity(R p) { return p * c_code<R>(); }
template <class R> __device__ __forceinline__ R larmor(R p, R b) { return p * c_code<R>() / b; }
template <class R> __device__ __forceinline__ R rel_factor(R v) { R r = v / c_code<R>(); return R(1) / m_sqrt(R(1) - r * r); }
template <class R> __device__ __forceinline__ R cyclotron(R v, R b) { return b / (rel_factor(v) * c_code<R>()); }
template <class R> __device__ __forceinline__ V3<R> vel_cart(V3<R> mom) { R m = norm(mom); return (vel_of(m) / m) * mom; }

// ---- spatial data (common/spatial_data.hh:55-135) ----------------------------------------------
constexpr unsigned kU = 0x1, kB = 0x2, kE = 0x4, kAll = 0x7, kGradU = 0x10, kGradB = 0x20, kDUdt = 0x100;
// Mask bit of this implementation: the caller needs only div U, div b, b.grad(b) and grad|B|, not
// the gradient matrices (Parker transport).
constexpr unsigned kDerivedOnly = 0x4000;

template <class R>
struct SD {
   V3<R> U, B, E, bhat, gradBmag, dUdt, region, bgradb;
   M3<R> gradU, gradB;
   R Bmag, dmax, divU, divbhat;
   R dr[3];
};

template <class R> __device__ __forceinline__ R sd_divU(const SD<R>& s) { return s.divU; }
template <class R> __device__ __forceinline__ V3<R> sd_curlB(const SD<R>& s)
{
   return {s.gradB.m[1][2] - s.gradB.m[2][1], s.gradB.m[2][0] - s.gradB.m[0][2], s.gradB.m[0][1] - s.gradB.m[1][0]};
}
template <class R> __device__ __forceinline__ R sd_divbhat(const SD<R>& s) { return s.divbhat; }
template <class R> __device__ __forceinline__ V3<R> sd_b_gradbhat(const SD<R>& s) { return s.bgradb; }

// div U, divbhat and bhat.grad(bhat) from the gradient matrices (common/spatial_data.hh:213-330)
template <class R> __device__ __forceinline__ R mat_divbhat(const SD<R>& s)
{
   return (trace(s.gradB) - dot(s.gradBmag, s.bhat)) / s.Bmag;
}
template <class R> __device__ __forceinline__ V3<R> mat_b_gradbhat(const SD<R>& s)
{
   V3<R> r;
   R o[3];
#pragma unroll
   for (int j = 0; j < 3; j++) {
      R acc = R(0);
#pragma unroll
      for (int i = 0; i < 3; i++) acc += s.bhat[i] * ((s.gradB.m[i][j] - s.gradBmag[i] * s.bhat[j]) / s.Bmag);
      o[j] = acc;
   }
   r = {o[0], o[1], o[2]};
   return r;
}

template <class R> __device__ __forceinline__ void zero(M3<R>& a)
{
#pragma unroll
   for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) a.m[i][j] = R(0);
}

// ---- backgrounds -------------------------------------------------------------------------------
// Smooth transition of SMOOTH_SHOCK_ORDER 4 (src/background_smooth_shock.cc:46-105) and SMOOTH_DISCONT_ORDER 4
// (src/background_smooth_discontinuity.cc:46-105); k is the class's tanh_width_factor
template <class R> __device__ __forceinline__ R shock_tr(R k, R x) { return R(0.5) * (R(1) + m_tanh(k * x)); }
template <class R> __device__ __forceinline__ R shock_trd(R k, R x) { R th = m_tanh(k * x); return R(0.5) * k * (R(1) - th * th); }

template <class R> __device__ __forceinline__ V3<R> eframe_to(const BgParamsT<R>& g, V3<R> a)
{
   return {a.x * g.eprime[0][0] + a.y * g.eprime[0][1] + a.z * g.eprime[0][2],
           a.x * g.eprime[1][0] + a.y * g.eprime[1][1] + a.z * g.eprime[1][2],
           a.x * g.eprime[2][0] + a.y * g.eprime[2][1] + a.z * g.eprime[2][2]};
}
template <class R> __device__ __forceinline__ V3<R> eframe_from(const BgParamsT<R>& g, V3<R> a)
{
   return {a.x * g.eprime[0][0] + a.y * g.eprime[1][0] + a.z * g.eprime[2][0],
           a.x * g.eprime[0][1] + a.y * g.eprime[1][1] + a.z * g.eprime[2][1],
           a.x * g.eprime[0][2] + a.y * g.eprime[1][2] + a.z * g.eprime[2][2]};
}

template <class R> __device__ __forceinline__ void derive_from_matrices(SD<R>& s)
{
   s.divU = trace(s.gradU);
   s.divbhat = mat_divbhat(s);
   s.bgradb = mat_b_gradbhat(s);
}

template <class R>
__device__ void grid_reader_values(const BgParamsT<R>& g, V3<R> pos, SD<R>& s);

// EvaluateBackground of the analytic backgrounds: U, B, E by mask, region; *ds is the smooth-shock
// coordinate (used by the derivatives); for a grid, the reader's interpolation.
template <int BG, class R>
__device__ __forceinline__ void eval_bg(const BgParamsT<R>& g, R t, V3<R> pos, unsigned mask, SD<R>& s, R& ds)
{
   if (BG == kBgUniform) {  // src/background_uniform.cc:63-72
      if (mask & kU) s.U = ld3(g.u0);
      if (mask & kB) s.B = ld3(g.B0);
      if (mask & kE) s.E = ld3(g.E0);
      s.region = mk(R(1), R(1), R(1));
   }
   else if (BG == kBgShock) {  // src/background_shock.cc:86-104
      if (dot(pos - ld3(g.r0), ld3(g.n_shock)) - g.v_shock * t > R(0)) {
         if (mask & kU) s.U = ld3(g.u0);
         if (mask & kB) s.B = ld3(g.B0);
         if (mask & kE) s.E = ld3(g.E0);
         s.region = mk(R(1), R(1), R(1));
      }
      else {
         if (mask & kU) s.U = ld3(g.u1);
         if (mask & kB) s.B = ld3(g.B1);
         if (mask & kE) s.E = ld3(g.E1);
         s.region = mk(R(2), R(2), R(2));
      }
   }
   else if (BG == kBgSmoothShock) {  // src/background_smooth_shock.cc:124-140
      ds = (dot(pos - ld3(g.r0), ld3(g.n_shock)) - g.v_shock * t) / g.width;
      R a1 = shock_tr(g.tanh_k, ds), a2 = R(1) - a1;
      if ((mask & kU) || (mask & kE)) s.U = a1 * ld3(g.u0) + a2 * ld3(g.u1);
      if (mask & kB) s.B = a1 * ld3(g.B0) + a2 * ld3(g.B1);
      if (mask & kE) s.E = R(-1) * (cross(s.U, s.B) / c_code<R>());  // InducedEfield: -(U x B) / c
      R rg = R(1) * a1 + R(2) * a2;
      s.region = mk(rg, rg, rg);
   }
   else if (BG == kBgDipole) {  // src/background_dipole.cc:64-80
      if (mask & kU) s.U = mk(R(0), R(0), R(0));
      if (mask & kB) {
         V3<R> pp = pos - ld3(g.r0), M = ld3(g.M);
         R r2 = norm(pp);
         R r5 = r2 * r2 * r2;
         r2 *= r2;
         r5 *= r2;
         s.B = (R(3) * dot(pp, M) * pp - r2 * M) / r5;
      }
      if (mask & kE) s.E = mk(R(0), R(0), R(0));
      s.region = mk(R(1), R(1), R(1));
   }
   else if (BG == kBgSolarWind) {  // src/background_solarwind.cc:111-255, switches at their defaults
      V3<R> pp = eframe_to(g, pos - ld3(g.r0));
      R r = norm(pp), r_mns = r - g.r_ref, costheta = pp.z / r, ur = g.ur0;
      s.region = mk(r < R(117.0 * 1.495978707E+13 / 1.0e10) ? R(1) : R(-1), R(-1), s.region.z);
      // U also when only E is asked for (the Lorentz mask): E = -U x B / c needs it (deviation D4)
      if (mask & (kU | kE)) s.U = eframe_from(g, ur * unit(pp));
      if (mask & kB) {
         R sintheta = m_sqrt(m_max(R(1) - costheta * costheta, R(0)));
         R sr = m_sqrt(pp.x * pp.x + pp.y * pp.y), cosphi, sinphi;
         if (sr < r * Lim<R>::tiny) { cosphi = R(0); sinphi = R(0); }
         else { cosphi = pp.x / sr; sinphi = pp.y / sr; }
         R q = g.r_ref / r;
         R Br = g.B0[0] * (q * q);
         R Bp = -Br * sintheta * r_mns * g.w0 / ur;
         s.B = eframe_from(g, mk(Br * sintheta * cosphi - Bp * sinphi, Br * sintheta * sinphi + Bp * cosphi, Br * costheta));
      }
      if (mask & kE) s.E = R(-1) * (cross(s.U, s.B) / c_code<R>());  // InducedEfield: -(U x B) / c
   }
   else if (BG == kBgGrid) grid_reader_values(g, pos, s);  // the points of numerical derivatives (order -1)
}

// EvaluateDmax (src/background_base.cc:378-382 and overrides). The smooth shock uses the shock
// distance at the evaluated point (the reference uses the previous evaluation's value because
// EvaluateDmax runs before EvaluateBackground in GetFields, src/background_base.cc:434-442).
template <int BG, class R>
__device__ __forceinline__ R eval_dmax(const BgParamsT<R>& g, R t, V3<R> pos)
{
   if (BG == kBgSmoothShock) {
      R ds = (dot(pos - ld3(g.r0), ld3(g.n_shock)) - g.v_shock * t) / g.width;
      return m_min(g.dmax_fraction * g.width * m_max(R(1), m_abs(ds)), g.dmax0);
   }
   if (BG == kBgDipole || BG == kBgSolarWind) return m_min(g.dmax_fraction * norm(pos - ld3(g.r0)), g.dmax0);
   if (BG == kBgGrid) return m_min(g.dmax0, g.zone_min);
   return g.dmax0;
}

// The Parker spiral and its derivatives in closed form in the global frame (analytic mode). With
// x = pos - r0, r = |x|, O = the rotation axis (eprime[2]), A = Br0 r_ref^2, k = A w0 / ur,
// f = (r - r_ref) / r^3, f' = (3 r_ref - 2 r) / r^4 and w = x cross O:
//   U = ur x / r,   B = A x / r^3 + k f w   (the field of src/background_solarwind.cc:111-249
//   without the angles: Br = A / r^2 along x/r, B_phi phi = k f w),
//   d_i U_j = ur (delta_ij / r - x_i x_j / r^3),  div U = 2 ur / r,
//   d_i B_j = A (delta_ij / r^3 - 3 x_i x_j / r^5) + k (f' x_i w_j / r + f eps_jil O_l),  div B = 0,
//   grad|B| = (grad B) b = A (b / r^3 - 3 (x.b) x / r^5) + k (f' (w.b) x / r + f O x b),
//   b^T grad B = A (b / r^3 - 3 (x.b) x / r^5) + k (f' (x.b) w / r + f b x O).
template <class R>
__device__ __forceinline__ bool solarwind_closed(const BgParamsT<R>& g, V3<R> pos, unsigned mask, SD<R>& s)
{
   V3<R> x = pos - ld3(g.r0), O = mk(g.eprime[2][0], g.eprime[2][1], g.eprime[2][2]);
   R r2 = norm2(x), r = m_sqrt(r2), ir = R(1) / r, ir2 = ir * ir, ir3 = ir2 * ir;
   s.dmax = m_min(g.dmax_fraction * r, g.dmax0);
   s.region = mk(r < R(117.0 * 1.495978707E+13 / 1.0e10) ? R(1) : R(-1), R(-1), s.region.z);
   R k = g.A * g.w0 / g.ur0;
   R f = (r - g.r_ref) * ir3;
   V3<R> w = cross(x, O);
   s.U = (g.ur0 * ir) * x;
   s.B = (g.A * ir3) * x + (k * f) * w;
   if (mask & kE) s.E = R(-1) * (cross(s.U, s.B) / c_code<R>());  // InducedEfield: -(U x B) / c
   s.Bmag = norm(s.B);
   if (!(s.Bmag >= Lim<R>::tiny)) return false;
   R iB = R(1) / s.Bmag;
   s.bhat = iB * s.B;
   if (!(mask & (kGradU | kGradB | kDUdt))) return true;
   R fp = (R(3) * g.r_ref - R(2) * r) * ir2 * ir2;
   R xb = dot(x, s.bhat), wb = dot(w, s.bhat);
   R a3 = g.A * ir3, a5 = R(3) * g.A * ir3 * ir2 * xb;
   s.gradBmag = (a3 * s.bhat - a5 * x) + ((k * fp * wb * ir) * x + (k * f) * cross(O, s.bhat));
   V3<R> bgB = (a3 * s.bhat - a5 * x) + ((k * fp * xb * ir) * w + (k * f) * cross(s.bhat, O));
   R bgm = dot(s.bhat, s.gradBmag);
   s.divU = R(2) * g.ur0 * ir;
   s.divbhat = -bgm * iB;
   s.bgradb = iB * (bgB - bgm * s.bhat);
   s.dUdt = mk(R(0), R(0), R(0));
   R xs[3] = {x.x, x.y, x.z};
#pragma unroll
   for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) s.gradU.m[i][j] = g.ur0 * ((i == j ? ir : R(0)) - xs[i] * xs[j] * ir3);
   if (!(mask & kDerivedOnly)) {
      R ws[3] = {w.x, w.y, w.z}, Os[3] = {O.x, O.y, O.z};
#pragma unroll
      for (int i = 0; i < 3; i++)
#pragma unroll
         for (int j = 0; j < 3; j++)
            s.gradB.m[i][j] = g.A * ((i == j ? ir3 : R(0)) - R(3) * xs[i] * xs[j] * ir3 * ir2) + k * (fp * xs[i] * ws[j] * ir);
      // f eps_jil O_l
      s.gradB.m[0][1] -= k * f * Os[2]; s.gradB.m[1][0] += k * f * Os[2];
      s.gradB.m[0][2] += k * f * Os[1]; s.gradB.m[2][0] -= k * f * Os[1];
      s.gradB.m[1][2] -= k * f * Os[0]; s.gradB.m[2][1] += k * f * Os[0];
   }
   return true;
}

// ---- gridded background ------------------------------------------------------------------------
// BackgroundServerCartesian with first-order interpolation, on one uniform block held in device
// memory: zone and offset as BlockBase::GetZoneOffset (src/block_base.cc:194-203), the 8-node
// stencil of ServerCartesianFront::InteriorInterpolationStencil (src/server_cartesian.cc:206-268),
// the variables of GetVariablesInterp1 (:551-666: U and B interpolated, |B| interpolated from the
// node magnitudes, E = -U x B / c, no region variable), dmax capped by the zone length
// (:687), and the gradients of GetGradientsInterp1 (:724-823) from the stencil's derivative
// weights. A node is 32 B in FP32 (two 16-byte loads), 64 B in FP64. A point whose stencil would
// leave the block is a field error.
__device__ __forceinline__ void load_node(const float* p, float* v)
{
   const float4 a = __ldg(reinterpret_cast<const float4*>(p)), b = __ldg(reinterpret_cast<const float4*>(p) + 1);
   v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z;
}
__device__ __forceinline__ void load_node(const double* p, double* v)
{
   const double2* q = reinterpret_cast<const double2*>(p);
   const double2 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2), d = __ldg(q + 3);
   v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y; v[4] = c.x; v[5] = c.y; v[6] = d.x;
}

// Block mode: the reference's Cartesian front end at first-order interpolation over its reader's
// blocks. The primary block is the one ReadCartesianGetNode finds for the position in file units
// (src/reader_cartesian.cc:264-277); its faces are the reader's corners scaled to code units, with
// the ghost layers of BlockBase::LoadDimensions (src/block_base.cc:133-152), and its zone length
// and zone-centre origin those of ConfigureProperties (:158-171); GetZoneOffset (:194-203) and the
// stencil (src/server_cartesian.cc:206-268) follow. Zones past the block's faces are its
// neighbours' zones, i.e. the same zones of the whole domain (:291-330). The sums are in fluid
// units and the Fluid/Particle ratios come after (:549-716, 724-865): E = -(U x B) / Fluid::c_code
// before its ratio, dmax capped by the block's smallest zone length (:687). A stencil that leaves
// the domain is a field error.
// Fluid-unit U and B to code units after the interpolation, E = -(U x B) / Fluid::c_code before its ratio
// (src/server_cartesian.cc:610-628, 710-716).
template <class R>
__device__ __forceinline__ void grid_convert(const BgParamsT<R>& g, const R var[6], SD<R>& s)
{
   const R vel = g.gunits[1], mag = g.gunits[2], cf = g.gunits[3];
   const V3<R> U = mk(var[0], var[1], var[2]), B = mk(var[3], var[4], var[5]), x = cross(U, B);
   s.E = mk((-x.x / cf) * mag, (-x.y / cf) * mag, (-x.z / cf) * mag);
   s.U = mk(U.x * vel, U.y * vel, U.z * vel);
   s.B = mk(B.x * mag, B.y * mag, B.z * mag);
}

// SERVER_INTERP_ORDER -1: the boss's interpolation, ReadCartesianGetBlockData (src/reader_cartesian.cc:193-254),
// over the whole domain in file units for the position scaled as the back end scales it (:1016); the zone
// index is truncated there, and here. Zero fields outside the domain (the front end's zero-initialised buffer).
template <class R>
__device__ void grid_reader_values(const BgParamsT<R>& g, V3<R> pos, SD<R>& s)
{
   R var[6] = {R(0), R(0), R(0), R(0), R(0), R(0)}, lo[3], hi[3];
   int z[3];
   bool inside = true;
#pragma unroll
   for (int k = 0; k < 3; k++) {
      const R pc = pos[k] / R(1.495978707e+13) * R(1.0e10);
      if (!(pc >= g.dom_min[k] && pc <= g.dom_max[k])) inside = false;
      const R o = (pc - g.dom_min[k]) / (g.blk_len[k] / R(kGridBlockZones)) - R(0.5);
      z[k] = (int)o;
      lo[k] = o - (R)z[k];
      hi[k] = R(1) - lo[k];
      if (z[k] < 0 || z[k] + 1 >= g.grid_n[k]) inside = false;
   }
   if (inside) {
      const int64_t nx = g.grid_n[0], nxy = nx * (int64_t)g.grid_n[1];
      const R* base = g.grid + ((int64_t)z[2] * nxy + (int64_t)z[1] * nx + z[0]) * kGridStride;
#pragma unroll
      for (int c = 0; c < 8; c++) {
         const int ci = c & 1, cj = (c >> 1) & 1, ck = (c >> 2) & 1;
         const R w = (ci ? lo[0] : hi[0]) * (cj ? lo[1] : hi[1]) * (ck ? lo[2] : hi[2]);
         R v[7];
         load_node(base + ((int64_t)ck * nxy + (int64_t)cj * nx + ci) * kGridStride, v);
#pragma unroll
         for (int q = 0; q < 6; q++) var[q] += w * v[q];
      }
   }
   grid_convert(g, var, s);
}

template <class R>
__device__ __forceinline__ bool grid_fields_blocks(const BgParamsT<R>& g, V3<R> pos, unsigned mask, SD<R>& s)
{
   const R len = g.gunits[0], vel = g.gunits[1], mag = g.gunits[2], cf = g.gunits[3];
   R lo[3], hi[3], zl[3], face[3];
   int gz[3], bk[3];
#pragma unroll
   for (int k = 0; k < 3; k++) {
      const R pc = pos[k] / R(1.495978707e+13) * R(1.0e10);  // pos / Fluid::unit_length * Particle::unit_length
      if (!(pc >= g.dom_min[k] && pc <= g.dom_max[k])) return false;
      const int b = (int)((pc - g.dom_min[k]) / g.blk_len[k]);
      if (b >= g.grid_nb[k]) return false;
      R fmn = g.dom_min[k] + g.blk_len[k] * (R)b, fmx = fmn + g.blk_len[k];
      fmn *= len;
      fmx *= len;
      int bs = kGridBlockZones;
      if (g.grid_ghost > 0) {
         const R incr = (fmx - fmn) * ((R)g.grid_ghost / (R)kGridBlockZones);
         fmn -= incr;
         fmx += incr;
         bs += 2 * g.grid_ghost;
      }
      zl[k] = (fmx - fmn) / (R)bs;
      face[k] = fmn;
      bk[k] = b;
      const R cent = fmn + R(0.5) * zl[k];
      const R o = (pos[k] - cent) / zl[k];
      int z = (int)o;
      if (o < R(0)) z--;
      lo[k] = o - (R)z;
      hi[k] = R(1) - lo[k];
      gz[k] = kGridBlockZones * b + z - g.grid_ghost;
      if (g.grid_order == 1 && (gz[k] < 0 || gz[k] + 1 >= g.grid_n[k])) return false;
   }
   const int64_t nx = g.grid_n[0], nxy = nx * (int64_t)g.grid_n[1];
   if (g.grid_order <= 0) {
      // GetVariablesInterp0 (src/server_cartesian.cc:479-540): the values of the zone holding the point,
      // BlockBase::GetZone (src/block_base.cc:180-185); or the reader's interpolation (order -1). |B| is the
      // norm of the converted B (BackgroundBase::EvaluateBmag); order 0 has zero gradients (:848-852),
      // order -1 numerical ones (get_fields).
      s.dmax = m_min(g.dmax0, m_min(zl[0], m_min(zl[1], zl[2])));
      if (g.grid_order == 0) {
         R var[6], v[7];
         int zz[3];
#pragma unroll
         for (int k = 0; k < 3; k++) {
            zz[k] = kGridBlockZones * bk[k] + (int)((pos[k] - face[k]) / zl[k]) - g.grid_ghost;
            if (zz[k] < 0 || zz[k] >= g.grid_n[k]) return false;
         }
         load_node(g.grid + ((int64_t)zz[2] * nxy + (int64_t)zz[1] * nx + zz[0]) * kGridStride, v);
#pragma unroll
         for (int q = 0; q < 6; q++) var[q] = v[q];
         grid_convert(g, var, s);
      }
      else grid_reader_values(g, pos, s);
      s.region = mk(R(0), R(0), R(0));
      s.Bmag = norm(s.B);
      if (!(s.Bmag >= Lim<R>::tiny)) return false;
      s.bhat = s.B / s.Bmag;
      zero(s.gradU);
      zero(s.gradB);
      s.gradBmag = mk(R(0), R(0), R(0));
      s.dUdt = mk(R(0), R(0), R(0));
      derive_from_matrices(s);
      return true;
   }
   const R* base = g.grid + ((int64_t)gz[2] * nxy + (int64_t)gz[1] * nx + gz[0]) * kGridStride;
   const bool grads = (mask & (kGradU | kGradB | kDUdt)) != 0;
   R var[6] = {R(0), R(0), R(0), R(0), R(0), R(0)}, bmag = R(0);
   R gr[6][3], gbm[3] = {R(0), R(0), R(0)};
#pragma unroll
   for (int q = 0; q < 6; q++) gr[q][0] = gr[q][1] = gr[q][2] = R(0);
#pragma unroll
   for (int c = 0; c < 8; c++) {
      const int ci = c & 1, cj = (c >> 1) & 1, ck = (c >> 2) & 1;
      const R fx = ci ? lo[0] : hi[0], fy = cj ? lo[1] : hi[1], fz = ck ? lo[2] : hi[2];
      R v[7];
      load_node(base + ((int64_t)ck * nxy + (int64_t)cj * nx + ci) * kGridStride, v);
      const R w = fx * fy * fz;
#pragma unroll
      for (int q = 0; q < 6; q++) var[q] += w * v[q];
      bmag += w * v[6];
      if (grads) {
         const R d0 = (ci ? fy * fz : -fy * fz) / zl[0];
         const R d1 = (cj ? fx * fz : -fx * fz) / zl[1];
         const R d2 = (ck ? fx * fy : -fx * fy) / zl[2];
#pragma unroll
         for (int q = 0; q < 6; q++) {
            gr[q][0] += d0 * v[q];
            gr[q][1] += d1 * v[q];
            gr[q][2] += d2 * v[q];
         }
         gbm[0] += d0 * v[6];
         gbm[1] += d1 * v[6];
         gbm[2] += d2 * v[6];
      }
   }
   s.dmax = m_min(g.dmax0, m_min(zl[0], m_min(zl[1], zl[2])));
   const V3<R> U = mk(var[0], var[1], var[2]), B = mk(var[3], var[4], var[5]);
   if (mask & kE) {
      const V3<R> x = cross(U, B);
      s.E = mk((-x.x / cf) * mag, (-x.y / cf) * mag, (-x.z / cf) * mag);
   }
   s.U = mk(U.x * vel, U.y * vel, U.z * vel);
   s.B = mk(B.x * mag, B.y * mag, B.z * mag);
   s.region = mk(R(0), R(0), R(0));
   s.Bmag = bmag * mag;
   if (!(s.Bmag >= Lim<R>::tiny)) return false;
   s.bhat = s.B / s.Bmag;
   if (!grads) return true;
#pragma unroll
   for (int u = 0; u < 3; u++) {
#pragma unroll
      for (int x = 0; x < 3; x++) {
         s.gradU.m[u][x] = gr[x][u] * vel;
         s.gradB.m[u][x] = gr[3 + x][u] * mag;
      }
   }
   s.gradBmag = mk(gbm[0] * mag, gbm[1] * mag, gbm[2] * mag);
   s.dUdt = mk(R(0), R(0), R(0));
   derive_from_matrices(s);
   return true;
}

template <class R>
__device__ __forceinline__ bool grid_fields(const BgParamsT<R>& g, V3<R> pos, unsigned mask, SD<R>& s)
{
   if (g.grid_nb[0] > 0) return grid_fields_blocks(g, pos, mask, s);
   R lo[3], hi[3];
   int z[3];
#pragma unroll
   for (int k = 0; k < 3; k++) {
      const R o = (pos[k] - g.cent_min[k]) / g.zone[k];
      if (!(o >= R(0) && o < (R)(g.grid_n[k] - 1))) return false;
      z[k] = (int)o;
      lo[k] = o - (R)z[k];
      hi[k] = R(1) - lo[k];
   }
   const int64_t nx = g.grid_n[0], nxy = nx * (int64_t)g.grid_n[1];
   const R* base = g.grid + ((int64_t)z[2] * nxy + (int64_t)z[1] * nx + z[0]) * kGridStride;
   const bool grads = (mask & (kGradU | kGradB | kDUdt)) != 0;
   R var[6] = {R(0), R(0), R(0), R(0), R(0), R(0)}, bmag = R(0);
   R gr[6][3], gbm[3] = {R(0), R(0), R(0)};
#pragma unroll
   for (int q = 0; q < 6; q++) gr[q][0] = gr[q][1] = gr[q][2] = R(0);
#pragma unroll
   for (int c = 0; c < 8; c++) {
      const int ci = c & 1, cj = (c >> 1) & 1, ck = (c >> 2) & 1;
      const R fx = ci ? lo[0] : hi[0], fy = cj ? lo[1] : hi[1], fz = ck ? lo[2] : hi[2];
      R v[7];
      load_node(base + ((int64_t)ck * nxy + (int64_t)cj * nx + ci) * kGridStride, v);
      const R w = fx * fy * fz;
#pragma unroll
      for (int q = 0; q < 6; q++) var[q] += w * v[q];
      bmag += w * v[6];
      if (grads) {
         const R d0 = (ci ? fy * fz : -fy * fz) / g.zone[0];
         const R d1 = (cj ? fx * fz : -fx * fz) / g.zone[1];
         const R d2 = (ck ? fx * fy : -fx * fy) / g.zone[2];
#pragma unroll
         for (int q = 0; q < 6; q++) {
            gr[q][0] += d0 * v[q];
            gr[q][1] += d1 * v[q];
            gr[q][2] += d2 * v[q];
         }
         gbm[0] += d0 * v[6];
         gbm[1] += d1 * v[6];
         gbm[2] += d2 * v[6];
      }
   }
   s.dmax = m_min(g.dmax0, g.zone_min);
   s.U = mk(var[0], var[1], var[2]);
   s.B = mk(var[3], var[4], var[5]);
   if (mask & kE) {
      const V3<R> x = cross(s.U, s.B);
      const R c = c_code<R>();
      s.E = mk(-(x.x / c), -(x.y / c), -(x.z / c));
   }
   s.region = mk(R(0), R(0), R(0));
   s.Bmag = bmag;
   if (!(s.Bmag >= Lim<R>::tiny)) return false;
   s.bhat = s.B / s.Bmag;
   if (!grads) return true;
#pragma unroll
   for (int u = 0; u < 3; u++)
#pragma unroll
      for (int x = 0; x < 3; x++) {
         s.gradU.m[u][x] = gr[x][u];
         s.gradB.m[u][x] = gr[3 + x][u];
      }
   s.gradBmag = mk(gbm[0], gbm[1], gbm[2]);
   s.dUdt = mk(R(0), R(0), R(0));
   derive_from_matrices(s);
   return true;
}

// BackgroundBase::NumericalDerivatives restricted to U and B (src/background_base.cc:228-312):
// central differences along the field-aligned basis with step r_g = min(r_L, dmax), rotated back
// to the global frame, then the time derivative of U with step 1/w_g.
template <int BG, class R>
__device__ __noinline__ void numerical_derivs(const BgParamsT<R>& g, R t, V3<R> pos, R p, SD<R>& s, unsigned mask)
{
   unsigned m1 = mask >> 4, m2 = m1 >> 4;
   if (m1 & kAll) {
      R r_g = m_min(larmor(p, s.Bmag), s.dmax);
      V3<R> fa[3];
      fa[2] = s.bhat;
      fa[0] = second_unit(s.bhat);
      fa[1] = cross(fa[2], fa[0]);
      M3<R> gu, gbv;
      R gbm[3];
#pragma unroll
      for (int xyz = 0; xyz < 3; xyz++) {
         SD<R> f, b;
         R dr = r_g, ds = R(0);
         V3<R> pt = pos + dr * fa[xyz];
         eval_bg<BG>(g, t, pt, m1, f, ds);
         dr *= R(2);
         pt = pt - dr * fa[xyz];
         eval_bg<BG>(g, t, pt, m1, b, ds);
         if (m1 & kU) { gu.m[xyz][0] = (f.U.x - b.U.x) / dr; gu.m[xyz][1] = (f.U.y - b.U.y) / dr; gu.m[xyz][2] = (f.U.z - b.U.z) / dr; }
         if (m1 & kB) {
            gbv.m[xyz][0] = (f.B.x - b.B.x) / dr; gbv.m[xyz][1] = (f.B.y - b.B.y) / dr; gbv.m[xyz][2] = (f.B.z - b.B.z) / dr;
            gbm[xyz] = (norm(f.B) - norm(b.B)) / dr;
         }
         s.dr[xyz] = dr;
      }
#pragma unroll
      for (int i = 0; i < 3; i++)
#pragma unroll
         for (int j = 0; j < 3; j++) {
            if (m1 & kU) s.gradU.m[i][j] = fa[0][i] * gu.m[0][j] + fa[1][i] * gu.m[1][j] + fa[2][i] * gu.m[2][j];
            if (m1 & kB) s.gradB.m[i][j] = fa[0][i] * gbv.m[0][j] + fa[1][i] * gbv.m[1][j] + fa[2][i] * gbv.m[2][j];
         }
      if (m1 & kB) {
         s.gradBmag = mk(fa[0].x * gbm[0] + fa[1].x * gbm[1] + fa[2].x * gbm[2],
                         fa[0].y * gbm[0] + fa[1].y * gbm[1] + fa[2].y * gbm[2],
                         fa[0].z * gbm[0] + fa[1].z * gbm[1] + fa[2].z * gbm[2]);
      }
   }
   if (m2 & kAll) {
      R v = vel_of(p);
      R w_g = m_min(cyclotron(v, s.Bmag), v / s.dmax);
      R dt = R(1) / w_g, ds = R(0);
      SD<R> f, b;
      eval_bg<BG>(g, t + dt, pos, m2, f, ds);
      dt *= R(2);
      eval_bg<BG>(g, t + dt * R(0.5) - dt, pos, m2, b, ds);
      if (m2 & kU) s.dUdt = (f.U - b.U) / dt;
   }
}

// BackgroundBase::GetFields (src/background_base.cc:425-456). Returns false on a field error
// (|B| below the reference's sp_tiny).
template <int BG, class R>
__device__ __forceinline__ bool get_fields(const BgParamsT<R>& g, int deriv_mode, R t, V3<R> pos, R p, unsigned mask,
                                           SD<R>& s)
{
   if (BG == kBgSolarWind && deriv_mode == 1) {
      s.dr[0] = s.dr[1] = s.dr[2] = R(0.0001) * g.dmax0;
      return solarwind_closed(g, pos, mask, s);
   }
   if (BG == kBgGrid) {
      s.dr[0] = s.dr[1] = s.dr[2] = R(0.0001) * g.dmax0;
      if (!grid_fields(g, pos, mask, s)) return false;
      // SERVER_INTERP_ORDER -1 raises BACKGROUND_grad_FAIL (src/server_cartesian.cc:843-846) and the background
      // takes numerical derivatives; the contexts that select it are FP64 (spx_set_option)
      if constexpr (sizeof(R) == sizeof(double)) {
         if (g.grid_nb[0] > 0 && g.grid_order == -1 && (mask & (kGradU | kGradB | kDUdt))) {
            numerical_derivs<BG>(g, t, pos, p, s, mask);
            derive_from_matrices(s);
         }
      }
      return true;
   }
   R ds = R(0);
   s.dmax = eval_dmax<BG>(g, t, pos);
   eval_bg<BG>(g, t, pos, mask, s, ds);
   if (mask & kB) {
      s.Bmag = norm(s.B);
      if (!(s.Bmag >= Lim<R>::tiny)) return false;
      s.bhat = s.B / s.Bmag;
   }
   s.dr[0] = s.dr[1] = s.dr[2] = R(0.0001) * g.dmax0;  // incr_dmax_ratio * dmax0 (src/background_base.cc:349)
   if (!(mask & (kGradU | kGradB | kDUdt))) return true;
   if (BG == kBgUniform || BG == kBgShock) {
      zero(s.gradU);
      zero(s.gradB);
      s.gradBmag = mk(R(0), R(0), R(0));
      s.dUdt = mk(R(0), R(0), R(0));
      s.divU = R(0);
      s.divbhat = R(0);
      s.bgradb = mk(R(0), R(0), R(0));
      return true;
   }
   else if (BG == kBgSmoothShock) {  // src/background_smooth_shock.cc:149-183
      R tr = shock_trd(g.tanh_k, ds);
      R fac = tr / g.width;
      V3<R> du = ld3(g.u0) - ld3(g.u1), db = ld3(g.B0) - ld3(g.B1), n = ld3(g.n_shock);
#pragma unroll
      for (int a = 0; a < 3; a++)
#pragma unroll
         for (int b = 0; b < 3; b++) {
            s.gradU.m[a][b] = n[a] * du[b] * fac;
            s.gradB.m[a][b] = n[a] * db[b] * fac;
         }
      s.gradBmag = mv(s.gradB, s.bhat);
      s.dUdt = (tr * g.v_shock / g.width) * (ld3(g.u1) - ld3(g.u0));
   }
   else if (BG == kBgDipole) {  // src/background_dipole.cc:86-115
      V3<R> pp = pos - ld3(g.r0), M = ld3(g.M);
      R r2 = norm(pp);
      R r5 = r2 * r2 * r2;
      r2 *= r2;
      r5 *= r2;
      R mr = dot(M, pp);
      zero(s.gradU);
#pragma unroll
      for (int a = 0; a < 3; a++)
#pragma unroll
         for (int b = 0; b < 3; b++)
            s.gradB.m[a][b] = R(3) * (M[a] * pp[b] + pp[a] * M[b] + mr * ((a == b ? R(1) : R(0)) - R(5) * (pp[a] * pp[b]) / r2)) / r5;
      s.gradBmag = mv(s.gradB, s.bhat);
      s.dUdt = mk(R(0), R(0), R(0));
   }
   else if (BG == kBgSolarWind) {
      numerical_derivs<BG>(g, t, pos, p, s, mask);
   }
   derive_from_matrices(s);
   return true;
}

// ---- diffusion ---------------------------------------------------------------------------------
// The reference evaluates one component per DiffusionBase::GetComponent call
// (src/diffusion_base.cc:105-121); every model computes K_perp and K_para from the same inputs,
// so both are formed here in one evaluation (the values are those of the two calls). Components a
// model does not set stay zero, as Kappa is zeroed in DiffusionBase::SetupDiffusion
// (src/diffusion_base.cc:80-81).
template <class R>
struct Kap {
   R perp, para;
};

// The field values the coefficient models read: |B|, U and the region indicators. Passed by value
// so the coefficient evaluation never takes the address of the lane's field record.
template <class R>
struct KapIn {
   R Bmag;
   V3<R> U, region;
};
template <class R> __device__ __forceinline__ KapIn<R> kap_in(const SD<R>& s) { return {s.Bmag, s.U, s.region}; }

// DiffusionWNLTRampVLISM::EvaluateDiffusion (src/diffusion_other.cc:301-324): on the Rankine half body
// through "pos", the largest turbulent scale grows linearly from l_max_HP at the nose (a[8]) to l_max at
// the sheath (a[9]), and the three variances scale with (k_min_ref / k_min)^(ps_index - 1). Beyond the
// sheath the constant values stand.
template <class R>
__device__ __forceinline__ void wnlt_ramp(const DiffParamsT<R>& d, V3<R> pos, R& kmin, R& a2a, R& a2t, R& a2l)
{
   const R r0 = norm(pos), z0 = m_sqrt(R(0.5) * r0 * (r0 + pos.z));
   if (z0 > d.a[9]) return;
   kmin = R(6.283185307179586476925286766559005768) / (d.a[7] + (d.a[1] - d.a[7]) * (z0 - d.a[8]) / (d.a[9] - d.a[8]));
   const R k_ratio = m_pow(d.a[3] / kmin, d.a[4]);
   a2a = d.a[0] * k_ratio;
   a2t = d.a[5] * k_ratio;
   a2l = d.a[6] * k_ratio;
}

// "mu" and "Omega" are DiffusionBase's pitch-angle cosine and cyclotron frequency, which only the WNLT models
// read; they are set once per GetComponent and not moved by the spatial difference quotients
// (src/diffusion_base.cc:105-174). The Parker types pass neither. DK >= 0 fixes the diffusion class at
// compile time (kernels specialised for one class); -1 dispatches on the descriptor.
template <class R, int DK = -1>
__device__ __forceinline__ Kap<R> kappa_pp(const DiffParamsT<R>& d, V3<R> pos, R p, R vmag, const KapIn<R>& s, R mu = R(0),
                                           R Omega = R(0))
{
   Kap<R> K{R(0), R(0)};
   switch (DK >= 0 ? DK : d.kind) {
   case kDfPara: K.para = d.a[0]; break;                      // src/diffusion_other.cc:381-385
   case kDfPerp: K.perp = d.a[0]; break;                      // :459-463
   case kDfFull: K.perp = d.a[0]; K.para = d.a[1]; break;     // :538-543
   case kDfFlowMomentum:                                      // :622-627
      K.para = d.a[0] * m_pow(norm(s.U) / d.a[1], d.a[2]) * m_pow(p / d.a[3], d.a[4]);
      K.perp = d.a[5] * K.para;
      break;
   case kDfKinEnergyRadial: {                                 // :713-723
      R r = norm(pos);
      R kap_mom = d.a[0] * m_pow(enr_kin(p) / d.a[1], d.a[3]);
      if (d.i0 == 0 || r < d.a[2]) K.para = kap_mom * m_pow(r / d.a[2], d.a[4]);
      else if (r < d.a[2] + d.a[7]) { R q = norm(s.U) / d.a[6]; K.para = kap_mom * (q * q); }
      else K.para = kap_mom * d.a[9];
      K.perp = d.a[5] * K.para;
      break;
   }
   case kDfRigidityB:                                         // :804-809
      K.para = (d.a[0] * vmag / R(3)) * m_pow(rigidity(p) / d.a[1], d.a[3]) * m_pow(s.Bmag / d.a[2], d.a[4]);
      K.perp = d.a[5] * K.para;
      break;
   case kDfStrauss2013:
   case kDfPotgieter2015: {                                   // :886-904, 968-986
      R lism = (d.i0 < 0) ? R(0) : (s.region[d.i0] > R(0) ? R(0) : R(1));
      R lk = lism * d.a[1] + (R(1) - lism) * d.a[0];
      R B0_eff = lism * s.Bmag + (R(1) - lism) * d.a[3];
      R rig = rigidity(p);
      if (d.kind == kDfStrauss2013)
         K.para = (lk * vmag / R(3)) * (rig < d.a[2] ? m_cbrt(rig / d.a[2]) : rig / d.a[2]) * (B0_eff / s.Bmag);
      else {
         R q = rig / d.a[2];
         K.para = lk * (vmag / c_code<R>()) * (rig < d.a[2] ? R(1) : m_sqrt(q * q * q)) * (B0_eff / s.Bmag);
      }
      K.perp = (lism * d.a[5] + (R(1) - lism) * d.a[4]) * K.para;
      break;
   }
   case kDfEmpiricalSOQLT: {                                  // :1049-1072
      R q = rigidity(p) / d.a[2];
      R c = m_cos(R(0.5) * s.region[d.i1 < 0 ? 0 : (d.i1 > 2 ? 2 : d.i1)]);
      R damp = R(1) + d.a[6] * (c * c);
      K.para = ((d.a[0] * vmag / R(3)) * m_cbrt(q * (R(1) + (q * q) * (q * q))) * (d.a[3] / s.Bmag)) / damp;
      R bmix = (d.i0 < 0) ? R(1) : (s.region[d.i0] < R(0) ? R(0) : R(1));
      R lam = (norm(pos) < d.a[5]) ? d.a[1] * (bmix + (R(1) - bmix) * d.a[4]) : d.a[1];
      K.perp = ((lam * vmag / R(3)) * m_cbrt(q * (R(1) + q * q)) * (d.a[3] / s.Bmag)) / damp;
      break;
   }
   case kDfWNLT: case kDfWNLTRamp: {                          // :215-228, 301-327
      R kmin = d.a[3], a2a = d.a[0], a2t = d.a[5], a2l = d.a[6];
      if (d.kind == kDfWNLTRamp) wnlt_ramp(d, pos, kmin, a2a, a2t, a2l);
      R q = mu / kmin;
      const R ct = R(0.5) * d.a[4] / (d.a[2] + R(1)) * (q * q) * a2t;
      q = vmag * (R(1) - mu * mu) / Omega;
      const R cl = R(0.125) * (q * q) * a2l;
      K.perp = vmag * m_sqrt(ct + cl);
      break;
   }
   default: break;
   }
   return K;
}

// Pitch-angle component D_mumu (Kappa[2]) of the pitch-angle models at "pos". The WNLT models give the
// QLT coefficient, with the ramp's local k_min and A2A: the reference defines
// USE_QLT_SCATT_WITH_WNLT_DIFF (src/diffusion_other.hh:137), so DiffusionWNLTConstant::EvaluateDiffusion
// returns before its hypergeometric correction (src/diffusion_other.cc:227-232).
template <class R>
__device__ __forceinline__ R kappa_mumu(const DiffParamsT<R>& d, V3<R> pos, R vmag, R Omega, R mu)
{
   R st2 = R(1) - mu * mu;
   if (d.kind == kDfIsotropic) return d.a[0] * st2;  // src/diffusion_other.cc:64-68
   if (d.kind == kDfQLT || d.kind == kDfWNLT || d.kind == kDfWNLTRamp) {  // src/diffusion_other.cc:145-149
      R kmin = d.a[3], a2a = d.a[0], a2t, a2l;
      if (d.kind == kDfWNLTRamp) wnlt_ramp(d, pos, kmin, a2a, a2t, a2l);
      return R(0.25) * R(3.141592653589793238462643383279502884) * d.a[4] * m_abs(Omega) * st2 *
             m_pow(vmag * kmin * m_abs(mu / Omega), d.a[4]) * a2a;
   }
   return R(0);
}

// d D_mumu / d mu: analytic for the isotropic model (src/diffusion_other.cc:76-79), else the
// one-sided difference of DiffusionBase::GetMuDerivative (src/diffusion_base.cc:226-255).
template <class R>
__device__ __forceinline__ R kappa_mumu_dmu(const DiffParamsT<R>& d, V3<R> pos, R vmag, R Omega, R mu, R dmumu)
{
   if (d.kind == kDfIsotropic) return R(-2) * d.a[0] * mu;
   if (d.kind != kDfQLT && d.kind != kDfWNLT && d.kind != kDfWNLTRamp) return R(0);
   R dmu = Lim<R>::small * (mu + Lim<R>::small < R(1) ? R(1) : R(-1));
   return (kappa_mumu(d, pos, vmag, Omega, mu + dmu) - dmumu) / dmu;
}

// Models whose gradient needs no field-gradient matrix (only grad|B| or grad U . U).
template <class R>
__device__ __forceinline__ bool kappa_grad_is_analytic(const DiffParamsT<R>& d, int dk = -1)
{
   const int kind = dk >= 0 ? dk : d.kind;
   return kind == kDfPara || kind == kDfPerp || kind == kDfFull || kind == kDfFlowMomentum ||
          kind == kDfKinEnergyRadial || kind == kDfRigidityB;
}

// Spatial gradients of K_perp and K_para: the analytic GetDirectionalDerivative overrides
// (src/diffusion_other.cc:395-398, 473-476, 553-556, 637-642, 732-742, 818-823), else the
// base-class central difference with the field moved along its gradient
// (src/diffusion_base.cc:131-174).
// Out-of-line evaluation for the difference quotients of the gradient (six calls a step).
template <class R>
__device__ __noinline__ Kap<R> kappa_pp_call(const DiffParamsT<R>& d, V3<R> pos, R p, R vmag, KapIn<R> s)
{
   return kappa_pp(d, pos, p, vmag, s);
}

template <class R>
__device__ __noinline__ Kap<R> kappa_wnlt_call(const DiffParamsT<R>& d, V3<R> pos, R p, R vmag, KapIn<R> s, R mu, R Omega)
{
   return kappa_pp(d, pos, p, vmag, s, mu, Omega);
}

// kPitch: the caller is a type with a pitch angle, for which the WNLT ramp (never compiled for Parker) exists.
// DK as for kappa_pp.
template <class R, bool kPitch = false, int DK = -1>
__device__ __forceinline__ void kappa_grad(const DiffParamsT<R>& d, V3<R> pos, R p, R vmag, const SD<R>& s, Kap<R> K, V3<R>& gperp,
                                           V3<R>& gpara, R mu = R(0), R Omega = R(0))
{
   switch (DK >= 0 ? DK : d.kind) {
   // DiffusionWNLTConstant reads neither the position nor |B| (mu and Omega stay fixed), so the base
   // class's difference quotient is exactly zero
   case kDfPara: case kDfPerp: case kDfFull: case kDfWNLT:
      gperp = mk(R(0), R(0), R(0));
      gpara = gperp;
      return;
   case kDfFlowMomentum: {
      R un2 = norm2(s.U);
      V3<R> gl = mk(dot(row(s.gradU, 0), s.U), dot(row(s.gradU, 1), s.U), dot(row(s.gradU, 2), s.U));
      gperp = (K.perp * d.a[2] / un2) * gl;
      gpara = (K.para * d.a[2] / un2) * gl;
      return;
   }
   case kDfKinEnergyRadial: {
      R r = norm(pos);
      V3<R> gl;
      if (d.i0 == 0 || r < d.a[2]) gl = (d.a[4] / (r * r)) * pos;
      else if (r < d.a[2] + d.a[7]) {
         R un2 = norm2(s.U);
         gl = (R(2) / un2) * mk(dot(row(s.gradU, 0), s.U), dot(row(s.gradU, 1), s.U), dot(row(s.gradU, 2), s.U));
      }
      else gl = mk(R(0), R(0), R(0));
      gperp = K.perp * gl;
      gpara = K.para * gl;
      return;
   }
   case kDfRigidityB: {
      V3<R> gl = (d.a[4] / s.Bmag) * s.gradBmag;
      gperp = K.perp * gl;
      gpara = K.para * gl;
      return;
   }
   default: {
      R gpe[3], gpa[3];
      KapIn<R> q = kap_in(s);
#pragma unroll
      for (int xyz = 0; xyz < 3; xyz++) {
         R dr = R(0.5) * s.dr[xyz];
         R e[3] = {R(0), R(0), R(0)};
         e[xyz] = dr;
         q.Bmag = s.Bmag + s.gradBmag[xyz] * dr;
         Kap<R> kf = kPitch && d.kind == kDfWNLTRamp ? kappa_wnlt_call(d, pos + mk(e[0], e[1], e[2]), p, vmag, q, mu, Omega)
                                           : kappa_pp_call(d, pos + mk(e[0], e[1], e[2]), p, vmag, q);
         q.Bmag = q.Bmag - s.gradBmag[xyz] * (R(2) * dr);
         e[xyz] = dr - R(2) * dr;
         Kap<R> kb = kPitch && d.kind == kDfWNLTRamp ? kappa_wnlt_call(d, pos + mk(e[0], e[1], e[2]), p, vmag, q, mu, Omega)
                                           : kappa_pp_call(d, pos + mk(e[0], e[1], e[2]), p, vmag, q);
         gpe[xyz] = (kf.perp - kb.perp) / (R(2) * dr);
         gpa[xyz] = (kf.para - kb.para) / (R(2) * dr);
      }
      gperp = mk(gpe[0], gpe[1], gpe[2]);
      gpara = mk(gpa[0], gpa[1], gpa[2]);
      return;
   }
   }
}

// ---- boundaries ---------------------------------------------------------------------------------
// Transient state of one boundary (src/boundary_base.hh): delta, delta_old, crossings left,
// crossed flag; TERMINAL is crossings_left == 1 (src/boundary_base.cc:150-151, 187-188).
template <class R>
struct alignas(sizeof(R) == 4 ? 16 : 8) BndState {
   R delta, delta_old;
   int crossings_left;
   int crossed;
};

// The boundary states of one lane, held in dynamic shared memory: state j of the block's lanes
// is one contiguous row, so a warp reads or writes a row with conflict-free vector accesses.
template <class R>
struct BndView {
   BndState<R>* p;  // this lane's state 0
   int stride;      // lanes per block
   __device__ __forceinline__ BndState<R> ld(int j) const { return p[j * stride]; }
   __device__ __forceinline__ void st(int j, const BndState<R>& b) const { p[j * stride] = b; }
};

// Outward normal of a reflecting spatial boundary at "pos" (the _normal of EvaluateBoundary).
template <class R>
__device__ V3<R> bnd_normal(const BndParamsT<R>& b, V3<R> pos)
{
   switch (b.kind) {
   case kBtPlaneAbsorb: case kBtPlaneReflect: case kBtPlanePass: return ld3(b.norm);
   case kBtBoxReflect: {
      R best = -Lim<R>::large;
      V3<R> nrm = mk(R(0), R(0), R(0));
      for (int s = 0; s < 3; s++) {
         V3<R> n = ld3(b.normals[s]);
         R d1 = -dot(pos - ld3(b.corner0), n);
         if (d1 > best) { best = d1; nrm = R(-1) * n; }
         R d2 = dot(pos - ld3(b.corner1), n);
         if (d2 > best) { best = d2; nrm = n; }
      }
      return nrm;
   }
   case kBtSphereAbsorb: case kBtSphereReflect: case kBtSpherePass: return unit(pos - ld3(b.origin));
   case kBtCylinderAbsorb: {
      V3<R> fa[3] = {ld3(b.fa[0]), ld3(b.fa[1]), ld3(b.fa[2])};
      V3<R> pr = to_basis(pos - ld3(b.origin), fa);
      pr.z = R(0);
      return from_basis(unit(pr), fa);
   }
   default: return mk(R(0), R(0), R(0));
   }
}

// EvaluateBoundary (src/boundary_time.cc, src/boundary_space.cc, src/boundary_momentum.cc), one
// evaluator per boundary class so that a loop over the boundaries of one class dispatches over that
// class's kinds only. For time boundaries the delta is formed from the accumulated time.
// BL 1: the boundary layout fixed at compile time (one expiry or pass time boundary and spheres, see
// BndLayout); its evaluators skip the other kinds.
template <int BL, class R, class A>
__device__ __forceinline__ void eval_time_bnd(const BndParamsT<R>& b, BndState<R>& st, const A& t)
{
   if (BL != 1 && b.kind == kBtTimeRecurrent) {
      R k = (R)((b.max_crossings - st.crossings_left) + 1);
      st.delta = (R)acc_diff(t, k * b.timemark, k * b.timemark_lo);
   }
   else st.delta = (R)acc_diff(t, b.timemark, b.timemark_lo);  // expire, pass
}

template <int BL, class R>
__device__ __forceinline__ void eval_space_bnd(const BndParamsT<R>& b, BndState<R>& st, V3<R> pos, V3<R> region)
{
   // spheres first: the usual inner and outer boundaries of the heliospheric set-ups
   if (BL == 1 || b.kind == kBtSphereAbsorb || b.kind == kBtSphereReflect || b.kind == kBtSpherePass) {
      st.delta = norm(pos - ld3(b.origin)) - b.radius;
      return;
   }
   switch (b.kind) {
   case kBtPlaneAbsorb: case kBtPlaneReflect: case kBtPlanePass:
      st.delta = dot(pos - ld3(b.origin), ld3(b.norm));
      break;
   case kBtBoxReflect: {
      st.delta = -Lim<R>::large;
#pragma unroll
      for (int s = 0; s < 3; s++) {
         V3<R> n = ld3(b.normals[s]);
         R d1 = -dot(pos - ld3(b.corner0), n);
         if (d1 > st.delta) st.delta = d1;
         R d2 = dot(pos - ld3(b.corner1), n);
         if (d2 > st.delta) st.delta = d2;
      }
      break;
   }
   case kBtRankineAbsorb: {
      V3<R> pr = pos - ld3(b.origin);
      R z = dot(pr, ld3(b.axis)), r = norm(pr);
      st.delta = r - b.z_nose * m_sqrt(R(2) / (R(1) + z / r));
      break;
   }
   case kBtCylinderAbsorb: {
      V3<R> fa[3] = {ld3(b.fa[0]), ld3(b.fa[1]), ld3(b.fa[2])};
      V3<R> pr = to_basis(pos - ld3(b.origin), fa);
      st.delta = m_sqrt(pr.x * pr.x + pr.y * pr.y) - b.radius;
      break;
   }
   case kBtRegionAbsorb: st.delta = region[b.region_ind] - b.region_val; break;
   }
}

template <class R>
__device__ __forceinline__ void eval_mom_bnd(const BndParamsT<R>& b, BndState<R>& st, V3<R> pos, V3<R> mom,
                                             V3<R> bhat, int traj)
{
   // BoundaryMirror::EvaluateBoundary (src/boundary_momentum.cc:329-339): the parallel momentum, which is
   // p mu for Focused, the native third component for the guiding-centre types and p . bhat for Lorentz
   if (b.kind == kBtMirror) {
      st.delta = (traj == kFocused) ? mom.x * mom.y : (traj == kGuiding ? mom.z : dot(mom, bhat));
      return;
   }
   st.delta = (traj == kLorentz ? norm(mom) : mom.x) - b.momentum;
   if (b.kind == kBtMomentumSlab && st.delta * st.delta_old < R(0)) {
      if (dot(pos - ld3(b.slab_r0), ld3(b.slab_n)) * dot(pos - ld3(b.slab_r1), ld3(b.slab_n)) > R(0)) st.delta_old = st.delta;
   }
   if (b.kind == kBtMomentumShell && st.delta * st.delta_old < R(0)) {
      R rd = norm(pos - ld3(b.slab_r0));
      if (rd < b.r1 || rd > b.r2) st.delta_old = st.delta;
   }
}

// CLS: the class of the boundary when the caller knows it (0 time, 1 space, 2 momentum), -1 from b.cls
template <int CLS, int BL = 0, class R, class A>
__device__ __forceinline__ void eval_bnd(const BndParamsT<R>& b, BndState<R>& st, const A& t, V3<R> pos, V3<R> mom,
                                         V3<R> bhat, V3<R> region, int traj)
{
   const int cls = CLS >= 0 ? CLS : b.cls;
   if (cls == 0) eval_time_bnd<BL>(b, st, t);
   else if (cls == 1) eval_space_bnd<BL>(b, st, pos, region);
   else eval_mom_bnd(b, st, pos, mom, bhat, traj);
}

// BoundaryBase::ResetBoundary (src/boundary_base.cc:138-162)
template <class R, class A>
__device__ __forceinline__ void reset_bnd(const BndParamsT<R>& b, BndState<R>& st, R scale, const A& t, V3<R> pos,
                                          V3<R> mom, V3<R> bhat, V3<R> region, int traj)
{
   st.crossings_left = b.max_crossings;
   st.delta_old = R(0);
   eval_bnd<-1>(b, st, t, pos, mom, bhat, region, traj);
   st.delta_old = st.delta;
   if (st.delta_old == R(0)) st.delta_old = -Lim<R>::tiny * m_abs(scale);
   st.crossed = 0;
}

// BoundaryBase::ComputeBoundary (src/boundary_base.cc:105-127)
template <int CLS, int BL = 0, class R, class A>
__device__ __forceinline__ void compute_bnd(const BndParamsT<R>& b, BndState<R>& st, const A& t, V3<R> pos, V3<R> mom,
                                            V3<R> bhat, V3<R> region, int traj)
{
   eval_bnd<CLS, BL>(b, st, t, pos, mom, bhat, region, traj);
   if (st.delta * st.delta_old <= R(0)) {
      st.crossed = 1;
      if (st.delta * st.delta_old == R(0)) st.delta = -st.delta_old;
   }
   else st.crossed = 0;
}

// BoundaryBase::RecordBoundary (src/boundary_base.cc:168-191)
template <int CLS, class R, class A>
__device__ __forceinline__ void record_bnd(const BndParamsT<R>& b, BndState<R>& st, const A& t, V3<R> pos, V3<R> mom,
                                           V3<R> bhat, V3<R> region, int traj)
{
   if (st.crossed) {
      st.crossings_left--;
      if (b.recurrent) eval_bnd<CLS>(b, st, t, pos, mom, bhat, region, traj);
      else st.delta_old = st.delta;
      st.crossed = 0;
   }
   else st.delta_old = st.delta;
}

}  // namespace spx
