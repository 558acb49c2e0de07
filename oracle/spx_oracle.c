/*
 * spx_oracle.c -- CPU restatement of SPECTRUM's test-particle stepping path (TEST ORACLE).
 *
 * Test infrastructure only (see spx_oracle.h). Each function names the reference code it
 * restates. Deviations from the reference are deliberate and listed here:
 *   D1 BackgroundSmoothShock::EvaluateDmax (src/background_smooth_shock.cc:193-197) uses the
 *      shock distance of the *previous* field evaluation of the object (it runs before
 *      EvaluateBackground in BackgroundBase::GetFields, src/background_base.cc:434-442); here it
 *      is the distance at the current point. With opts->reference_quirks the reference's
 *      behaviour is reproduced instead (the object's distance persists across the trajectories of
 *      a run; it starts at 0), so the restatement can be compared with the reference bit for bit.
 *   D2 DistributionTemplated::AddEvent (src/distribution_templated.cc:145-181) computes a
 *      negative bin for left outliers beyond one bin width when bin_outside is set; here such
 *      events go to bin 0, which is what the code intends.
 *   D3 Trajectories run independently: samplers that step through a sequence
 *      (InitialSpaceLine, InitialTimeInterval with n_intervals > 0) give trajectory k the k-th
 *      element instead of continuing a per-process counter.
 * Everything else, including the order of floating-point operations where it matters, follows
 * the reference.
 */
#include "spx_oracle.h"
#include "spx_rng.h"
#include "spx_rk_tables.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* With nudge_libm (a test option) every result of the transcendental functions below is moved one
 * ulp away from zero: a model of another libm rounding them differently in the last bit, with which
 * the parity tests measure a problem's conditioning. The macros leave sqrt and the arithmetic alone
 * (both round correctly everywhere); inside each macro the name refers to the function itself. */
static int g_nudge_libm = 0;
static double nudged(double v) { return g_nudge_libm ? nextafter(v, v >= 0.0 ? INFINITY : -INFINITY) : v; }
#define exp(x) nudged(exp(x))
#define log(x) nudged(log(x))
#define log10(x) nudged(log10(x))
#define pow(x, y) nudged(pow(x, y))
#define sin(x) nudged(sin(x))
#define cos(x) nudged(cos(x))
#define tanh(x) nudged(tanh(x))
#define acos(x) nudged(acos(x))
#define asin(x) nudged(asin(x))
#define atan2(y, x) nudged(atan2(y, x))
#define cbrt(x) nudged(cbrt(x))

/* ------------------------------------------------------------------------------------------ */
/* constants: common/definitions.hh:54-66, common/specie.hh:30-82, common/physical_constants.hh */
/* ------------------------------------------------------------------------------------------ */
#define SP_LARGE 1.0E+20
#define SP_LITTLE 1.0E-5
#define SP_SMALL 1.0E-8
#define SP_TINY 1.0E-15
#define M_2PI_ 6.283185307179586476925286766559005768E+0
#define M_PI_ 3.141592653589793238462643383279502884E+0

static const double c_light = 2.99792458e+10;
#define AU_CM 1.495978707e+13 /* Fluid::unit_length, the astronomical unit in cm */
static double unit_velocity(void) { return 0.1 * c_light; }
static double c_code(void) { return c_light / unit_velocity(); }
static const double p_mass = 1.0;   /* proton mass / unit_mass */
static const double p_charge = 1.0; /* proton charge / unit_charge */

/* trajectory status bits (src/trajectory_base.hh:45-57) */
#define TRAJ_FINISH 0x0010u
#define TRAJ_TIME_CROSSED 0x0020u
#define TRAJ_SPATIAL_CROSSED 0x0040u
#define TRAJ_MOMENTUM_CROSSED 0x0080u
#define TRAJ_DISCARD 0x0100u

#define MAX_TRAJ_STEPS 10000000   /* src/trajectory_base.hh:38 */
#define MAX_TIME_ADAPT 100        /* src/trajectory_base.hh:41 */

/* mask bits (common/spatial_data.hh:23-48) */
#define BG_U 0x0001u
#define BG_B 0x0002u
#define BG_E 0x0004u
#define BG_ALL 0x0007u
#define BG_gradU 0x0010u
#define BG_gradB 0x0020u
#define BG_gradE 0x0040u
#define BG_dUdt 0x0100u
#define BG_dBdt 0x0200u
#define BG_dEdt 0x0400u

/* ------------------------------------------------------------------------------------------ */
/* vector helpers (common/vectors.hh, common/vectors.cc)                                      */
/* ------------------------------------------------------------------------------------------ */
typedef struct { double x[3]; } v3;

static v3 V(double a, double b, double c) { v3 r = {{a, b, c}}; return r; }
static v3 vadd(v3 a, v3 b) { return V(a.x[0] + b.x[0], a.x[1] + b.x[1], a.x[2] + b.x[2]); }
static v3 vsub(v3 a, v3 b) { return V(a.x[0] - b.x[0], a.x[1] - b.x[1], a.x[2] - b.x[2]); }
static v3 vscale(double s, v3 a) { return V(s * a.x[0], s * a.x[1], s * a.x[2]); }
static v3 vdiv(v3 a, double s) { return V(a.x[0] / s, a.x[1] / s, a.x[2] / s); }
static double vdot(v3 a, v3 b) { return a.x[0] * b.x[0] + a.x[1] * b.x[1] + a.x[2] * b.x[2]; }
static double vnorm2(v3 a) { return a.x[0] * a.x[0] + a.x[1] * a.x[1] + a.x[2] * a.x[2]; }
static double vnorm(v3 a) { return sqrt(vnorm2(a)); }
static v3 vcross(v3 a, v3 b)
{
   return V(a.x[1] * b.x[2] - a.x[2] * b.x[1], a.x[2] * b.x[0] - a.x[0] * b.x[2], a.x[0] * b.x[1] - a.x[1] * b.x[0]);
}
static v3 vunit(v3 a) { double n = vnorm(a); return V(a.x[0] / n, a.x[1] / n, a.x[2] / n); }
static const v3 cart_unit[3] = {{{1.0, 0.0, 0.0}}, {{0.0, 1.0, 0.0}}, {{0.0, 0.0, 1.0}}};

/* GetSecondUnitVec, common/vectors.cc:453-468 */
static v3 second_unit(v3 f)
{
   int m;
   if (fabs(f.x[0]) < fabs(f.x[1])) m = (fabs(f.x[0]) < fabs(f.x[2])) ? 0 : 2;
   else m = (fabs(f.x[1]) < fabs(f.x[2])) ? 1 : 2;
   return vunit(vcross(f, cart_unit[m]));
}
/* GeoVector::ChangeToBasis / ChangeFromBasis, common/vectors.cc:58-95 */
static v3 to_basis(v3 a, const v3 b[3]) { return V(vdot(a, b[0]), vdot(a, b[1]), vdot(a, b[2])); }
static v3 from_basis(v3 a, const v3 b[3])
{
   return V(a.x[0] * b[0].x[0] + a.x[1] * b[1].x[0] + a.x[2] * b[2].x[0],
            a.x[0] * b[0].x[1] + a.x[1] * b[1].x[1] + a.x[2] * b[2].x[1],
            a.x[0] * b[0].x[2] + a.x[1] * b[1].x[2] + a.x[2] * b[2].x[2]);
}

typedef struct { double m[3][3]; } m3;
static m3 mzero(void) { m3 r; memset(&r, 0, sizeof r); return r; }
/* matrix * vector: rows dotted with the vector (common/matrix.hh:480-483) */
static v3 mvmul(const m3* a, v3 v)
{
   return V(a->m[0][0] * v.x[0] + a->m[0][1] * v.x[1] + a->m[0][2] * v.x[2],
            a->m[1][0] * v.x[0] + a->m[1][1] * v.x[1] + a->m[1][2] * v.x[2],
            a->m[2][0] * v.x[0] + a->m[2][1] * v.x[1] + a->m[2][2] * v.x[2]);
}
/* vector * matrix (common/matrix.hh:493-500) */
static v3 vmmul(v3 v, const m3* a)
{
   v3 r;
   int j;
   for (j = 0; j < 3; j++) r.x[j] = v.x[0] * a->m[0][j] + v.x[1] * a->m[1][j] + v.x[2] * a->m[2][j];
   return r;
}
static double mtrace(const m3* a) { return a->m[0][0] + a->m[1][1] + a->m[2][2]; }

/* ------------------------------------------------------------------------------------------ */
/* kinematics (common/physics.hh:246-510)                                                     */
/* ------------------------------------------------------------------------------------------ */
static double enr_tot(double p) { double c = c_code(); return sqrt(p * p + (p_mass * c) * (p_mass * c)) * c; }
static double enr_kin(double p) { double c = c_code(); return enr_tot(p) - p_mass * (c * c); }
static double vel_of(double p) { double c = c_code(); return p * (c * c) / enr_tot(p); }
static double mom_of(double e) { double c = c_code(); return sqrt(e * (e + 2.0 * p_mass * (c * c))) / c; }
static double rigidity(double p) { return p * c_code() / fabs(p_charge); }
static double larmor(double p, double b) { return p * c_code() / (fabs(p_charge) * b); }
static double rel_factor(double v) { double r = v / c_code(); return 1.0 / sqrt(1.0 - r * r); }
static double cyclotron(double v, double b) { return p_charge * b / (rel_factor(v) * p_mass * c_code()); }
/* Particle::Vel<Cartesian>(GeoVector): mom rescaled by v(|p|)/|p| */
static v3 vel_cart(v3 mom) { double m = vnorm(mom); return vscale(vel_of(m) / m, mom); }
/* Particle::Vel<SphericalRMP>: length is mom[0] */
static v3 vel_rmp(v3 mom) { double m = mom.x[0]; return vscale(vel_of(m) / m, mom); }

/* ------------------------------------------------------------------------------------------ */
/* spatial data (common/spatial_data.hh:55-135)                                               */
/* ------------------------------------------------------------------------------------------ */
typedef struct {
   unsigned mask;
   v3 U, B, E;
   m3 gradU, gradB;
   v3 dUdt, dBdt;
   double Bmag, dBmagdt;
   v3 gradBmag, bhat, region;
   double dmax;
   double dr[3]; /* "safe" increments for diffusion derivatives (BackgroundBase::SetupBackground) */
} spdata;

static double sd_divU(const spdata* s) { return mtrace(&s->gradU); }
static v3 sd_curlB(const spdata* s)
{
   return V(s->gradB.m[1][2] - s->gradB.m[2][1], s->gradB.m[2][0] - s->gradB.m[0][2], s->gradB.m[0][1] - s->gradB.m[1][0]);
}
/* divbhat, gradbhat: common/spatial_data.hh:288-330 */
static double sd_divbhat(const spdata* s) { return (mtrace(&s->gradB) - vdot(s->gradBmag, s->bhat)) / s->Bmag; }
static m3 sd_gradbhat(const spdata* s)
{
   m3 r;
   int i, j;
   for (i = 0; i < 3; i++)
      for (j = 0; j < 3; j++) r.m[i][j] = (s->gradB.m[i][j] - s->gradBmag.x[i] * s->bhat.x[j]) / s->Bmag;
   return r;
}

/* ------------------------------------------------------------------------------------------ */
/* spec parsing                                                                               */
/* ------------------------------------------------------------------------------------------ */
typedef struct {
   const uint8_t* p;
   size_t n, pos;
   int bad;
} rd_t;

static int rd_rec(rd_t* r, void* dst, size_t size)
{
   if (r->pos >= r->n) { r->bad = 1; return -1; }
   size_t len = r->p[r->pos];
   if (r->pos + 1 + len > r->n || (size && len != size)) { r->bad = 1; return -1; }
   if (dst) memcpy(dst, r->p + r->pos + 1, len);
   r->pos += 1 + len;
   return (int)len;
}
static double rd_d(rd_t* r) { double v = 0; rd_rec(r, &v, 8); return v; }
static int rd_i(rd_t* r) { int32_t v = 0; rd_rec(r, &v, 4); return v; }
static int rd_b(rd_t* r) { uint8_t v = 0; rd_rec(r, &v, 1); return v; }
static v3 rd_v(rd_t* r) { v3 v = {{0, 0, 0}}; rd_rec(r, v.x, 24); return v; }
static void rd_mi(rd_t* r, int out[3]) { int32_t v[3] = {0, 0, 0}; rd_rec(r, v, 12); out[0] = v[0]; out[1] = v[1]; out[2] = v[2]; }
static int rd_ints(rd_t* r, int* out, int max)
{
   int32_t tmp[64];
   int len = rd_rec(r, tmp, 0), k;
   if (len < 0 || len % 4 || len / 4 > max || len / 4 > 64) { r->bad = 1; return 0; }
   for (k = 0; k < len / 4; k++) out[k] = tmp[k];
   return len / 4;
}

#define MAXB 8
#define MAXD 4

enum { BG_UNIFORM = 1, BG_SHOCK, BG_SMOOTHSHOCK, BG_DIPOLE, BG_SOLARWIND, BG_GRID, BG_DISCONT, BG_SMOOTHDISCONT };
typedef struct {
   int kind;
   double t0, dmax0;
   v3 r0, u0, B0;
   /* shock (src/background_shock.cc:56-80) */
   v3 n_shock, u1, B1, E0, E1;
   double v_shock, compression, width, dmax_fraction;
   double tanh_k;  /* the smooth transition's tanh_width_factor */
   /* dipole */
   v3 M;
   /* solar wind */
   v3 Omega, eprime[3];
   double w0, r_ref, ur0;
} bg_t;

/* the guiding-centre types: Guiding, GuidingScatt, GuidingDiff, GuidingDiffScatt (configure.ac:239-242) */
#define IS_GC(tt) ((tt) >= 201 && (tt) <= 204)
enum { DF_ISO = 1, DF_QLT, DF_PARA, DF_PERP, DF_FULL, DF_FLOWMOM, DF_KINRAD, DF_RIGB, DF_STRAUSS, DF_POTGIETER, DF_EMPIRICAL,
       DF_WNLT, DF_WNLT_RAMP };
typedef struct {
   int kind;
   double a[10];
   int i0, i1, i2;
} df_t;

enum { BT_TIME = 1, BT_TIME_PASS, BT_TIME_REC, BT_PLANE_ABS = 10, BT_PLANE_REF, BT_PLANE_PASS, BT_BOX_REF, BT_SPH_ABS,
       BT_SPH_REF, BT_RANKINE, BT_CYL, BT_REGION, BT_SPH_PASS, BT_MOM_INJ = 30, BT_MOM_PASS, BT_MOM_SLAB, BT_MOM_SHELL,
       BT_MIRROR };
typedef struct {
   int kind, cls; /* cls: 0 time, 1 space, 2 momentum */
   int reflect, recurrent;
   int max_crossings, n_actions, actions[MAXD];
   double timemark, momentum, radius, z_nose, r1, r2, region_val;
   int region_ind;
   v3 origin, norm, corner0, corner1, normals[3], axis, fa[3], slab_r0, slab_r1, slab_n;
   /* transient */
   double delta, delta_old, scale;
   v3 normal;
   int crossings_left, crossed, terminal;
} bnd_t;

enum { IT_FIXED = 1, IT_INTERVAL, IS_FIXED = 10, IS_LINE, IS_CIRCLE, IS_BOX, IS_SPHERE, IS_SECTOR, IS_RANKINE,
       IS_CYLINDER, IS_CYL_SECTOR,
       IM_FIXED = 30, IM_BEAM, IM_RING, IM_SHELL, IM_THICK, IM_MAXWELL, IM_LOGE_PITCH = 40, IS_EQ_BAND };
typedef struct {
   int kind;
   double a[8];
   v3 v0, v1, v2;
   int n_int, flag;
} ini_t;

enum { DS_TIME = 1, DS_POS, DS_MOM, DS_POSMOM, DS_SPEC, DS_SPECBENT, DS_CUM1, DS_CUM2, DS_DIVFLOW, DS_LOSSCONE,
       DS_ANISO_LISM, DS_TIMEMU = 20 };
typedef struct {
   int kind, width;
   int n_bins[3], log_bins[3], bin_outside[3], dims;
   double limits0[3], bin_size[3];
   int n_actions;
   double val_hot, val_cold;
   int val_time, val_coord, pos_idx, mom_idx;
   double J0, T0, pow_law, T_b, pow_law_comb, bend, A0;
   v3 rot[3], u_lism, grad_perp; /* DistributionAnisotropyLISM */
   int64_t offset_bins;
} dist_t;

typedef struct {
   uint64_t seed;
   uint32_t n_traj, problem;
   int has_bg, has_diff, has_src, src_kind;  /* src_kind 1 SourceConstant, 2 SourceMomentumInjection,
                                                3 SourceSphericalShockInjection */
   bg_t bg;
   df_t df;
   double src_p_inj, src_rate, src_r_sh, src_w_sh;
   v3 src_r0;
   int nbt, nbs, nbm;
   bnd_t bt[MAXB], bs[MAXB], bm[MAXB];
   ini_t it, is, im;
   int has_it, has_is, has_im;
   int nd;
   dist_t d[MAXD];
} prob_t;

static int name_is(const char* name, size_t nl, const char* s) { return strlen(s) == nl && memcmp(name, s, nl) == 0; }

static void setup_bg(bg_t* g, rd_t* r, int kind)
{
   memset(g, 0, sizeof *g);
   g->kind = kind;
   /* BackgroundBase::SetupBackground, src/background_base.cc:342-346 */
   g->t0 = rd_d(r);
   g->r0 = rd_v(r);
   g->u0 = rd_v(r);
   g->B0 = rd_v(r);
   g->dmax0 = rd_d(r);
   if (kind == BG_SHOCK || kind == BG_SMOOTHSHOCK) {
      /* src/background_shock.cc:56-80 */
      v3 u0n, u0t, B0n, B0t;
      g->n_shock = rd_v(r);
      g->v_shock = rd_d(r);
      g->compression = rd_d(r);
      g->n_shock = vunit(g->n_shock);
      u0n = vscale(vdot(g->u0, g->n_shock) - g->v_shock, g->n_shock);
      u0t = vsub(g->u0, vscale(vdot(g->u0, g->n_shock), g->n_shock));
      B0n = vscale(vdot(g->B0, g->n_shock), g->n_shock);
      B0t = vsub(g->B0, B0n);
      g->u1 = vadd(vadd(vdiv(u0n, g->compression), vscale(g->v_shock, g->n_shock)), u0t);
      g->B1 = vadd(B0n, vscale(g->compression, B0t));
      g->E0 = vscale(-1.0, vdiv(vcross(g->u0, g->B0), c_code()));
      g->E1 = vscale(-1.0, vdiv(vcross(g->u1, g->B1), c_code()));
      if (kind == BG_SMOOTHSHOCK) {
         g->width = rd_d(r);
         g->dmax_fraction = rd_d(r);
      }
      g->tanh_k = 8.0;  /* src/background_smooth_shock.hh:23 */
   }
   else if (kind == BG_DISCONT || kind == BG_SMOOTHDISCONT) {
      /* BackgroundDiscontinuity::SetupBackground, src/background_discontinuity.cc:51-63, and the smooth
       * one's width and dmax fraction (src/background_smooth_discontinuity.cc:109-116), steepness 4 (its
       * .hh:49). EvaluateBackground, the derivatives and EvaluateDmax have the shock's forms
       * (src/background_discontinuity.cc:75-104, src/background_smooth_discontinuity.cc:121-178), so the
       * two run as a shock and a smooth shock with this downstream state. */
      g->n_shock = rd_v(r);
      g->v_shock = rd_d(r);
      g->u1 = rd_v(r);
      g->B1 = rd_v(r);
      g->n_shock = vunit(g->n_shock);
      g->E0 = vscale(-1.0, vdiv(vcross(g->u0, g->B0), c_code()));
      g->E1 = vscale(-1.0, vdiv(vcross(g->u1, g->B1), c_code()));
      g->tanh_k = 4.0;
      if (kind == BG_SMOOTHDISCONT) {
         g->width = rd_d(r);
         g->dmax_fraction = rd_d(r);
      }
      g->kind = (kind == BG_DISCONT) ? BG_SHOCK : BG_SMOOTHSHOCK;
   }
   else if (kind == BG_UNIFORM) {
      g->E0 = vscale(-1.0, vdiv(vcross(g->u0, g->B0), c_code()));
   }
   else if (kind == BG_DIPOLE) {
      /* src/background_dipole.cc:48-58 */
      g->r_ref = rd_d(r);
      g->dmax_fraction = rd_d(r);
      g->M = vscale(g->r_ref * g->r_ref * g->r_ref, g->B0);
   }
   else if (kind == BG_SOLARWIND) {
      /* src/background_solarwind.cc:58-84 */
      g->Omega = rd_v(r);
      g->r_ref = rd_d(r);
      g->dmax_fraction = rd_d(r);
      g->w0 = vnorm(g->Omega);
      g->eprime[2] = (g->w0 < SP_TINY) ? cart_unit[2] : vunit(g->Omega);
      g->eprime[0] = second_unit(g->eprime[2]);
      g->eprime[1] = vcross(g->eprime[2], g->eprime[0]);
      g->ur0 = fabs(g->u0.x[0]);
   }
}

static void setup_df(df_t* d, rd_t* r, int kind)
{
   int k;
   memset(d, 0, sizeof *d);
   d->kind = kind;
   switch (kind) {
   case DF_ISO: case DF_PARA: case DF_PERP: d->a[0] = rd_d(r); break;
   case DF_QLT: for (k = 0; k < 3; k++) d->a[k] = rd_d(r); d->a[3] = M_2PI_ / d->a[1]; d->a[4] = d->a[2] - 1.0; break;
   case DF_WNLT: case DF_WNLT_RAMP:
      /* src/diffusion_other.cc:202-208 (A2A, l_max, ps_index as QLT, then A2T, A2L) and :281-295 (l_max_HP,
       * z_nose, z_sheath) */
      for (k = 0; k < 3; k++) d->a[k] = rd_d(r);
      d->a[3] = M_2PI_ / d->a[1]; d->a[4] = d->a[2] - 1.0;
      d->a[5] = rd_d(r); d->a[6] = rd_d(r);
      if (kind == DF_WNLT_RAMP) { d->a[7] = rd_d(r); d->a[8] = rd_d(r); d->a[9] = rd_d(r); }
      break;
   case DF_FULL: d->a[0] = rd_d(r); d->a[1] = rd_d(r); break;
   case DF_FLOWMOM: for (k = 0; k < 6; k++) d->a[k] = rd_d(r); break;
   case DF_KINRAD:
      for (k = 0; k < 6; k++) d->a[k] = rd_d(r);
      d->i0 = rd_i(r);
      d->a[6] = rd_d(r); d->a[7] = rd_d(r); d->a[8] = rd_d(r);
      d->a[9] = 1.0 / d->a[8] * (1.0 / d->a[8]);
      break;
   case DF_RIGB: for (k = 0; k < 6; k++) d->a[k] = rd_d(r); break;
   case DF_STRAUSS: case DF_POTGIETER: d->i0 = rd_i(r); for (k = 0; k < 6; k++) d->a[k] = rd_d(r); break;
   case DF_EMPIRICAL:
      d->a[0] = rd_d(r); d->a[1] = rd_d(r); d->a[2] = rd_d(r); d->a[3] = rd_d(r);
      d->i0 = rd_i(r); d->a[4] = rd_d(r); d->a[5] = rd_d(r); d->i1 = rd_i(r); d->a[6] = rd_d(r);
      break;
   }
}

static void setup_bnd(bnd_t* b, rd_t* r, int kind)
{
   memset(b, 0, sizeof *b);
   b->kind = kind;
   /* BoundaryBase::SetupBoundary, src/boundary_base.cc:138-141 */
   b->max_crossings = rd_i(r);
   b->n_actions = rd_ints(r, b->actions, MAXD);
   switch (kind) {
   case BT_TIME: case BT_TIME_PASS: case BT_TIME_REC:
      b->cls = 0;
      b->timemark = rd_d(r);
      if (kind == BT_TIME) b->max_crossings = 1;
      if (kind == BT_TIME_PASS) b->max_crossings = -1;
      if (kind == BT_TIME_REC) b->recurrent = 1;
      break;
   case BT_PLANE_ABS: case BT_PLANE_REF: case BT_PLANE_PASS:
      b->cls = 1;
      b->origin = rd_v(r);
      b->norm = vunit(rd_v(r));
      if (kind == BT_PLANE_ABS) b->max_crossings = 1;
      if (kind == BT_PLANE_REF) b->reflect = 1;
      break;
   case BT_BOX_REF:
      b->cls = 1;
      b->reflect = 1;
      b->corner0 = rd_v(r);
      b->normals[0] = rd_v(r);
      b->normals[1] = rd_v(r);
      b->normals[2] = rd_v(r);
      b->corner1 = vadd(vadd(vadd(b->corner0, b->normals[0]), b->normals[1]), b->normals[2]);
      b->normals[0] = vunit(b->normals[0]);
      b->normals[1] = vunit(b->normals[1]);
      b->normals[2] = vunit(b->normals[2]);
      break;
   case BT_SPH_ABS: case BT_SPH_REF: case BT_SPH_PASS:
      b->cls = 1;
      b->origin = rd_v(r);
      b->radius = rd_d(r);
      if (kind == BT_SPH_ABS) b->max_crossings = 1;
      if (kind == BT_SPH_REF) b->reflect = 1;
      break;
   case BT_RANKINE:
      b->cls = 1;
      b->origin = rd_v(r);
      b->axis = rd_v(r);
      b->z_nose = rd_d(r);
      b->max_crossings = 1;
      break;
   case BT_CYL:
      b->cls = 1;
      b->origin = rd_v(r);
      b->fa[2] = vunit(rd_v(r));
      b->radius = rd_d(r);
      b->fa[0] = second_unit(b->fa[2]);
      b->fa[1] = vcross(b->fa[2], b->fa[0]);
      b->max_crossings = 1;
      break;
   case BT_REGION:
      b->cls = 1;
      b->region_ind = rd_i(r);
      b->region_val = rd_d(r);
      b->max_crossings = 1;
      break;
   case BT_MOM_INJ: case BT_MOM_PASS: case BT_MOM_SLAB: case BT_MOM_SHELL:
      b->cls = 2;
      b->momentum = rd_d(r);
      if (kind != BT_MOM_PASS) b->max_crossings = 1;
      if (kind == BT_MOM_SLAB) { b->slab_r0 = rd_v(r); b->slab_r1 = rd_v(r); b->slab_n = rd_v(r); }
      if (kind == BT_MOM_SHELL) { b->slab_r0 = rd_v(r); b->r1 = rd_d(r); b->r2 = rd_d(r); }
      break;
   case BT_MIRROR:
      b->cls = 2;
      b->reflect = 1;
      break;
   }
}

static void setup_ini(ini_t* q, rd_t* r, int kind)
{
   memset(q, 0, sizeof *q);
   q->kind = kind;
   switch (kind) {
   case IT_FIXED: q->a[0] = rd_d(r); break;
   case IT_INTERVAL: q->a[0] = rd_d(r); q->a[1] = rd_d(r); q->n_int = rd_i(r); break;
   case IS_FIXED: q->v0 = rd_v(r); break;
   case IS_LINE: case IS_BOX: q->v0 = rd_v(r); q->v1 = rd_v(r); q->n_int = rd_i(r); break;
   case IS_CIRCLE: {
      /* src/initial_space.cc:190-202 */
      v3 normal;
      double radius;
      q->v0 = rd_v(r);
      normal = vunit(rd_v(r));
      radius = rd_d(r);
      q->v1 = vscale(radius, second_unit(normal));
      q->v2 = vcross(normal, q->v1);
      break;
   }
   case IS_SPHERE: q->v0 = rd_v(r); q->a[0] = rd_d(r); break;
   case IS_SECTOR:
      /* src/initial_space.cc:357-377 */
      q->v0 = rd_v(r);
      q->a[0] = rd_d(r);
      q->a[1] = rd_d(r); if (q->a[1] < 0.0) q->a[1] = 0.0;
      q->a[2] = rd_d(r); if (q->a[2] > M_PI_) q->a[2] = M_PI_; if (q->a[2] < q->a[1]) q->a[2] = q->a[1];
      q->a[3] = rd_d(r);
      q->a[4] = rd_d(r); if (q->a[4] > M_2PI_) q->a[4] = M_2PI_; if (q->a[4] < q->a[3]) q->a[4] = q->a[3];
      q->a[5] = cos(q->a[1]);
      q->a[6] = cos(q->a[2]);
      break;
   case IS_CYLINDER: case IS_CYL_SECTOR:
      /* InitialSpaceCylinder(Sector)::SetupInitial (src/initial_space.cc:561-570, 621-631): origin, height vector,
       * radius vector x; radius vector y = unit(height) x radius x; the sector's azimuths clamped to
       * [phi1, min(phi2, 2 pi)] */
      q->v0 = rd_v(r);
      q->v1 = rd_v(r);
      q->v2 = rd_v(r);
      {
         v3 ry = vcross(vunit(q->v1), q->v2);
         q->a[0] = ry.x[0]; q->a[1] = ry.x[1]; q->a[2] = ry.x[2];
      }
      if (kind == IS_CYL_SECTOR) {
         q->a[3] = rd_d(r);
         q->a[4] = rd_d(r);
         if (q->a[4] > M_2PI_) q->a[4] = M_2PI_;
         if (q->a[4] < q->a[3]) q->a[4] = q->a[3];
      }
      break;
   case IS_RANKINE:
      q->v0 = rd_v(r); q->a[0] = rd_d(r); q->a[1] = rd_d(r);
      q->a[2] = (2.0 * q->a[0] * q->a[0] - q->a[1] * q->a[1]) / (q->a[1] * q->a[1]);
      break;
   case IS_EQ_BAND: q->v0 = rd_v(r); q->a[0] = rd_d(r); q->a[1] = rd_d(r); q->a[2] = rd_d(r); break;
   case IM_FIXED: q->v0 = rd_v(r); break;
   case IM_BEAM: case IM_SHELL: q->a[0] = rd_d(r); break;
   case IM_RING: q->a[0] = rd_d(r); q->a[1] = rd_d(r); q->a[2] = cos(q->a[1]); q->a[3] = sin(q->a[1]); break;
   case IM_THICK:
      q->a[0] = rd_d(r); q->a[1] = rd_d(r); q->flag = rd_b(r);
      if (q->flag) { q->a[0] = log10(q->a[0]); q->a[1] = log10(q->a[1]); }
      break;
   case IM_MAXWELL:
      q->a[0] = rd_d(r); q->a[1] = rd_d(r) / sqrt(2.0); q->a[2] = rd_d(r) / sqrt(2.0);
      break;
   case IM_LOGE_PITCH: q->a[0] = rd_d(r); q->a[1] = rd_d(r); q->a[2] = rd_d(r); q->a[3] = rd_d(r); break;
   }
}

static int setup_dist(dist_t* d, rd_t* r, int kind)
{
   int ijk;
   double minv[3], maxv[3];
   v3 mn, mx;
   memset(d, 0, sizeof *d);
   d->kind = kind;
   d->width = (kind == DS_CUM1 || kind == DS_LOSSCONE) ? 3 : (kind == DS_CUM2 ? 9 : 1);
   /* DistributionTemplated::SetupDistribution, src/distribution_templated.cc:92-137 */
   rd_mi(r, d->n_bins);
   mn = rd_v(r);
   mx = rd_v(r);
   rd_mi(r, d->log_bins);
   rd_mi(r, d->bin_outside);
   rd_rec(r, NULL, 0);  /* unit_distro */
   rd_rec(r, NULL, 0);  /* unit_val */
   rd_b(r);             /* keep_records */
   d->dims = 0;
   for (ijk = 0; ijk < 3; ijk++) {
      if (d->n_bins[ijk] > 0) d->dims |= 1 << ijk;
      if (d->n_bins[ijk] < 1) d->n_bins[ijk] = 1;
      minv[ijk] = d->log_bins[ijk] ? log10(mn.x[ijk]) : mn.x[ijk];
      maxv[ijk] = d->log_bins[ijk] ? log10(mx.x[ijk]) : mx.x[ijk];
      d->limits0[ijk] = minv[ijk];
      d->bin_size[ijk] = (maxv[ijk] - minv[ijk]) / d->n_bins[ijk];
   }
   switch (kind) {
   case DS_TIME: case DS_POS: case DS_MOM: case DS_POSMOM: case DS_TIMEMU:
      /* DistributionUniform::SetupDistribution, src/distribution_other.cc:40-60 */
      d->val_hot = rd_d(r);
      d->val_cold = rd_d(r);
      d->n_actions = 2;
      if (kind == DS_TIME) d->val_time = rd_i(r);
      if (kind == DS_POS || kind == DS_MOM) { d->val_time = rd_i(r); d->val_coord = rd_i(r); }
      if (kind == DS_POSMOM) { d->val_time = rd_i(r); d->pos_idx = rd_i(r); d->mom_idx = rd_i(r); }
      break;
   case DS_SPEC: case DS_SPECBENT:
      d->J0 = rd_d(r); d->T0 = rd_d(r); d->pow_law = rd_d(r); d->val_cold = rd_d(r);
      d->n_actions = 2;
      if (kind == DS_SPECBENT) {
         double plb;
         d->T_b = rd_d(r); plb = rd_d(r); d->bend = rd_d(r);
         d->pow_law_comb = (d->pow_law - plb) / d->bend;
      }
      break;
   case DS_CUM1: case DS_CUM2: d->n_actions = 1; break;
   case DS_DIVFLOW: d->A0 = rd_d(r); d->pow_law = rd_d(r); d->val_cold = rd_d(r); d->n_actions = 2; break;
   case DS_LOSSCONE:
      /* DistributionLossCone::SetupDistribution, src/distribution_other.cc:826-840: one action, all three
       * dimensions active */
      d->val_time = rd_i(r);
      d->val_coord = rd_i(r);
      d->n_actions = 1;
      if (d->dims != 7) return -3;
      break;
   case DS_ANISO_LISM:
      /* DistributionAnisotropyLISM::SetupDistribution, src/distribution_other.cc:388-409: the binning
       * frame, the LISM flow, the momentum slope, the perpendicular density gradient; five actions; its
       * set-up accepts dims 5 only */
      d->rot[0] = rd_v(r);
      d->rot[1] = rd_v(r);
      d->rot[2] = rd_v(r);
      d->u_lism = rd_v(r);
      d->pow_law = rd_d(r);
      d->grad_perp = rd_v(r);
      d->n_actions = 5;
      if (d->dims != 5) return -3;
      break;
   }
   return 0;
}

static int kind_of(uint32_t role, const char* nm, size_t nl)
{
#define K(s, v) if (name_is(nm, nl, s)) return v;
   if (role == 0) {
      K("BackgroundUniform", BG_UNIFORM) K("BackgroundShock", BG_SHOCK) K("BackgroundSmoothShock", BG_SMOOTHSHOCK)
      K("BackgroundDiscontinuity", BG_DISCONT) K("BackgroundSmoothDiscontinuity", BG_SMOOTHDISCONT)
      K("BackgroundDipole", BG_DIPOLE) K("BackgroundSolarWind", BG_SOLARWIND)
      K("BackgroundServerCartesian", BG_GRID)
   }
   else if (role == 1) {
      K("DiffusionIsotropicConstant", DF_ISO) K("DiffusionQLTConstant", DF_QLT) K("DiffusionParaConstant", DF_PARA)
      K("DiffusionPerpConstant", DF_PERP) K("DiffusionFullConstant", DF_FULL)
      K("DiffusionFlowMomentumPowerLaw", DF_FLOWMOM) K("DiffusionKineticEnergyRadialDistancePowerLaw", DF_KINRAD)
      K("DiffusionRigidityMagneticFieldPowerLaw", DF_RIGB) K("DiffusionStraussEtAl2013", DF_STRAUSS)
      K("DiffusionPotgieterEtAl2015", DF_POTGIETER) K("DiffusionEmpiricalSOQLTandUNLT", DF_EMPIRICAL)
      K("DiffusionWNLTConstant", DF_WNLT) K("DiffusionWNLTRampVLISM", DF_WNLT_RAMP)
   }
   else if (role == 2) {
      K("SourceConstant", 1) K("SourceMomentumInjection", 2) K("SourceSphericalShockInjection", 3)
   }
   else if (role == 3) {
      K("BoundaryTimeExpire", BT_TIME) K("BoundaryTimePass", BT_TIME_PASS) K("BoundaryTimeRecurrent", BT_TIME_REC)
      K("BoundaryPlaneAbsorb", BT_PLANE_ABS) K("BoundaryPlaneReflect", BT_PLANE_REF) K("BoundaryPlanePass", BT_PLANE_PASS)
      K("BoundaryBoxReflect", BT_BOX_REF) K("BoundarySphereAbsorb", BT_SPH_ABS) K("BoundarySphereReflect", BT_SPH_REF)
      K("BoundaryRankineAbsorb", BT_RANKINE) K("BoundaryCylinderAbsorb", BT_CYL) K("BoundaryRegionAbsorb", BT_REGION)
      K("BoundarySpherePass", BT_SPH_PASS) K("BoundaryMomentumInject", BT_MOM_INJ) K("BoundaryMomentumPass", BT_MOM_PASS)
      K("BoundaryMomentumInjectRestrictSlab", BT_MOM_SLAB) K("BoundaryMomentumInjectRestrictShell", BT_MOM_SHELL)
      K("BoundaryMirror", BT_MIRROR)
   }
   else if (role == 4) {
      K("InitialTimeFixed", IT_FIXED) K("InitialTimeInterval", IT_INTERVAL) K("InitialSpaceFixed", IS_FIXED)
      K("InitialSpaceLine", IS_LINE) K("InitialSpaceCircle", IS_CIRCLE) K("InitialSpaceBox", IS_BOX)
      K("InitialSpaceSphere", IS_SPHERE) K("InitialSpaceSphereSector", IS_SECTOR)
      K("InitialSpaceRankineHalfBody", IS_RANKINE) K("InitialSpaceEquatorialBand", IS_EQ_BAND)
      K("InitialSpaceCylinder", IS_CYLINDER) K("InitialSpaceCylinderSector", IS_CYL_SECTOR)
      K("InitialMomentumFixed", IM_FIXED) K("InitialMomentumBeam", IM_BEAM) K("InitialMomentumRing", IM_RING)
      K("InitialMomentumShell", IM_SHELL) K("InitialMomentumThickShell", IM_THICK)
      K("InitialMomentumMaxwell", IM_MAXWELL) K("InitialMomentumLogEnergyPitchBand", IM_LOGE_PITCH)
   }
   else if (role == 5) {
      K("DistributionTimeUniform", DS_TIME) K("DistributionPositionUniform", DS_POS)
      K("DistributionMomentumUniform", DS_MOM) K("DistributionPositionMomentumUniform", DS_POSMOM)
      K("DistributionSpectrumKineticEnergyPowerLaw", DS_SPEC)
      K("DistributionSpectrumKineticEnergyBentPowerLaw", DS_SPECBENT)
      K("DistributionPositionCumulativeOrder1", DS_CUM1) K("DistributionPositionCumulativeOrder2", DS_CUM2)
      K("DistributionDivergenceFlowPowerLaw", DS_DIVFLOW) K("DistributionTimeMu", DS_TIMEMU)
      K("DistributionLossCone", DS_LOSSCONE) K("DistributionAnisotropyLISM", DS_ANISO_LISM)
   }
#undef K
   return -1;
}

static int get_u32(const uint8_t* s, size_t n, size_t* pos, uint32_t* v)
{
   if (*pos + 4 > n) return -1;
   memcpy(v, s + *pos, 4);
   *pos += 4;
   return 0;
}

static int parse_spec(const uint8_t* s, size_t n, prob_t* pb, char* err, size_t el)
{
   size_t pos = 0;
   uint32_t ver, nps, maxatt, np, i;
   memset(pb, 0, sizeof *pb);
   if (n < 8 || memcmp(s, "SPXS", 4) != 0) { snprintf(err, el, "bad spec magic"); return -1; }
   pos = 4;
   if (get_u32(s, n, &pos, &ver) || ver != 1) { snprintf(err, el, "bad spec version"); return -1; }
   if (pos + 8 > n) return -1;
   memcpy(&pb->seed, s + pos, 8);
   pos += 8;
   if (get_u32(s, n, &pos, &pb->n_traj) || get_u32(s, n, &pos, &pb->problem) || get_u32(s, n, &pos, &nps) ||
       get_u32(s, n, &pos, &maxatt) || get_u32(s, n, &pos, &np)) { snprintf(err, el, "truncated spec"); return -1; }
   for (i = 0; i < np; i++) {
      uint32_t role, nl, nrec, bl;
      const char* nm;
      int kind;
      rd_t r;
      if (get_u32(s, n, &pos, &role) || get_u32(s, n, &pos, &nl) || pos + nl > n) { snprintf(err, el, "truncated spec"); return -1; }
      nm = (const char*)(s + pos);
      pos += nl;
      if (get_u32(s, n, &pos, &nrec) || get_u32(s, n, &pos, &bl) || pos + bl > n) { snprintf(err, el, "truncated spec"); return -1; }
      r.p = s + pos; r.n = bl; r.pos = 0; r.bad = 0;
      pos += bl;
      kind = kind_of(role, nm, nl);
      if (kind < 0) { snprintf(err, el, "unknown plugin %.*s", (int)nl, nm); return -2; }
      if (role == 0) { setup_bg(&pb->bg, &r, kind); pb->has_bg = 1; }
      else if (role == 1) { setup_df(&pb->df, &r, kind); pb->has_diff = 1; }
      else if (role == 2) {
         /* SourceConstant::SetupSource reads S0 (src/source_other.cc:41-50); SourceMomentumInjection p_inj
          * and the rate (:98-107) */
         pb->src_kind = kind;
         if (kind == 1) pb->src_rate = rd_d(&r);
         else if (kind == 2) { pb->src_p_inj = rd_d(&r); pb->src_rate = rd_d(&r); }
         else {  /* SourceSphericalShockInjection::SetupSource, src/source_other.cc:150-160 */
            pb->src_p_inj = rd_d(&r); pb->src_r0 = rd_v(&r); pb->src_r_sh = rd_d(&r); pb->src_w_sh = rd_d(&r);
            pb->src_rate = rd_d(&r);
         }
         pb->has_src = 1;
      }
      else if (role == 3) {
         bnd_t b;
         setup_bnd(&b, &r, kind);
         if (b.cls == 0 && pb->nbt < MAXB) pb->bt[pb->nbt++] = b;
         else if (b.cls == 1 && pb->nbs < MAXB) pb->bs[pb->nbs++] = b;
         else if (b.cls == 2 && pb->nbm < MAXB) pb->bm[pb->nbm++] = b;
         else { snprintf(err, el, "too many boundaries"); return -2; }
      }
      else if (role == 4) {
         ini_t q;
         setup_ini(&q, &r, kind);
         if (kind < 10) { pb->it = q; pb->has_it = 1; }
         else if (kind < 30 || kind == IS_EQ_BAND) { pb->is = q; pb->has_is = 1; }
         else { pb->im = q; pb->has_im = 1; }
      }
      else if (role == 5) {
         if (pb->nd >= MAXD) { snprintf(err, el, "too many distributions"); return -2; }
         if (setup_dist(&pb->d[pb->nd++], &r, kind)) {
            snprintf(err, el, "set-up of %.*s incomplete (active dimensions)", (int)nl, nm);
            return -3;
         }
      }
      if (r.bad) { snprintf(err, el, "malformed blob for %.*s", (int)nl, nm); return -3; }
   }
   (void)nps;
   (void)maxatt;
   return 0;
}

/* ------------------------------------------------------------------------------------------ */
/* trajectory object                                                                          */
/* ------------------------------------------------------------------------------------------ */
/* A Butcher table (common/rk_config.hh:36-65) */
typedef struct {
   int number, stages, order, adaptive;
   double a[SPX_RK_MAX_STAGES], b[SPX_RK_MAX_STAGES][SPX_RK_MAX_STAGES], v[SPX_RK_MAX_STAGES], w[SPX_RK_MAX_STAGES];
} rk_t;

/* adaptive step control of RKStep (common/rk_config.hh:25-34) and Integrate's limit on consecutive
 * rejected steps (src/trajectory_base.hh:41) */
#define RK_TOL_ABS 1.0e-9
#define RK_TOL_REL 1.0e-9
#define RK_SAFETY 2.0
#define RK_ADJUST 0.995
#define MAX_TIME_ADAPTATIONS 100

typedef struct {
   const prob_t* pb;
   const spx_oracle_opts* o;
   const rk_t* rk;
   int time_adaptations;
   /* RNG */
   uint32_t traj_id, attempt;
   uint64_t n_normal, n_uniform, n_init_normal;
   /* state (Params, TrajectoryBase) */
   double t, dt, dt_physical, dt_adaptive, amp, wgt;
   v3 pos, mom, vel;
   double t0;
   v3 pos0, mom0;
   spdata sp, sp0;
   unsigned status;
   uint64_t segments;
   double local_t, local_amp, local_wgt;
   v3 local_pos, local_mom;
   /* |B| extrema along the trajectory (TrajectoryBase with RECORD_BMAG_EXTREMA, src/trajectory_base.cc:
      581-592, 884-888, 959-962), read by DistributionLossCone */
   double bmag_min, bmag_max;
   /* the last stored point of the trajectory (Store(), read back by Load()) */
   double stored_t;
   v3 stored_pos, stored_mom;
   bnd_t bt[MAXB], bs[MAXB], bm[MAXB];
   int bactive_t, bactive_s, bactive_m;
   /* Parker */
   v3 drift_vel, divK, dr_perp;
   double Kperp, Kpara;
   /* Focused, GuidingScatt */
   double Dmumu, Vmu;
   /* Guiding: the modified fields E*, B* of the last drift evaluation */
   v3 e_star, b_star;
   /* GuidingDiff: field-aligned frame, perpendicular drift and displacement of the step */
   v3 fa[3], v_perp;
   /* SourceMomentumInjection state (del_mom_old, src/source_other.cc:113-119) */
   double src_del_old;
   /* BackgroundSmoothShock::ds_shock of the last field evaluation; like the reference's background
      object it lives on across the trajectories of a run (used with reference_quirks, D1) */
   double bg_ds_prev;
   /* distributions */
   int32_t* counts;
   double* sums;
   int64_t* n_events;
   int error;
} trj_t;

/* The normal deviates of one random block; with nudge_libm each is moved one ulp away from zero. */
static void normals4(const uint32_t b[4], double n[4])
{
   int i;
   spx_normals4(b, n);
   if (g_nudge_libm)
      for (i = 0; i < 4; i++) n[i] = nextafter(n[i], n[i] >= 0.0 ? INFINITY : -INFINITY);
}

static double next_uniform(trj_t* T)
{
   uint64_t k = T->n_uniform++;
   uint32_t b[4];
   spx_rng_block(T->pb->seed, (uint32_t)(k / 4), T->traj_id, T->pb->problem, SPX_RNG_INIT, T->attempt, b);
   return spx_u01(b[k % 4]);
}

static double next_init_normal(trj_t* T)
{
   uint64_t k = T->n_init_normal++;
   uint32_t b[4];
   double n[4];
   spx_rng_block(T->pb->seed, (uint32_t)(k / 4), T->traj_id, T->pb->problem, SPX_RNG_INIT_NORMAL, T->attempt, b);
   normals4(b, n);
   return n[k % 4];
}

/* ------------------------------------------------------------------------------------------ */
/* backgrounds                                                                                */
/* ------------------------------------------------------------------------------------------ */

/* Smooth shock transition (SMOOTH_SHOCK_ORDER 4, src/background_smooth_shock.cc:46-105) */
static double shock_tr(double k, double x) { return 0.5 * (1.0 + tanh(k * x)); }
static double shock_trd(double k, double x) { double th = tanh(k * x); return 0.5 * k * (1.0 - th * th); }

/* EvaluateBackground of each analytic background; fills U, B, E (by mask) and region. Returns
 * the smooth-shock coordinate through *ds (used by EvaluateDmax and the derivatives). */
static void grid_reader_values(v3 pos, spdata* s);

static void eval_bg(const bg_t* g, double t, v3 pos, unsigned mask, spdata* s, double* ds)
{
   switch (g->kind) {
   case BG_GRID: /* the points of numerical derivatives under SERVER_INTERP_ORDER -1 */
      grid_reader_values(pos, s);
      break;
   case BG_UNIFORM: /* src/background_uniform.cc:63-72 */
      if (mask & BG_U) s->U = g->u0;
      if (mask & BG_B) s->B = g->B0;
      if (mask & BG_E) s->E = g->E0;
      s->region = V(1.0, 1.0, 1.0);
      break;
   case BG_SHOCK: /* src/background_shock.cc:86-104 */
      if (vdot(vsub(pos, g->r0), g->n_shock) - g->v_shock * t > 0) {
         if (mask & BG_U) s->U = g->u0;
         if (mask & BG_B) s->B = g->B0;
         if (mask & BG_E) s->E = g->E0;
         s->region = V(1.0, 1.0, 1.0);
      }
      else {
         if (mask & BG_U) s->U = g->u1;
         if (mask & BG_B) s->B = g->B1;
         if (mask & BG_E) s->E = g->E1;
         s->region = V(2.0, 2.0, 2.0);
      }
      break;
   case BG_SMOOTHSHOCK: { /* src/background_smooth_shock.cc:124-140 */
      double a1, a2;
      *ds = (vdot(vsub(pos, g->r0), g->n_shock) - g->v_shock * t) / g->width;
      a1 = shock_tr(g->tanh_k, *ds);
      a2 = 1.0 - a1;
      if ((mask & BG_U) || (mask & BG_E)) s->U = vadd(vscale(a1, g->u0), vscale(a2, g->u1));
      if (mask & BG_B) s->B = vadd(vscale(a1, g->B0), vscale(a2, g->B1));
      if (mask & BG_E) s->E = vscale(-1.0, vdiv(vcross(s->U, s->B), c_code()));
      {
         double rg = 1.0 * a1 + 2.0 * a2;
         s->region = V(rg, rg, rg);
      }
      break;
   }
   case BG_DIPOLE: /* src/background_dipole.cc:64-80 */
      if (mask & BG_U) s->U = V(0, 0, 0);
      if (mask & BG_B) {
         v3 pp = vsub(pos, g->r0);
         double r2 = vnorm(pp);
         double r5 = r2 * r2 * r2;
         r2 *= r2;
         r5 *= r2;
         s->B = vdiv(vsub(vscale(3.0 * vdot(pp, g->M), pp), vscale(r2, g->M)), r5);
      }
      if (mask & BG_E) s->E = V(0, 0, 0);
      s->region = V(1.0, 1.0, 1.0);
      break;
   case BG_SOLARWIND: { /* src/background_solarwind.cc:111-255, all switches at their defaults */
      v3 pp = to_basis(vsub(pos, g->r0), g->eprime);
      double r = vnorm(pp), r_mns = r - g->r_ref, costheta, ur, Br0 = g->B0.x[0];
      costheta = pp.x[2] / r;
      s->region = V(r < (117.0 * 1.495978707E+13 / 1.0e10) ? 1.0 : -1.0, -1.0, s->region.x[2]);
      ur = g->ur0;
      /* D4: U also when only E is asked for (the Lorentz mask), as BackgroundSmoothShock does
       * (src/background_smooth_shock.cc:148); the reference's solar wind leaves U unset then and forms
       * E from an uninitialised velocity */
      if (mask & (BG_U | BG_E)) s->U = from_basis(vscale(ur, vunit(pp)), g->eprime);
      if (mask & BG_B) {
         double sintheta = sqrt(fmax(1.0 - costheta * costheta, 0.0));
         double sr = sqrt(pp.x[0] * pp.x[0] + pp.x[1] * pp.x[1]);
         double cosphi, sinphi, Br, Bp;
         v3 Bl;
         if (sr < r * SP_TINY) { cosphi = 0.0; sinphi = 0.0; }
         else { cosphi = pp.x[0] / sr; sinphi = pp.x[1] / sr; }
         Br = Br0 * ((g->r_ref / r) * (g->r_ref / r));
         Bp = -Br * sintheta * r_mns * g->w0 / ur;
         Bl = V(Br * sintheta * cosphi - Bp * sinphi, Br * sintheta * sinphi + Bp * cosphi, Br * costheta);
         s->B = from_basis(Bl, g->eprime);
      }
      if (mask & BG_E) s->E = vscale(-1.0, vdiv(vcross(s->U, s->B), c_code()));
      break;
   }
   }
}

/* EvaluateDmax (src/background_base.cc:378-382 and the overrides); see D1 for the smooth shock */
static double eval_dmax(const bg_t* g, double t, v3 pos)
{
   switch (g->kind) {
   case BG_SMOOTHSHOCK: {
      double ds = (vdot(vsub(pos, g->r0), g->n_shock) - g->v_shock * t) / g->width;
      return fmin(g->dmax_fraction * g->width * fmax(1.0, fabs(ds)), g->dmax0);
   }
   case BG_DIPOLE: case BG_SOLARWIND: return fmin(g->dmax_fraction * vnorm(vsub(pos, g->r0)), g->dmax0);
   default: return g->dmax0;
   }
}

/* Analytic gradients of the Parker spiral (deriv_mode 1). With x the position in the rotation
 * frame, r = |x|, A = Br0 r_ref^2, k = A w0 / ur and w = (x2, -x1, 0):
 *   B = A x / r^3 + k (r - r_ref) / r^3 w,   U = ur x / r,
 *   d_i B_j = A (delta_ij / r^3 - 3 x_i x_j / r^5) + k (f'(r) x_i w_j / r + f(r) dw_j/dx_i),
 *   f = (r - r_ref) / r^3, f' = (3 r_ref - 2 r) / r^4,
 *   d_i U_j = ur (delta_ij / r - x_i x_j / r^3).
 * The reference's own analytic branch (SOLARWIND_DERIVATIVE_METHOD 0) is not buildable. */
static void solarwind_grad(const bg_t* g, v3 pos, spdata* s)
{
   v3 x = to_basis(vsub(pos, g->r0), g->eprime);
   double r = vnorm(x), r2 = r * r, r3 = r2 * r, r5 = r3 * r2;
   double A = g->B0.x[0] * g->r_ref * g->r_ref, k = A * g->w0 / g->ur0;
   double f = (r - g->r_ref) / r3, fp = (3.0 * g->r_ref - 2.0 * r) / (r2 * r2);
   double w[3] = {x.x[1], -x.x[0], 0.0};
   double gb[3][3], gu[3][3], R[3][3];
   int i, j, a, b;
   for (i = 0; i < 3; i++)
      for (j = 0; j < 3; j++) {
         double dij = (i == j) ? 1.0 : 0.0;
         gb[i][j] = A * (dij / r3 - 3.0 * x.x[i] * x.x[j] / r5) + k * (fp * x.x[i] * w[j] / r);
         gu[i][j] = g->ur0 * (dij / r - x.x[i] * x.x[j] / r3);
      }
   gb[0][1] += k * f * (-1.0);
   gb[1][0] += k * f * (1.0);
   /* rotate: grad_global = E^T grad' E with E rows = eprime */
   for (i = 0; i < 3; i++)
      for (j = 0; j < 3; j++) R[i][j] = g->eprime[i].x[j];
   for (i = 0; i < 3; i++)
      for (j = 0; j < 3; j++) {
         double sb = 0.0, su = 0.0;
         for (a = 0; a < 3; a++)
            for (b = 0; b < 3; b++) {
               sb += R[a][i] * gb[a][b] * R[b][j];
               su += R[a][i] * gu[a][b] * R[b][j];
            }
         s->gradB.m[i][j] = sb;
         s->gradU.m[i][j] = su;
      }
   s->gradBmag = mvmul(&s->gradB, s->bhat);
   s->dUdt = V(0, 0, 0);
   s->dBdt = V(0, 0, 0);
   s->dBmagdt = 0.0;
}

/* BackgroundBase::NumericalDerivatives (src/background_base.cc:228-312), restricted to U and B
 * (E gradients are not used on the path). Spatial derivatives along the field-aligned basis with
 * step r_g = min(r_L, dmax), then a time derivative of U with step 1/w_g. */
static void numerical_derivs(const bg_t* g, double t, v3 pos, v3 mom_pmu, spdata* s)
{
   unsigned m1 = s->mask >> 4, m2 = m1 >> 4;
   v3 fa[3];
   int xyz, i, j;
   if (m1 & BG_ALL) {
      double r_g = fmin(larmor(mom_pmu.x[0], s->Bmag), s->dmax);
      m3 gu = mzero(), gbv = mzero();
      v3 gbm = V(0, 0, 0);
      fa[2] = s->bhat;
      fa[0] = second_unit(s->bhat);
      fa[1] = vcross(fa[2], fa[0]);
      for (xyz = 0; xyz < 3; xyz++) {
         spdata f, b;
         double dr = r_g, ds = 0.0;
         v3 p = vadd(pos, vscale(dr, fa[xyz]));
         memset(&f, 0, sizeof f);
         memset(&b, 0, sizeof b);
         eval_bg(g, t, p, m1, &f, &ds);
         dr *= 2.0;
         p = vsub(p, vscale(dr, fa[xyz]));
         eval_bg(g, t, p, m1, &b, &ds);
         for (j = 0; j < 3; j++) {
            if (m1 & BG_U) gu.m[xyz][j] = (f.U.x[j] - b.U.x[j]) / dr;
            if (m1 & BG_B) gbv.m[xyz][j] = (f.B.x[j] - b.B.x[j]) / dr;
         }
         if (m1 & BG_B) gbm.x[xyz] = (vnorm(f.B) - vnorm(b.B)) / dr;
         s->dr[xyz] = dr;
      }
      /* rot_mat = transpose(fa_basis); grad = rot_mat * grad_fa */
      for (i = 0; i < 3; i++)
         for (j = 0; j < 3; j++) {
            if (m1 & BG_U) s->gradU.m[i][j] = fa[0].x[i] * gu.m[0][j] + fa[1].x[i] * gu.m[1][j] + fa[2].x[i] * gu.m[2][j];
            if (m1 & BG_B) s->gradB.m[i][j] = fa[0].x[i] * gbv.m[0][j] + fa[1].x[i] * gbv.m[1][j] + fa[2].x[i] * gbv.m[2][j];
         }
      if (m1 & BG_B)
         for (i = 0; i < 3; i++) s->gradBmag.x[i] = fa[0].x[i] * gbm.x[0] + fa[1].x[i] * gbm.x[1] + fa[2].x[i] * gbm.x[2];
   }
   if (m2 & BG_ALL) {
      double v = vel_of(mom_pmu.x[0]);
      double w_g = fmin(cyclotron(v, s->Bmag), v / s->dmax);
      double dt = 1.0 / w_g, ds = 0.0;
      spdata f, b;
      memset(&f, 0, sizeof f);
      memset(&b, 0, sizeof b);
      eval_bg(g, t + dt, pos, m2, &f, &ds);
      dt *= 2.0;
      eval_bg(g, t + dt * 0.5 - dt, pos, m2, &b, &ds);
      if (m2 & BG_U) s->dUdt = vdiv(vsub(f.U, b.U), dt);
      if (m2 & BG_B) { s->dBdt = vdiv(vsub(f.B, b.B), dt); s->dBmagdt = (vnorm(f.B) - vnorm(b.B)) / dt; }
   }
}

/* ------------------------------------------------------------------------------------------ */
/* gridded background: BackgroundServerCartesian, first-order interpolation, one uniform block  */
/* ------------------------------------------------------------------------------------------ */
static struct {
   int n[3];
   v3 cent, zone;
   double zone_min;
   double* v; /* 8 per node: U, B, |B|, unused */
   /* block mode (the reference's Cartesian server over its reader's data): nb[0] nb[1] nb[2] blocks
    * of 4^3 zones over [dmin, dmax] (file units), values in fluid units, ghost cells per block side */
   int nb[3], ghost;
   int order;       /* SERVER_INTERP_ORDER: 1 the stencil, 0 the zone's values, -1 the reader's interpolation */
   v3 dmin, dmax, blen;
   double units[4]; /* Fluid/Particle length, velocity and magnetic ratios; Fluid::c_code */
} g_grid;

void spx_oracle_set_grid(const int64_t n[3], const double cent_min[3], const double zone_length[3],
                         const double* values)
{
   int64_t i, nodes = n[0] * n[1] * n[2];
   int k, q;
   g_grid.nb[0] = g_grid.nb[1] = g_grid.nb[2] = 0;
   free(g_grid.v);
   g_grid.v = (double*)calloc((size_t)nodes * 8, sizeof(double));
   for (k = 0; k < 3; k++) {
      g_grid.n[k] = (int)n[k];
      g_grid.cent.x[k] = cent_min[k];
      g_grid.zone.x[k] = zone_length[k];
   }
   g_grid.zone_min = fmin(zone_length[0], fmin(zone_length[1], zone_length[2]));
   for (i = 0; i < nodes; i++) {
      const double* v = values + 6 * i;
      double* o = g_grid.v + 8 * i;
      for (q = 0; q < 6; q++) o[q] = v[q];
      o[6] = sqrt(v[3] * v[3] + v[4] * v[4] + v[5] * v[5]);  /* src/server_cartesian.cc:566-569 */
   }
}

/* Block mode: the reader's layout (src/reader_cartesian.cc:117-166) -- blocks x fastest, in each
 * block 4^3 zones x fastest, six values per zone -- regrouped by dimension (its variables_by_dimen)
 * with |B| per node appended. */
void spx_oracle_set_grid_blocks(const int nb[3], const double dmin[3], const double dmax[3], int ghost,
                                const double* values, const double units[4])
{
   int64_t nodes, b, z;
   int k, q, n[3];
   for (k = 0; k < 3; k++) n[k] = 4 * nb[k];
   nodes = (int64_t)n[0] * n[1] * n[2];
   free(g_grid.v);
   g_grid.v = (double*)calloc((size_t)nodes * 8, sizeof(double));
   for (k = 0; k < 3; k++) {
      g_grid.n[k] = n[k];
      g_grid.nb[k] = nb[k];
      g_grid.dmin.x[k] = dmin[k];
      g_grid.dmax.x[k] = dmax[k];
      g_grid.blen.x[k] = (dmax[k] - dmin[k]) / (double)nb[k];  /* block_length, :97 */
   }
   for (k = 0; k < 4; k++) g_grid.units[k] = units[k];
   g_grid.ghost = ghost;
   g_grid.order = 1;
   for (b = 0; b < (int64_t)nb[0] * nb[1] * nb[2]; b++) {
      int64_t bi = b % nb[0], bj = (b / nb[0]) % nb[1], bk = b / ((int64_t)nb[0] * nb[1]);
      for (z = 0; z < 64; z++) {
         int64_t i = 4 * bi + z % 4, j = 4 * bj + (z / 4) % 4, kk = 4 * bk + z / 16;
         const double* v = values + 6 * (64 * b + z);
         double* o = g_grid.v + 8 * (i + n[0] * (j + (int64_t)n[1] * kk));
         for (q = 0; q < 6; q++) o[q] = v[q];
         o[6] = sqrt(v[3] * v[3] + v[4] * v[4] + v[5] * v[5]);  /* src/server_cartesian.cc:566-569 */
      }
   }
}

/* SERVER_INTERP_ORDER of the block mode (1, 0 or -1) */
void spx_oracle_set_grid_order(int order) { g_grid.order = order; }

/* The reference's unit conversion for server data (common/physics.hh:18-55 Fluid,
 * common/specie.hh:25-64 Particle): Fluid/Particle length, velocity, magnetic ratios, Fluid::c_code. */
void spx_oracle_grid_units(double out[4])
{
   const double m_p = 1.67262192596e-24, e = 4.8032044e-10;
   const double p_vel = 0.1 * c_light, p_len = 1.0e10, p_time = p_len / p_vel;
   const double p_mag = (m_p * p_vel) / (e * p_time), f_vel = 1.0e7, f_mag = f_vel * sqrt(m_p * 1.0);
   out[0] = AU_CM / p_len;
   out[1] = f_vel / p_vel;
   out[2] = f_mag / p_mag;
   out[3] = c_light / f_vel;
}

/* The primary block of "pos" and its stencil geometry, block mode: ReadCartesianGetNode
 * (src/reader_cartesian.cc:264-277) on the position in file units; the block's faces as the reader
 * and BlockBase::LoadDimensions form them (:291-300, src/block_base.cc:133-152, ghost layers
 * included); ConfigureProperties (:158-171); GetZoneOffset (:194-203). Nonzero outside the domain. */
static int grid_block_geometry(v3 pos, int bidx[3], v3* cent, v3* zl, int zone[3], double off[3], v3* face)
{
   int k;
   const double len = g_grid.units[0];
   for (k = 0; k < 3; k++) {
      double pc = pos.x[k] / AU_CM * 1.0e10;  /* pos / Fluid::unit_length * Particle::unit_length */
      if (pc < g_grid.dmin.x[k] || pc > g_grid.dmax.x[k]) return 1;
      bidx[k] = (int)((pc - g_grid.dmin.x[k]) / g_grid.blen.x[k]);
      if (bidx[k] >= g_grid.nb[k]) return 1;
   }
   for (k = 0; k < 3; k++) {
      double fmin_ = g_grid.dmin.x[k] + g_grid.blen.x[k] * bidx[k], fmax_ = fmin_ + g_grid.blen.x[k];
      double o;
      int bs = 4;
      fmin_ *= len;
      fmax_ *= len;
      if (g_grid.ghost > 0) {
         double incr = (fmax_ - fmin_) * ((double)g_grid.ghost / 4.0);
         fmin_ -= incr;
         fmax_ += incr;
         bs += 2 * g_grid.ghost;
      }
      zl->x[k] = (fmax_ - fmin_) / (double)bs;
      cent->x[k] = fmin_ + 0.5 * zl->x[k];
      face->x[k] = fmin_;
      o = (pos.x[k] - cent->x[k]) / zl->x[k];
      zone[k] = (int)o;
      if (o < 0.0) zone[k]--;
      off[k] = o - (double)zone[k];
   }
   return 0;
}

/* InteriorInterpolationStencil (src/server_cartesian.cc:206-268): weights and their derivatives */
static void grid_stencil(const double lo[3], const double hi[3], v3 zl, double w[8], double der[24])
{
   int c;
   for (c = 0; c < 8; c++) {
      int ci = c & 1, cj = (c >> 1) & 1, ck = (c >> 2) & 1;
      double fx = ci ? lo[0] : hi[0], fy = cj ? lo[1] : hi[1], fz = ck ? lo[2] : hi[2];
      w[c] = fx * fy * fz;
      der[3 * c + 0] = (ci ? fy * fz : -fy * fz) / zl.x[0];
      der[3 * c + 1] = (cj ? fx * fz : -fx * fz) / zl.x[1];
      der[3 * c + 2] = (ck ? fx * fy : -fx * fy) / zl.x[2];
   }
}

int spx_oracle_grid_stencil(const double pos[3], int node[3], double cent_min[3], double zone_length[3], int zone[3],
                            double offset[3], double w[8], double der[24])
{
   v3 cent, zl;
   double hi[3];
   int k;
   v3 face;
   if (g_grid.nb[0] == 0 || grid_block_geometry(V(pos[0], pos[1], pos[2]), node, &cent, &zl, zone, offset, &face)) return 1;
   for (k = 0; k < 3; k++) {
      hi[k] = 1.0 - offset[k];
      cent_min[k] = cent.x[k];
      zone_length[k] = zl.x[k];
   }
   grid_stencil(offset, hi, zl, w, der);
   return 0;
}

/* GetZoneOffset (src/block_base.cc:194-203), InteriorInterpolationStencil
 * (src/server_cartesian.cc:206-268), GetVariablesInterp1 (:551-666), GetVariables' dmax cap (:687)
 * and GetGradientsInterp1 (:724-823) for a point inside the block. Nonzero outside. */
static int grid_fields_blocks(double dmax0, v3 pos, spdata* s);

static int grid_fields(double dmax0, v3 pos, unsigned mask, spdata* s)
{
   double lo[3], hi[3], w[8], der[24], var[6] = {0, 0, 0, 0, 0, 0}, grads[6][3], gbm[3] = {0, 0, 0};
   int z[3], k, c, q, u;
   int64_t nx = g_grid.n[0], nxy = nx * g_grid.n[1];
   if (!g_grid.v) return 1;
   (void)mask;
   if (g_grid.nb[0] > 0) return grid_fields_blocks(dmax0, pos, s);
   for (k = 0; k < 3; k++) {
      double o = (pos.x[k] - g_grid.cent.x[k]) / g_grid.zone.x[k];
      if (!(o >= 0.0 && o < (double)(g_grid.n[k] - 1))) return 1;
      z[k] = (int)o;
      lo[k] = o - z[k];
      hi[k] = 1.0 - lo[k];
   }
   for (c = 0; c < 8; c++) {
      int ci = c & 1, cj = (c >> 1) & 1, ck = (c >> 2) & 1;
      double fx = ci ? lo[0] : hi[0], fy = cj ? lo[1] : hi[1], fz = ck ? lo[2] : hi[2];
      w[c] = fx * fy * fz;
      der[3 * c + 0] = (ci ? fy * fz : -fy * fz) / g_grid.zone.x[0];
      der[3 * c + 1] = (cj ? fx * fz : -fx * fz) / g_grid.zone.x[1];
      der[3 * c + 2] = (ck ? fx * fy : -fx * fy) / g_grid.zone.x[2];
   }
   for (q = 0; q < 6; q++) grads[q][0] = grads[q][1] = grads[q][2] = 0.0;
   s->Bmag = 0.0;
   for (c = 0; c < 8; c++) {
      int ci = c & 1, cj = (c >> 1) & 1, ck = (c >> 2) & 1;
      const double* v = g_grid.v + 8 * ((z[2] + ck) * nxy + (int64_t)(z[1] + cj) * nx + (z[0] + ci));
      for (q = 0; q < 6; q++) var[q] += w[c] * v[q];
      s->Bmag += w[c] * v[6];
      for (q = 0; q < 6; q++)
         for (u = 0; u < 3; u++) grads[q][u] += der[3 * c + u] * v[q];
      for (u = 0; u < 3; u++) gbm[u] += der[3 * c + u] * v[6];
   }
   s->dmax = fmin(dmax0, g_grid.zone_min);
   for (k = 0; k < 3; k++) {
      s->U.x[k] = var[k];
      s->B.x[k] = var[3 + k];
   }
   {
      v3 x = vcross(s->U, s->B);
      for (k = 0; k < 3; k++) s->E.x[k] = -(x.x[k] / c_code());
   }
   s->region = V(0.0, 0.0, 0.0);
   if (s->Bmag < SP_TINY) return 1;
   s->bhat = vdiv(s->B, s->Bmag);
   for (u = 0; u < 3; u++)
      for (k = 0; k < 3; k++) {
         s->gradU.m[u][k] = grads[k][u];
         s->gradB.m[u][k] = grads[3 + k][u];
      }
   for (u = 0; u < 3; u++) s->gradBmag.x[u] = gbm[u];
   s->dUdt = V(0, 0, 0);
   s->dBdt = V(0, 0, 0);
   s->dBmagdt = 0.0;
   return 0;
}

/* Block mode: GetVariables / GetGradients of the Cartesian front end at first order
 * (src/server_cartesian.cc:549-716, 724-865). The weights come from the primary block's stencil; the
 * values of zones past its faces are its neighbours' (the same global zones). Sums in fluid units,
 * then the unit ratios; E = -(U x B) / Fluid::c_code before its ratio; dmax capped by the block's
 * smallest zone length. A stencil that leaves the domain is a field error. */
/* U, B and E from fluid-unit values, converted after the interpolation (src/server_cartesian.cc:610-628, 710-716) */
static void grid_convert(const double var[6], spdata* s)
{
   const double vel = g_grid.units[1], mag = g_grid.units[2], cf = g_grid.units[3];
   v3 U = V(var[0], var[1], var[2]), B = V(var[3], var[4], var[5]), x = vcross(U, B);
   int k;
   for (k = 0; k < 3; k++) {
      s->E.x[k] = (-x.x[k] / cf) * mag;
      s->U.x[k] = U.x[k] * vel;
      s->B.x[k] = B.x[k] * mag;
   }
}

/* SERVER_INTERP_ORDER -1: the boss's interpolation, ReadCartesianGetBlockData (src/reader_cartesian.cc:193-254),
 * over the whole domain in file units, for the position scaled as the back end scales it (:1016); the zone
 * index is truncated, as there. Zero fields outside the domain (the front end's zero-initialised buffer). */
static void grid_reader_values(v3 pos, spdata* s)
{
   double pc[3], lo[3], hi[3], var[6] = {0, 0, 0, 0, 0, 0};
   int z[3], k, c, q;
   int64_t nx = g_grid.n[0], nxy = nx * g_grid.n[1];
   for (k = 0; k < 3; k++) {
      pc[k] = pos.x[k] / AU_CM * 1.0e10;
      if (pc[k] < g_grid.dmin.x[k] || pc[k] > g_grid.dmax.x[k]) { grid_convert(var, s); return; }
   }
   for (k = 0; k < 3; k++) {
      double o = (pc[k] - g_grid.dmin.x[k]) / (g_grid.blen.x[k] / 4.0) - 0.5;
      z[k] = (int)o;
      lo[k] = o - (double)z[k];
      hi[k] = 1.0 - lo[k];
      if (z[k] < 0 || z[k] + 1 >= g_grid.n[k]) { grid_convert(var, s); return; }
   }
   for (c = 0; c < 8; c++) {
      int ci = c & 1, cj = (c >> 1) & 1, ck = (c >> 2) & 1;
      double fx = ci ? lo[0] : hi[0], fy = cj ? lo[1] : hi[1], fz = ck ? lo[2] : hi[2], w = fx * fy * fz;
      const double* v = g_grid.v + 8 * ((z[2] + ck) * nxy + (int64_t)(z[1] + cj) * nx + (z[0] + ci));
      for (q = 0; q < 6; q++) var[q] += w * v[q];
   }
   grid_convert(var, s);
}

static int grid_fields_blocks(double dmax0, v3 pos, spdata* s)
{
   int bidx[3], zone[3], k, c, q, u, g[3];
   v3 cent, zl;
   double lo[3], hi[3], w[8], der[24], var[6] = {0, 0, 0, 0, 0, 0}, grads[6][3], gbm[3] = {0, 0, 0}, bm = 0.0;
   const double vel = g_grid.units[1], mag = g_grid.units[2], cf = g_grid.units[3];
   int64_t nx = g_grid.n[0], nxy = nx * g_grid.n[1];
   v3 face;
   if (grid_block_geometry(pos, bidx, &cent, &zl, zone, lo, &face)) return 1;
   if (g_grid.order <= 0) {
      /* GetVariablesInterp0 (src/server_cartesian.cc:479-540): the values of the zone holding the point,
       * BlockBase::GetZone (src/block_base.cc:180-185); or the reader's interpolation (order -1). |B| is
       * the norm of the converted B (BackgroundBase::EvaluateBmag); order 0 has zero gradients (:848-852),
       * order -1 numerical ones (the caller). */
      s->dmax = fmin(dmax0, fmin(zl.x[0], fmin(zl.x[1], zl.x[2])));
      if (g_grid.order == 0) {
         for (k = 0; k < 3; k++) {
            g[k] = 4 * bidx[k] + (int)((pos.x[k] - face.x[k]) / zl.x[k]) - g_grid.ghost;
            if (g[k] < 0 || g[k] >= g_grid.n[k]) return 1;
         }
         {
            const double* v = g_grid.v + 8 * (g[2] * nxy + (int64_t)g[1] * nx + g[0]);
            for (q = 0; q < 6; q++) var[q] = v[q];
         }
         grid_convert(var, s);
      }
      else grid_reader_values(pos, s);
      s->region = V(0.0, 0.0, 0.0);
      s->Bmag = vnorm(s->B);
      if (s->Bmag < SP_TINY) return 1;
      s->bhat = vdiv(s->B, s->Bmag);
      s->gradU = mzero();
      s->gradB = mzero();
      s->gradBmag = V(0, 0, 0);
      s->dUdt = V(0, 0, 0);
      s->dBdt = V(0, 0, 0);
      s->dBmagdt = 0.0;
      return 0;
   }
   for (k = 0; k < 3; k++) {
      hi[k] = 1.0 - lo[k];
      g[k] = 4 * bidx[k] + zone[k] - g_grid.ghost;  /* global zone of the stencil's corner 0 */
      if (g[k] < 0 || g[k] + 1 >= g_grid.n[k]) return 1;
   }
   grid_stencil(lo, hi, zl, w, der);
   for (q = 0; q < 6; q++) grads[q][0] = grads[q][1] = grads[q][2] = 0.0;
   for (c = 0; c < 8; c++) {
      int ci = c & 1, cj = (c >> 1) & 1, ck = (c >> 2) & 1;
      const double* v = g_grid.v + 8 * ((g[2] + ck) * nxy + (int64_t)(g[1] + cj) * nx + (g[0] + ci));
      for (q = 0; q < 6; q++) var[q] += w[c] * v[q];
      bm += w[c] * v[6];
      for (q = 0; q < 6; q++)
         for (u = 0; u < 3; u++) grads[q][u] += der[3 * c + u] * v[q];
      for (u = 0; u < 3; u++) gbm[u] += der[3 * c + u] * v[6];
   }
   s->dmax = fmin(dmax0, fmin(zl.x[0], fmin(zl.x[1], zl.x[2])));
   {
      v3 U = V(var[0], var[1], var[2]), B = V(var[3], var[4], var[5]), x = vcross(U, B);
      for (k = 0; k < 3; k++) {
         s->E.x[k] = (-x.x[k] / cf) * mag;
         s->U.x[k] = U.x[k] * vel;
         s->B.x[k] = B.x[k] * mag;
      }
   }
   s->Bmag = bm * mag;
   s->region = V(0.0, 0.0, 0.0);
   if (s->Bmag < SP_TINY) return 1;
   s->bhat = vdiv(s->B, s->Bmag);
   for (u = 0; u < 3; u++) {
      for (k = 0; k < 3; k++) {
         s->gradU.m[u][k] = grads[k][u] * vel;
         s->gradB.m[u][k] = grads[3 + k][u] * mag;
      }
      s->gradBmag.x[u] = gbm[u] * mag;
   }
   s->dUdt = V(0, 0, 0);
   s->dBdt = V(0, 0, 0);
   s->dBmagdt = 0.0;
   return 0;
}

/* The gridded background's fields at one point, in the grid harness's order: U[3] B[3] Bmag E[3] dmax
 * gradU[9] gradB[9] gradBmag[3]. Nonzero on a field error. */
int spx_oracle_grid_fields(const double pos[3], double dmax0, double out[32])
{
   spdata s;
   int k, a, b;
   memset(&s, 0, sizeof s);
   if (grid_fields(dmax0, V(pos[0], pos[1], pos[2]), 0xffffu, &s)) return 1;
   for (k = 0; k < 3; k++) {
      out[k] = s.U.x[k];
      out[3 + k] = s.B.x[k];
      out[7 + k] = s.E.x[k];
      out[29 + k] = s.gradBmag.x[k];
   }
   out[6] = s.Bmag;
   out[10] = s.dmax;
   for (a = 0; a < 3; a++)
      for (b = 0; b < 3; b++) {
         out[11 + 3 * a + b] = s.gradU.m[a][b];
         out[20 + 3 * a + b] = s.gradB.m[a][b];
      }
   return 0;
}

/* BackgroundBase::GetFields (src/background_base.cc:425-456). Returns nonzero on a field error. */
static int get_fields(trj_t* T, double t, v3 pos, v3 mom_pmu, unsigned mask, spdata* s)
{
   const bg_t* g = &T->pb->bg;
   double ds = 0.0;
   int i;
   s->mask = mask;
   if (g->kind == BG_GRID) {
      for (i = 0; i < 3; i++) s->dr[i] = 0.0001 * g->dmax0;
      if (grid_fields(g->dmax0, pos, mask, s)) return 1;
      /* SERVER_INTERP_ORDER -1 raises BACKGROUND_grad_FAIL (src/server_cartesian.cc:843-846), and the
       * background then takes numerical derivatives (src/background_server.cc, EvaluateBackgroundDerivatives) */
      if (g_grid.nb[0] > 0 && g_grid.order == -1) numerical_derivs(g, t, pos, mom_pmu, s);
      return 0;
   }
   if (g->kind == BG_SMOOTHSHOCK && T->o->reference_quirks)  /* D1 as the reference has it */
      s->dmax = fmin(g->dmax_fraction * g->width * fmax(1.0, fabs(T->bg_ds_prev)), g->dmax0);
   else
      s->dmax = eval_dmax(g, t, pos);
   eval_bg(g, t, pos, mask, s, &ds);
   if (g->kind == BG_SMOOTHSHOCK) T->bg_ds_prev = ds;
   if (mask & BG_B) {
      s->Bmag = vnorm(s->B);
      if (s->Bmag < SP_TINY) return 1;
      s->bhat = vdiv(s->B, s->Bmag);
   }
   for (i = 0; i < 3; i++) s->dr[i] = 0.0001 * g->dmax0;  /* incr_dmax_ratio * dmax0 */
   /* EvaluateBackgroundDerivatives */
   switch (g->kind) {
   case BG_UNIFORM: case BG_SHOCK:
      s->gradU = mzero(); s->gradB = mzero();
      s->gradBmag = V(0, 0, 0); s->dUdt = V(0, 0, 0); s->dBdt = V(0, 0, 0); s->dBmagdt = 0.0;
      break;
   case BG_SMOOTHSHOCK: { /* src/background_smooth_shock.cc:149-183 */
      double fac = shock_trd(g->tanh_k, ds) / g->width;
      v3 du = vsub(g->u0, g->u1), db = vsub(g->B0, g->B1);
      int a, b;
      for (a = 0; a < 3; a++)
         for (b = 0; b < 3; b++) {
            s->gradU.m[a][b] = g->n_shock.x[a] * du.x[b] * fac;
            s->gradB.m[a][b] = g->n_shock.x[a] * db.x[b] * fac;
         }
      s->gradBmag = mvmul(&s->gradB, s->bhat);
      s->dUdt = vscale(shock_trd(g->tanh_k, ds) * g->v_shock / g->width, vsub(g->u1, g->u0));
      s->dBdt = vscale(shock_trd(g->tanh_k, ds) * g->v_shock / g->width, vsub(g->B1, g->B0));
      s->dBmagdt = 0.0;
      break;
   }
   case BG_DIPOLE: { /* src/background_dipole.cc:86-115 */
      v3 pp = vsub(pos, g->r0);
      double r2 = vnorm(pp), r5 = r2 * r2 * r2, mdotr;
      int a, b;
      r2 *= r2;
      r5 *= r2;
      mdotr = vdot(g->M, pp);
      s->gradU = mzero();
      for (a = 0; a < 3; a++)
         for (b = 0; b < 3; b++) {
            double unit = (a == b) ? 1.0 : 0.0;
            s->gradB.m[a][b] = 3.0 * (g->M.x[a] * pp.x[b] + pp.x[a] * g->M.x[b] + mdotr * (unit - 5.0 * (pp.x[a] * pp.x[b]) / r2)) / r5;
         }
      s->gradBmag = mvmul(&s->gradB, s->bhat);
      s->dUdt = V(0, 0, 0); s->dBdt = V(0, 0, 0); s->dBmagdt = 0.0;
      break;
   }
   case BG_SOLARWIND:
      if (T->o->deriv_mode == 1) {
         if (mask & (BG_gradU | BG_gradB | BG_dUdt | BG_dBdt)) solarwind_grad(g, pos, s);
      }
      else numerical_derivs(g, t, pos, mom_pmu, s);
      break;
   }
   return 0;
}

/* ------------------------------------------------------------------------------------------ */
/* diffusion (src/diffusion_base.cc:105-217, src/diffusion_other.cc)                          */
/* ------------------------------------------------------------------------------------------ */
typedef struct {
   double K[3];
   double vmag, mu, st2, Omega;
} dstate;

/* DiffusionWNLTRampVLISM::EvaluateDiffusion (src/diffusion_other.cc:301-324): the largest turbulent scale grows
 * linearly from l_max_HP at the heliopause nose to l_max at the sheath, on the Rankine half body through "pos";
 * the three variances scale with (k_min_ref / k_min)^(ps_index - 1). Beyond the sheath the constant values. */
static void wnlt_ramp(const df_t* d, v3 pos, double* kmin, double* a2a, double* a2t, double* a2l)
{
   double r0 = vnorm(pos), z0 = sqrt(0.5 * r0 * (r0 + pos.x[2])), k_ratio;
   if (z0 > d->a[9]) return;
   *kmin = M_2PI_ / (d->a[7] + (d->a[1] - d->a[7]) * (z0 - d->a[8]) / (d->a[9] - d->a[8]));
   k_ratio = pow(d->a[3] / *kmin, d->a[4]);
   *a2a = d->a[0] * k_ratio;
   *a2t = d->a[5] * k_ratio;
   *a2l = d->a[6] * k_ratio;
}

static void eval_diff(const df_t* d, int comp, double t, v3 pos, v3 mom, const spdata* s, dstate* st)
{
   double* K = st->K;
   double p = mom.x[0];
   (void)t;
   switch (d->kind) {
   case DF_ISO:
      if (comp == 0 || comp == 1) return;
      K[2] = d->a[0] * (1.0 - st->mu * st->mu);
      break;
   case DF_QLT:
      if (comp == 0 || comp == 1) return;
      K[2] = 0.25 * M_PI_ * d->a[4] * fabs(st->Omega) * st->st2 * pow(st->vmag * d->a[3] * fabs(st->mu / st->Omega), d->a[4]) * d->a[0];
      break;
   case DF_WNLT: case DF_WNLT_RAMP: {
      /* DiffusionWNLTConstant::EvaluateDiffusion (src/diffusion_other.cc:215-243). The reference defines
       * USE_QLT_SCATT_WITH_WNLT_DIFF (src/diffusion_other.hh:137), so after K_perp the pitch-angle component is the
       * QLT one and the hypergeometric correction is never reached. */
      double kmin = d->a[3], a2a = d->a[0], a2t = d->a[5], a2l = d->a[6], ct, cl, q;
      if (comp == 1) return;
      if (d->kind == DF_WNLT_RAMP) wnlt_ramp(d, pos, &kmin, &a2a, &a2t, &a2l);
      q = st->mu / kmin;
      ct = 0.5 * d->a[4] / (d->a[2] + 1.0) * (q * q) * a2t;
      q = st->vmag * st->st2 / st->Omega;
      cl = 0.125 * (q * q) * a2l;
      K[0] = st->vmag * sqrt(ct + cl);
      if (comp == 0) return;
      K[2] = 0.25 * M_PI_ * d->a[4] * fabs(st->Omega) * st->st2 * pow(st->vmag * kmin * fabs(st->mu / st->Omega), d->a[4]) * a2a;
      break;
   }
   case DF_PARA: if (comp == 0 || comp == 2) return; K[1] = d->a[0]; break;
   case DF_PERP: if (comp == 1 || comp == 2) return; K[0] = d->a[0]; break;
   case DF_FULL: if (comp == 2) return; K[0] = d->a[0]; K[1] = d->a[1]; break;
   case DF_FLOWMOM:
      if (comp == 2) return;
      K[1] = d->a[0] * pow(vnorm(s->U) / d->a[1], d->a[2]) * pow(p / d->a[3], d->a[4]);
      K[0] = d->a[5] * K[1];
      break;
   case DF_KINRAD: {
      double r = vnorm(pos), kap_mom;
      if (comp == 2) return;
      kap_mom = d->a[0] * pow(enr_kin(p) / d->a[1], d->a[3]);
      if (d->i0 == 0 || r < d->a[2]) K[1] = kap_mom * pow(r / d->a[2], d->a[4]);
      else if (r < d->a[2] + d->a[7]) { double q = vnorm(s->U) / d->a[6]; K[1] = kap_mom * (q * q); }
      else K[1] = kap_mom * d->a[9];
      K[0] = d->a[5] * K[1];
      break;
   }
   case DF_RIGB:
      if (comp == 2) return;
      K[1] = (d->a[0] * st->vmag / 3.0) * pow(rigidity(p) / d->a[1], d->a[3]) * pow(s->Bmag / d->a[2], d->a[4]);
      K[0] = d->a[5] * K[1];
      break;
   case DF_STRAUSS: case DF_POTGIETER: {
      double lism, lam_or_kap, B0_eff, rig, kr;
      if (comp == 2) return;
      lism = (d->i0 < 0) ? 0.0 : (s->region.x[d->i0] > 0.0 ? 0.0 : 1.0);
      lam_or_kap = lism * d->a[1] + (1.0 - lism) * d->a[0];
      B0_eff = lism * s->Bmag + (1.0 - lism) * d->a[3];
      rig = rigidity(p);
      if (d->kind == DF_STRAUSS)
         K[1] = (lam_or_kap * st->vmag / 3.0) * (rig < d->a[2] ? cbrt(rig / d->a[2]) : rig / d->a[2]) * (B0_eff / s->Bmag);
      else {
         double q = rig / d->a[2];
         K[1] = lam_or_kap * (st->vmag / c_code()) * (rig < d->a[2] ? 1.0 : sqrt(q * q * q)) * (B0_eff / s->Bmag);
      }
      if (comp == 0) {
         kr = lism * d->a[5] + (1.0 - lism) * d->a[4];
         K[0] = kr * K[1];
      }
      break;
   }
   case DF_EMPIRICAL: {
      double lam = 0.0, rig_dep = 0.0, rig = rigidity(p), q = rig / d->a[2], bmix, c;
      if (comp == 2) return;
      if (comp == 1) { rig_dep = cbrt(q * (1.0 + (q * q) * (q * q))); lam = d->a[0]; }
      else if (comp == 0) {
         rig_dep = cbrt(q * (1.0 + q * q));
         bmix = (s->region.x[d->i0 < 0 ? 0 : d->i0] < 0.0) ? 0.0 : 1.0;
         if (d->i0 < 0) bmix = 1.0;
         if (vnorm(pos) < d->a[5]) lam = d->a[1] * (bmix + (1.0 - bmix) * d->a[4]);
         else lam = d->a[1];
      }
      K[comp] = (lam * st->vmag / 3.0) * rig_dep * (d->a[3] / s->Bmag);
      c = cos(0.5 * s->region.x[d->i1]);
      K[comp] /= 1.0 + d->a[6] * (c * c);
      break;
   }
   }
}

/* DiffusionBase::GetComponent (src/diffusion_base.cc:105-121) */
static double get_component(trj_t* T, int comp, double t, v3 pos, v3 mom, const spdata* s, dstate* st)
{
   st->vmag = vel_of(mom.x[0]);
   st->Omega = cyclotron(st->vmag, s->Bmag);
   if (T->o->traj_type != 206 && T->o->traj_type != 207) {
      st->mu = mom.x[1];
      st->st2 = 1.0 - st->mu * st->mu;
   }
   eval_diff(&T->pb->df, comp, t, pos, mom, s, st);
   return st->K[comp];
}

/* GetDirectionalDerivative: analytic overrides where the reference has them
 * (src/diffusion_other.cc:395-398, 473-476, 553-556, 637-642, 732-742, 818-823), else the
 * base-class central difference (src/diffusion_base.cc:131-217). */
static double dir_derivative(trj_t* T, int comp, int xyz, double t, v3 pos, v3 mom, const spdata* s, dstate* st)
{
   const df_t* d = &T->pb->df;
   switch (d->kind) {
   case DF_PARA: case DF_PERP: case DF_FULL: return 0.0;
   case DF_FLOWMOM: {
      double un = vnorm(s->U);
      v3 row = V(s->gradU.m[xyz][0], s->gradU.m[xyz][1], s->gradU.m[xyz][2]);
      return st->K[comp] * d->a[2] * vdot(row, s->U) / (un * un);
   }
   case DF_KINRAD: {
      double r = vnorm(pos);
      if (d->i0 == 0 || r < d->a[2]) return st->K[comp] * d->a[4] * pos.x[xyz] / (r * r);
      else if (r < d->a[2] + d->a[7]) {
         double un = vnorm(s->U);
         v3 row = V(s->gradU.m[xyz][0], s->gradU.m[xyz][1], s->gradU.m[xyz][2]);
         return st->K[comp] * 2.0 * vdot(row, s->U) / (un * un);
      }
      return 0.0;
   }
   case DF_RIGB: return st->K[comp] * d->a[4] * s->gradBmag.x[xyz] / s->Bmag;
   default: {
      spdata s2 = *s;
      dstate s_saved = *st, sf, sb;
      double dr = 0.5 * s->dr[xyz], kf, kb;
      v3 p2 = pos;
      int j;
      sf = *st;
      p2.x[xyz] += dr;
      for (j = 0; j < 3; j++) s2.B.x[j] += s->gradB.m[xyz][j] * dr;
      s2.Bmag += s->gradBmag.x[xyz] * dr;
      eval_diff(d, comp, t, p2, mom, &s2, &sf);
      kf = sf.K[comp];
      dr *= 2.0;
      sb = sf;
      p2.x[xyz] -= dr;
      for (j = 0; j < 3; j++) s2.B.x[j] -= s->gradB.m[xyz][j] * dr;
      s2.Bmag -= s->gradBmag.x[xyz] * dr;
      eval_diff(d, comp, t, p2, mom, &s2, &sb);
      kb = sb.K[comp];
      *st = s_saved;
      return (kf - kb) / dr;
   }
   }
}

/* DiffusionBase::GetMuDerivative (src/diffusion_base.cc:226-255); isotropic: -2 D0 mu */
static double mu_derivative(trj_t* T, int comp, double t, v3 pos, v3 mom, const spdata* s, dstate* st)
{
   const df_t* d = &T->pb->df;
   if (d->kind == DF_ISO) return -2.0 * d->a[0] * st->mu;
   if (d->kind == DF_PARA || d->kind == DF_PERP || d->kind == DF_FULL || d->kind == DF_FLOWMOM ||
       d->kind == DF_KINRAD || d->kind == DF_RIGB || (d->kind >= DF_STRAUSS && d->kind <= DF_EMPIRICAL)) return 0.0;
   {
      dstate s2 = *st;
      double dmu = SP_SMALL * (st->mu + SP_SMALL < 1.0 ? 1.0 : -1.0);
      s2.mu += dmu;
      s2.st2 = 1.0 - s2.mu * s2.mu;
      eval_diff(d, comp, t, pos, mom, s, &s2);
      return (s2.K[comp] - st->K[comp]) / dmu;
   }
}

/* ------------------------------------------------------------------------------------------ */
/* boundaries (src/boundary_base.cc:105-191 and subclasses)                                   */
/* ------------------------------------------------------------------------------------------ */
static void eval_bnd(trj_t* T, bnd_t* b, double t, v3 pos, v3 mom, v3 bhat, v3 region)
{
   int tt = T->o->traj_type;
   switch (b->kind) {
   case BT_TIME: case BT_TIME_PASS: b->delta = t - b->timemark; break;
   case BT_TIME_REC: b->delta = t - ((b->max_crossings - b->crossings_left) + 1) * b->timemark; break;
   case BT_PLANE_ABS: case BT_PLANE_REF: case BT_PLANE_PASS:
      b->delta = vdot(vsub(pos, b->origin), b->norm);
      b->normal = b->norm;
      break;
   case BT_BOX_REF: {
      int s;
      double dt_;
      b->delta = -SP_LARGE;
      for (s = 0; s < 3; s++) {
         dt_ = -vdot(vsub(pos, b->corner0), b->normals[s]);
         if (dt_ > b->delta) { b->delta = dt_; b->normal = vscale(-1.0, b->normals[s]); }
         dt_ = vdot(vsub(pos, b->corner1), b->normals[s]);
         if (dt_ > b->delta) { b->delta = dt_; b->normal = b->normals[s]; }
      }
      break;
   }
   case BT_SPH_ABS: case BT_SPH_REF: case BT_SPH_PASS:
      b->delta = vnorm(vsub(pos, b->origin)) - b->radius;
      b->normal = vunit(vsub(pos, b->origin));
      break;
   case BT_RANKINE: {
      v3 pr = vsub(pos, b->origin);
      double z = vdot(pr, b->axis), r = vnorm(pr);
      b->delta = r - b->z_nose * sqrt(2.0 / (1.0 + z / r));
      break;
   }
   case BT_CYL: {
      v3 pr = to_basis(vsub(pos, b->origin), b->fa);
      b->delta = sqrt(pr.x[0] * pr.x[0] + pr.x[1] * pr.x[1]) - b->radius;
      pr.x[2] = 0.0;
      b->normal = from_basis(vunit(pr), b->fa);
      break;
   }
   case BT_REGION: b->delta = region.x[b->region_ind] - b->region_val; b->normal = V(0, 0, 0); break;
   case BT_MOM_INJ: case BT_MOM_PASS: case BT_MOM_SLAB: case BT_MOM_SHELL:
      if (tt == 200 || IS_GC(tt)) b->delta = vnorm(mom) - b->momentum;
      else b->delta = mom.x[0] - b->momentum;
      if (b->kind == BT_MOM_SLAB && b->delta * b->delta_old < 0.0) {
         if (vdot(vsub(pos, b->slab_r0), b->slab_n) * vdot(vsub(pos, b->slab_r1), b->slab_n) > 0.0) b->delta_old = b->delta;
      }
      if (b->kind == BT_MOM_SHELL && b->delta * b->delta_old < 0.0) {
         double rd = vnorm(vsub(pos, b->slab_r0));
         if (rd < b->r1 || rd > b->r2) b->delta_old = b->delta;
      }
      break;
   case BT_MIRROR:
      if (tt == 205) b->delta = mom.x[0] * mom.x[1];
      else if (IS_GC(tt)) b->delta = mom.x[2];  /* the parallel component */
      else b->delta = vdot(mom, bhat);
      break;
   }
}

static void reset_bnd(trj_t* T, bnd_t* b, double scale, double t, v3 pos, v3 mom, v3 bhat, v3 region)
{
   b->scale = fabs(scale);
   b->crossings_left = b->max_crossings;
   b->terminal = (b->crossings_left == 1);
   b->delta_old = 0.0;
   eval_bnd(T, b, t, pos, mom, bhat, region);
   b->delta_old = b->delta;
   if (b->delta_old == 0.0) b->delta_old = -SP_TINY * b->scale;
   b->crossed = 0;
}

static void compute_bnd(trj_t* T, bnd_t* b, double t, v3 pos, v3 mom, v3 bhat, v3 region)
{
   eval_bnd(T, b, t, pos, mom, bhat, region);
   if (b->delta * b->delta_old <= 0.0) {
      b->crossed = 1;
      if (b->delta * b->delta_old == 0.0) b->delta = -b->delta_old;
   }
   else b->crossed = 0;
}

static void record_bnd(trj_t* T, bnd_t* b, double t, v3 pos, v3 mom, v3 bhat, v3 region)
{
   if (b->crossed) {
      b->crossings_left--;
      if (b->recurrent) eval_bnd(T, b, t, pos, mom, bhat, region);
      else b->delta_old = b->delta;
      b->crossed = 0;
   }
   else b->delta_old = b->delta;
   b->terminal = (b->crossings_left == 1);
}

/* ------------------------------------------------------------------------------------------ */
/* distributions (src/distribution_base.cc:174-194, src/distribution_templated.cc:145-181)    */
/* ------------------------------------------------------------------------------------------ */
static void pos_to_rtp(v3* p)
{
   double r = vnorm(*p), phi = atan2(p->x[1], p->x[0]);
   if (phi < 0.0) phi += M_2PI_;
   p->x[1] = acos(p->x[2] / r);
   p->x[0] = r;
   p->x[2] = phi;
}

static void process_trajectory(trj_t* T, int di, int action)
{
   const dist_t* d = &T->pb->d[di];
   v3 value = V(0, 0, 0);
   double w[9] = {0};
   int nw = d->width, ijk, k;
   int bin[3] = {0, 0, 0};
   int64_t lin;
   int tt = T->o->traj_type;
   const spdata* s1 = &T->sp0;
   const spdata* s2 = &T->sp;  /* the fields of the step's start point, as in the reference */
   if (action >= d->n_actions) { T->error = 1; return; }
   /* EvaluateValue */
   switch (d->kind) {
   case DS_TIME: value.x[0] = (d->val_time == 0) ? T->t0 : T->t; break;
   case DS_POS: case DS_LOSSCONE:
      value = (d->val_time == 0) ? T->pos0 : T->pos;
      if (d->val_coord == 1) pos_to_rtp(&value);
      break;
   case DS_MOM: {
      v3 m = (d->val_time == 0) ? T->mom0 : T->mom;
      v3 bh = (d->val_time == 0) ? s1->bhat : s2->bhat;
      if (d->val_coord == 0 || (tt != 200 && tt != 199 && !IS_GC(tt))) value = m;
      else if (tt == 199) value = V(m.x[2], 0.0, 0.0);  /* src/distribution_other.cc:276-279 */
      else if (tt == 200) { value.x[0] = vnorm(m); value.x[1] = vdot(m, bh) / value.x[0]; value.x[2] = 0.0; }
      else { value.x[0] = vnorm(m); value.x[1] = m.x[2] / value.x[0]; value.x[2] = 0.0; }
      break;
   }
   case DS_POSMOM: {
      v3 p = (d->val_time == 0) ? T->pos0 : T->pos, m = (d->val_time == 0) ? T->mom0 : T->mom;
      value.x[0] = (d->pos_idx == 3) ? vnorm(p) : p.x[d->pos_idx];
      value.x[1] = m.x[d->mom_idx];
      break;
   }
   case DS_SPEC: case DS_SPECBENT:
      /* src/distribution_other.cc:553-561: Fieldline takes the parallel component */
      value.x[0] = enr_kin((tt >= 200 && tt <= 204) ? vnorm(T->mom0) : (tt == 199 ? T->mom0.x[2] : T->mom0.x[0]));
      break;
   case DS_CUM1: case DS_CUM2: value.x[0] = T->t; break;
   case DS_DIVFLOW: value = T->mom0; break;
   case DS_TIMEMU:
      value.x[0] = T->t;
      value.x[1] = (tt == 200) ? vdot(T->mom, s2->bhat) / vnorm(T->mom) : IS_GC(tt) ? T->mom.x[2] / vnorm(T->mom) : T->mom.x[1];
      break;
   case DS_ANISO_LISM: {
      /* DistributionAnisotropyLISM::EvaluateValue, src/distribution_other.cc:416-426: the first point's
       * momentum in the binning frame (GeoVector::ChangeToBasis), as spherical (r, theta, phi); theta
       * and phi binned. The reference leaves the third value unset while binning dims 5; 0 here. */
      v3 q = V(vdot(T->mom0, d->rot[0]), vdot(T->mom0, d->rot[1]), vdot(T->mom0, d->rot[2]));
      pos_to_rtp(&q);
      value = V(q.x[1], q.x[2], 0.0);
      break;
   }
   }
   /* EvaluateWeight */
   switch (d->kind) {
   case DS_TIME: case DS_POS: case DS_MOM: case DS_POSMOM: case DS_TIMEMU:
      w[0] = (action == 0) ? d->val_hot : d->val_cold;
      break;
   case DS_SPEC: case DS_SPECBENT:
      if (action == 0) {
         double m2 = (tt >= 200 && tt <= 204) ? vnorm(T->mom) : (tt == 199 ? T->mom.x[2] : T->mom.x[0]);
         double ke = enr_kin(m2), v = vel_of(m2);
         w[0] = d->J0 * v * pow(ke / d->T0, d->pow_law) / (m2 * m2);
         if (d->kind == DS_SPECBENT) w[0] /= pow(1.0 + pow(ke / d->T_b, d->pow_law_comb), d->bend);
      }
      else w[0] = d->val_cold;
      break;
   case DS_CUM1: {
      v3 dp = vsub(T->pos, T->pos0);
      w[0] = dp.x[0]; w[1] = dp.x[1]; w[2] = dp.x[2];
      break;
   }
   case DS_CUM2: {
      v3 dp = vsub(T->pos, T->pos0);
      int i, j;
      for (i = 0; i < 3; i++)
         for (j = 0; j < 3; j++) w[3 * i + j] = dp.x[i] * dp.x[j];
      break;
   }
   case DS_DIVFLOW: w[0] = (action == 0) ? d->A0 * pow(fabs(sd_divU(s2)), d->pow_law) : d->val_cold; break;
   case DS_LOSSCONE:
      /* DistributionLossCone::RecordLossCone, src/distribution_other.cc:858-862: the |B| extrema along
       * the trajectory and the loss-cone half-angle at the first or the second point */
      w[0] = T->bmag_min;
      w[1] = T->bmag_max;
      w[2] = asin(sqrt(((d->val_time == 0) ? s1->Bmag : s2->Bmag) / T->bmag_max));
      break;
   case DS_ANISO_LISM: {
      /* src/distribution_other.cc:433-483; the relative momentum p2 - RelFactor1(|p2|) m U_LISM
       * (common/physics.hh:260-263) of EvaluateValue, m = 1 and q = 1 for the proton in code units */
      double m1 = vnorm(T->mom0), m2 = vnorm(T->mom), rf = sqrt(1.0 + (m2 / 1.0 / c_code()) * (m2 / 1.0 / c_code()));
      v3 rel = vsub(T->mom, vscale(rf * 1.0, d->u_lism)), ru;
      double rn = vnorm(rel);
      ru = V(rel.x[0] / rn, rel.x[1] / rn, rel.x[2] / rn);
      if (action == 0) {  /* ComptonGettingFactor */
         v3 mh = V(T->mom0.x[0] / m1, T->mom0.x[1] / m1, T->mom0.x[2] / m1);
         w[0] = 1.0 - vdot(vscale(d->pow_law, d->u_lism), mh) / vel_of(m1);
      }
      else if (action == 1) w[0] = pow(rn / m1, d->pow_law);           /* MomPowerLawAnisotropy */
      else if (action == 2) w[0] = vdot(ru, s2->bhat);                 /* FirstLegendreAnisotropy */
      else if (action == 3) {                                           /* SecondLegendreAnisotropy */
         double c = vdot(ru, s2->bhat);
         w[0] = 0.5 * (3.0 * (c * c) - 1.0);
      }
      else {                                                            /* bCrossGradientAnisotropy */
         double rl = rn * c_code() / (fabs(1.0) * s2->Bmag);
         w[0] = vdot(d->grad_perp, vadd(T->pos, vscale(rl, vcross(ru, s2->bhat))));
      }
      break;
   }
   }
   /* AddEvent */
   for (ijk = 0; ijk < 3; ijk++) {
      double val;
      if (!(d->dims & (1 << ijk))) continue;
      val = (d->log_bins[ijk] ? log10(value.x[ijk]) : value.x[ijk]) - d->limits0[ijk];
      if (val != val) return;
      /* a "left" outlier is dropped unless bin_outside; the bin is then still val / bin_size,
       * which is how a negative bin width (max < min) bins correctly */
      if (val < 0.0 && !d->bin_outside[ijk]) return;
      {
         double q = val / d->bin_size[ijk];
         if (q >= (double)d->n_bins[ijk]) bin[ijk] = d->n_bins[ijk];
         else if (q <= -1.0) bin[ijk] = 0; /* D2 */
         else bin[ijk] = (int)q;
      }
      if (bin[ijk] >= d->n_bins[ijk]) {
         if (d->bin_outside[ijk]) bin[ijk] = d->n_bins[ijk] - 1;
         else return;
      }
   }
   lin = (int64_t)d->n_bins[2] * ((int64_t)d->n_bins[1] * bin[0] + bin[1]) + bin[2];
   {
      double e = exp(T->wgt);
      for (k = 0; k < nw; k++) T->sums[(d->offset_bins + lin) * nw + k] += w[k] * e + T->amp;
   }
   T->counts[d->offset_bins + lin]++;
   T->n_events[di]++;
}

static void distro_events(trj_t* T, const bnd_t* b)
{
   int di;
   for (di = 0; di < T->pb->nd; di++) {
      int action = (di < b->n_actions) ? b->actions[di] : -1;
      if (action >= 0) process_trajectory(T, di, action);
   }
}

/* ------------------------------------------------------------------------------------------ */
/* initial conditions (src/initial_*.cc)                                                      */
/* ------------------------------------------------------------------------------------------ */
static double sample_time(trj_t* T)
{
   const ini_t* q = &T->pb->it;
   if (q->kind == IT_INTERVAL) {
      if (q->n_int <= 0) return q->a[0] + (q->a[1] - q->a[0]) * next_uniform(T);
      return q->a[0] + ((double)T->traj_id + 0.5) * ((q->a[1] - q->a[0]) / (double)q->n_int);  /* D3 */
   }
   return q->a[0];
}

static v3 sample_pos(trj_t* T)
{
   const ini_t* q = &T->pb->is;
   switch (q->kind) {
   case IS_LINE:
      if (q->n_int <= 0) return vadd(q->v0, vscale(next_uniform(T), vsub(q->v1, q->v0)));
      return vadd(q->v0, vscale((double)T->traj_id + 0.5, vdiv(vsub(q->v1, q->v0), (double)q->n_int)));  /* D3 */
   case IS_BOX: {
      v3 p;
      int xyz;
      for (xyz = 0; xyz < 3; xyz++) p.x[xyz] = q->v0.x[xyz] + (q->v1.x[xyz] - q->v0.x[xyz]) * next_uniform(T);
      return p;
   }
   case IS_CIRCLE: {
      double phi = M_2PI_ * next_uniform(T);
      return vadd(vadd(q->v0, vscale(cos(phi), q->v1)), vscale(sin(phi), q->v2));
   }
   case IS_SPHERE: case IS_SECTOR: {
      double ct, st, phi;
      if (q->kind == IS_SPHERE) {
         ct = -1.0 + 2.0 * next_uniform(T);
         st = sqrt(1.0 - ct * ct);
         phi = M_2PI_ * next_uniform(T);
      }
      else {
         ct = q->a[5] + (q->a[6] - q->a[5]) * next_uniform(T);
         st = sqrt(1.0 - ct * ct);
         phi = q->a[3] + (q->a[4] - q->a[3]) * next_uniform(T);
      }
      return vadd(q->v0, V(q->a[0] * st * cos(phi), q->a[0] * st * sin(phi), q->a[0] * ct));
   }
   case IS_RANKINE: {
      double ct = q->a[2] + (1.0 - q->a[2]) * next_uniform(T);
      double r = q->a[0] * sqrt(2.0 / (1.0 + ct)), z = r * ct, s = sqrt(r * r - z * z);
      double phi = M_2PI_ * next_uniform(T);
      return vadd(q->v0, V(s * cos(phi), s * sin(phi), z));
   }
   case IS_CYLINDER: case IS_CYL_SECTOR: {
      /* src/initial_space.cc:576-583, 638-645 */
      double z = next_uniform(T), phi;
      v3 ry = V(q->a[0], q->a[1], q->a[2]);
      if (q->kind == IS_CYLINDER) phi = M_2PI_ * next_uniform(T);
      else phi = q->a[3] + (q->a[4] - q->a[3]) * next_uniform(T);
      return vadd(vadd(vadd(q->v0, vscale(cos(phi), q->v2)), vscale(sin(phi), ry)), vscale(z, q->v1));
   }
   case IS_EQ_BAND: {
      double L = q->a[1] + (q->a[2] - q->a[1]) * next_uniform(T);
      double phi = M_2PI_ * next_uniform(T);
      return vadd(q->v0, V(L * q->a[0] * cos(phi), L * q->a[0] * sin(phi), 0.0));
   }
   default: return q->v0;
   }
}

/* GetMomSample(axis): src/initial_base.cc:133-143 and the momentum samplers */
static v3 sample_mom(trj_t* T, v3 axis_in)
{
   const ini_t* q = &T->pb->im;
   int tt = T->o->traj_type;
   v3 axis = vunit(axis_in);
   switch (q->kind) {
   case IM_FIXED: return q->v0;  /* Lorentz and Fieldline only */
   case IM_BEAM:
      if (tt == 200) return vscale(q->a[0], axis);
      if (IS_GC(tt)) return V(0.0, 0.0, q->a[0]);
      return V(q->a[0], 0.0, 0.0);
   case IM_RING:
      if (tt == 200) {
         double phi = M_2PI_ * next_uniform(T);
         v3 e1 = second_unit(axis), e2 = vcross(axis, e1);
         v3 m = vscale(q->a[0] * q->a[2], axis);
         return vadd(m, vscale(q->a[0] * q->a[3], vadd(vscale(cos(phi), e1), vscale(sin(phi), e2))));
      }
      if (IS_GC(tt)) return V(q->a[0] * q->a[3], 0.0, q->a[0] * q->a[2]);
      return V(q->a[0], q->a[2], 0.0);
   case IM_SHELL: case IM_THICK: {
      double p = q->a[0];
      if (q->kind == IM_THICK) {
         if (q->flag) p = pow(10.0, q->a[0] + (q->a[1] - q->a[0]) * next_uniform(T));
         else p = q->a[0] + (q->a[1] - q->a[0]) * next_uniform(T);
      }
      if (tt == 206 || tt == 207) return V(p, 0.0, 0.0);
      if (tt == 199) return V(0.0, 0.0, p);  /* src/initial_momentum.cc:290-291, 390-391 */
      if (tt == 205) {
         double mu = -1.0 + 2.0 * next_uniform(T);
         return V(p, mu, 0.0);
      }
      if (IS_GC(tt)) {
         double mu = -1.0 + 2.0 * next_uniform(T), st = sqrt(1.0 - mu * mu);
         return V(p * st, 0.0, p * mu);
      }
      {
         double mu = -1.0 + 2.0 * next_uniform(T), st = sqrt(1.0 - mu * mu), phi = M_2PI_ * next_uniform(T);
         return V(p * st * cos(phi), p * st * sin(phi), p * mu);
      }
   }
   case IM_MAXWELL: {
      double p_para, p_perp;
      /* Fieldline: the mean momentum along the line, no draws (src/initial_momentum.cc:522-525) */
      if (tt == 199) return V(0.0, 0.0, q->a[0]);
      p_para = q->a[0] + q->a[1] * next_init_normal(T);
      p_perp = q->a[2] * sqrt(-2.0 * log(next_uniform(T)));
      if (tt == 200) {
         double phi = M_2PI_ * next_uniform(T);
         v3 e1 = second_unit(axis), e2 = vcross(axis, e1);
         return vadd(vscale(p_para, axis), vscale(p_perp, vadd(vscale(cos(phi), e1), vscale(sin(phi), e2))));
      }
      if (IS_GC(tt)) return V(p_perp, 0.0, p_para);
      {
         double p = sqrt(p_para * p_para + p_perp * p_perp);
         if (tt == 205) return V(p, p_para / p, 0.0);
         return V(p, 0.0, 0.0);
      }
   }
   case IM_LOGE_PITCH: {
      double le1 = log(q->a[0]), le2 = log(q->a[1]);
      double e = exp(le1 + (le2 - le1) * next_uniform(T));
      double mu = q->a[2] + (q->a[3] - q->a[2]) * next_uniform(T);
      double p = mom_of(e);
      if (tt == 200) {
         double psi = M_2PI_ * next_uniform(T), st = sqrt(1.0 - mu * mu);
         v3 e1 = second_unit(axis), e2 = vcross(axis, e1);
         return vadd(vscale(p * mu, axis), vscale(p * st, vadd(vscale(cos(psi), e1), vscale(sin(psi), e2))));
      }
      if (tt == 205) return V(p, mu, 0.0);
      if (IS_GC(tt)) return V(p * sqrt(1.0 - mu * mu), 0.0, p * mu);
      return V(p, 0.0, 0.0);
   }
   }
   return V(0, 0, 0);
}

/* ------------------------------------------------------------------------------------------ */
/* trajectory machinery                                                                       */
/* ------------------------------------------------------------------------------------------ */
static int is_parker(const trj_t* T) { return T->o->traj_type == 206 || T->o->traj_type == 207; }
static int is_guiding(const trj_t* T) { return IS_GC(T->o->traj_type); }
static int is_guiding_diff(const trj_t* T) { return T->o->traj_type == 203 || T->o->traj_type == 204; }
static int fwd(const trj_t* T) { return T->o->time_flow == 0; }

/* ConvertMomentum: Parker/Focused native (p, mu, -); Lorentz (|p|, p.b/|p|, 0)
 * (src/trajectory_lorentz.hh:84-87); Fieldline (|p_para|, 0, 0) (src/trajectory_fieldline.hh:80-83) */
static v3 convert_mom(const trj_t* T)
{
   if (T->o->traj_type == 199) return V(fabs(T->mom.x[2]), 0.0, 0.0);
   if (T->o->traj_type == 200) {
      double m = vnorm(T->mom);
      return V(m, vdot(T->mom, T->sp.bhat) / m, 0.0);
   }
   /* Guiding: (p_perp, -, p_para) -> (p, mu, 0), src/trajectory_guiding.hh:113-116 */
   if (is_guiding(T)) return V(sqrt(T->mom.x[0] * T->mom.x[0] + T->mom.x[2] * T->mom.x[2]), T->mom.x[2] / vnorm(T->mom), 0.0);
   return T->mom;
}

static unsigned traj_mask(const trj_t* T)
{
   switch (T->o->traj_type) {
   case 199: return BG_B;                                         /* src/trajectory_fieldline.cc:37-38, .hh:30 */
   case 200: return BG_E | BG_B;                                  /* src/trajectory_lorentz.cc:36 */
   case 205: return BG_ALL | BG_gradB | BG_gradU | BG_dUdt;       /* src/trajectory_focused.cc:40 */
   /* src/trajectory_guiding.cc:51-52 adds dB/dt, which is zero for every static background */
   case 201: case 202: case 203: case 204: return BG_ALL | BG_gradB;
   default: return BG_U | BG_B | BG_gradU | BG_gradB;             /* src/trajectory_parker.cc:204 */
   }
}

static int common_fields(trj_t* T)
{
   if (get_fields(T, T->t, T->pos, convert_mom(T), T->sp.mask, &T->sp)) {
      T->status |= TRAJ_DISCARD;
      return 1;
   }
   return 0;
}

static void set_vel_load(trj_t* T)
{
   /* Load()/LoadLocal(): Cartesian velocity, except Focused which uses (p, mu, phi) */
   T->vel = (T->o->traj_type == 205) ? vel_rmp(T->mom) : vel_cart(T->mom);
}

/* TrajectoryParker::DiffusionCoeff (src/trajectory_parker.cc:83-153) */
static int parker_diffusion_coeff(trj_t* T)
{
   dstate st;
   memset(&st, 0, sizeof st);
   if (T->o->deriv_mode == 0) {
      /* TRAJ_PARKER_DIVK_METHOD 0: central differences of the full tensor */
      double delta = fmin(larmor(T->mom.x[0], T->sp.Bmag), T->sp.dmax);
      int i, j;
      T->Kperp = get_component(T, 0, T->t, T->pos, T->mom, &T->sp, &st);
      T->Kpara = get_component(T, 1, T->t, T->pos, T->mom, &T->sp, &st);
      T->divK = V(0, 0, 0);
      for (j = 0; j < 3; j++) {
         spdata sf, sb;
         dstate df, db;
         double kpf, kaf, kpb, kab;
         v3 pt = vadd(T->pos, vscale(delta, cart_unit[j]));
         memset(&sf, 0, sizeof sf);
         memset(&sb, 0, sizeof sb);
         memset(&df, 0, sizeof df);
         memset(&db, 0, sizeof db);
         if (get_fields(T, T->t, pt, T->mom, BG_U | BG_B, &sf)) return 1;
         kpf = get_component(T, 0, T->t, pt, T->mom, &sf, &df);
         kaf = get_component(T, 1, T->t, pt, T->mom, &sf, &df);
         pt.x[j] -= 2.0 * delta;
         if (get_fields(T, T->t, pt, T->mom, BG_U | BG_B, &sb)) return 1;
         kpb = get_component(T, 0, T->t, pt, T->mom, &sb, &db);
         kab = get_component(T, 1, T->t, pt, T->mom, &sb, &db);
         for (i = 0; i < 3; i++) {
            double kf = kpf * (i == j ? 1.0 : 0.0) + (kaf - kpf) * sf.bhat.x[j] * sf.bhat.x[i];
            double kb = kpb * (i == j ? 1.0 : 0.0) + (kab - kpb) * sb.bhat.x[j] * sb.bhat.x[i];
            T->divK.x[i] += 0.5 * (kf - kb) / delta;
         }
      }
   }
   else {
      /* TRAJ_PARKER_DIVK_METHOD 1 */
      v3 gKpe, gKpa, t1, t2;
      m3 gbh;
      int i;
      double divb;
      T->Kperp = get_component(T, 0, T->t, T->pos, T->mom, &T->sp, &st);
      for (i = 0; i < 3; i++) gKpe.x[i] = dir_derivative(T, 0, i, T->t, T->pos, T->mom, &T->sp, &st);
      T->Kpara = get_component(T, 1, T->t, T->pos, T->mom, &T->sp, &st);
      for (i = 0; i < 3; i++) gKpa.x[i] = dir_derivative(T, 1, i, T->t, T->pos, T->mom, &T->sp, &st);
      gbh = sd_gradbhat(&T->sp);
      divb = sd_divbhat(&T->sp);
      t1 = vsub(gKpa, gKpe);
      /* bhatbhat * (gKpa - gKpe) = bhat (bhat . d) */
      t2 = vscale(vdot(T->sp.bhat, t1), T->sp.bhat);
      T->divK = vadd(vadd(gKpe, t2), vscale(T->Kpara - T->Kperp, vadd(vscale(divb, T->sp.bhat), vmmul(T->sp.bhat, &gbh))));
   }
   return 0;
}

static int parker_slopes(trj_t* T, v3* sp, v3* sm, double* sa)
{
   T->drift_vel = T->sp.U;  /* DriftCoeff without TRAJ_PARKER_USE_B_DRIFTS */
   if (parker_diffusion_coeff(T)) return 1;
   *sp = fwd(T) ? vadd(T->drift_vel, T->divK) : vsub(T->drift_vel, T->divK);
   *sm = V(-T->mom.x[0] * sd_divU(&T->sp) / 3.0, 0.0, 0.0);
   *sa = 0.0;
   if (T->o->traj_type == 207 && T->pb->has_src && T->pb->src_kind == 1) *sa = T->pb->src_rate;  /* SourceConstant */
   else if (T->o->traj_type == 207 && T->pb->has_src) {
      /* TrajectoryParkerSource::Slopes -> SourceMomentumInjection::EvaluateSource
       * (src/trajectory_parker_source.cc:58-66, src/source_other.cc:113-119): a crossing of
       * p_inj since the previous step start gives rate / dt, with dt still the previous step's */
      double del = T->mom.x[0] - T->pb->src_p_inj;
      if (del * T->src_del_old < 0.0) {
         if (T->pb->src_kind == 2) *sa = T->pb->src_rate / T->dt;
         else {
            /* SourceSphericalShockInjection::EvaluateSource (src/source_other.cc:166-177): only in the shell */
            double r = vnorm(vsub(T->pos, T->pb->src_r0));
            if (T->pb->src_r_sh <= r && r <= T->pb->src_r_sh + T->pb->src_w_sh) *sa = T->pb->src_rate / T->dt;
         }
      }
      T->src_del_old = del;
   }
   return 0;
}

/* TimeBoundaryProximityCheck, src/trajectory_base.cc:151-179 */
static void time_proximity(trj_t* T)
{
   int b;
   double c = c_code(), delta, dn;
   dn = fwd(T) ? -SP_LARGE * T->sp.dmax / c : SP_LARGE * T->sp.dmax / c;
   for (b = 0; b < T->pb->nbt; b++) {
      delta = T->bt[b].delta;
      if (fwd(T)) { if (delta <= 0.0 && delta > dn) dn = delta; }
      else { if (delta >= 0.0 && delta < dn) dn = delta; }
   }
   if (fwd(T)) { if (T->dt >= -dn) T->dt = fmax(-(1.0 + SP_LITTLE) * dn, SP_SMALL * T->sp.dmax / c); }
   else { if (T->dt >= dn) T->dt = fmax((1.0 + SP_LITTLE) * dn, SP_SMALL * T->sp.dmax / c); }
}

static void store(trj_t* T)
{
   T->segments++;
   T->stored_t = T->t;
   T->stored_pos = T->pos;
   T->stored_mom = T->mom;
}

/* HandleBoundaries, src/trajectory_base.cc:413-535 */
/* ReverseMomentum: the base negates the vector (src/trajectory_base.cc:139-142), Focused its mu
 * (src/trajectory_focused.hh:141-144), Guiding its parallel component (src/trajectory_guiding.hh:123-126),
 * Parker does nothing (src/trajectory_parker.hh:129-131) */
static void reverse_momentum(trj_t* T)
{
   switch (T->o->traj_type) {
   case 205: T->mom.x[1] = -T->mom.x[1]; break;
   case 201: case 202: case 203: case 204: T->mom.x[2] = -T->mom.x[2]; break;
   case 206: case 207: break;
   default: T->mom = vscale(-1.0, T->mom);
   }
}

static void handle_boundaries(trj_t* T)
{
   int b;
   v3 mp = convert_mom(T);
   (void)mp;
   for (b = 0; b < T->pb->nbt; b++) compute_bnd(T, &T->bt[b], T->t, T->pos, T->mom, T->sp.bhat, T->sp.region);
   for (b = 0; b < T->pb->nbs; b++) compute_bnd(T, &T->bs[b], T->t, T->pos, T->mom, T->sp.bhat, T->sp.region);
   for (b = 0; b < T->pb->nbm; b++) compute_bnd(T, &T->bm[b], T->t, T->pos, T->mom, T->sp.bhat, T->sp.region);
   for (b = 0; b < T->pb->nbm; b++) {
      if (T->bm[b].crossed) {
         T->bactive_m = b;
         if (T->bm[b].reflect) {}
         else if (T->bm[b].terminal) T->status |= TRAJ_MOMENTUM_CROSSED | TRAJ_FINISH;
      }
   }
   if (T->bactive_m >= 0) { distro_events(T, &T->bm[T->bactive_m]); T->bactive_m = -1; }
   for (b = 0; b < T->pb->nbs; b++) {
      bnd_t* bd = &T->bs[b];
      if (bd->crossed) {
         T->bactive_s = b;
         if (bd->reflect) {
            T->pos = vsub(T->pos, vscale(2.0 * bd->delta, bd->normal));
            reverse_momentum(T);
            compute_bnd(T, bd, T->t, T->pos, T->mom, T->sp.bhat, T->sp.region);
            bd->crossings_left--;
         }
         else if (bd->terminal) T->status |= TRAJ_SPATIAL_CROSSED | TRAJ_FINISH;
      }
   }
   if (T->bactive_s >= 0) { distro_events(T, &T->bs[T->bactive_s]); T->bactive_s = -1; }
   for (b = 0; b < T->pb->nbt; b++) {
      if (T->bt[b].crossed) {
         T->bactive_t = b;
         if (T->bt[b].terminal) T->status |= TRAJ_TIME_CROSSED | TRAJ_FINISH;
      }
   }
   if (T->bactive_t >= 0) { distro_events(T, &T->bt[T->bactive_t]); T->bactive_t = -1; }
   for (b = 0; b < T->pb->nbt; b++) record_bnd(T, &T->bt[b], T->t, T->pos, T->mom, T->sp.bhat, T->sp.region);
   for (b = 0; b < T->pb->nbs; b++) record_bnd(T, &T->bs[b], T->t, T->pos, T->mom, T->sp.bhat, T->sp.region);
   for (b = 0; b < T->pb->nbm; b++) record_bnd(T, &T->bm[b], T->t, T->pos, T->mom, T->sp.bhat, T->sp.region);
}

/* SpaceTerminateCheck, src/trajectory_base.cc:188-237 */
static int space_terminate(trj_t* T)
{
   int b = 0;
   T->bactive_s = -1;
   while (T->bactive_s == -1 && b < T->pb->nbs) {
      compute_bnd(T, &T->bs[b], T->t, T->pos, T->mom, T->sp.bhat, T->sp.region);
      if (T->bs[b].crossed && T->bs[b].terminal) {
         T->status |= TRAJ_SPATIAL_CROSSED | TRAJ_FINISH;
         T->bactive_s = b;
      }
      else b++;
   }
   if (T->bactive_s >= 0) distro_events(T, &T->bs[T->bactive_s]);
   if ((T->status & TRAJ_SPATIAL_CROSSED) && (T->status & TRAJ_FINISH)) { store(T); return 1; }
   return 0;
}

/* Butcher tables (common/rk_config.hh:72-520), from the exact table the library shares
 * (spx_rk_tables.h, pinned to the reference's header by tests/test_rk_tables.py). RKSlopes reads only
 * the strictly lower triangle of b; the rest stays zero. */
static int rk_load(int number, rk_t* R)
{
   int k, i, j;
   memset(R, 0, sizeof *R);
   for (k = 0; k < SPX_RK_N_TABLES; k++) {
      const spx_rk_entry* e = &spx_rk_index[k];
      const double* c = spx_rk_coeffs + e->offset;
      if (e->number != number) continue;
      R->number = number;
      R->stages = e->stages;
      R->order = e->order;
      R->adaptive = e->adaptive;
      for (i = 0; i < e->stages; i++) R->a[i] = *c++;
      for (i = 1; i < e->stages; i++)
         for (j = 0; j < i; j++) R->b[i][j] = *c++;
      for (i = 0; i < e->stages; i++) R->v[i] = *c++;
      for (i = 0; i < e->stages; i++) R->w[i] = *c++;
      return 0;
   }
   return -1;
}

static void lorentz_slopes(trj_t* T, v3* sp, v3* sm)
{
   /* src/trajectory_lorentz.cc:67-71 */
   *sp = T->vel;
   *sm = vscale(p_charge, vadd(T->sp.E, vdiv(vcross(T->vel, T->sp.B), c_code())));
}

/* TrajectoryFocused::DriftCoeff / Slopes, src/trajectory_focused.cc:62-128 */
static void focused_drift(trj_t* T)
{
   double ct2 = T->mom.x[1] * T->mom.x[1], st2 = 1.0 - ct2;
   const spdata* s = &T->sp;
   /* the operations in the reference's order: ((0.5 st2) (b x grad B)) / B, and ((0.5 st2) b) (B . curl B) */
   v3 bxg = vcross(s->bhat, s->gradBmag);
   v3 dv = vdiv(vscale(0.5 * st2, bxg), s->Bmag);
   v3 curlB = sd_curlB(s);
   v3 bgb = vmmul(s->B, &s->gradB);
   v3 cur = vadd(vscale(vdot(s->B, curlB), vscale(0.5 * st2, s->bhat)), vscale(ct2, vcross(s->bhat, bgb)));
   dv = vadd(dv, vdiv(cur, s->Bmag * s->Bmag));
   dv = vscale(larmor(T->mom.x[0], s->Bmag) * T->vel.x[0], dv);
   T->drift_vel = vadd(dv, vadd(s->U, vscale(T->vel.x[0] * T->mom.x[1], s->bhat)));
}

static void focused_slopes(trj_t* T, v3* sp, v3* sm)
{
   const spdata* s = &T->sp;
   double st2, bbgu = 0.0, bcd, divU;
   v3 cd;
   int i, j;
   focused_drift(T);
   *sp = T->drift_vel;
   st2 = 1.0 - T->mom.x[1] * T->mom.x[1];
   /* bb : grad U as GeoMatrix::operator% sums it: row by row, each row a dot product
    * (common/matrix.hh:556-561) */
   for (i = 0; i < 3; i++) {
      double row = 0.0;
      for (j = 0; j < 3; j++) row = (j == 0) ? s->bhat.x[i] * s->bhat.x[j] * s->gradU.m[i][j]
                                             : row + s->bhat.x[i] * s->bhat.x[j] * s->gradU.m[i][j];
      bbgu += row;
   }
   cd = vadd(s->dUdt, vmmul(s->U, &s->gradU));
   bcd = 2.0 * vdot(s->bhat, cd) / T->vel.x[0];
   divU = sd_divU(s);
   sm->x[0] = 0.5 * T->mom.x[0] * ((3.0 * st2 - 2.0) * bbgu - st2 * divU - T->mom.x[1] * bcd);
   sm->x[1] = 0.5 * st2 * (T->vel.x[0] * sd_divbhat(s) - bcd + T->mom.x[1] * (divU - 3.0 * bbgu));
   sm->x[2] = 0.0;
}

static void focused_momentum_correction(trj_t* T)
{
   if (T->mom.x[1] > 1.0) T->mom.x[1] = 1.0;
   else if (T->mom.x[1] < -1.0) T->mom.x[1] = -1.0;
}

/* TrajectoryGuiding::ModifiedFields and DriftCoeff (src/trajectory_guiding.cc:60-96). The fields are
 * static, so dB/dt and dBmag/dt are zero; dbhat/dt = (dB/dt - dBmag/dt bhat) / Bmag is formed from
 * those zeros all the same, so that signed zeros propagate as in the reference. */
static void guiding_drift(trj_t* T)
{
   const spdata* s = &T->sp;
   double c = c_code();
   double rL = larmor(T->mom.x[0], s->Bmag), rR = larmor(T->mom.x[2], s->Bmag);
   v3 dbhatdt = vdiv(vsub(V(0.0, 0.0, 0.0), vscale(0.0, s->bhat)), s->Bmag);
   v3 curlbhat = vdiv(vsub(sd_curlB(s), vcross(s->gradBmag, s->bhat)), s->Bmag);
   v3 e_star = vsub(vsub(s->E, vdiv(vscale(rR * s->Bmag, dbhatdt), c)), vdiv(vscale(rL * T->vel.x[0], s->gradBmag), 2.0 * c));
   v3 b_star = vadd(s->B, vscale(rR * s->Bmag, curlbhat));
   T->e_star = e_star;
   T->b_star = b_star;
   T->drift_vel = vdiv(vadd(vscale(T->vel.x[2], b_star), vscale(c, vcross(e_star, s->bhat))), vdot(b_star, s->bhat));
}

/* TrajectoryGuiding::Slopes with PPERP_METHOD 1 (src/trajectory_guiding.cc:104-117) */
static void guiding_slopes(trj_t* T, v3* sp, v3* sm)
{
   const spdata* s = &T->sp;
   guiding_drift(T);
   *sp = T->drift_vel;
   sm->x[0] = 0.5 * T->mom.x[0] / s->Bmag * (0.0 + vdot(T->drift_vel, s->gradBmag));
   sm->x[1] = 0.0;
   sm->x[2] = p_charge * vdot(T->e_star, T->b_star) / vdot(T->b_star, s->bhat);
}

/* TrajectoryGuidingDiff::DiffusionCoeff (src/trajectory_guiding_diff.cc:61-86): the field-aligned frame,
 * D_perp (component 0) and the perpendicular part of its gradient, V_perp */
static void guiding_diff_coeff(trj_t* T)
{
   dstate st;
   v3 g, fa[3], m = convert_mom(T);
   int i;
   memset(&st, 0, sizeof st);
   fa[2] = T->sp.bhat;
   fa[0] = second_unit(T->sp.bhat);
   fa[1] = vcross(fa[2], fa[0]);
   for (i = 0; i < 3; i++) T->fa[i] = fa[i];
   T->Kperp = get_component(T, 0, T->t, T->pos, m, &T->sp, &st);
   for (i = 0; i < 3; i++) g.x[i] = dir_derivative(T, 0, i, T->t, T->pos, m, &T->sp, &st);
   T->v_perp = from_basis(V(vdot(g, fa[0]), vdot(g, fa[1]), 0.0), fa);
}

/* sqrt(2 D_perp) at a displaced point: CommonFields(t, pos, ...) into a separate record, then GetComponent(0, ...)
 * (src/trajectory_guiding_diff.cc:152-155). "dmax" receives that evaluation's dmax, which the background's
 * GetSafeIncr reads for the next increment (src/background_base.cc:409-413). The reference's record there has an
 * uninitialised field mask; here it takes the trajectory's. */
static double perp_slope_at(trj_t* T, double t, v3 pos, v3 m, double* dmax)
{
   spdata s;
   dstate st;
   memset(&st, 0, sizeof st);
   s = T->sp;
   if (get_fields(T, t, pos, m, T->sp.mask, &s)) {
      T->status |= TRAJ_DISCARD;
      return 0.0;
   }
   *dmax = s.dmax;
   return sqrt(2.0 * get_component(T, 0, t, pos, m, &s, &st));
}

#define INCR_DMAX_RATIO 0.0001  /* src/background_base.hh:42 */

/* TrajectoryGuidingDiff::EulerPerpDiffSlopes (src/trajectory_guiding_diff.cc:103-122), STOCHASTIC_METHOD_PERP 0:
 * two normals (the next of the trajectory's count, as for the pitch-angle step). With perp_method 1 the Milstein
 * terms of MilsteinPerpDiffSlopes (:129-176), with 2 the RK2PerpDiffSlopes stages (:182-300); both draw one uniform
 * for the sign of the Levy-area stand-in. Returns 1 when an RK2 trial point crosses a terminal boundary. */
static int guiding_perp_step(trj_t* T)
{
   dstate st;
   v3 m = convert_mom(T);
   double n[4], n1, n2, dwx, dwy, d;
   uint32_t b[4];
   memset(&st, 0, sizeof st);
   spx_rng_block(T->pb->seed, (uint32_t)T->n_normal++, T->traj_id, T->pb->problem, SPX_RNG_STEP, T->attempt, b);
   normals4(b, n);
   n1 = n[0];
   spx_rng_block(T->pb->seed, (uint32_t)T->n_normal++, T->traj_id, T->pb->problem, SPX_RNG_STEP, T->attempt, b);
   normals4(b, n);
   n2 = n[0];
   dwx = sqrt(T->dt) * n1;
   dwy = sqrt(T->dt) * n2;
   d = get_component(T, 0, T->t, T->pos, m, &T->sp, &st);
   T->Kperp = d;
   {
      v3 fa[3], xhat, yhat, p;
      int i;
      const double dt = T->dt, b0 = sqrt(2.0 * d);
      double dmax = T->sp.dmax, dx, dy, bx, by, dbdx, dbdy, vxy, drx, dry;
      for (i = 0; i < 3; i++) fa[i] = T->fa[i];
      if (T->o->perp_method != 1 && T->o->perp_method != 2) {
         T->dr_perp = from_basis(V(b0 * dwx, b0 * dwy, 0.0), fa);
         return 0;
      }
      xhat = from_basis(V(1.0, 0.0, 0.0), fa);
      yhat = from_basis(V(0.0, 1.0, 0.0), fa);
      if (T->o->perp_method == 1) {
         dx = INCR_DMAX_RATIO * dmax;
         bx = perp_slope_at(T, T->t, vadd(T->pos, vscale(dx, xhat)), m, &dmax);
         dbdx = (bx - b0) / dx;
         dy = INCR_DMAX_RATIO * dmax;
         by = perp_slope_at(T, T->t, vadd(T->pos, vscale(dy, yhat)), m, &dmax);
         dbdy = (by - b0) / dy;
         vxy = next_uniform(T) < 0.5 ? dt : -dt;
         drx = b0 * dwx + 0.5 * b0 * (dbdx * (dwx * dwx - dt) + dbdy * (dwx * dwy - vxy));
         dry = b0 * dwy + 0.5 * b0 * (dbdy * (dwy * dwy - dt) + dbdx * (dwx * dwy + vxy));
      }
      else {
         const double g = 1.0 / sqrt(3.0);
         double b1, b2, bxx, byy, bxy, d2x, d2y, d2xy, rx, ry, bmid;
         v3 dpos = from_basis(V(b0 * dwx, b0 * dwy, 0.0), fa);
         T->pos = vadd(T->pos, vscale(g, dpos));
         if (space_terminate(T)) return 1;
         b1 = perp_slope_at(T, T->t + dt, T->pos, m, &dmax);
         T->pos = T->local_pos;
         T->pos = vsub(T->pos, V(dpos.x[0] / (3.0 * g), dpos.x[1] / (3.0 * g), dpos.x[2] / (3.0 * g)));
         if (space_terminate(T)) return 1;
         b2 = perp_slope_at(T, T->t + dt, T->pos, m, &dmax);
         T->pos = T->local_pos;
         dx = INCR_DMAX_RATIO * dmax;
         bxx = perp_slope_at(T, T->t, vadd(T->pos, vscale(dx, xhat)), m, &dmax);
         dx *= 0.5;
         bx = perp_slope_at(T, T->t, vadd(T->pos, vscale(dx, xhat)), m, &dmax);
         dbdx = (bx - b0) / dx;
         d2x = (bxx - 2.0 * bx + b0) / (dx * dx);
         dy = INCR_DMAX_RATIO * dmax;
         byy = perp_slope_at(T, T->t, vadd(T->pos, vscale(dy, yhat)), m, &dmax);
         dy *= 0.5;
         by = perp_slope_at(T, T->t, vadd(T->pos, vscale(dy, yhat)), m, &dmax);
         dbdy = (by - b0) / dy;
         d2y = (byy - 2.0 * by + b0) / (dy * dy);
         p = vadd(vadd(T->pos, vscale(dx, xhat)), vscale(dy, yhat));
         bxy = perp_slope_at(T, T->t, p, m, &dmax);
         d2xy = (bxy - bx - by + b0) / (dx * dy);
         vxy = next_uniform(T) < 0.5 ? dt : -dt;
         rx = 0.5 * b0 * (dbdx * (dwx * dwx - dt) + dbdy * (dwx * dwy - vxy)) + dt * (b0 * b0) * (d2y * dwx - d2xy * dwy) / 6.0;
         ry = 0.5 * b0 * (dbdy * (dwy * dwy - dt) + dbdx * (dwx * dwy + vxy)) + dt * (b0 * b0) * (d2x * dwy - d2xy * dwx) / 6.0;
         bmid = 0.5 * (b0 + (b1 + 3.0 * (g * g) * b2) / (1.0 + 3.0 * (g * g)));
         drx = bmid * dwx + rx;
         dry = bmid * dwy + ry;
      }
      T->dr_perp = from_basis(V(drx, dry, 0.0), fa);
      return 0;
   }
}

/* TrajectoryFieldline::Slopes, src/trajectory_fieldline.cc:58-66: along b at the parallel speed
 * (which_field_to_follow is BACKGROUND_B, src/trajectory_fieldline.hh:30) */
static void fieldline_slopes(trj_t* T, v3* sp, v3* sm)
{
   *sp = vscale(T->vel.x[2], T->sp.bhat);
   *sm = V(0.0, 0.0, 0.0);
}

static void slopes_rk(trj_t* T, v3* sp, v3* sm)
{
   if (T->o->traj_type == 199) fieldline_slopes(T, sp, sm);
   else if (T->o->traj_type == 200) lorentz_slopes(T, sp, sm);
   else if (is_guiding(T)) {
      guiding_slopes(T, sp, sm);
      if (is_guiding_diff(T)) {
         /* TrajectoryGuidingDiff::Slopes (src/trajectory_guiding_diff.cc:327-336) */
         guiding_diff_coeff(T);
         *sp = fwd(T) ? vadd(*sp, T->v_perp) : vsub(*sp, T->v_perp);
      }
   }
   else focused_slopes(T, sp, sm);
}

static void physical_step_rk(trj_t* T)
{
   if (T->o->traj_type == 199) {
      /* src/trajectory_fieldline.cc:47-50, cfl_adv_tf = 0.5 (src/trajectory_fieldline.hh:27) */
      T->dt_physical = 0.5 * T->sp.dmax / fabs(T->vel.x[2]);
   }
   else if (T->o->traj_type == 200) {
      /* src/trajectory_lorentz.cc:51-59 */
      double vn = vnorm(T->vel);
      double Om = fmax(cyclotron(vn, T->sp.Bmag), SP_TINY);
      T->dt_physical = M_2PI_ / Om / T->o->steps_per_orbit;
      T->dt_physical = fmin(T->dt_physical, 0.1 * T->sp.dmax / vn);
   }
   else if (is_guiding_diff(T)) {
      /* TrajectoryGuidingDiff::PhysicalStep (src/trajectory_guiding_diff.cc:343-351) */
      v3 dv = fwd(T) ? vadd(T->drift_vel, T->v_perp) : vsub(T->drift_vel, T->v_perp);
      T->dt_physical = 0.5 * T->sp.dmax / (vnorm(dv) + 0.5 * vnorm(T->vel));
      T->dt_physical = fmin(T->dt_physical, 0.5 * (T->sp.dmax * T->sp.dmax) / T->Kperp);
   }
   else if (is_guiding(T)) {
      /* src/trajectory_guiding.cc:81-86 */
      T->dt_physical = 0.5 * T->sp.dmax / (vnorm(T->drift_vel) + 0.5 * vnorm(T->vel));
   }
   else {
      /* src/trajectory_focused.cc:87-91 */
      T->dt_physical = 0.5 * T->sp.dmax / (vnorm(T->drift_vel) + 0.5 * T->vel.x[0]);
   }
}

/* Euler pitch-angle scattering, after TrajectoryGuidingScatt (src/trajectory_guiding_scatt.cc:61-110, 255-262) */
static void pa_coeffs(trj_t* T)
{
   dstate st;
   v3 m = convert_mom(T);
   memset(&st, 0, sizeof st);
   T->Dmumu = get_component(T, 2, T->t, T->pos, m, &T->sp, &st);
   T->Vmu = mu_derivative(T, 2, T->t, T->pos, m, &T->sp, &st);
}

static void pa_physical_step(trj_t* T)
{
   const double dthetamax = 2.0 * M_PI_ / 180.0;
   double amu = is_guiding(T) ? fabs(T->mom.x[2] / vnorm(T->mom)) : fabs(T->mom.x[1]);
   double dmumax = sqrt(1.0 - amu) * dthetamax + 0.5 * amu * (dthetamax * dthetamax);
   T->dt_physical = fmin(T->dt_physical, 0.5 * (dmumax * dmumax) / T->Dmumu);
   T->dt_physical = fmin(T->dt_physical, 0.5 * dmumax / fabs(T->Vmu));
}

/* The k-th normal of a guiding-centre trajectory, redraws included, is the first of the SPX_RNG_STEP
 * block with index k (one normal per block). */
static double gc_normal(trj_t* T)
{
   double n[4];
   uint32_t b[4];
   spx_rng_block(T->pb->seed, (uint32_t)T->n_normal++, T->traj_id, T->pb->problem, SPX_RNG_STEP, T->attempt, b);
   normals4(b, n);
   return n[0];
}

/* D_mumu at (p, mu) of the step's point (GetComponent(2, ...) with a modified momentum) */
static double dmumu_at(trj_t* T, double t, double p, double mu)
{
   dstate st;
   memset(&st, 0, sizeof st);
   return get_component(T, 2, t, T->pos, V(p, mu, 0.0), &T->sp, &st);
}

/* The pitch-angle steps of TrajectoryGuidingScatt (src/trajectory_guiding_scatt.cc:61-247):
 * STOCHASTIC_METHOD_MU 0 Euler (:61-84), 1 Milstein (:91-130), 2 RK2 (:137-247), each redrawing while
 * |mu| > 1 (here at most 256 times, then mu is clamped). */
static void guiding_pa_scatter(trj_t* T)
{
   v3 mc = convert_mom(T);
   const double dt = T->dt;
   double mu_new;
   int tries = 0;
   if (T->o->mu_method == 1) {
      double mu = T->mom.x[2] / vnorm(T->mom);
      double b = sqrt(2.0 * T->Dmumu);
      double dmu = SP_SMALL * (mu + SP_SMALL < 1.0 ? 1.0 : -1.0);
      double b1 = (sqrt(2.0 * dmumu_at(T, T->t, mc.x[0], mc.x[1] + dmu)) - b) / dmu;
      do {
         double dw = sqrt(dt) * gc_normal(T);
         mu_new = mu + T->Vmu * dt + b * dw + 0.5 * b * b1 * (dw * dw - dt);
      } while (fabs(mu_new) > 1.0 && ++tries < 256);
   }
   else if (T->o->mu_method == 2) {
      const double gambar = 1.0 / sqrt(3.0);
      double mu = T->mom.x[2] / vnorm(T->mom);
      double sv0 = T->Vmu, sv1 = 0.0, sd0 = sqrt(2.0 * T->Dmumu), sd1 = 0.0, sd2 = 0.0;
      do {
         double dw = sqrt(dt) * gc_normal(T), d, dn, dmu, dfit;
         mu_new = mu + sd0 * dw;
         mu_new += sv0 * dt;
         if (fabs(mu_new) > 1.0) continue;
         d = dmumu_at(T, T->t + dt, mc.x[0], mu_new);
         dmu = SP_SMALL * (mu_new + SP_SMALL < 1.0 ? 1.0 : -1.0);
         dn = dmumu_at(T, T->t + dt, mc.x[0], mu_new + dmu);
         sv1 = (dn - d) / dmu;
         mu_new = mu + gambar * sd0 * dw;
         mu_new += sv0 * dt;
         if (fabs(mu_new) > 1.0) continue;
         sd1 = sqrt(2.0 * dmumu_at(T, T->t + dt, mc.x[0], mu_new));
         mu_new = mu - sd0 / (3.0 * gambar) * dw;
         mu_new += sv0 * dt;
         if (fabs(mu_new) > 1.0) continue;
         sd2 = sqrt(2.0 * dmumu_at(T, T->t + dt, mc.x[0], mu_new));
         dmu = SP_SMALL * (mu + SP_SMALL < 1.0 ? 1.0 : -1.0);
         dfit = (sqrt(2.0 * dmumu_at(T, T->t, mc.x[0], mu + dmu)) - sd0) / dmu;
         mu_new = mu + (0.5 * sd0 + (sd1 + 3.0 * (gambar * gambar) * sd2) / (2.0 + 6.0 * (gambar * gambar))) * dw;
         mu_new += 0.5 * dt * (sv0 + sv1);
         mu_new += 0.5 * sd0 * dfit * (dw * dw - dt);
      } while (fabs(mu_new) > 1.0 && ++tries < 256);
   }
   else {
      do {
         mu_new = mc.x[1] + T->Vmu * dt + sqrt(2.0 * T->Dmumu * dt) * gc_normal(T);
      } while (fabs(mu_new) > 1.0 && ++tries < 256);
   }
   if (fabs(mu_new) > 1.0) mu_new = (mu_new > 0.0) ? 1.0 : -1.0;
   T->mom.x[0] = mc.x[0] * sqrt(1.0 - mu_new * mu_new);
   T->mom.x[2] = mc.x[0] * mu_new;
   T->vel = vel_cart(T->mom);
}

static void pa_scatter(trj_t* T, uint32_t step)
{
   /* the first four draws of a step come from its SPX_RNG_STEP block, redraws beyond that from
    * SPX_RNG_EXTRA blocks of the same step */
   double mu_new, n[4];
   uint32_t b[4];
   int k = 0, blk = 0;
   spx_rng_block(T->pb->seed, step, T->traj_id, T->pb->problem, SPX_RNG_STEP, T->attempt, b);
   normals4(b, n);
   do {
      if (k == 4) {
         spx_rng_block(T->pb->seed, step * 64u + (uint32_t)blk, T->traj_id, T->pb->problem, SPX_RNG_EXTRA, T->attempt, b);
         normals4(b, n);
         blk++;
         k = 0;
      }
      mu_new = T->mom.x[1] + T->Vmu * T->dt + sqrt(2.0 * T->Dmumu * T->dt) * n[k++];
   } while (fabs(mu_new) > 1.0 && blk < 64);
   if (fabs(mu_new) > 1.0) mu_new = (mu_new > 0.0) ? 1.0 : -1.0;
   T->mom.x[1] = mu_new;
}

/* RKStep, src/trajectory_base.cc:366-406: the step with the table's weights v, and for an adaptive
 * table the lower-order position with the weights w, the error against rk_tol_abs + rk_tol_rel
 * (|r| + |r_lo|), the next dt_adaptive and the rejection of a step whose error exceeds 1. Returns 1
 * for a rejected step (FINISH is cleared, as the reference does). */
static int rk_step(trj_t* T, const v3* slp, const v3* slm, const double* sla)
{
   const rk_t* R = T->rk;
   v3 pos_lo = T->pos;
   int il;
   double err;
   if (fwd(T)) T->t += T->dt; else T->t -= T->dt;
   for (il = 0; il < R->stages; il++) {
      if (fwd(T)) {
         T->pos = vadd(T->pos, vscale(T->dt * R->v[il], slp[il]));
         T->mom = vadd(T->mom, vscale(T->dt * R->v[il], slm[il]));
         if (R->adaptive) pos_lo = vadd(pos_lo, vscale(T->dt * R->w[il], slp[il]));
      }
      else {
         T->pos = vsub(T->pos, vscale(T->dt * R->v[il], slp[il]));
         T->mom = vsub(T->mom, vscale(T->dt * R->v[il], slm[il]));
         if (R->adaptive) pos_lo = vsub(pos_lo, vscale(T->dt * R->w[il], slp[il]));
      }
      if (sla) T->amp += T->dt * R->v[il] * sla[il] * exp(T->wgt);
   }
   T->vel = vel_cart(T->mom);
   if (!R->adaptive) return 0;
   err = RK_TOL_ABS + RK_TOL_REL * (vnorm(T->pos) + vnorm(pos_lo));
   err = sqrt(vnorm2(vsub(T->pos, pos_lo)) / (err * err));
   T->dt_adaptive = T->dt * RK_ADJUST * pow(err, -1.0 / R->order);
   T->dt_adaptive = fmin(T->dt * RK_SAFETY, T->dt_adaptive);
   T->dt_adaptive = fmax(T->dt / RK_SAFETY, T->dt_adaptive);
   if (err > 1.0 + SP_TINY) {
      T->status &= ~TRAJ_FINISH;
      return 1;
   }
   return 0;
}

/* After a rejected step the next Advance starts with Load(), which puts back time, position and
 * momentum of the last stored point (src/trajectory_base.hh:507-515); the amplitude and log-weight
 * keep the rejected step's increments. The reference keeps the fields of the rejected step's last
 * stage point too (nothing re-evaluates them before the next Slopes); with reference_quirks that is
 * reproduced, else (deviation D6, shared with the CUDA kernels) the fields are those of the restored
 * point, as at the start of the rejected step. */
static uint64_t g_rejections = 0;  /* rejected steps of the last spx_oracle_run */

static void rk_reject(trj_t* T)
{
   g_rejections++;
   T->t = T->stored_t;
   T->pos = T->stored_pos;
   T->mom = T->stored_mom;
   set_vel_load(T);
   if (!T->o->reference_quirks) common_fields(T);
}

/* RKAdvance, src/trajectory_base.cc:545-579 (Lorentz and Focused) */
static int rk_advance(trj_t* T)
{
   const rk_t* R = T->rk;
   v3 slp[SPX_RK_MAX_STAGES], slm[SPX_RK_MAX_STAGES];
   int is, il;
   int scatt = (T->o->traj_type == 205 && T->o->pa_scattering) || T->o->traj_type == 202 || T->o->traj_type == 204;
   int perp = is_guiding_diff(T);
   set_vel_load(T);
   if (scatt) {
      /* TrajectoryGuidingScatt::Advance (src/trajectory_guiding_scatt.cc:277-310) and
       * TrajectoryGuidingDiffScatt::Advance (src/trajectory_guiding_diff_scatt.cc:84-145) */
      if (perp) guiding_diff_coeff(T);
      pa_coeffs(T);
      if (is_guiding(T)) guiding_drift(T);
      else focused_drift(T);
      physical_step_rk(T);
      pa_physical_step(T);
      T->dt = fmin(T->dt_physical, T->dt_adaptive);
      time_proximity(T);
      if (is_guiding(T)) guiding_pa_scatter(T);
      else pa_scatter(T, (uint32_t)T->segments);
      set_vel_load(T);
   }
   T->local_t = T->t; T->local_pos = T->pos; T->local_mom = T->mom; T->local_amp = T->amp; T->local_wgt = T->wgt;
   slopes_rk(T, &slp[0], &slm[0]);
   if (!scatt) {
      physical_step_rk(T);
      T->dt = fmin(T->dt_physical, T->dt_adaptive);
      time_proximity(T);
   }
   if (perp && guiding_perp_step(T)) return 1;
   /* RKSlopes */
   for (is = 1; is < R->stages; is++) {
      for (il = 0; il < is; il++) {
         if (fwd(T)) {
            T->t += R->a[is] * T->dt;
            T->pos = vadd(T->pos, vscale(T->dt * R->b[is][il], slp[il]));
            T->mom = vadd(T->mom, vscale(T->dt * R->b[is][il], slm[il]));
         }
         else {
            T->t -= R->a[is] * T->dt;
            T->pos = vsub(T->pos, vscale(T->dt * R->b[is][il], slp[il]));
            T->mom = vsub(T->mom, vscale(T->dt * R->b[is][il], slm[il]));
         }
      }
      if (space_terminate(T)) return 1;
      if (common_fields(T)) return 1;
      if (T->o->traj_type == 205) focused_momentum_correction(T);
      T->vel = vel_cart(T->mom);  /* src/trajectory_base.cc:344 uses the Cartesian form for all types */
      slopes_rk(T, &slp[is], &slm[is]);
      T->t = T->local_t; T->pos = T->local_pos; T->mom = T->local_mom; T->amp = T->local_amp; T->wgt = T->local_wgt;
      set_vel_load(T);
   }
   /* RKStep; a rejected step of an adaptive table is not taken */
   if (rk_step(T, slp, slm, NULL)) {
      rk_reject(T);
      return 0;
   }
   if (perp) T->pos = vadd(T->pos, T->dr_perp);
   handle_boundaries(T);
   if (!(T->status & TRAJ_FINISH)) {
      if (common_fields(T)) return 1;
      if (T->o->traj_type == 205) focused_momentum_correction(T);
   }
   store(T);
   return 1;
}

/* TrajectoryParker::Advance, src/trajectory_parker.cc:255-306, with any Butcher table: the slopes of
 * the step's start, PhysicalStep, the stochastic displacement (EulerDiffSlopes), RKSlopes with the
 * Parker slopes at each stage point (TrajectoryParkerSource evaluates its source there too,
 * src/trajectory_parker_source.cc:58-66), RKStep, then the displacement. Returns 0 for a step an
 * adaptive table rejected. */
static int parker_advance(trj_t* T)
{
   const rk_t* R = T->rk;
   v3 slp[SPX_RK_MAX_STAGES], slm[SPX_RK_MAX_STAGES], fa[3];
   double sla[SPX_RK_MAX_STAGES], dWx, dWy, dWz;
   dstate st;
   uint32_t b[4];
   double n[4];
   int is, il;
   set_vel_load(T);
   T->local_t = T->t; T->local_pos = T->pos; T->local_mom = T->mom; T->local_amp = T->amp; T->local_wgt = T->wgt;
   if (parker_slopes(T, &slp[0], &slm[0], &sla[0])) return 1;
   /* PhysicalStep, src/trajectory_parker.cc:212-221 */
   T->dt_physical = 0.5 * T->sp.dmax / vnorm(fwd(T) ? vadd(T->drift_vel, T->divK) : vsub(T->drift_vel, T->divK));
   T->dt_physical = fmin(T->dt_physical, 0.5 * (T->sp.dmax * T->sp.dmax) / fmax(T->Kperp, T->Kpara));
   T->dt_physical = fmin(T->dt_physical, 0.5 * 3.0 * 0.01 / fabs(sd_divU(&T->sp)));
   T->dt = fmin(T->dt_physical, T->dt_adaptive);
   time_proximity(T);
   /* EulerDiffSlopes, src/trajectory_parker.cc:159-180: the trajectory's next three normals */
   fa[2] = T->sp.bhat;
   fa[0] = second_unit(T->sp.bhat);
   fa[1] = vcross(fa[2], fa[0]);
   spx_rng_block(T->pb->seed, (uint32_t)(T->n_normal / 3), T->traj_id, T->pb->problem, SPX_RNG_STEP, T->attempt, b);
   normals4(b, n);
   T->n_normal += 3;
   dWx = sqrt(T->dt) * n[0];
   dWy = sqrt(T->dt) * n[1];
   dWz = sqrt(T->dt) * n[2];
   memset(&st, 0, sizeof st);
   T->Kperp = get_component(T, 0, T->t, T->pos, T->mom, &T->sp, &st);
   T->Kpara = get_component(T, 1, T->t, T->pos, T->mom, &T->sp, &st);
   T->dr_perp = V(sqrt(2.0 * T->Kperp) * dWx, sqrt(2.0 * T->Kperp) * dWy, sqrt(2.0 * T->Kpara) * dWz);
   T->dr_perp = from_basis(T->dr_perp, fa);
   /* RKSlopes */
   for (is = 1; is < R->stages; is++) {
      for (il = 0; il < is; il++) {
         if (fwd(T)) {
            T->t += R->a[is] * T->dt;
            T->pos = vadd(T->pos, vscale(T->dt * R->b[is][il], slp[il]));
            T->mom = vadd(T->mom, vscale(T->dt * R->b[is][il], slm[il]));
         }
         else {
            T->t -= R->a[is] * T->dt;
            T->pos = vsub(T->pos, vscale(T->dt * R->b[is][il], slp[il]));
            T->mom = vsub(T->mom, vscale(T->dt * R->b[is][il], slm[il]));
         }
      }
      if (space_terminate(T)) return 1;
      if (common_fields(T)) return 1;
      T->vel = vel_cart(T->mom);
      if (parker_slopes(T, &slp[is], &slm[is], &sla[is])) return 1;
      T->t = T->local_t; T->pos = T->local_pos; T->mom = T->local_mom; T->amp = T->local_amp; T->wgt = T->local_wgt;
      set_vel_load(T);
   }
   /* RKStep, then the stochastic displacement */
   if (rk_step(T, slp, slm, sla)) {
      rk_reject(T);
      return 0;
   }
   T->pos = vadd(T->pos, T->dr_perp);
   handle_boundaries(T);
   if (!(T->status & TRAJ_FINISH)) if (common_fields(T)) return 1;
   store(T);
   return 1;
}

/* SetStart (src/trajectory_base.cc:867-939 and the trajectory overrides) */
static int set_start(trj_t* T)
{
   int b;
   double c = c_code();
   T->status = 0;
   T->segments = 0;
   T->n_normal = T->n_uniform = T->n_init_normal = 0;
   T->t = sample_time(T);
   T->pos = sample_pos(T);
   T->mom = sample_mom(T, V(1.0, 1.0, 1.0));
   memset(&T->sp, 0, sizeof T->sp);
   T->sp.mask = traj_mask(T);
   if (common_fields(T)) return 1;
   T->mom = sample_mom(T, T->sp.bhat);
   set_vel_load(T);
   T->sp0 = T->sp;
   T->bmag_min = T->bmag_max = T->sp.Bmag;
   T->dt_adaptive = SP_LARGE * T->sp.dmax / c;
   T->t0 = T->t; T->pos0 = T->pos; T->mom0 = T->mom;
   T->bactive_t = T->bactive_s = T->bactive_m = -1;
   for (b = 0; b < T->pb->nbt; b++) {
      T->bt[b] = T->pb->bt[b];
      reset_bnd(T, &T->bt[b], T->sp.dmax / c, T->t, T->pos, T->mom, T->sp.bhat, T->sp.region);
   }
   for (b = 0; b < T->pb->nbs; b++) {
      T->bs[b] = T->pb->bs[b];
      reset_bnd(T, &T->bs[b], T->sp.dmax, T->t, T->pos, T->mom, T->sp.bhat, T->sp.region);
   }
   for (b = 0; b < T->pb->nbm; b++) {
      T->bm[b] = T->pb->bm[b];
      reset_bnd(T, &T->bm[b], vnorm(T->mom), T->t, T->pos, T->mom, T->sp.bhat, T->sp.region);
   }
   T->amp = 0.0;
   T->wgt = 0.0;
   T->stored_t = T->t; T->stored_pos = T->pos; T->stored_mom = T->mom;
   T->time_adaptations = 0;
   /* TrajectoryParkerSource::SetStart initialises the source (src/trajectory_parker_source.cc:43-50) */
   if (T->o->traj_type == 207 && T->pb->has_src) T->src_del_old = T->mom.x[0] - T->pb->src_p_inj;
   return 0;
}

/* Integrate, src/trajectory_base.cc:946-995; returns 0 finished, 1 discarded */
static int integrate(trj_t* T)
{
   double c = c_code();
   while (!(T->status & TRAJ_FINISH) && !(T->status & TRAJ_DISCARD)) {
      int advanced = is_parker(T) ? parker_advance(T) : rk_advance(T);
      if (advanced) {  /* UpdateBmagExtrema with the fields the step ended with */
         T->bmag_min = fmin(T->bmag_min, T->sp.Bmag);
         T->bmag_max = fmax(T->bmag_max, T->sp.Bmag);
      }
      if (T->error) return 1;
      if (T->status & TRAJ_DISCARD) return 1;
      if (T->segments > MAX_TRAJ_STEPS) { T->status |= TRAJ_DISCARD; return 1; }
      /* consecutive steps an adaptive table rejected (src/trajectory_base.cc:969-979) */
      if (advanced) T->time_adaptations = 0;
      else if (++T->time_adaptations > MAX_TIME_ADAPTATIONS) { T->status |= TRAJ_DISCARD; return 1; }
      if (T->dt < SP_TINY * T->sp.dmax / c) { T->status |= TRAJ_DISCARD; return 1; }
      if (!isnormal(T->dt)) { T->status |= TRAJ_DISCARD; return 1; }
   }
   return (T->status & TRAJ_DISCARD) ? 1 : 0;
}

int spx_oracle_distro_sizes(const uint8_t* spec, size_t spec_len, int max, int64_t* n_bins, int* width)
{
   static prob_t pb;
   char err[64];
   int d;
   if (parse_spec(spec, spec_len, &pb, err, sizeof err)) return -1;
   for (d = 0; d < pb.nd && d < max; d++) {
      n_bins[d] = (int64_t)pb.d[d].n_bins[0] * pb.d[d].n_bins[1] * pb.d[d].n_bins[2];
      width[d] = pb.d[d].width;
   }
   return pb.nd;
}

int spx_oracle_run(const uint8_t* spec, size_t spec_len, const spx_oracle_opts* opts, uint32_t first, uint32_t n,
                   spx_oracle_traj* traj_out, int32_t* counts, double* sums, int64_t* n_events, char* err, size_t err_len)
{
   prob_t* pb = (prob_t*)calloc(1, sizeof(prob_t));
   trj_t* T = (trj_t*)calloc(1, sizeof(trj_t));
   int64_t off = 0;
   uint32_t k;
   int d, rc = 0;
   if (!pb || !T) { free(pb); free(T); return -10; }
   g_nudge_libm = opts->nudge_libm;
   g_rejections = 0;
   rc = parse_spec(spec, spec_len, pb, err, err_len);
   if (rc) { free(pb); free(T); return rc; }
   if (!pb->has_bg || !pb->has_it || !pb->has_is || !pb->has_im || pb->nbt == 0) {
      snprintf(err, err_len, "incomplete problem: background, three initial conditions and a time boundary are required");
      free(pb); free(T);
      return -4;
   }
   if ((opts->traj_type == 206 || opts->traj_type == 207 || (opts->traj_type >= 202 && opts->traj_type <= 204)) &&
       !pb->has_diff) {
      snprintf(err, err_len, "Parker, GuidingScatt, GuidingDiff and GuidingDiffScatt trajectories need a diffusion model");
      free(pb); free(T);
      return -4;
   }
   /* Fieldline: no momentum boundaries (BoundaryMomentum::EvaluateBoundary sets no delta for it,
    * src/boundary_momentum.cc:69-75; BoundaryMirror is not compiled for it, src/boundary_momentum.hh:225),
    * no beam or ring initials (src/initial_momentum.hh:86, 131), and no divergence-flow distribution (its
    * weight reads grad U, which the field-line mask never evaluates) */
   if (opts->traj_type == 199) {
      int bad = pb->nbm > 0 || pb->im.kind == IM_BEAM || pb->im.kind == IM_RING || pb->im.kind == IM_LOGE_PITCH;
      for (d = 0; d < pb->nd; d++) bad |= pb->d[d].kind == DS_DIVFLOW;
      if (bad) {
         snprintf(err, err_len, "a plugin class that TrajectoryFieldline does not have");
         free(pb); free(T);
         return -4;
      }
   }
   else if (pb->im.kind == IM_FIXED && opts->traj_type != 200) {
      /* InitialMomentumFixed is compiled for Lorentz and Fieldline only (src/initial_momentum.hh:21) */
      snprintf(err, err_len, "InitialMomentumFixed needs Lorentz or Fieldline trajectories");
      free(pb); free(T);
      return -4;
   }
   for (d = 0; d < pb->nd; d++) {
      /* DistributionAnisotropyLISM exists for Lorentz trajectories only (src/distribution_other.hh:245) */
      if (pb->d[d].kind == DS_ANISO_LISM && opts->traj_type != 200) {
         snprintf(err, err_len, "DistributionAnisotropyLISM needs Lorentz trajectories");
         free(pb); free(T);
         return -4;
      }
      pb->d[d].offset_bins = off;
      off += (int64_t)pb->d[d].n_bins[0] * pb->d[d].n_bins[1] * pb->d[d].n_bins[2];
   }
   {
      static rk_t tab;
      if (rk_load(opts->rk, &tab)) {
         snprintf(err, err_len, "unknown Runge-Kutta table %d", opts->rk);
         free(pb); free(T);
         return -6;
      }
      T->rk = &tab;
   }
   T->pb = pb;
   T->o = opts;
   T->counts = counts;
   T->sums = sums;
   T->n_events = n_events;
   for (k = first; k < first + n; k++) {
      uint32_t attempt = 0;
      int done = 0;
      while (!done && (int)attempt < opts->max_attempts) {
         T->traj_id = k;
         T->attempt = attempt;
         T->error = 0;
         attempt++;
         if (set_start(T)) continue;
         if (integrate(T) == 0) done = 1;
         if (T->error) { snprintf(err, err_len, "distribution action out of range"); free(pb); free(T); return -5; }
      }
      if (traj_out) {
         spx_oracle_traj* o = &traj_out[k - first];
         int i;
         o->attempts = attempt;
         o->status = T->status | (done ? 0u : 0x10000u);
         o->steps = T->segments;
         o->t = T->t;
         o->t0 = T->t0;
         for (i = 0; i < 3; i++) {
            o->pos[i] = T->pos.x[i]; o->mom[i] = T->mom.x[i];
            o->pos0[i] = T->pos0.x[i]; o->mom0[i] = T->mom0.x[i];
         }
         o->amp = T->amp;
         o->logwgt = T->wgt;
      }
   }
   free(pb);
   free(T);
   return 0;
}

uint64_t spx_oracle_rejections(void) { return g_rejections; }

#ifdef SPX_OPCOUNT
/* the op-counting build (oracle/opcount.hh): the counts since the last reset */
spx_opcount_t spx_opcount;
void spx_oracle_opcount(uint64_t out[6])
{
   out[0] = spx_opcount.add; out[1] = spx_opcount.mul; out[2] = spx_opcount.div;
   out[3] = spx_opcount.sqrt; out[4] = spx_opcount.trans; out[5] = spx_opcount.philox;
   memset(&spx_opcount, 0, sizeof spx_opcount);
}
#endif

void spx_oracle_normals(uint64_t seed, uint32_t index, uint32_t traj, uint32_t problem, uint32_t attempt, double out[4])
{
   uint32_t b[4];
   spx_rng_block(seed, index, traj, problem, SPX_RNG_STEP, attempt, b);
   spx_normals4(b, out);
}

void spx_oracle_uniforms(uint64_t seed, uint32_t index, uint32_t traj, uint32_t problem, uint32_t attempt, double out[4])
{
   uint32_t b[4];
   int i;
   spx_rng_block(seed, index, traj, problem, SPX_RNG_INIT, attempt, b);
   for (i = 0; i < 4; i++) out[i] = spx_u01(b[i]);
}

void spx_oracle_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
   spx_philox4x32_10(ctr, key, out);
}
