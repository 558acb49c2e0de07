// spx_device.cuh -- device math for the stepping kernels: 3-vectors over a real type R,
// compensated float-float accumulators, Philox4x32-10 streams and Box-Muller normals.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace spx {

// ---- scalar math overloads ------------------------------------------------------------------
__device__ __forceinline__ double m_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float m_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double m_rsqrt(double x) { return 1.0 / sqrt(x); }
__device__ __forceinline__ float m_rsqrt(float x) { return rsqrtf(x); }
__device__ __forceinline__ double m_log(double x) { return log(x); }
__device__ __forceinline__ float m_log(float x) { return logf(x); }
__device__ __forceinline__ double m_log10(double x) { return log10(x); }
__device__ __forceinline__ float m_log10(float x) { return log10f(x); }
__device__ __forceinline__ double m_exp(double x) { return exp(x); }
__device__ __forceinline__ float m_exp(float x) { return expf(x); }
__device__ __forceinline__ double m_pow(double x, double y) { return pow(x, y); }
__device__ __forceinline__ float m_pow(float x, float y) { return powf(x, y); }
__device__ __forceinline__ double m_tanh(double x) { return tanh(x); }
__device__ __forceinline__ float m_tanh(float x) { return tanhf(x); }
__device__ __forceinline__ double m_cbrt(double x) { return cbrt(x); }
__device__ __forceinline__ float m_cbrt(float x) { return cbrtf(x); }
__device__ __forceinline__ double m_cos(double x) { return cos(x); }
__device__ __forceinline__ float m_cos(float x) { return cosf(x); }
__device__ __forceinline__ double m_sin(double x) { return sin(x); }
__device__ __forceinline__ float m_sin(float x) { return sinf(x); }
__device__ __forceinline__ double m_acos(double x) { return acos(x); }
__device__ __forceinline__ float m_acos(float x) { return acosf(x); }
__device__ __forceinline__ double m_atan2(double y, double x) { return atan2(y, x); }
__device__ __forceinline__ float m_atan2(float y, float x) { return atan2f(y, x); }
__device__ __forceinline__ double m_abs(double x) { return fabs(x); }
__device__ __forceinline__ float m_abs(float x) { return fabsf(x); }
__device__ __forceinline__ double m_min(double a, double b) { return fmin(a, b); }
__device__ __forceinline__ float m_min(float a, float b) { return fminf(a, b); }
__device__ __forceinline__ double m_max(double a, double b) { return fmax(a, b); }
__device__ __forceinline__ float m_max(float a, float b) { return fmaxf(a, b); }
__device__ __forceinline__ void m_sincospi(double x, double* s, double* c) { sincospi(x, s, c); }
__device__ __forceinline__ void m_sincospi(float x, float* s, float* c) { sincospif(x, s, c); }

template <class R> struct Lim;
template <> struct Lim<double> {
   static constexpr double large = 1.0E+20;
   static constexpr double little = 1.0E-5;
   static constexpr double small = 1.0E-8;
   static constexpr double tiny = 1.0E-15;
};
// In FP32 the reference's 1e-15 "machine precision" guard and 1e20 "large" keep their roles with
// values a float can represent.
template <> struct Lim<float> {
   static constexpr float large = 1.0E+20f;
   static constexpr float little = 1.0E-5f;
   static constexpr float small = 1.0E-8f;
   static constexpr float tiny = 1.0E-15f;
};

// ---- 3-vectors ------------------------------------------------------------------------------
template <class R>
struct V3 {
   R x, y, z;
   __device__ __forceinline__ R operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
template <class R> __device__ __forceinline__ V3<R> mk(R a, R b, R c) { return V3<R>{a, b, c}; }
template <class R> __device__ __forceinline__ V3<R> operator+(V3<R> a, V3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class R> __device__ __forceinline__ V3<R> operator-(V3<R> a, V3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class R> __device__ __forceinline__ V3<R> operator*(R s, V3<R> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class R> __device__ __forceinline__ V3<R> operator/(V3<R> a, R s) { return {a.x / s, a.y / s, a.z / s}; }
template <class R> __device__ __forceinline__ R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class R> __device__ __forceinline__ R norm2(V3<R> a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
template <class R> __device__ __forceinline__ R norm(V3<R> a) { return m_sqrt(norm2(a)); }
template <class R> __device__ __forceinline__ V3<R> cross(V3<R> a, V3<R> b)
{
   return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class R> __device__ __forceinline__ V3<R> unit(V3<R> a) { R n = norm(a); return {a.x / n, a.y / n, a.z / n}; }
template <class R> __device__ __forceinline__ V3<R> ld3(const R* p) { return {p[0], p[1], p[2]}; }

// GetSecondUnitVec (common/vectors.cc:453-468)
template <class R>
__device__ __forceinline__ V3<R> second_unit(V3<R> f)
{
   V3<R> r;
   R ax = m_abs(f.x), ay = m_abs(f.y), az = m_abs(f.z);
   int m = (ax < ay) ? ((ax < az) ? 0 : 2) : ((ay < az) ? 1 : 2);
   if (m == 0) r = {R(0), f.z, -f.y};          // f x e_x
   else if (m == 1) r = {-f.z, R(0), f.x};     // f x e_y
   else r = {f.y, -f.x, R(0)};                 // f x e_z
   return unit(r);
}
// GeoVector::ChangeToBasis / ChangeFromBasis (common/vectors.cc:58-95)
template <class R>
__device__ __forceinline__ V3<R> to_basis(V3<R> a, const V3<R> (&b)[3]) { return {dot(a, b[0]), dot(a, b[1]), dot(a, b[2])}; }
template <class R>
__device__ __forceinline__ V3<R> from_basis(V3<R> a, const V3<R> (&b)[3])
{
   return {a.x * b[0].x + a.y * b[1].x + a.z * b[2].x, a.x * b[0].y + a.y * b[1].y + a.z * b[2].y,
           a.x * b[0].z + a.y * b[1].z + a.z * b[2].z};
}

// 3x3 matrices, m[i][j] = d_i F_j for gradients (common/spatial_data.hh:30-32)
template <class R>
struct M3 {
   R m[3][3];
};
template <class R> __device__ __forceinline__ V3<R> row(const M3<R>& a, int i) { return {a.m[i][0], a.m[i][1], a.m[i][2]}; }
template <class R> __device__ __forceinline__ V3<R> mv(const M3<R>& a, V3<R> v)
{
   return {dot(row(a, 0), v), dot(row(a, 1), v), dot(row(a, 2), v)};
}
template <class R> __device__ __forceinline__ V3<R> vm(V3<R> v, const M3<R>& a)
{
   return {v.x * a.m[0][0] + v.y * a.m[1][0] + v.z * a.m[2][0], v.x * a.m[0][1] + v.y * a.m[1][1] + v.z * a.m[2][1],
           v.x * a.m[0][2] + v.y * a.m[1][2] + v.z * a.m[2][2]};
}
template <class R> __device__ __forceinline__ R trace(const M3<R>& a) { return a.m[0][0] + a.m[1][1] + a.m[2][2]; }

// ---- accumulators ---------------------------------------------------------------------------
// Time, position and momentum magnitude are accumulated in A = double for the FP64 kernel and in
// a compensated float pair for the FP32 kernel (Knuth two-sum; the pair carries ~48 bits).
struct FF {
   float hi, lo;
};

__device__ __forceinline__ void acc_set(double& a, double v) { a = v; }
__device__ __forceinline__ void acc_set(FF& a, double v) { a.hi = (float)v; a.lo = (float)(v - (double)a.hi); }
__device__ __forceinline__ void acc_setf(FF& a, float v) { a.hi = v; a.lo = 0.0f; }
__device__ __forceinline__ void acc_setf(double& a, double v) { a = v; }
__device__ __forceinline__ double acc_val(double a) { return a; }
__device__ __forceinline__ float acc_val(FF a) { return a.hi + a.lo; }
__device__ __forceinline__ double acc_dbl(double a) { return a; }
__device__ __forceinline__ double acc_dbl(FF a) { return (double)a.hi + (double)a.lo; }
__device__ __forceinline__ void acc_add(double& a, double b) { a += b; }
__device__ __forceinline__ void acc_add(FF& a, float b)
{
   float s = __fadd_rn(a.hi, b);
   float bp = __fsub_rn(s, a.hi);
   float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bp)), __fsub_rn(b, bp));
   float lo = __fadd_rn(a.lo, e);
   float hi = __fadd_rn(s, lo);
   a.lo = __fsub_rn(lo, __fsub_rn(hi, s));
   a.hi = hi;
}
// a - (m + m_lo), with the mark split into a float and its remainder
__device__ __forceinline__ double acc_diff(double a, double m, double) { return a - m; }
__device__ __forceinline__ float acc_diff(FF a, float m, float m_lo) { return __fsub_rn(a.hi, m) + (a.lo - m_lo); }

template <class R> struct AccOf;
template <> struct AccOf<double> { using type = double; };
template <> struct AccOf<float> { using type = FF; };

template <class A> struct AV3 {
   A x, y, z;
};
template <class R, class A>
__device__ __forceinline__ V3<R> val3(const AV3<A>& a) { return {(R)acc_val(a.x), (R)acc_val(a.y), (R)acc_val(a.z)}; }
template <class R, class A>
__device__ __forceinline__ void add3(AV3<A>& a, V3<R> d) { acc_add(a.x, d.x); acc_add(a.y, d.y); acc_add(a.z, d.z); }

// ---- Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) --------------------------------------
// key = {seed lo, seed hi}; counter = {index, trajectory id, problem id, purpose << 24 | attempt}
constexpr uint32_t kRngStep = 0u, kRngInit = 1u, kRngExtra = 2u, kRngInitNormal = 3u;

__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k)
{
#pragma unroll
   for (int r = 0; r < 10; r++) {
      if (r) {
         k.x += 0x9E3779B9u;
         k.y += 0xBB67AE85u;
      }
      uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
      uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
      c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
   }
   return c;
}

__device__ __forceinline__ uint4 rng_block(uint64_t seed, uint32_t index, uint32_t traj, uint32_t problem,
                                           uint32_t purpose, uint32_t attempt)
{
   return philox4x32_10(make_uint4(index, traj, problem, (purpose << 24) | (attempt & 0xffffffu)),
                        make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)));
}

// u = (x + 1/2) 2^-32 in (0,1)
__device__ __forceinline__ double u01d(uint32_t x) { return ((double)x + 0.5) * 2.3283064365386962890625e-10; }
__device__ __forceinline__ float u01f(uint32_t x) { return __fmaf_rn((float)x, 2.3283064365386962890625e-10f, 1.16415321826934814453125e-10f); }
template <class R> __device__ __forceinline__ R u01(uint32_t x);
template <> __device__ __forceinline__ double u01<double>(uint32_t x) { return u01d(x); }
template <> __device__ __forceinline__ float u01<float>(uint32_t x) { return u01f(x); }

// sin and cos of 2 pi u for u in (0,1). Double: sincospi. Float: the angle reduced to [-pi, pi]
// (2 pi (u - rint(u)), the same sine and cosine) and the special-function unit's approximations,
// absolute error below 2^-21 on that interval; sincospif is a software routine of some thirty
// instructions that the fast-math build does not replace.
__device__ __forceinline__ void sincos_2pi(double u, double* s, double* c) { sincospi(2.0 * u, s, c); }
__device__ __forceinline__ void sincos_2pi(float u, float* s, float* c)
{
   __sincosf(6.28318530717958647692f * (u - rintf(u)), s, c);
}

// Four standard normals (Box-Muller on (u0,u1) and (u2,u3)): n0 = r cos(2 pi u1), n1 = r sin(2 pi u1)
template <class R>
__device__ __forceinline__ void normals4(uint4 b, R n[4])
{
   R r0 = m_sqrt(R(-2) * m_log(u01<R>(b.x)));
   R r1 = m_sqrt(R(-2) * m_log(u01<R>(b.z)));
   R s0, c0, s1, c1;
   sincos_2pi(u01<R>(b.y), &s0, &c0);
   sincos_2pi(u01<R>(b.w), &s1, &c1);
   n[0] = r0 * c0;
   n[1] = r0 * s0;
   n[2] = r1 * c1;
   n[3] = r1 * s1;
}

}  // namespace spx
