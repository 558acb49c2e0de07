/* opcount.hh -- an operation-counting build of the oracle (test infrastructure only).
 *
 * Force-included before oracle/spx_oracle.c compiled as C++ (make -C oracle opcount): every double
 * of the restatement becomes an spx_cd, a double that counts the arithmetic done on it, so a run of
 * the oracle reports how many operations an accepted step of a workload takes in the minimal
 * formulation the restatement follows. Additions and subtractions, multiplications, divisions,
 * square roots and the transcendental functions are counted separately (a fused multiply-add is
 * its multiplication and its addition); negation, comparisons, fabs, fmin and fmax are not
 * floating-point work and are not counted. The random streams (oracle/spx_rng.h) are compiled
 * before the substitution, with plain doubles: their Philox blocks are counted per call instead. */
#ifndef SPX_OPCOUNT_HH
#define SPX_OPCOUNT_HH

#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <cmath>
#include <cstddef>

#include "spx_rng.h"

extern "C" {
/* counts since the last spx_opcount_reset: add, mul, div, sqrt, transcendental, Philox blocks */
typedef struct { uint64_t add, mul, div, sqrt, trans, philox; } spx_opcount_t;
extern spx_opcount_t spx_opcount;
}

struct spx_cd {
   double v;
   spx_cd() = default;
   constexpr spx_cd(double x) : v(x) {}
   explicit operator double() const { return v; }
   explicit operator int() const { return (int)v; }
   explicit operator long() const { return (long)v; }
   explicit operator unsigned() const { return (unsigned)v; }
   explicit operator unsigned long() const { return (unsigned long)v; }
   explicit operator long long() const { return (long long)v; }
   explicit operator unsigned long long() const { return (unsigned long long)v; }
   explicit operator bool() const { return v != 0.0; }
   spx_cd operator-() const { return spx_cd(-v); }
   spx_cd& operator+=(spx_cd o) { spx_opcount.add++; v += o.v; return *this; }
   spx_cd& operator-=(spx_cd o) { spx_opcount.add++; v -= o.v; return *this; }
   spx_cd& operator*=(spx_cd o) { spx_opcount.mul++; v *= o.v; return *this; }
   spx_cd& operator/=(spx_cd o) { spx_opcount.div++; v /= o.v; return *this; }
   spx_cd& operator++() { spx_opcount.add++; v += 1.0; return *this; }
};
static_assert(sizeof(spx_cd) == sizeof(double), "spx_cd must have the layout of a double");

inline spx_cd operator+(spx_cd a, spx_cd b) { spx_opcount.add++; return spx_cd(a.v + b.v); }
inline spx_cd operator-(spx_cd a, spx_cd b) { spx_opcount.add++; return spx_cd(a.v - b.v); }
inline spx_cd operator*(spx_cd a, spx_cd b) { spx_opcount.mul++; return spx_cd(a.v * b.v); }
inline spx_cd operator/(spx_cd a, spx_cd b) { spx_opcount.div++; return spx_cd(a.v / b.v); }
inline bool operator<(spx_cd a, spx_cd b) { return a.v < b.v; }
inline bool operator<=(spx_cd a, spx_cd b) { return a.v <= b.v; }
inline bool operator>(spx_cd a, spx_cd b) { return a.v > b.v; }
inline bool operator>=(spx_cd a, spx_cd b) { return a.v >= b.v; }
inline bool operator==(spx_cd a, spx_cd b) { return a.v == b.v; }
inline bool operator!=(spx_cd a, spx_cd b) { return a.v != b.v; }
inline bool operator!(spx_cd a) { return a.v == 0.0; }

inline spx_cd sqrt(spx_cd a) { spx_opcount.sqrt++; return spx_cd(std::sqrt(a.v)); }
#define SPX_TRANS1(f) inline spx_cd f(spx_cd a) { spx_opcount.trans++; return spx_cd(std::f(a.v)); }
SPX_TRANS1(exp) SPX_TRANS1(log) SPX_TRANS1(log10) SPX_TRANS1(sin) SPX_TRANS1(cos) SPX_TRANS1(tan)
SPX_TRANS1(tanh) SPX_TRANS1(acos) SPX_TRANS1(asin) SPX_TRANS1(atan) SPX_TRANS1(cbrt)
#undef SPX_TRANS1
inline spx_cd pow(spx_cd a, spx_cd b) { spx_opcount.trans++; return spx_cd(std::pow(a.v, b.v)); }
inline spx_cd atan2(spx_cd a, spx_cd b) { spx_opcount.trans++; return spx_cd(std::atan2(a.v, b.v)); }
inline spx_cd fabs(spx_cd a) { return spx_cd(std::fabs(a.v)); }
inline spx_cd fmin(spx_cd a, spx_cd b) { return spx_cd(std::fmin(a.v, b.v)); }
inline spx_cd fmax(spx_cd a, spx_cd b) { return spx_cd(std::fmax(a.v, b.v)); }
inline spx_cd floor(spx_cd a) { return spx_cd(std::floor(a.v)); }
inline spx_cd nextafter(spx_cd a, spx_cd b) { return spx_cd(std::nextafter(a.v, b.v)); }
inline bool isnormal(spx_cd a) { return std::isnormal(a.v); }
inline bool isfinite(spx_cd a) { return std::isfinite(a.v); }
inline bool isnan(spx_cd a) { return std::isnan(a.v); }

/* the random streams' work: one Philox4x32-10 block per call */
inline void spx_normals4(const uint32_t b[4], spx_cd n[4]) { spx_normals4(b, reinterpret_cast<double*>(n)); }
inline void spx_rng_block_counted(uint64_t seed, uint32_t index, uint32_t traj, uint32_t problem, uint32_t purpose,
                                  uint32_t attempt, uint32_t out[4])
{
   spx_opcount.philox++;
   spx_rng_block(seed, index, traj, problem, purpose, attempt, out);
}
#define spx_rng_block spx_rng_block_counted

#define double spx_cd

#endif
