/*
 * spx_rng.h -- CPU statement of the counter-based random streams (test infrastructure).
 *
 * This header is part of the ORACLE: it is used by the CPU restatement in oracle/spx_oracle.c
 * and by the GSL stand-in that lets the reference's own sources run with the same random
 * numbers (oracle/ref_glue). Nothing in the product library includes it; the CUDA kernels
 * carry their own implementation (spectrum_gb300/csrc/spx_device.cuh) and the tests check the two
 * against each other.
 *
 * Generator: Philox4x32-10, the published counter-based generator of Salmon, Moraes, Dror and
 * Shaw, "Parallel random numbers: as easy as 1, 2, 3" (SC'11): ten rounds of the 4x32 Philox
 * S-box with multipliers 0xD2511F53 / 0xCD9E8D57 and Weyl key increments 0x9E3779B9 /
 * 0xBB67AE85.
 *
 * Stream layout (shared with the CUDA kernels):
 *   key     = { seed & 0xffffffff, seed >> 32 }
 *   counter = { index, trajectory id, problem id, (purpose << 24) | attempt }
 *   purpose SPX_RNG_STEP : index = step number; the block's four normals feed that step
 *   purpose SPX_RNG_INIT : index = k/4 for the k-th uniform drawn by the initial samplers
 *   purpose SPX_RNG_EXTRA: index = step * 64 + k; spare normals for rejection loops
 *   purpose SPX_RNG_INIT_NORMAL: index = j/4 for the j-th normal drawn while a trajectory is set
 *                        up (before its first step)
 * The reference draws its noise through gsl_ran_ugaussian / gsl_rng_uniform
 * (common/random.hh:99-122); the stand-in in oracle/ref_glue maps those calls onto the same
 * layout so the reference and this restatement see identical random numbers.
 *
 * Uniforms: u = (x + 0.5) * 2^-32 in (0,1), never 0 or 1.
 * Normals:  Box-Muller on the pairs (u0,u1) and (u2,u3):
 *           n0 = r cos(2 pi u1), n1 = r sin(2 pi u1), r = sqrt(-2 ln u0), same for (u2,u3).
 */
#ifndef SPX_ORACLE_RNG_H
#define SPX_ORACLE_RNG_H

#include <math.h>
#include <stdint.h>

#define SPX_RNG_STEP 0u
#define SPX_RNG_INIT 1u
#define SPX_RNG_EXTRA 2u
#define SPX_RNG_INIT_NORMAL 3u

static inline void spx_philox_round(uint32_t c[4], const uint32_t k[2])
{
   uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
   uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
   uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
   uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
   uint32_t n0 = hi1 ^ c[1] ^ k[0];
   uint32_t n2 = hi0 ^ c[3] ^ k[1];
   c[0] = n0;
   c[1] = lo1;
   c[2] = n2;
   c[3] = lo0;
}

/* Philox4x32-10 of counter "ctr" under key "key"; result in out[4]. */
static inline void spx_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
   uint32_t c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
   uint32_t k[2] = {key[0], key[1]};
   int r;
   for (r = 0; r < 10; r++) {
      if (r) {
         k[0] += 0x9E3779B9u;
         k[1] += 0xBB67AE85u;
      }
      spx_philox_round(c, k);
   }
   out[0] = c[0];
   out[1] = c[1];
   out[2] = c[2];
   out[3] = c[3];
}

static inline void spx_rng_block(uint64_t seed, uint32_t index, uint32_t traj, uint32_t problem,
                                 uint32_t purpose, uint32_t attempt, uint32_t out[4])
{
   uint32_t key[2] = {(uint32_t)(seed & 0xffffffffu), (uint32_t)(seed >> 32)};
   uint32_t ctr[4] = {index, traj, problem, (purpose << 24) | (attempt & 0xffffffu)};
   spx_philox4x32_10(ctr, key, out);
}

static inline double spx_u01(uint32_t x)
{
   return ((double)x + 0.5) * 2.3283064365386962890625e-10;
}

/* Four standard normals from one block (two Box-Muller pairs). */
static inline void spx_normals4(const uint32_t b[4], double n[4])
{
   const double two_pi = 6.283185307179586476925286766559;
   double r0 = sqrt(-2.0 * log(spx_u01(b[0])));
   double r1 = sqrt(-2.0 * log(spx_u01(b[2])));
   double a0 = two_pi * spx_u01(b[1]);
   double a1 = two_pi * spx_u01(b[3]);
   n[0] = r0 * cos(a0);
   n[1] = r0 * sin(a0);
   n[2] = r1 * cos(a1);
   n[3] = r1 * sin(a1);
}

#endif
