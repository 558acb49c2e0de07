/* GSL stand-in for running the reference sources as a test oracle (never part of the product).
 *
 * The reference draws every random number through common/random.hh:99-122, i.e. through
 * gsl_rng_uniform, gsl_ran_ugaussian and gsl_ran_rayleigh. This file implements those calls on
 * the Philox streams defined in oracle/spx_rng.h so that a reference trajectory and the CUDA
 * kernels consume identical random numbers:
 *   - the k-th normal of a trajectory is component k % nps of the SPX_RNG_STEP block with
 *     index k / nps, where nps ("normals per step", <= 4) is fixed by the harness for the
 *     trajectory type (3 for Parker: dWx, dWy, dWz in src/trajectory_parker.cc:159-180);
 *   - the k-th uniform is component k % 4 of the SPX_RNG_INIT block with index k / 4;
 *   - normals drawn while the trajectory is set up (between spx_standin_begin and
 *     spx_standin_steps) come from the SPX_RNG_INIT_NORMAL stream instead.
 * The harness selects the trajectory and attempt with spx_standin_begin() before SetStart(). */
#include <cstdio>
#include <cstdlib>
#include <cstdint>
#include "gsl/gsl_rng.h"
#include "gsl/gsl_randist.h"
#include "gsl/gsl_sf_hyperg.h"
#include "spx_rng.h"
#include "gsl_standin_ctl.h"

struct spx_gsl_rng {
   uint64_t seed;
   uint32_t traj, problem, attempt;
   uint64_t normal_idx, uniform_idx, init_normal_idx;
   int nps;
   int in_setup;
};

static spx_gsl_rng g_rng = {0, 0, 0, 0, 0, 0, 0, 3, 1};
static const gsl_rng_type g_type = {"spx-philox4x32-10"};
const gsl_rng_type* gsl_rng_default = &g_type;

gsl_rng* gsl_rng_alloc(const gsl_rng_type*) { return &g_rng; }
void gsl_rng_set(const gsl_rng*, unsigned long) {}
void gsl_rng_free(gsl_rng*) {}

double gsl_rng_uniform(const gsl_rng* r)
{
   gsl_rng* s = const_cast<gsl_rng*>(r);
   uint64_t k = s->uniform_idx++;
   uint32_t b[4];
   spx_rng_block(s->seed, (uint32_t)(k / 4), s->traj, s->problem, SPX_RNG_INIT, s->attempt, b);
   return spx_u01(b[k % 4]);
}

double gsl_ran_ugaussian(const gsl_rng* r)
{
   gsl_rng* s = const_cast<gsl_rng*>(r);
   uint32_t b[4];
   double n[4];
   if (s->in_setup) {
      uint64_t j = s->init_normal_idx++;
      spx_rng_block(s->seed, (uint32_t)(j / 4), s->traj, s->problem, SPX_RNG_INIT_NORMAL, s->attempt, b);
      spx_normals4(b, n);
      return n[j % 4];
   }
   uint64_t k = s->normal_idx++;
   spx_rng_block(s->seed, (uint32_t)(k / s->nps), s->traj, s->problem, SPX_RNG_STEP, s->attempt, b);
   spx_normals4(b, n);
   return n[k % s->nps];
}

double gsl_ran_rayleigh(const gsl_rng* r, double sigma)
{
   return sigma * sqrt(-2.0 * log(gsl_rng_uniform(r)));
}

double gsl_sf_hyperg_2F1(double, double, double, double) { return NAN; }

void spx_standin_configure(uint64_t seed, int normals_per_step)
{
   if (normals_per_step < 1 || normals_per_step > 4) {
      std::fprintf(stderr, "gsl stand-in: normals per step must be 1..4\n");
      std::exit(2);
   }
   g_rng.seed = seed;
   g_rng.nps = normals_per_step;
}

void spx_standin_begin(uint32_t traj, uint32_t problem, uint32_t attempt)
{
   g_rng.traj = traj;
   g_rng.problem = problem;
   g_rng.attempt = attempt;
   g_rng.normal_idx = 0;
   g_rng.uniform_idx = 0;
   g_rng.init_normal_idx = 0;
   g_rng.in_setup = 1;
}

void spx_standin_steps(void) { g_rng.in_setup = 0; }

uint64_t spx_standin_normals_drawn(void) { return g_rng.normal_idx; }
