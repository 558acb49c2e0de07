/* Stand-in for <gsl/gsl_rng.h> used only to compile the reference sources as a test oracle.
 * It provides the four calls common/random.hh makes (alloc, set, free, uniform) on top of the
 * Philox streams of oracle/spx_rng.h; see gsl_standin.cc. */
#ifndef SPX_GSL_RNG_STANDIN_H
#define SPX_GSL_RNG_STANDIN_H
#ifdef __cplusplus
extern "C" {
#endif
typedef struct spx_gsl_rng_type { const char* name; } gsl_rng_type;
typedef struct spx_gsl_rng gsl_rng;
extern const gsl_rng_type* gsl_rng_default;
gsl_rng* gsl_rng_alloc(const gsl_rng_type* type);
void gsl_rng_set(const gsl_rng* r, unsigned long seed);
void gsl_rng_free(gsl_rng* r);
double gsl_rng_uniform(const gsl_rng* r);
#ifdef __cplusplus
}
#endif
#endif
