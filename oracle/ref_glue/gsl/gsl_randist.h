/* Stand-in for <gsl/gsl_randist.h> (test oracle only); see gsl_standin.cc. */
#ifndef SPX_GSL_RANDIST_STANDIN_H
#define SPX_GSL_RANDIST_STANDIN_H
#include "gsl_rng.h"
#ifdef __cplusplus
extern "C" {
#endif
double gsl_ran_ugaussian(const gsl_rng* r);
double gsl_ran_rayleigh(const gsl_rng* r, double sigma);
#ifdef __cplusplus
}
#endif
#endif
