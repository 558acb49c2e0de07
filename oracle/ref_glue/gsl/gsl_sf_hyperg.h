/* Stand-in for <gsl/gsl_sf_hyperg.h> (test oracle only). Only the WNLT diffusion models call it;
 * they are outside the ported path, so the stand-in returns NaN to make any accidental use loud. */
#ifndef SPX_GSL_SF_HYPERG_STANDIN_H
#define SPX_GSL_SF_HYPERG_STANDIN_H
#ifdef __cplusplus
extern "C" {
#endif
double gsl_sf_hyperg_2F1(double a, double b, double c, double x);
#ifdef __cplusplus
}
#endif
#endif
