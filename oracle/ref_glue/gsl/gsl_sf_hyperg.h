/* Stand-in for <gsl/gsl_sf_hyperg.h> (test oracle only). Only the WNLT diffusion models name it, in a branch
 * that USE_QLT_SCATT_WITH_WNLT_DIFF (src/diffusion_other.hh:137) makes unreachable, so the stand-in returns
 * NaN to make any use loud. */
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
