/* Stand-in for <gsl/gsl_const_cgsm.h> (test oracle only). The values are the ones the
 * reference itself uses when it is built without GSL (common/physical_constants.hh:20-81), so a
 * build with this stand-in has the same unit system as a GSL-less build. */
#ifndef SPX_GSL_CONST_CGSM_STANDIN_H
#define SPX_GSL_CONST_CGSM_STANDIN_H
#define GSL_CONST_CGSM_SPEED_OF_LIGHT (2.99792458e+10)
#define GSL_CONST_CGSM_MASS_ELECTRON (9.1093837139E-28)
#define GSL_CONST_CGSM_MASS_MUON (1.883531627E-25)
#define GSL_CONST_CGSM_MASS_PROTON (1.67262192596E-24)
#define GSL_CONST_CGSM_MASS_NEUTRON (1.67492750057E-24)
#define GSL_CONST_CGSM_ELECTRON_VOLT (1.602176634E-12)
#define GSL_CONST_CGSM_BOLTZMANN (1.380649E-16)
#define GSL_CONST_CGSM_ASTRONOMICAL_UNIT (1.495978707E+13)
#endif
