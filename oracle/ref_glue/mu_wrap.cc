/* mu_wrap.cc -- the reference's TrajectoryGuidingScatt compiled with another pitch-angle scheme (test
 * oracle only). The reference's header fixes STOCHASTIC_METHOD_MU to 0 (Euler); this unit includes that
 * header, redefines the macro to SPX_MU (1 Milstein, 2 RK2), then includes the unmodified
 * src/trajectory_guiding_scatt.cc, whose own include of the header is then a no-op. oracle/Makefile
 * compiles it in place of that source for the guidingscatt_mu1 / _mu2 harness variants. */
#include "config.h"
#include "src/trajectory_guiding_scatt.hh"
#undef STOCHASTIC_METHOD_MU
#define STOCHASTIC_METHOD_MU SPX_MU
#include "src/trajectory_guiding_scatt.cc"
