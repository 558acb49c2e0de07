/* perp_wrap.cc -- the reference's guiding-centre perpendicular-diffusion types compiled with another
 * perpendicular scheme (test oracle only). The reference's header fixes STOCHASTIC_METHOD_PERP to 0 (Euler);
 * this unit includes that header, redefines the macro to SPX_PERP (1 Milstein, 2 RK2), then includes the
 * unmodified source named by SPX_PERP_UNIT (1 src/trajectory_guiding_diff.cc, 2 src/trajectory_guiding_diff_scatt.cc),
 * whose own include of the header is then a no-op. oracle/Makefile compiles it in place of those sources for the
 * *_perp1 / *_perp2 harness variants. */
#include "config.h"
#include "src/trajectory_guiding_diff.hh"
#undef STOCHASTIC_METHOD_PERP
#define STOCHASTIC_METHOD_PERP SPX_PERP
#if SPX_PERP_UNIT == 1
#include "src/trajectory_guiding_diff.cc"
#else
#include "src/trajectory_guiding_diff_scatt.cc"
#endif
