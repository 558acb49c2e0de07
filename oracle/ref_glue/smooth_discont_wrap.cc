/* smooth_discont_wrap.cc -- the reference's BackgroundSmoothDiscontinuity (test oracle only). Its
 * EvaluateBackground and EvaluateBackgroundDerivatives name c_code without a namespace
 * (src/background_smooth_discontinuity.cc:131, 154, 163), so the unit does not compile as shipped. The
 * class's electric field is the particle-frame -(U x B) / c of the smooth shock it mirrors
 * (src/background_smooth_shock.cc:150), so this unit makes Particle::c_code visible in namespace Spectrum
 * and then includes the unmodified source. oracle/Makefile compiles it in place of that source. */
#include "config.h"
#include "src/background_smooth_discontinuity.hh"
namespace Spectrum {
using Particle::c_code;
}
#include "src/background_smooth_discontinuity.cc"
