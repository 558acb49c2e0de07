/* Control calls of the GSL stand-in (test oracle only). */
#ifndef SPX_GSL_STANDIN_CTL_H
#define SPX_GSL_STANDIN_CTL_H
#include <cstdint>
void spx_standin_configure(uint64_t seed, int normals_per_step);
void spx_standin_begin(uint32_t traj, uint32_t problem, uint32_t attempt);
uint64_t spx_standin_normals_drawn(void);
void spx_standin_steps(void);
#endif
