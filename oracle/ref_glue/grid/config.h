/* Hand-written stand-in for the reference's autotools config.h (test oracle only), for the grid
 * harness: a parallel build with the Cartesian data server at first-order interpolation, the way
 * configure.ac:301-350 fixes SERVER_TYPE, SERVER_INTERP_ORDER and SERVER_NUM_GHOST_CELLS. The ghost
 * cell count and the interpolation order come from oracle/Makefile (-DSPX_GRID_GHOST, -DSPX_GRID_ORDER). */
#ifndef SPX_REF_GRID_CONFIG_H
#define SPX_REF_GRID_CONFIG_H

#define USE_GSL 1
#define USE_MPI 1
#define EXEC_SERIAL 0
#define EXEC_PARALLEL 1
#define EXEC_TYPE EXEC_PARALLEL

#define SERVER_SELF 299
#define SERVER_CARTESIAN 300
#define SERVER_BATL 301
#define SERVER_TYPE SERVER_CARTESIAN
#ifndef SPX_GRID_ORDER
#define SPX_GRID_ORDER 1
#endif
#define SERVER_INTERP_ORDER SPX_GRID_ORDER

#ifndef SPX_GRID_GHOST
#error "SPX_GRID_GHOST must give the ghost cells per block side (0 or 1)"
#endif
#define SERVER_NUM_GHOST_CELLS SPX_GRID_GHOST

#endif
