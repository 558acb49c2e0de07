/*
 * spx_oracle.h -- CPU restatement of SPECTRUM's test-particle stepping path (TEST ORACLE).
 *
 * This is test infrastructure, not product: only tests/, __graft_entry__.smoke() and the CPU
 * baseline leg of bench.py may load it. It restates, in plain C, the per-trajectory algorithm of
 * the reference (src/trajectory_base.cc, src/trajectory_parker.cc, src/trajectory_lorentz.cc,
 * src/trajectory_focused.cc and the plugins they call), driven by the same plugin blobs and the
 * same Philox random streams (oracle/spx_rng.h) as the CUDA library, so the CUDA results can be
 * compared with it trajectory by trajectory. Its own parity with the reference is pinned by
 * running the reference's sources through oracle/ref_glue (see tests/test_oracle_vs_reference.py).
 */
#ifndef SPX_ORACLE_H
#define SPX_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Final state of one trajectory; same fields as the reference harness output. */
typedef struct {
   uint32_t attempts;
   uint32_t status;      /* reference TRAJ_* bits (src/trajectory_base.hh:45-57); 0x10000 = gave up */
   uint64_t steps;
   double t, pos[3], mom[3];
   double t0, pos0[3], mom0[3];
   double amp, logwgt;
} spx_oracle_traj;

typedef struct {
   int traj_type;          /* 200 Lorentz, 201-204 guiding centre, 205 Focused, 206 Parker, 207 Parker+source */
   int time_flow;          /* 0 forward, 1 backward */
   int rk;                 /* Butcher table number of common/rk_config.hh (any but 30) */
   int deriv_mode;         /* 0: the reference's compiled-in defaults; 1: analytic derivatives */
   double steps_per_orbit; /* Lorentz orbit resolution (reference: 100, src/trajectory_lorentz.hh:26) */
   int pa_scattering;      /* Focused: add the Euler pitch-angle scattering step */
   int max_attempts;       /* retries of a discarded trajectory (src/simulation.cc:262-288) */
   int reference_quirks;   /* 1: reproduce deviations D1 (the smooth shock's dmax from the previous field
                              evaluation) and D6 (after a rejected adaptive step, the fields of that step's
                              last stage point) as the reference has them, to compare with the reference's
                              own output; 0: the corrected behaviour the CUDA kernels share */
   int mu_method;          /* guiding-centre pitch-angle step: 0 Euler, 1 Milstein, 2 RK2 (STOCHASTIC_METHOD_MU) */
   int perp_method;        /* guiding-centre perpendicular step: 0 Euler, 1 Milstein, 2 RK2 (STOCHASTIC_METHOD_PERP) */
   int nudge_libm;         /* 1: every normal deviate and every result of exp, log, pow, sin, cos, tanh and
                              the inverse trigonometric functions one ulp larger in magnitude: a model of
                              the last-bit differences between two libm implementations; the parity tests
                              measure a problem's conditioning with it */
} spx_oracle_opts;

/*
 * Run trajectories [first, first + n) of the problem in "spec" (format of
 * oracle/ref_glue/harness.cc). traj_out may be NULL. counts/sums/n_events receive the
 * distributions back to back in plugin order (sums has width 1, 3 or 9 doubles per bin);
 * they are accumulated into, not cleared. Returns 0 or a negative error code; err gets a message.
 */
int spx_oracle_run(const uint8_t* spec, size_t spec_len, const spx_oracle_opts* opts, uint32_t first,
                   uint32_t n, spx_oracle_traj* traj_out, int32_t* counts, double* sums, int64_t* n_events,
                   char* err, size_t err_len);

/* Steps an adaptive Butcher table rejected during the last spx_oracle_run. */
uint64_t spx_oracle_rejections(void);

/* The op-counting build only (make -C oracle opcount): additions, multiplications, divisions, square
 * roots, transcendental calls and Philox blocks since the previous call, which resets them. */
void spx_oracle_opcount(uint64_t out[6]);

/* Sizes of the distributions of a spec: returns the number of distributions, fills up to
 * "max" entries of n_bins[] and width[]. Negative on a malformed spec. */
int spx_oracle_distro_sizes(const uint8_t* spec, size_t spec_len, int max, int64_t* n_bins, int* width);

/* The four normals of one step block and four uniforms of one init block, for RNG cross-checks. */
void spx_oracle_normals(uint64_t seed, uint32_t index, uint32_t traj, uint32_t problem, uint32_t attempt,
                        double out[4]);
void spx_oracle_uniforms(uint64_t seed, uint32_t index, uint32_t traj, uint32_t problem, uint32_t attempt,
                         double out[4]);
/* The block of a gridded background (BackgroundServerCartesian): n[0] x n[1] x n[2] nodes at
 * cent_min + (i, j, k) * zone_length, six values per node (U, B), x fastest. One grid at a time. */
void spx_oracle_set_grid(const int64_t n[3], const double cent_min[3], const double zone_length[3],
                         const double* values);

/* The gridded background in the layout of the reference's Cartesian reader (block mode): nb[0] x
 * nb[1] x nb[2] blocks of 4^3 zones over [dmin, dmax] in file units (au), blocks x fastest and in
 * each block zones x fastest, six fluid-unit values per zone (U, B); "ghost" ghost cells per block
 * side; units = {Fluid/Particle length ratio, velocity ratio, magnetic ratio, Fluid::c_code}. */
void spx_oracle_set_grid_blocks(const int nb[3], const double dmin[3], const double dmax[3], int ghost,
                                const double* values, const double units[4]);
/* The fields of the gridded background (either mode) at one point: U[3] B[3] Bmag E[3] dmax gradU[9]
 * gradB[9] gradBmag[3]. Nonzero on a field error. */
int spx_oracle_grid_fields(const double pos[3], double dmax0, double out[32]);
/* SERVER_INTERP_ORDER of the block mode: 1 (default), 0 or -1. */
void spx_oracle_set_grid_order(int order);
/* The Fluid/Particle length, velocity and magnetic ratios and Fluid::c_code of the reference. */
void spx_oracle_grid_units(double out[4]);
/* The primary block and stencil of "pos" in block mode (block indices, zone-centre origin, zone
 * length, zone, offset, the eight weights and 24 derivative weights). Nonzero outside the domain. */
int spx_oracle_grid_stencil(const double pos[3], int node[3], double cent_min[3], double zone_length[3], int zone[3],
                            double offset[3], double w[8], double der[24]);

/* Philox4x32-10 of one counter under one key (for the generator's known-answer tests). */
void spx_oracle_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

#ifdef __cplusplus
}
#endif
#endif
