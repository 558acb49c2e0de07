/*
 * spx.h -- C ABI of spectrum_gb300, the GB300 (sm_103a) implementation of SPECTRUM's
 * test-particle stepping path (the per-trajectory loop of the method of stochastic
 * characteristics).
 *
 * The reference exposes this path as a C++ plugin surface: a user builds DataContainer
 * parameter blobs and calls SimulationWorker::Add{Background,Diffusion,Source,Boundary,Initial,
 * Distribution}, SetTasks, MainLoop and reads the distributions back (src/simulation.hh:93-138;
 * each Add* clones a prototype and calls SetupObject, src/trajectory_base.cc:644-741). This ABI
 * carries the same information across a plain-C boundary: plugins arrive as the reference's own
 * DataContainer bytes (common/data_container.cc:139-224: per record one size byte then the
 * payload), configure-time choices (configure.ac:236-295) arrive as spx_create arguments, and the
 * MPI trajectory farm (src/simulation.cc:253-305, 743-767) is replaced by one device-resident
 * launch. Nothing here allocates on behalf of the caller's buffers; blobs are copied at call
 * time. All device work is ordered on the context's own CUDA stream.
 *
 * Reference exceptions map to return codes (below); per-trajectory failures (the reference's
 * TRAJ_DISCARD, src/trajectory_base.cc:964-992) are retried with a new random stream, as
 * src/simulation.cc:262-288 does, and counted in spx_stats instead of being returned.
 */
#ifndef SPX_H
#define SPX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- return codes ---------------------------------------------------------------------- */
#define SPX_OK 0
#define SPX_ERR_INVALID_ARG -1      /* null pointer, unknown enum value */
#define SPX_ERR_UNKNOWN_PLUGIN -2   /* kind not known for this role / trajectory type */
#define SPX_ERR_BAD_BLOB -3         /* blob shorter than the class's parameter list */
#define SPX_ERR_INCOMPLETE -4       /* TrajectoryBase::IsSimmulationReady false (src/trajectory_base.cc:608-632) */
#define SPX_ERR_CUDA -5             /* a CUDA runtime call failed */
#define SPX_ERR_OUT_OF_MEMORY -6
#define SPX_ERR_LIMIT -7            /* more than 4 boundaries per class or 4 distributions, or trajectory ids beyond 2^32 */
#define SPX_ERR_STATE -8            /* call out of order (e.g. spx_run before spx_add_problem) */
#define SPX_ERR_DEVICE -9           /* the kernel reported an error (e.g. action beyond the ActionTable) */
#define SPX_ERR_NO_DEVICE -11       /* no CUDA device, or not an sm_103 device */
#define SPX_ERR_IO -12              /* spx_dump / spx_restore file error */
#define SPX_ERR_TOO_LARGE -13       /* size beyond a fixed capacity */
#define SPX_ERR_MISMATCH -14        /* a dump file of another distribution class or parameter set */

/* ---- enumerations ---------------------------------------------------------------------- */
/* trajectory types: the numbers of configure.ac:236-244 */
#define SPX_TRAJ_FIELDLINE 199      /* field-line tracer: B only, no momentum boundaries */
#define SPX_TRAJ_LORENTZ 200
#define SPX_TRAJ_GUIDING 201        /* guiding centre, static backgrounds (uniform, dipole, solar wind, grid) */
#define SPX_TRAJ_GUIDING_SCATT 202  /* guiding centre with pitch-angle scattering (SPX_OPT_MU_METHOD); needs a diffusion model */
#define SPX_TRAJ_GUIDING_DIFF 203   /* guiding centre with perpendicular diffusion (SPX_OPT_PERP_METHOD); needs a diffusion model */
#define SPX_TRAJ_GUIDING_DIFF_SCATT 204  /* both stochastic steps; needs a diffusion model */
#define SPX_TRAJ_FOCUSED 205
#define SPX_TRAJ_PARKER 206
#define SPX_TRAJ_PARKER_SOURCE 207
/* time flow: configure.ac:263-280 */
#define SPX_FORWARD 0
#define SPX_BACKWARD 1
/* arithmetic: plain FP64 drop-in, or FP32 bulk with float-float accumulation */
#define SPX_FP64 0
#define SPX_MIXED 1
/* plugin roles */
#define SPX_ROLE_BACKGROUND 0
#define SPX_ROLE_DIFFUSION 1
#define SPX_ROLE_SOURCE 2
#define SPX_ROLE_BOUNDARY 3
#define SPX_ROLE_INITIAL 4
#define SPX_ROLE_DISTRIBUTION 5
/* options (spx_set_option) */
#define SPX_OPT_STEPS_PER_ORBIT 1   /* Lorentz orbit resolution; reference constant 100 (src/trajectory_lorentz.hh:26) */
#define SPX_OPT_DERIV_MODE 2        /* 0: the reference's compiled-in derivative methods; 1: analytic */
#define SPX_OPT_PA_SCATTERING 3     /* Focused: Euler pitch-angle scattering step (1) or none (0) */
#define SPX_OPT_RECORD_FINAL 4      /* keep the final state of every trajectory (spx_get_records) */
#define SPX_OPT_MAX_ATTEMPTS 5      /* retries of a discarded trajectory, default 100 */
#define SPX_OPT_RUN_INDEX 6         /* index of the next run: problem p's trajectory ids start at index * n_traj(p);
                                       each run advances it by one (set per rank to shard one job over GPUs) */
#define SPX_OPT_RECORD_CAPACITY 7   /* records kept per distribution with keep_records, default 65536 */
#define SPX_OPT_MU_METHOD 8         /* GuidingScatt / GuidingDiffScatt pitch-angle scheme, the reference's compile-time
                                       STOCHASTIC_METHOD_MU (src/trajectory_guiding_scatt.hh:24): 0 Euler (default),
                                       1 Milstein, 2 RK2 */
#define SPX_OPT_PERP_METHOD 9       /* GuidingDiff / GuidingDiffScatt perpendicular scheme, the reference's compile-time
                                       STOCHASTIC_METHOD_PERP (src/trajectory_guiding_diff.hh:19): 0 Euler (default),
                                       1 Milstein, 2 RK2 */
#define SPX_OPT_SPECIALIZE 10       /* 1 (default): SPX_MIXED Parker contexts whose problems share the diffusion class
                                       FullConstant or RigidityMagneticFieldPowerLaw run on kernels compiled for that
                                       class, and, where every problem has one expiry or pass time boundary, two
                                       spheres and no momentum boundary, for that layout; 2: for the class only;
                                       0: on the kernel that dispatches at run time. 1 and 2 also run SPX_MIXED
                                       TrajectoryGuiding contexts on kernels without the scattering and
                                       perpendicular steps of the other guiding-centre types. The Parker kernels
                                       give the same trajectories bit for bit; the guiding-centre one the same
                                       steps and outcomes, with positions equal to FP32 rounding (the compiler
                                       contracts some multiply-adds differently). */
#define SPX_OPT_GRID_INTERP 12      /* SERVER_INTERP_ORDER of a block-layout grid (spx_set_background_blocks):
                                       1 (default) the 8-zone stencil with its gradients, 0 the values of the zone
                                       holding the point with zero gradients, -1 the reader's interpolation over
                                       the domain with numerical gradients (SPX_FP64 contexts only) */
#define SPX_OPT_STEP_CAP 11         /* 0 (default): off. N > 0: spx_run stops every trajectory after N steps, as the
                                       autotuner's timing samples do: a steady-state throughput sample with no drain
                                       of the queue; trajectories stopped by the cap are neither finished nor binned */
/* plugin kinds: see spectrum_gb300/plugins.py; e.g. background 1 uniform, 3 smooth shock,
 * 4 dipole, 5 solar wind, 7 discontinuity, 8 smooth discontinuity; diffusion 5 full constant, 8 rigidity/field power law; boundary
 * 1 time expire, 10 plane absorb, 14 sphere absorb, 30 momentum inject; distribution 2 position
 * uniform, 5 kinetic-energy power-law spectrum. */

/* ---- types ----------------------------------------------------------------------------- */
typedef struct spx_ctx* spx_ctx_t;

typedef struct {
   int block_size;      /* threads per block; 0 = autotuned */
   int blocks_per_sm;   /* resident blocks per SM for the persistent launch; 0 = autotuned */
   int steps_per_sync;  /* steps between lane refills of the work queue; 0 = autotuned */
   int schedule;        /* 0 = one thread per trajectory (plain grid), 1 = persistent work queue */
} spx_tuning;

typedef struct {
   double kernel_ms;        /* device time of the last spx_run (CUDA events on the context stream) */
   int64_t trajectories;    /* trajectories finished in the last spx_run */
   int64_t steps;           /* accepted steps in the last spx_run */
   int64_t retries;         /* discarded attempts that were re-run with a new random stream */
   int64_t given_up;        /* trajectories discarded max_attempts times */
   int64_t events;          /* distribution events recorded */
   int kernel_launches;     /* kernels launched by the last spx_run */
   spx_tuning tuning;       /* the launch shape used */
} spx_stats;

typedef struct {
   uint32_t attempts, status;   /* status: reference TRAJ_* bits (src/trajectory_base.hh:45-57) */
   uint64_t steps;
   double t, pos[3], mom[3];
   double t0, pos0[3], mom0[3];
   double amp, logwgt;
} spx_traj_record;

/* ---- calls ----------------------------------------------------------------------------- */
/* Create a context on the current CUDA device. Replaces CreateSimulation
 * (src/simulation.cc:899-907) plus the configure-time choice of TRAJ_TYPE, TRAJ_TIME_FLOW and
 * RK_INTEGRATOR_TYPE (configure.ac:236-295). rk_method is any Butcher table of
 * common/rk_config.hh:72-520 but 30 (which does not compile in the reference), with the
 * reference's adaptive step control and step rejection for the adaptive ones
 * (src/trajectory_base.cc:366-406); the Parker types apply it to their drift and add the
 * Euler-Maruyama displacement after the step (src/trajectory_parker.cc:255-306). Euler (0), and the
 * classic RK4 (25) for the Runge-Kutta types, run in both arithmetics; the other tables in SPX_FP64
 * only (SPX_MIXED gives SPX_ERR_INVALID_ARG: FP32 cannot meet the tables' 1e-9 error tolerance).
 * The arguments are checked before the device is looked for. */
int spx_create(spx_ctx_t* ctx, int traj_kind, int time_flow, int rk_method, int precision);

/* Set an SPX_OPT_* option (no reference counterpart: these are the reference's compile-time
 * constants made run-time). */
int spx_set_option(spx_ctx_t ctx, int option, double value);

/* Add one plugin; replaces SimulationWorker::Add{Background,Diffusion,Source,Boundary,Initial,
 * Distribution} (src/simulation.hh:105-123, src/trajectory_base.cc:644-741). blob/blob_len/
 * n_records are exactly DataContainer::data()/length()/size(). */
int spx_add_plugin(spx_ctx_t ctx, int role, int kind, const uint8_t* blob, size_t blob_len, size_t n_records);

/* Add a problem of n_traj trajectories (0 allowed: an empty member of a batch) built from the plugins added so far, with optional
 * per-problem replacements: override_blob is a sequence of records
 * { u32 role, u32 slot, u32 kind, u32 n_records, u32 blob_len, u8 blob[blob_len] } replacing the
 * slot-th plugin of that role. Replaces SetTasks(n_traj, batch_size) (src/simulation.cc:509); many
 * problems (energies, mean free paths) run in one launch. */
int spx_add_problem(spx_ctx_t ctx, int64_t n_traj, uint64_t seed, const uint8_t* override_blob, size_t override_len);

/* The data of a gridded background (kind 6, BackgroundServerCartesian with first-order
 * interpolation, src/server_cartesian.cc:206-840): one uniform block of n[0] x n[1] x n[2] nodes,
 * node (i, j, k) at cent_min + (i, j, k) * zone_length, six doubles per node (U, then B, in code
 * units), x fastest. Replaces the data files the reference's server reads (the fname_pattern of
 * AddBackground, src/simulation.hh:111) and its MPI block server: the block is copied to device
 * memory now (this call allocates), shared by all problems of the context. Points whose 8-node
 * stencil leaves the block are field errors (the trajectory is discarded and retried). */
int spx_set_background_grid(spx_ctx_t ctx, const int64_t n[3], const double cent_min[3], const double zone_length[3],
                            const double* values);

/* The data of a gridded background (kind 6) as the reference's Cartesian server holds it: the
 * layout of its reader's data file (src/reader_cartesian.cc:28-166), n_blocks[0] x n_blocks[1] x
 * n_blocks[2] blocks of 4 x 4 x 4 zones spanning [domain_min, domain_max] (the .info header, in
 * au), blocks x fastest and in each block zones x fastest, six doubles per zone (U, then B, in the
 * reference's fluid units). Each point is interpolated in its own block with that block's
 * zone-centre origin and zone length, as the front end does (src/server_cartesian.cc:274-330,
 * 549-865), with ghost_cells (0 or 1) ghost layers per block side (SERVER_NUM_GHOST_CELLS); the
 * values of zones past a block's faces are its neighbours'. Fields are converted to code units
 * after the sums with the ratios spx_grid_units gives. Copies to device memory now (this call
 * allocates); replaces a grid set by spx_set_background_grid. Replaces the server's data file and
 * MPI block service. */
int spx_set_background_blocks(spx_ctx_t ctx, const int32_t n_blocks[3], const double domain_min[3],
                              const double domain_max[3], int ghost_cells, const double* values);

/* The unit conversion of the reference's data server (src/server_cartesian.cc:710-716): out[0..3] =
 * Fluid/Particle ratios of length, velocity and magnetic field, and Fluid::c_code
 * (common/physics.hh:18-55, common/specie.hh:25-64). Needs no device. */
void spx_grid_units(double out[4]);

/* Integrate every trajectory of every problem; replaces MainLoop (src/simulation.cc:818-835).
 * Enqueues on the context stream and returns; tuning may be NULL (autotuned). Each call draws
 * fresh trajectory ids, so repeated calls add new trajectories to the distributions. */
int spx_run(spx_ctx_t ctx, const spx_tuning* tuning);

/* Wait for the last spx_run and report its statistics (stats may be NULL). */
int spx_sync(spx_ctx_t ctx, spx_stats* stats);

/* Choose the launch shape (block size, refill interval, schedule) by timing candidates on a sample
 * of the context's problems: about sample_traj trajectories (0: two per resident lane), each
 * stopped after 2048 steps, on separate buffers and random streams. spx_run with a NULL tuning
 * then uses the fastest; best (may be NULL) receives it. No reference counterpart: the
 * reference's MPI farm has no launch shape to tune. */
int spx_autotune(spx_ctx_t ctx, int64_t sample_traj, spx_tuning* best);

/* Size of the fixed device array spx_run_static works in (every GPU that loads the library holds
 * it until the process exits): 41 problems in SPX_MIXED, 64 in SPX_FP64. */
#define SPX_STATIC_SCRATCH_BYTES (512u * 1024u)

/* spx_run without any device allocation. No counterpart in the reference: it is for callers that
 * cannot call cudaMalloc -- code running inside a host framework that owns all device memory
 * through its own pool, or on a latency-critical path where cudaMalloc's implicit device
 * synchronisation is not acceptable. The caller passes device buffers for the outputs, laid out
 * as one array over all (problem, distribution) pairs in order, each as spx_get_distribution_info
 * sizes it: int32 counts[n_counts], double sums[n_sums], and n_events[problem * 4 + distribution]
 * (n_events_len >= 4 * problems); the kernel adds into them, so the caller zeroes them first.
 * With SPX_OPT_RECORD_FINAL set, records[n_records] (device memory, one per trajectory over all
 * problems in order) receives the final states. The run counters and the device copies of the
 * problem descriptors live in a fixed array of SPX_STATIC_SCRATCH_BYTES; a context whose
 * descriptors do not fit is rejected with SPX_ERR_TOO_LARGE. The call allocates no device memory
 * (no cudaMalloc, cudaFree or allocating library routine); it blocks until the launch is done
 * and fills stats (may be NULL). The launch shape is chosen as spx_run chooses it (tuning, else the
 * spx_autotune result, else the defaults). The first call on a device looks up the array's address
 * there (and may load the library's device code), so make it before any stream capture; the
 * address is kept for the life of the process, so resetting the device (cudaDeviceReset) while the
 * library is loaded is not supported. All calls share
 * the array and it keeps the last call's contents (each call clears the counters it needs):
 * calls whose launches overlap on the GPU race and give wrong results. Trajectory ids continue
 * from spx_run's, so a sequence of spx_run_static calls draws the same trajectories as the same
 * sequence of spx_run calls; spx_sync reports spx_run launches only. Distribution records
 * (keep_records) are not kept by this call: it has no buffer for them. */
int spx_run_static(spx_ctx_t ctx, const spx_tuning* tuning, int32_t* counts, int64_t n_counts, double* sums,
                   int64_t n_sums, unsigned long long* n_events, int64_t n_events_len, spx_traj_record* records,
                   int64_t n_records, spx_stats* stats);

/* Shape of a distribution: number of bins and doubles per bin (1, 3 or 9). */
int spx_get_distribution_info(spx_ctx_t ctx, int problem, int distro, int64_t* n_bins, int* width);

/* Copy one distribution to host memory: int32 counts[n_bins], double sums[n_bins*width] and the
 * event count; any pointer may be NULL. Layout of DistributionTemplated (counts, distro,
 * n_events; src/distribution_templated.cc:145-181), bins linearised by MultiIndex::LinIdx
 * (common/multi_index.hh:138-141). */
int spx_get_distribution(spx_ctx_t ctx, int problem, int distro, int32_t* counts, double* sums, int64_t* n_events);

/* Final states of the trajectories of one problem (SPX_OPT_RECORD_FINAL must be set). Returns the
 * number written (<= max_records) or an error code. */
int64_t spx_get_records(spx_ctx_t ctx, int problem, spx_traj_record* out, int64_t max_records);

/* The records of a distribution whose container set keep_records (DistributionTemplated::AddRecord,
 * src/distribution_templated.cc:188-192; the values_record / weights_record arrays): the value
 * (3 doubles) and the weight (width doubles, spx_get_distribution_info) of every processed event,
 * outliers included, in the order the device appended them. At most SPX_OPT_RECORD_CAPACITY are
 * stored; *n_events receives the number recorded. Returns the number written (<= max_records), or
 * SPX_ERR_STATE when the distribution keeps no records. */
int64_t spx_get_distribution_records(spx_ctx_t ctx, int problem, int distro, double* values, double* weights,
                                     int64_t max_records, int64_t* n_events);

/* Clear all distributions (DistributionTemplated::ResetDistribution). */
int spx_reset_distributions(spx_ctx_t ctx);

/* Write / read all distributions and the run index (this library's whole-run checkpoint, the role of
 * src/simulation.cc:592-594, 714-720); distribution records are not part of it (spx_dump_distribution
 * writes them). */
int spx_dump(spx_ctx_t ctx, const char* path);
int spx_restore(spx_ctx_t ctx, const char* path);

/* One distribution in the reference's own dump-file layout, so that files pass both ways between
 * this library and the reference's post-processing and restart:
 * spx_dump_distribution replaces DistributionTemplated::Dump (src/distribution_templated.cc:394-425),
 * which the reference calls as distro_file_name + index + ".out" (src/simulation.cc:590-594, 790-793);
 * spx_restore_distribution replaces DistributionTemplated::Restore (src/distribution_templated.cc:433-466),
 * called for the distributions flagged by SimulationMaster::RestoreDistro (src/simulation.cc:714-720).
 * The file's class name and parameter container must equal the distribution's: SPX_ERR_MISMATCH
 * otherwise (the reference returns without restoring), SPX_ERR_IO for a missing or short file.
 * Distribution records (keep_records) are not kept on the device: dumps carry empty record arrays
 * and a restore reads past any. */
int spx_dump_distribution(spx_ctx_t ctx, int problem, int distro, const char* path);
int spx_restore_distribution(spx_ctx_t ctx, int problem, int distro, const char* path);

const char* spx_strerror(int code);
void spx_destroy(spx_ctx_t ctx);

/* Library version string. */
const char* spx_version(void);

#ifdef __cplusplus
}
#endif
#endif
