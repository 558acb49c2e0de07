// spx_capi.cu -- the C ABI of include/spx.h: contexts, plugin and problem set-up, launches on the
// context's stream, statistics, distribution read-back and checkpoints.
//
// A context owns one CUDA stream and its device buffers: the problem descriptors in FP64 and FP32,
// the run counters (the work-queue head among them), the distribution counts and sums, the event
// counters and, when asked for, the per-trajectory final records. Problems are snapshots of the
// plugins added before them plus per-problem replacements; all problems of a context share one
// trajectory type, time flow, Runge-Kutta table and background class (these select the kernel).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/spx.h"
#include "spx_launch.hh"
#include "spx_parse.hh"
#include "spx_rk_tables.h"

static_assert(sizeof(spx_traj_record) == sizeof(spx::TrajRecord), "record layouts differ");

namespace {

struct PluginBlob {
   int role, kind;
   uint32_t n_records;
   std::vector<uint8_t> blob;
};

struct ProblemHost {
   spx::ProblemDesc pd;
   int64_t n_traj;
   // the parameter blob of each distribution slot: the container a reference dump file carries
   PluginBlob dist[spx::kMaxDistro];
};

}  // namespace

struct spx_ctx {
   int device = 0;
   cudaStream_t stream = nullptr;
   cudaEvent_t ev0 = nullptr, ev1 = nullptr;
   int traj = 0, flow = 0, rk = 0, precision = 0;
   // the Butcher table: general (not Euler or, for the RK types, the classic RK4) tables run on the
   // *_f64rk / *_f64fdrk kernels, which read it from constant memory
   bool general_rk = false;
   // SPX_OPT_SPECIALIZE: 1 the FP32 Parker kernels compiled for the problems' diffusion class and, where
   // it matches, their boundary layout; 2 for the diffusion class only; 0 the kernels that dispatch at
   // run time (all give the same trajectories)
   int specialize = 1;
   uint32_t step_cap = 0;  // SPX_OPT_STEP_CAP
   int rk_stages = 1, rk_order = 1, rk_adaptive = 0, rk_offset = 0;
   double steps_per_orbit = 100.0;
   int deriv_mode = 0, pa_scattering = 0, record_final = 0, max_attempts = 100, mu_method = 0, perp_method = 0;
   std::vector<PluginBlob> base;
   std::vector<ProblemHost> problems;
   int bg_kind = 0;
   bool dirty = true;
   int64_t run_index = 0;
   int64_t total_traj = 0;
   int64_t n_counts = 0, n_sums = 0;
   // device buffers
   spx::ProblemDesc* d_pd = nullptr;
   void* d_pr = nullptr;
   spx::RunCounters* d_ctr = nullptr;
   int32_t* d_counts = nullptr;
   double* d_sums = nullptr;
   unsigned long long* d_nev = nullptr;
   spx::TrajRecord* d_rec = nullptr;
   int64_t rec_cap = 0;
   bool launched = false;
   spx_stats last{};
   int sm_count = 0;
   // spx_run replays one captured graph (counter reset, timing events, the step kernel); only the
   // kernel's arguments change between runs (the run index), so they are updated in place
   cudaGraph_t graph = nullptr;
   cudaGraphExec_t gexec = nullptr;
   cudaGraphNode_t gkernel = nullptr;
   cudaKernelNodeParams gparams{};
   unsigned char gkey[192] = {};
   // launch shape chosen by spx_autotune (used by spx_run when it gets no tuning)
   bool has_tuned = false;
   spx_tuning tuned{};
   // the gridded background (spx_set_background_grid): geometry and the node values on the device
   bool has_grid = false;
   int grid_n[3] = {0, 0, 0};
   double grid_cent[3] = {0, 0, 0}, grid_zone[3] = {0, 0, 0};
   // block mode (spx_set_background_blocks): blocks per axis (0: one uniform block), ghost layers,
   // domain in file units and block length
   int grid_nb[3] = {0, 0, 0}, grid_ghost = 0, grid_order = 1;
   double grid_dmin[3] = {0, 0, 0}, grid_dmax[3] = {0, 0, 0}, grid_blen[3] = {0, 0, 0};
   double* d_grid64 = nullptr;
   float* d_grid32 = nullptr;
   // distribution records (keep_records): per such distribution rec_capacity slots of 3 values and
   // width weights, and one event counter per (problem, distribution)
   int64_t rec_capacity = 65536;
   double* d_rvals = nullptr;
   double* d_rwts = nullptr;
   unsigned long long* d_rn = nullptr;
   int64_t n_rvals = 0, n_rwts = 0;
};

namespace {

// the Butcher tables a context may select (spx_rk_tables.h)
constexpr spx_rk_entry kRkIndex[SPX_RK_N_TABLES] = SPX_RK_INDEX_INIT;

int cuda_err(cudaError_t e) { return e == cudaSuccess ? SPX_OK : (e == cudaErrorMemoryAllocation ? SPX_ERR_OUT_OF_MEMORY : SPX_ERR_CUDA); }

#define SPX_CUDA(call)                              \
   do {                                             \
      cudaError_t e__ = (call);                     \
      if (e__ != cudaSuccess) return cuda_err(e__); \
   } while (0)

void free_buffers(spx_ctx* c)
{
   cudaFree(c->d_pd);
   cudaFree(c->d_pr);
   cudaFree(c->d_ctr);
   cudaFree(c->d_counts);
   cudaFree(c->d_sums);
   cudaFree(c->d_nev);
   cudaFree(c->d_rec);
   cudaFree(c->d_rvals);
   cudaFree(c->d_rwts);
   cudaFree(c->d_rn);
   c->d_rvals = nullptr;
   c->d_rwts = nullptr;
   c->d_rn = nullptr;
   c->n_rvals = c->n_rwts = 0;
   c->d_pd = nullptr;
   c->d_pr = nullptr;
   c->d_ctr = nullptr;
   c->d_counts = nullptr;
   c->d_sums = nullptr;
   c->d_nev = nullptr;
   c->d_rec = nullptr;
   c->rec_cap = 0;
}

// Geometry and device address of the context's grid in a descriptor copy (gridded backgrounds).
void apply_grid(const spx_ctx* c, spx::ProblemDesc& pd)
{
   if (pd.bg.kind != spx::kBgGrid) return;
   for (int k = 0; k < 3; k++) {
      pd.bg.cent_min[k] = c->grid_cent[k];
      pd.bg.zone[k] = c->grid_zone[k];
      pd.bg.grid_n[k] = c->grid_n[k];
   }
   pd.bg.zone_min = std::min(c->grid_zone[0], std::min(c->grid_zone[1], c->grid_zone[2]));
   pd.bg.grid = c->d_grid64;
   for (int k = 0; k < 3; k++) {
      pd.bg.grid_nb[k] = c->grid_nb[k];
      pd.bg.dom_min[k] = c->grid_dmin[k];
      pd.bg.dom_max[k] = c->grid_dmax[k];
      pd.bg.blk_len[k] = c->grid_blen[k];
   }
   pd.bg.grid_ghost = c->grid_ghost;
   pd.bg.grid_order = c->grid_nb[0] > 0 ? c->grid_order : 1;  // a uniform grid interpolates at first order
   spx_grid_units(pd.bg.gunits);
}

void apply_grid(const spx_ctx* c, spx::ProblemDescT<float>& pd)
{
   if (pd.bg.kind == spx::kBgGrid) pd.bg.grid = c->d_grid32;
}

// A gridded background needs its grid before anything runs.
bool grid_missing(const spx_ctx* c) { return c->bg_kind == spx::kBgGrid && !c->has_grid; }

// Lay out the distributions of all problems, allocate and upload (called when problems changed).
int upload(spx_ctx* c)
{
   int n = (int)c->problems.size();
   int64_t off_c = 0, off_s = 0, first = 0;
   for (int k = 0; k < n; k++) {
      spx::ProblemDesc& pd = c->problems[k].pd;
      pd.first = first;
      pd.n_traj = c->problems[k].n_traj;
      first += pd.n_traj;
      for (int d = 0; d < pd.nd; d++) {
         int64_t nb = (int64_t)pd.d[d].n_bins[0] * pd.d[d].n_bins[1] * pd.d[d].n_bins[2];
         pd.d[d].offset_counts = off_c;
         pd.d[d].offset_sums = off_s;
         off_c += nb;
         off_s += nb * pd.d[d].width;
      }
   }
   c->total_traj = first;
   bool resize = (off_c != c->n_counts) || (off_s != c->n_sums) || c->d_pd == nullptr;
   if (resize) {
      cudaFree(c->d_pd);
      cudaFree(c->d_pr);
      cudaFree(c->d_counts);
      cudaFree(c->d_sums);
      cudaFree(c->d_nev);
      c->d_pd = nullptr;
      c->d_pr = nullptr;
      c->d_counts = nullptr;
      c->d_sums = nullptr;
      c->d_nev = nullptr;
      SPX_CUDA(cudaMalloc(&c->d_pd, sizeof(spx::ProblemDesc) * n));
      size_t rsz = c->precision == SPX_FP64 ? sizeof(spx::ProblemDescT<double>) : sizeof(spx::ProblemDescT<float>);
      SPX_CUDA(cudaMalloc(&c->d_pr, rsz * n));
      SPX_CUDA(cudaMalloc(&c->d_counts, sizeof(int32_t) * std::max<int64_t>(off_c, 1)));
      SPX_CUDA(cudaMalloc(&c->d_sums, sizeof(double) * std::max<int64_t>(off_s, 1)));
      SPX_CUDA(cudaMalloc(&c->d_nev, sizeof(unsigned long long) * n * spx::kMaxDistro));
      SPX_CUDA(cudaMemsetAsync(c->d_counts, 0, sizeof(int32_t) * std::max<int64_t>(off_c, 1), c->stream));
      SPX_CUDA(cudaMemsetAsync(c->d_sums, 0, sizeof(double) * std::max<int64_t>(off_s, 1), c->stream));
      SPX_CUDA(cudaMemsetAsync(c->d_nev, 0, sizeof(unsigned long long) * n * spx::kMaxDistro, c->stream));
      c->n_counts = off_c;
      c->n_sums = off_s;
   }
   if (c->d_ctr == nullptr) SPX_CUDA(cudaMalloc(&c->d_ctr, sizeof(spx::RunCounters)));
   if (grid_missing(c)) return SPX_ERR_STATE;
   // record buffers of the keep_records distributions (DistributionBase::AddRecord)
   int64_t rv = 0, rw = 0;
   for (int k = 0; k < n; k++)
      for (int d = 0; d < c->problems[k].pd.nd; d++)
         if (c->problems[k].pd.d[d].keep_records) {
            rv += 3 * c->rec_capacity;
            rw += (int64_t)c->problems[k].pd.d[d].width * c->rec_capacity;
         }
   if (rv != c->n_rvals || rw != c->n_rwts || (rv > 0 && c->d_rn == nullptr)) {
      cudaFree(c->d_rvals);
      cudaFree(c->d_rwts);
      cudaFree(c->d_rn);
      c->d_rvals = c->d_rwts = nullptr;
      c->d_rn = nullptr;
      c->n_rvals = c->n_rwts = 0;
      if (rv > 0) {
         SPX_CUDA(cudaMalloc(&c->d_rvals, sizeof(double) * rv));
         SPX_CUDA(cudaMalloc(&c->d_rwts, sizeof(double) * rw));
         SPX_CUDA(cudaMalloc(&c->d_rn, sizeof(unsigned long long) * n * spx::kMaxDistro));
         SPX_CUDA(cudaMemsetAsync(c->d_rn, 0, sizeof(unsigned long long) * n * spx::kMaxDistro, c->stream));
         c->n_rvals = rv;
         c->n_rwts = rw;
      }
   }
   std::vector<spx::ProblemDesc> hd(n);
   rv = rw = 0;
   for (int k = 0; k < n; k++) {
      hd[k] = c->problems[k].pd;
      apply_grid(c, hd[k]);
      for (int d = 0; d < hd[k].nd; d++) {
         spx::DistParams& dp = hd[k].d[d];
         dp.rec_vals = dp.rec_wts = nullptr;
         dp.rec_n = nullptr;
         dp.rec_cap = 0;
         if (!dp.keep_records || c->d_rn == nullptr) continue;
         dp.rec_vals = c->d_rvals + rv;
         dp.rec_wts = c->d_rwts + rw;
         dp.rec_n = c->d_rn + (int64_t)k * spx::kMaxDistro + d;
         dp.rec_cap = c->rec_capacity;
         rv += 3 * c->rec_capacity;
         rw += (int64_t)dp.width * c->rec_capacity;
      }
   }
   SPX_CUDA(cudaMemcpyAsync(c->d_pd, hd.data(), sizeof(spx::ProblemDesc) * n, cudaMemcpyHostToDevice, c->stream));
   if (c->precision == SPX_FP64) {
      SPX_CUDA(cudaMemcpyAsync(c->d_pr, hd.data(), sizeof(spx::ProblemDesc) * n, cudaMemcpyHostToDevice, c->stream));
   }
   else {
      std::vector<spx::ProblemDescT<float>> hf(n);
      for (int k = 0; k < n; k++) {
         spx::convert_problem(hd[k], hf[k]);
         apply_grid(c, hf[k]);
      }
      SPX_CUDA(cudaMemcpyAsync(c->d_pr, hf.data(), sizeof(spx::ProblemDescT<float>) * n, cudaMemcpyHostToDevice,
                               c->stream));
      SPX_CUDA(cudaStreamSynchronize(c->stream));  // hf is a host temporary
   }
   SPX_CUDA(cudaStreamSynchronize(c->stream));
   if (c->record_final && c->rec_cap < c->total_traj) {
      cudaFree(c->d_rec);
      c->d_rec = nullptr;
      SPX_CUDA(cudaMalloc(&c->d_rec, sizeof(spx::TrajRecord) * c->total_traj));
      c->rec_cap = c->total_traj;
   }
   c->dirty = false;
   return SPX_OK;
}

// The diffusion class every problem of the context shares, or -1 (kernels specialised for it exist for
// the FP32 Parker types: spx_k_parker_f32rb.cu, spx_k_parker_f32fc.cu).
int common_diffusion(const spx_ctx* c)
{
   int k = -2;
   for (const auto& p : c->problems) {
      if (k == -2) k = p.pd.df.kind;
      else if (k != p.pd.df.kind) return -1;
   }
   return k < 0 ? -1 : k;
}

int parker_f32_special(const spx_ctx* c)
{
   if (c->precision != SPX_MIXED || c->general_rk || c->specialize == 0) return -1;
   if (c->traj != SPX_TRAJ_PARKER && c->traj != SPX_TRAJ_PARKER_SOURCE) return -1;
   const int k = common_diffusion(c);
   return (k == spx::kDfRigidityB || k == spx::kDfFull) ? k : -1;
}

// TrajectoryGuiding proper in FP32, Euler or RK4: the kernels without the scattering and perpendicular steps.
bool guiding_plain(const spx_ctx* c)
{
   return c->precision == SPX_MIXED && !c->general_rk && c->specialize != 0 && c->traj == SPX_TRAJ_GUIDING &&
          !c->pa_scattering;
}

// Whether every problem has the boundary layout spx::kLayoutSpheres: one expiry or pass time boundary,
// two spheres, no momentum boundary.
bool layout_spheres(const spx_ctx* c)
{
   if (c->specialize != 1 || c->problems.empty()) return false;
   for (const auto& p : c->problems) {
      const spx::ProblemDesc& d = p.pd;
      if (d.nbt != 1 || d.nbs != 2 || d.nbm != 0) return false;
      if ((d.bt[0].kind != spx::kBtTimeExpire && d.bt[0].kind != spx::kBtTimePass) || d.bt[0].recurrent) return false;
      for (int i = 0; i < 2; i++) {
         const int k = d.bs[i].kind;
         if (k != spx::kBtSphereAbsorb && k != spx::kBtSphereReflect && k != spx::kBtSpherePass) return false;
      }
   }
   return true;
}

cudaError_t launch(spx_ctx* c, const spx::LaunchArgs& a)
{
   const bool f64 = c->precision == SPX_FP64, fd = f64 && c->deriv_mode == 0;
   const int bg = c->bg_kind;
   if (c->general_rk) {  // FP64 only (spx_create)
      switch (c->traj) {
      case SPX_TRAJ_PARKER:
      case SPX_TRAJ_PARKER_SOURCE: return fd ? spx::launch_parker_f64fdrk(bg, a) : spx::launch_parker_f64rk(bg, a);
      case SPX_TRAJ_LORENTZ: return fd ? spx::launch_lorentz_f64fdrk(bg, a) : spx::launch_lorentz_f64rk(bg, a);
      case SPX_TRAJ_FOCUSED: return fd ? spx::launch_focused_f64fdrk(bg, a) : spx::launch_focused_f64rk(bg, a);
      case SPX_TRAJ_FIELDLINE: return spx::launch_fieldline_f64rk(bg, a);
      default: return fd ? spx::launch_guiding_f64fdrk(bg, a) : spx::launch_guiding_f64rk(bg, a);
      }
   }
   if (guiding_plain(c)) return spx::launch_guiding_f32p(bg, a);
   switch (parker_f32_special(c)) {
   case spx::kDfRigidityB: return layout_spheres(c) ? spx::launch_parker_f32rbs(bg, a) : spx::launch_parker_f32rb(bg, a);
   case spx::kDfFull: return layout_spheres(c) ? spx::launch_parker_f32fcs(bg, a) : spx::launch_parker_f32fc(bg, a);
   default: break;
   }
   switch (c->traj) {
   case SPX_TRAJ_PARKER:
   case SPX_TRAJ_PARKER_SOURCE:
      return fd ? spx::launch_parker_f64fd(bg, a) : f64 ? spx::launch_parker_f64(bg, a) : spx::launch_parker_f32(bg, a);
   case SPX_TRAJ_LORENTZ:
      return fd ? spx::launch_lorentz_f64fd(bg, a) : f64 ? spx::launch_lorentz_f64(bg, a) : spx::launch_lorentz_f32(bg, a);
   case SPX_TRAJ_FOCUSED:
      return fd ? spx::launch_focused_f64fd(bg, a) : f64 ? spx::launch_focused_f64(bg, a) : spx::launch_focused_f32(bg, a);
   case SPX_TRAJ_GUIDING:
   case SPX_TRAJ_GUIDING_SCATT:
   case SPX_TRAJ_GUIDING_DIFF:
   case SPX_TRAJ_GUIDING_DIFF_SCATT:
      return fd ? spx::launch_guiding_f64fd(bg, a) : f64 ? spx::launch_guiding_f64(bg, a) : spx::launch_guiding_f32(bg, a);
   case SPX_TRAJ_FIELDLINE: return f64 ? spx::launch_fieldline_f64(bg, a) : spx::launch_fieldline_f32(bg, a);
   default: return cudaErrorInvalidValue;
   }
}

int occupancy(spx_ctx* c, int block, int slots)
{
   const bool f64 = c->precision == SPX_FP64, fd = f64 && c->deriv_mode == 0;
   const int bg = c->bg_kind;
   if (c->general_rk) {
      switch (c->traj) {
      case SPX_TRAJ_PARKER:
      case SPX_TRAJ_PARKER_SOURCE:
         return fd ? spx::occupancy_parker_f64fdrk(bg, block, slots) : spx::occupancy_parker_f64rk(bg, block, slots);
      case SPX_TRAJ_LORENTZ:
         return fd ? spx::occupancy_lorentz_f64fdrk(bg, block, slots) : spx::occupancy_lorentz_f64rk(bg, block, slots);
      case SPX_TRAJ_FOCUSED:
         return fd ? spx::occupancy_focused_f64fdrk(bg, block, slots) : spx::occupancy_focused_f64rk(bg, block, slots);
      case SPX_TRAJ_FIELDLINE: return spx::occupancy_fieldline_f64rk(bg, block, slots);
      default:
         return fd ? spx::occupancy_guiding_f64fdrk(bg, block, slots) : spx::occupancy_guiding_f64rk(bg, block, slots);
      }
   }
   if (guiding_plain(c)) return spx::occupancy_guiding_f32p(bg, block, slots);
   switch (parker_f32_special(c)) {
   case spx::kDfRigidityB:
      return layout_spheres(c) ? spx::occupancy_parker_f32rbs(bg, block, slots) : spx::occupancy_parker_f32rb(bg, block, slots);
   case spx::kDfFull:
      return layout_spheres(c) ? spx::occupancy_parker_f32fcs(bg, block, slots) : spx::occupancy_parker_f32fc(bg, block, slots);
   default: break;
   }
   switch (c->traj) {
   case SPX_TRAJ_PARKER:
   case SPX_TRAJ_PARKER_SOURCE:
      return fd ? spx::occupancy_parker_f64fd(bg, block, slots)
                : f64 ? spx::occupancy_parker_f64(bg, block, slots) : spx::occupancy_parker_f32(bg, block, slots);
   case SPX_TRAJ_LORENTZ:
      return fd ? spx::occupancy_lorentz_f64fd(bg, block, slots)
                : f64 ? spx::occupancy_lorentz_f64(bg, block, slots) : spx::occupancy_lorentz_f32(bg, block, slots);
   case SPX_TRAJ_FOCUSED:
      return fd ? spx::occupancy_focused_f64fd(bg, block, slots)
                : f64 ? spx::occupancy_focused_f64(bg, block, slots) : spx::occupancy_focused_f32(bg, block, slots);
   case SPX_TRAJ_GUIDING:
   case SPX_TRAJ_GUIDING_SCATT:
   case SPX_TRAJ_GUIDING_DIFF:
   case SPX_TRAJ_GUIDING_DIFF_SCATT:
      return fd ? spx::occupancy_guiding_f64fd(bg, block, slots)
                : f64 ? spx::occupancy_guiding_f64(bg, block, slots) : spx::occupancy_guiding_f32(bg, block, slots);
   case SPX_TRAJ_FIELDLINE:
      return f64 ? spx::occupancy_fieldline_f64(bg, block, slots) : spx::occupancy_fieldline_f32(bg, block, slots);
   default: return 0;
   }
}

// Boundary states a lane holds: the largest boundary count of the context's problems.
int bnd_slots(const spx_ctx* c)
{
   int n = 1;
   for (const auto& p : c->problems) n = std::max(n, p.pd.nbt + p.pd.nbs + p.pd.nbm);
   return n;
}

bool valid_ctx(spx_ctx* c) { return c != nullptr; }

// the context's Butcher table, and whether |B| extrema are tracked (a problem has a
// DistributionLossCone), in a run configuration
void set_rk(const spx_ctx* c, spx::RunConfig& cfg)
{
   cfg.rk_stages = c->rk_stages;
   cfg.rk_order = c->rk_order;
   cfg.rk_adaptive = c->rk_adaptive;
   cfg.rk_offset = c->rk_offset;
   cfg.track_bmag = 0;
   for (const auto& p : c->problems)
      for (int d = 0; d < p.pd.nd; d++)
         if (p.pd.d[d].kind == spx::kDsLossCone) cfg.track_bmag = 1;
}

// The launch shape of a run: the caller's, else the one spx_autotune chose, else the defaults (the
// FP64 drop-in keeps one thread per trajectory; the FP32 stepper takes the persistent queue in
// blocks of 64 refilled every 8 steps, the shape that measured fastest on the modulation batch).
// Unset fields are completed and checked; blocks per SM is capped by the kernel's occupancy for
// "slots" boundary states per lane. Shared by spx_run and spx_run_static.
int resolve_tuning(spx_ctx* c, const spx_tuning* tuning, int slots, spx_tuning& tu)
{
   tu = spx_tuning{};
   if (tuning) tu = *tuning;
   else if (c->has_tuned) tu = c->tuned;
   else {
      tu.schedule = c->precision == SPX_MIXED ? 1 : 0;
      if (tu.schedule) {
         tu.block_size = 64;
         tu.steps_per_sync = 8;
      }
   }
   if (tu.schedule != 0 && tu.schedule != 1) return SPX_ERR_INVALID_ARG;
   if (tu.block_size <= 0) tu.block_size = 128;
   if (tu.block_size % 32 || tu.block_size > 128) return SPX_ERR_INVALID_ARG;
   if (tu.steps_per_sync <= 0) tu.steps_per_sync = tu.schedule ? 16 : 1 << 30;
   int occ = occupancy(c, tu.block_size, slots);
   if (occ <= 0) occ = 1;
   if (tu.blocks_per_sm <= 0 || tu.blocks_per_sm > occ) tu.blocks_per_sm = occ;
   return SPX_OK;
}


// What a captured graph depends on: launch shape, the run configuration apart from the run
// index, and the device buffers. A different key means a new capture.
struct GraphKey {
   unsigned grid, block, slots;
   int queue;
   spx::RunConfig cfg;
   const void* ptr[7];
};
static_assert(sizeof(GraphKey) <= sizeof(spx_ctx::gkey), "graph key does not fit");

void graph_key(const spx::LaunchArgs& a, unsigned char* out)
{
   GraphKey k;
   std::memset(&k, 0, sizeof k);
   k.grid = a.grid.x;
   k.block = a.block.x;
   k.slots = (unsigned)a.bnd_slots;
   k.queue = a.queue;
   k.cfg = a.cfg;
   k.cfg.run_index = 0;
   const void* p[7] = {a.problems_r, a.problems_d, a.ctr, a.counts, a.sums, a.n_events, a.records};
   std::memcpy(k.ptr, p, sizeof p);
   std::memset(out, 0, sizeof(spx_ctx::gkey));
   std::memcpy(out, &k, sizeof k);
}

void drop_graph(spx_ctx* c)
{
   if (c->gexec) cudaGraphExecDestroy(c->gexec);
   if (c->graph) cudaGraphDestroy(c->graph);
   c->gexec = nullptr;
   c->graph = nullptr;
   c->gkernel = nullptr;
}

// Capture [clear the run counters, start event, step kernel, stop event] on the context stream.
int capture_graph(spx_ctx* c, const spx::LaunchArgs& a)
{
   drop_graph(c);
   cudaGetLastError();  // a launch check below must not report an earlier call's error
   SPX_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
   cudaError_t e = cudaMemsetAsync(c->d_ctr, 0, sizeof(spx::RunCounters), c->stream);
   // inside a capture a plain event record only orders streams; the timing events must become
   // event-record nodes of the graph
   if (e == cudaSuccess) e = cudaEventRecordWithFlags(c->ev0, c->stream, cudaEventRecordExternal);
   if (e == cudaSuccess) e = launch(c, a);
   if (e == cudaSuccess) e = cudaEventRecordWithFlags(c->ev1, c->stream, cudaEventRecordExternal);
   cudaGraph_t g = nullptr;
   cudaError_t e2 = cudaStreamEndCapture(c->stream, &g);
   if (e == cudaSuccess) e = e2;
   if (e != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();
      return cuda_err(e);
   }
   size_t n = 0;
   SPX_CUDA(cudaGraphGetNodes(g, nullptr, &n));
   std::vector<cudaGraphNode_t> nodes(n);
   SPX_CUDA(cudaGraphGetNodes(g, nodes.data(), &n));
   for (cudaGraphNode_t node : nodes) {
      cudaGraphNodeType t;
      SPX_CUDA(cudaGraphNodeGetType(node, &t));
      if (t == cudaGraphNodeTypeKernel) {
         c->gkernel = node;
         SPX_CUDA(cudaGraphKernelNodeGetParams(node, &c->gparams));
      }
   }
   c->graph = g;
   if (c->gkernel == nullptr) return SPX_ERR_CUDA;
   SPX_CUDA(cudaGraphInstantiate(&c->gexec, g, 0));
   graph_key(a, c->gkey);
   return SPX_OK;
}

// One run: replay the captured graph with this run's kernel arguments.
int run_graph(spx_ctx* c, const spx::LaunchArgs& a)
{
   unsigned char key[sizeof(spx_ctx::gkey)];
   graph_key(a, key);
   if (c->gexec == nullptr || std::memcmp(key, c->gkey, sizeof key) != 0) {
      int rc = capture_graph(c, a);
      if (rc != SPX_OK) return rc;
   }
   // the step kernel's parameter list: (problems_r, problems_d, cfg, ctr, counts, sums, n_events,
   // records, queue)
   const void* pr = a.problems_r;
   const spx::ProblemDesc* pd = a.problems_d;
   spx::RunConfig cfg = a.cfg;
   spx::RunCounters* ctr = a.ctr;
   int32_t* counts = a.counts;
   double* sums = a.sums;
   unsigned long long* nev = a.n_events;
   spx::TrajRecord* rec = a.records;
   int queue = a.queue;
   void* args[9] = {&pr, &pd, &cfg, &ctr, &counts, &sums, &nev, &rec, &queue};
   cudaKernelNodeParams p = c->gparams;
   p.kernelParams = args;
   p.extra = nullptr;
   SPX_CUDA(cudaGraphExecKernelNodeSetParams(c->gexec, c->gkernel, &p));
   SPX_CUDA(cudaGraphLaunch(c->gexec, c->stream));
   return SPX_OK;
}

}  // namespace

namespace {

// The class names the reference gives its distribution classes (src/distribution_other.hh:72-573):
// the first field of a DistributionTemplated dump file, and what a restore checks it against.
const char* distro_class_name(int kind)
{
   switch (kind) {
   case spx::kDsTimeUniform: return "DistributionTimeUniform";
   case spx::kDsPositionUniform: return "DistributionPositionUniform";
   case spx::kDsMomentumUniform: return "DistributionMomentumUniform";
   case spx::kDsPositionMomentumUniform: return "DistributionPositionMomentumUniform";
   case spx::kDsSpectrumPowerLaw: return "DistributionSpectrumKineticEnergyPowerLaw";
   case spx::kDsSpectrumBentPowerLaw: return "DistributionSpectrumKineticEnergyBentPowerLaw";
   case spx::kDsCumulative1: return "DistributionPositionCumulativeOrder1";
   case spx::kDsCumulative2: return "DistributionPositionCumulativeOrder2";
   case spx::kDsDivergenceFlow: return "DistributionDivergenceFlowPowerLaw";
   case spx::kDsLossCone: return "DistributionLossCone";
   case spx::kDsAnisotropyLISM: return "DistributionAnisotropyLISM";
   case spx::kDsTimeMu: return "DistributionTimeMu";  // a class of this library only
   default: return nullptr;
   }
}

template <class T>
bool put(FILE* f, const T* v, size_t n) { return n == 0 || std::fwrite(v, sizeof(T), n, f) == n; }

template <class T>
bool get(FILE* f, T* v, size_t n) { return n == 0 || std::fread(v, sizeof(T), n, f) == n; }

}  // namespace

extern "C" {

int spx_create(spx_ctx_t* out, int traj_kind, int time_flow, int rk_method, int precision)
{
   if (!out) return SPX_ERR_INVALID_ARG;
   *out = nullptr;
   if (traj_kind != SPX_TRAJ_PARKER && traj_kind != SPX_TRAJ_PARKER_SOURCE && traj_kind != SPX_TRAJ_LORENTZ &&
       traj_kind != SPX_TRAJ_FOCUSED && traj_kind != SPX_TRAJ_FIELDLINE &&
       (traj_kind < SPX_TRAJ_GUIDING || traj_kind > SPX_TRAJ_GUIDING_DIFF_SCATT))
      return SPX_ERR_INVALID_ARG;
   if (time_flow != SPX_FORWARD && time_flow != SPX_BACKWARD) return SPX_ERR_INVALID_ARG;
   if (precision != SPX_FP64 && precision != SPX_MIXED) return SPX_ERR_INVALID_ARG;
   // The Butcher table (RK_INTEGRATOR_TYPE, common/rk_config.hh:72-520): any of the reference's tables
   // but 30, which does not compile there. Euler, and the classic RK4 for the RK types, run on kernels
   // with the coefficients unrolled, in both arithmetics; the other tables run on the FP64 kernels of
   // any table (their error control works at the reference's 1e-9 tolerance, which FP32 cannot reach).
   const spx_rk_entry* tab = nullptr;
   for (const auto& e : kRkIndex)
      if (e.number == rk_method) tab = &e;
   if (!tab) return SPX_ERR_INVALID_ARG;
   const bool parker = traj_kind == SPX_TRAJ_PARKER || traj_kind == SPX_TRAJ_PARKER_SOURCE;
   const bool general = !(rk_method == 0 || (rk_method == 25 && !parker));
   if (general && precision != SPX_FP64) return SPX_ERR_INVALID_ARG;
   int ndev = 0;
   if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
      cudaGetLastError();
      return SPX_ERR_NO_DEVICE;
   }
   auto c = std::make_unique<spx_ctx>();
   if (cudaGetDevice(&c->device) != cudaSuccess) return SPX_ERR_NO_DEVICE;
   cudaDeviceProp prop;
   if (cudaGetDeviceProperties(&prop, c->device) != cudaSuccess) return SPX_ERR_NO_DEVICE;
   if (prop.major != 10 || prop.minor != 3) return SPX_ERR_NO_DEVICE;  // built for sm_103a only
   c->sm_count = prop.multiProcessorCount;
   c->traj = traj_kind;
   c->flow = time_flow;
   c->rk = rk_method;
   c->general_rk = general;
   c->rk_stages = tab->stages;
   c->rk_order = tab->order;
   c->rk_adaptive = tab->adaptive;
   c->rk_offset = tab->offset;
   c->precision = precision;
   if (precision == SPX_MIXED) c->deriv_mode = 1;
   // TrajectoryGuidingScatt is the guiding-centre stepper with its pitch-angle step always on
   if (traj_kind == SPX_TRAJ_GUIDING_SCATT || traj_kind == SPX_TRAJ_GUIDING_DIFF_SCATT) c->pa_scattering = 1;
   if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) return SPX_ERR_CUDA;
   if (cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess) return SPX_ERR_CUDA;
   *out = c.release();
   return SPX_OK;
}

int spx_set_option(spx_ctx_t c, int option, double value)
{
   if (!valid_ctx(c)) return SPX_ERR_INVALID_ARG;
   switch (option) {
   case SPX_OPT_STEPS_PER_ORBIT:
      if (!(value > 0.0)) return SPX_ERR_INVALID_ARG;
      c->steps_per_orbit = value;
      return SPX_OK;
   case SPX_OPT_DERIV_MODE:
      if (value != 0.0 && value != 1.0) return SPX_ERR_INVALID_ARG;
      // the FP32 kernels compute analytic derivatives only
      if (c->precision == SPX_MIXED && value == 0.0) return SPX_ERR_INVALID_ARG;
      c->deriv_mode = (int)value;
      return SPX_OK;
   case SPX_OPT_PA_SCATTERING:
      // an option of the focused stepper only; GuidingScatt scatters by its type
      if (c->traj == SPX_TRAJ_GUIDING_SCATT || c->traj == SPX_TRAJ_GUIDING_DIFF_SCATT)
         return value != 0.0 ? SPX_OK : SPX_ERR_INVALID_ARG;
      if (c->traj != SPX_TRAJ_FOCUSED && value != 0.0) return SPX_ERR_INVALID_ARG;
      c->pa_scattering = value != 0.0;
      return SPX_OK;
   case SPX_OPT_RECORD_FINAL:
      c->record_final = value != 0.0;
      c->dirty = true;
      return SPX_OK;
   case SPX_OPT_MAX_ATTEMPTS:
      if (!(value >= 1.0)) return SPX_ERR_INVALID_ARG;
      c->max_attempts = (int)value;
      return SPX_OK;
   case SPX_OPT_MU_METHOD:
      // the pitch-angle scheme of the guiding-centre scattering types (STOCHASTIC_METHOD_MU)
      if (value != 0.0 && value != 1.0 && value != 2.0) return SPX_ERR_INVALID_ARG;
      if (value != 0.0 && c->traj != SPX_TRAJ_GUIDING_SCATT && c->traj != SPX_TRAJ_GUIDING_DIFF_SCATT)
         return SPX_ERR_INVALID_ARG;
      c->mu_method = (int)value;
      return SPX_OK;
   case SPX_OPT_PERP_METHOD:
      // the perpendicular scheme of the guiding-centre diffusion types (STOCHASTIC_METHOD_PERP)
      if (value != 0.0 && value != 1.0 && value != 2.0) return SPX_ERR_INVALID_ARG;
      if (value != 0.0 && c->traj != SPX_TRAJ_GUIDING_DIFF && c->traj != SPX_TRAJ_GUIDING_DIFF_SCATT)
         return SPX_ERR_INVALID_ARG;
      c->perp_method = (int)value;
      return SPX_OK;
   case SPX_OPT_RECORD_CAPACITY:
      // records kept per keep_records distribution; further events are counted, not stored
      if (!(value >= 0.0) || value != (double)(int64_t)value || value > 2147483647.0) return SPX_ERR_INVALID_ARG;
      c->rec_capacity = (int64_t)value;
      c->dirty = true;
      return SPX_OK;
   case SPX_OPT_SPECIALIZE:
      // 0: no specialised kernel; 1: diffusion class and boundary layout; 2: diffusion class only
      // (a captured launch is re-captured)
      if (value != 0.0 && value != 1.0 && value != 2.0) return SPX_ERR_INVALID_ARG;
      c->specialize = (int)value;
      drop_graph(c);
      return SPX_OK;
   case SPX_OPT_GRID_INTERP:
      // the reader's interpolation needs numerical gradients, which the FP64 kernels carry
      if (value != 1.0 && value != 0.0 && value != -1.0) return SPX_ERR_INVALID_ARG;
      if (value == -1.0 && c->precision != SPX_FP64) return SPX_ERR_INVALID_ARG;
      c->grid_order = (int)value;
      c->dirty = true;
      drop_graph(c);
      return SPX_OK;
   case SPX_OPT_STEP_CAP:
      if (!(value >= 0.0) || value != (double)(int64_t)value || value > 4294967295.0) return SPX_ERR_INVALID_ARG;
      c->step_cap = (uint32_t)value;
      drop_graph(c);
      return SPX_OK;
   case SPX_OPT_RUN_INDEX:
      // shards of one job: rank r starting at index r draws trajectory ids disjoint from the others'
      if (!(value >= 0.0) || value != (double)(int64_t)value || value > 4294967295.0) return SPX_ERR_INVALID_ARG;
      c->run_index = (int64_t)value;
      return SPX_OK;
   default: return SPX_ERR_INVALID_ARG;
   }
}

int spx_add_plugin(spx_ctx_t c, int role, int kind, const uint8_t* blob, size_t blob_len, size_t n_records)
{
   if (!valid_ctx(c) || (blob_len && !blob) || role < 0 || role > SPX_ROLE_DISTRIBUTION) return SPX_ERR_INVALID_ARG;
   if (n_records > 0xffffffffu) return SPX_ERR_INVALID_ARG;
   // parse now so a malformed blob is reported where it is added
   spx::ProblemDesc probe;
   std::memset(&probe, 0, sizeof probe);
   int rc = spx::parse_plugin(probe, c->traj, role, kind, blob, blob_len, -1);
   if (rc != SPX_OK) return rc;
   if (role == SPX_ROLE_SOURCE && c->traj != SPX_TRAJ_PARKER_SOURCE) return SPX_ERR_UNKNOWN_PLUGIN;
   if (role == SPX_ROLE_BACKGROUND && !spx::background_allowed(c->traj, probe.bg.kind)) return SPX_ERR_UNKNOWN_PLUGIN;
   c->base.push_back(PluginBlob{role, kind, (uint32_t)n_records, std::vector<uint8_t>(blob, blob + blob_len)});
   return SPX_OK;
}

int spx_add_problem(spx_ctx_t c, int64_t n_traj, uint64_t seed, const uint8_t* ov, size_t ov_len)
{
   if (!valid_ctx(c) || n_traj < 0 || n_traj > 0xffffffffLL || (ov_len && !ov)) return SPX_ERR_INVALID_ARG;
   ProblemHost ph;
   std::memset(&ph.pd, 0, sizeof ph.pd);
   for (const auto& p : c->base) {
      int rc = spx::parse_plugin(ph.pd, c->traj, p.role, p.kind, p.blob.data(), p.blob.size(), -1);
      if (rc != SPX_OK) return rc;
      if (p.role == SPX_ROLE_DISTRIBUTION) ph.dist[ph.pd.nd - 1] = p;
   }
   size_t pos = 0;
   while (pos < ov_len) {
      uint32_t hdr[5];
      if (pos + sizeof hdr > ov_len) return SPX_ERR_BAD_BLOB;
      std::memcpy(hdr, ov + pos, sizeof hdr);
      pos += sizeof hdr;
      if (pos + hdr[4] > ov_len) return SPX_ERR_BAD_BLOB;
      int role = (int)hdr[0], slot = (int)hdr[1], kind = (int)hdr[2];
      bool slotted = role == SPX_ROLE_BOUNDARY || role == SPX_ROLE_DISTRIBUTION;
      int rc = spx::parse_plugin(ph.pd, c->traj, role, kind, ov + pos, hdr[4], slotted ? slot : -1);
      if (rc != SPX_OK) return rc;
      if (role == SPX_ROLE_DISTRIBUTION) ph.dist[slot] = PluginBlob{role, kind, hdr[3], std::vector<uint8_t>(ov + pos, ov + pos + hdr[4])};
      pos += hdr[4];
   }
   int rc = spx::check_ready(ph.pd, c->traj);
   if (rc != SPX_OK) return rc;
   if (c->problems.empty()) c->bg_kind = ph.pd.bg.kind;
   else if (ph.pd.bg.kind != c->bg_kind) return SPX_ERR_INVALID_ARG;  // one background class per context
   if (c->problems.size() >= 65536) return SPX_ERR_LIMIT;
   ph.pd.problem_id = (uint32_t)c->problems.size();
   ph.pd.seed = seed;
   ph.n_traj = n_traj;
   c->problems.push_back(ph);
   c->dirty = true;
   return SPX_OK;
}

// BackgroundServerCartesian's data: one uniform block of n[0] x n[1] x n[2] nodes, node (i, j, k) at
// cent_min + (i, j, k) * zone_length, six values per node (U then B, code units), x fastest. The
// values are copied to device memory now, in the context's arithmetic, with |B| of every node
// appended (the magnitude the reference interpolates, src/server_cartesian.cc:566-569).
int spx_set_background_grid(spx_ctx_t c, const int64_t n[3], const double cent_min[3], const double zone_length[3],
                            const double* values)
{
   if (!valid_ctx(c) || !n || !cent_min || !zone_length || !values) return SPX_ERR_INVALID_ARG;
   int64_t nodes = 1;
   for (int k = 0; k < 3; k++) {
      if (n[k] < 2 || n[k] > 1000000 || !(zone_length[k] > 0.0) || !std::isfinite(cent_min[k])) return SPX_ERR_INVALID_ARG;
      nodes *= n[k];
   }
   if (nodes > ((int64_t)1 << 31)) return SPX_ERR_TOO_LARGE;
   SPX_CUDA(cudaSetDevice(c->device));
   SPX_CUDA(cudaStreamSynchronize(c->stream));
   cudaFree(c->d_grid64);
   cudaFree(c->d_grid32);
   c->d_grid64 = nullptr;
   c->d_grid32 = nullptr;
   c->has_grid = false;
   const size_t count = (size_t)nodes * spx::kGridStride;
   std::vector<double> h(count, 0.0);
   for (int64_t i = 0; i < nodes; i++) {
      const double* v = values + 6 * i;
      double* o = h.data() + spx::kGridStride * i;
      for (int q = 0; q < 6; q++) o[q] = v[q];
      const double bx2 = v[3] * v[3], by2 = v[4] * v[4], bz2 = v[5] * v[5];
      o[6] = std::sqrt(bx2 + by2 + bz2);
   }
   if (c->precision == SPX_FP64) {
      SPX_CUDA(cudaMalloc(&c->d_grid64, sizeof(double) * count));
      SPX_CUDA(cudaMemcpy(c->d_grid64, h.data(), sizeof(double) * count, cudaMemcpyHostToDevice));
   }
   else {
      std::vector<float> f(h.begin(), h.end());
      SPX_CUDA(cudaMalloc(&c->d_grid32, sizeof(float) * count));
      SPX_CUDA(cudaMemcpy(c->d_grid32, f.data(), sizeof(float) * count, cudaMemcpyHostToDevice));
   }
   for (int k = 0; k < 3; k++) {
      c->grid_n[k] = (int)n[k];
      c->grid_cent[k] = cent_min[k];
      c->grid_zone[k] = zone_length[k];
      c->grid_nb[k] = 0;
   }
   c->grid_ghost = 0;
   c->has_grid = true;
   c->dirty = true;
   return SPX_OK;
}

void spx_grid_units(double out[4])
{
   if (!out) return;
   // the reference's unit systems: Fluid (au, 100 km/s, m_p cm^-3) and Particle (1e10 cm, c/10, m_p, e)
   const double au = 1.495978707e+13, c_light = 2.99792458e+10, m_p = 1.67262192596e-24, e = 4.8032044e-10;
   const double p_vel = 0.1 * c_light, p_len = 1.0e10;
   const double p_time = p_len / p_vel, p_mag = (m_p * p_vel) / (e * p_time);
   const double f_vel = 1.0e7, f_mag = f_vel * std::sqrt(m_p * 1.0);
   out[0] = au / p_len;
   out[1] = f_vel / p_vel;
   out[2] = f_mag / p_mag;
   out[3] = c_light / f_vel;
}

int spx_set_background_blocks(spx_ctx_t c, const int32_t n_blocks[3], const double domain_min[3],
                              const double domain_max[3], int ghost_cells, const double* values)
{
   if (!valid_ctx(c) || !n_blocks || !domain_min || !domain_max || !values) return SPX_ERR_INVALID_ARG;
   if (ghost_cells < 0 || ghost_cells > 1) return SPX_ERR_INVALID_ARG;
   const int bz = spx::kGridBlockZones;
   int64_t blocks = 1;
   for (int k = 0; k < 3; k++) {
      if (n_blocks[k] < 1 || n_blocks[k] > 100000 || !std::isfinite(domain_min[k]) || !std::isfinite(domain_max[k]) ||
          !(domain_max[k] > domain_min[k]))
         return SPX_ERR_INVALID_ARG;
      blocks *= n_blocks[k];
   }
   if (blocks * bz * bz * bz > ((int64_t)1 << 31)) return SPX_ERR_TOO_LARGE;
   SPX_CUDA(cudaSetDevice(c->device));
   SPX_CUDA(cudaStreamSynchronize(c->stream));
   cudaFree(c->d_grid64);
   cudaFree(c->d_grid32);
   c->d_grid64 = nullptr;
   c->d_grid32 = nullptr;
   c->has_grid = false;
   int n[3];
   for (int k = 0; k < 3; k++) n[k] = bz * n_blocks[k];
   const int64_t nodes = (int64_t)n[0] * n[1] * n[2];
   const size_t count = (size_t)nodes * spx::kGridStride;
   // the reader's regrouping by dimension (src/reader_cartesian.cc:136-162), |B| of every zone appended
   std::vector<double> h(count, 0.0);
   for (int64_t b = 0; b < blocks; b++) {
      const int64_t bi = b % n_blocks[0], bj = (b / n_blocks[0]) % n_blocks[1], bk = b / ((int64_t)n_blocks[0] * n_blocks[1]);
      for (int z = 0; z < bz * bz * bz; z++) {
         const int64_t i = bz * bi + z % bz, j = bz * bj + (z / bz) % bz, k = bz * bk + z / (bz * bz);
         const double* v = values + 6 * (bz * bz * bz * b + z);
         double* o = h.data() + spx::kGridStride * (i + n[0] * (j + (int64_t)n[1] * k));
         for (int q = 0; q < 6; q++) o[q] = v[q];
         const double bx2 = v[3] * v[3], by2 = v[4] * v[4], bz2 = v[5] * v[5];
         o[6] = std::sqrt(bx2 + by2 + bz2);
      }
   }
   if (c->precision == SPX_FP64) {
      SPX_CUDA(cudaMalloc(&c->d_grid64, sizeof(double) * count));
      SPX_CUDA(cudaMemcpy(c->d_grid64, h.data(), sizeof(double) * count, cudaMemcpyHostToDevice));
   }
   else {
      std::vector<float> f(h.begin(), h.end());
      SPX_CUDA(cudaMalloc(&c->d_grid32, sizeof(float) * count));
      SPX_CUDA(cudaMemcpy(c->d_grid32, f.data(), sizeof(float) * count, cudaMemcpyHostToDevice));
   }
   for (int k = 0; k < 3; k++) {
      c->grid_n[k] = n[k];
      c->grid_nb[k] = n_blocks[k];
      c->grid_dmin[k] = domain_min[k];
      c->grid_dmax[k] = domain_max[k];
      c->grid_blen[k] = (domain_max[k] - domain_min[k]) / (double)n_blocks[k];  // block_length (:97)
      c->grid_cent[k] = 0.0;
      c->grid_zone[k] = 1.0;
   }
   c->grid_ghost = ghost_cells;
   c->has_grid = true;
   c->dirty = true;
   return SPX_OK;
}

int spx_run(spx_ctx_t c, const spx_tuning* tuning)
{
   if (!valid_ctx(c)) return SPX_ERR_INVALID_ARG;
   if (c->problems.empty()) return SPX_ERR_STATE;
   SPX_CUDA(cudaSetDevice(c->device));
   if (c->dirty) {
      int rc = upload(c);
      if (rc != SPX_OK) return rc;
   }
   spx_tuning tu;
   const int slots = bnd_slots(c);
   const int trc = resolve_tuning(c, tuning, slots, tu);
   if (trc != SPX_OK) return trc;
   spx::LaunchArgs a;
   a.block = dim3(tu.block_size);
   int64_t grid;
   if (tu.schedule == 1) grid = (int64_t)c->sm_count * tu.blocks_per_sm;  // persistent: fill the GPU once
   else grid = (c->total_traj + tu.block_size - 1) / tu.block_size;      // one thread per trajectory
   grid = std::max<int64_t>(1, std::min<int64_t>(grid, 0x7fffffff));
   a.grid = dim3((unsigned)grid);
   a.stream = c->stream;
   a.problems_r = c->d_pr;
   a.problems_d = c->d_pd;
   a.cfg.traj_kind = c->traj;
   a.cfg.time_flow = c->flow;
   a.cfg.rk = c->rk;
   set_rk(c, a.cfg);
   a.cfg.deriv_mode = c->deriv_mode;
   a.cfg.pa_scattering = c->pa_scattering;
   a.cfg.mu_method = c->mu_method;
   a.cfg.perp_method = c->perp_method;
   a.cfg.max_attempts = c->max_attempts;
   a.cfg.steps_per_orbit = c->steps_per_orbit;
   a.cfg.steps_per_orbit_f = (float)c->steps_per_orbit;
   a.cfg.record_final = c->record_final;
   a.cfg.n_problems = (int)c->problems.size();
   a.cfg.steps_per_sync = tu.steps_per_sync;
   a.cfg.step_cap = c->step_cap;
   a.cfg.total_traj = c->total_traj;
   a.cfg.run_index = c->run_index;
   a.ctr = c->d_ctr;
   a.counts = c->d_counts;
   a.sums = c->d_sums;
   a.n_events = c->d_nev;
   a.records = c->d_rec;
   a.queue = tu.schedule;
   a.bnd_slots = slots;
   if (c->record_final && c->d_rec == nullptr) return SPX_ERR_STATE;
   // trajectory ids of this run, run_index * n_traj ... (run_index + 1) * n_traj - 1, must fit 32 bits
   for (const auto& p : c->problems)
      if ((uint64_t)(c->run_index + 1) * (uint64_t)p.n_traj > 0x100000000ull) return SPX_ERR_LIMIT;
   int grc = run_graph(c, a);
   if (grc != SPX_OK) return grc;
   c->run_index++;  // the next run draws the ids after these (new random streams)
   c->launched = true;
   c->last = spx_stats{};
   c->last.tuning = tu;
   c->last.kernel_launches = 1;
   return SPX_OK;
}

// The autotuner: time candidate launch shapes on a sample of the context's problems (each problem
// keeps its share of trajectories, every trajectory stops after a fixed number of steps) and keep
// the fastest by accepted steps per second. The sample runs on buffers of its own with other
// random streams, so the context's distributions and trajectory ids are untouched.
int spx_autotune(spx_ctx_t c, int64_t sample_traj, spx_tuning* best)
{
   if (!valid_ctx(c)) return SPX_ERR_INVALID_ARG;
   if (c->problems.empty() || grid_missing(c)) return SPX_ERR_STATE;
   SPX_CUDA(cudaSetDevice(c->device));
   const int n = (int)c->problems.size();
   const bool f64 = c->precision == SPX_FP64;
   const int slots = bnd_slots(c);
   if (sample_traj <= 0) sample_traj = (int64_t)c->sm_count * 4 * 128 * 2;  // about two per resident lane
   int64_t total = 0;
   for (const auto& p : c->problems) total += p.n_traj;
   std::vector<spx::ProblemDesc> hd(n);
   int64_t off_c = 0, off_s = 0, first = 0;
   for (int k = 0; k < n; k++) {
      hd[k] = c->problems[k].pd;
      apply_grid(c, hd[k]);
      int64_t nk = std::max<int64_t>(1, (int64_t)((double)c->problems[k].n_traj * sample_traj / std::max<int64_t>(total, 1)));
      hd[k].n_traj = nk;
      hd[k].first = first;
      hd[k].seed ^= 0x9E3779B97F4A7C15ull;
      first += nk;
      for (int d = 0; d < hd[k].nd; d++) {
         int64_t nb = (int64_t)hd[k].d[d].n_bins[0] * hd[k].d[d].n_bins[1] * hd[k].d[d].n_bins[2];
         hd[k].d[d].offset_counts = off_c;
         hd[k].d[d].offset_sums = off_s;
         off_c += nb;
         off_s += nb * hd[k].d[d].width;
      }
   }
   struct DevBuf {
      void* p = nullptr;
      ~DevBuf() { cudaFree(p); }
   } b_pd, b_pr, b_ctr, b_counts, b_sums, b_nev;
   SPX_CUDA(cudaMalloc(&b_pd.p, sizeof(spx::ProblemDesc) * n));
   SPX_CUDA(cudaMalloc(&b_pr.p, f64 ? sizeof(spx::ProblemDesc) * n : sizeof(spx::ProblemDescT<float>) * n));
   SPX_CUDA(cudaMalloc(&b_ctr.p, sizeof(spx::RunCounters)));
   SPX_CUDA(cudaMalloc(&b_counts.p, sizeof(int32_t) * std::max<int64_t>(off_c, 1)));
   SPX_CUDA(cudaMalloc(&b_sums.p, sizeof(double) * std::max<int64_t>(off_s, 1)));
   SPX_CUDA(cudaMalloc(&b_nev.p, sizeof(unsigned long long) * n * spx::kMaxDistro));
   SPX_CUDA(cudaMemcpy(b_pd.p, hd.data(), sizeof(spx::ProblemDesc) * n, cudaMemcpyHostToDevice));
   if (f64) SPX_CUDA(cudaMemcpy(b_pr.p, hd.data(), sizeof(spx::ProblemDesc) * n, cudaMemcpyHostToDevice));
   else {
      std::vector<spx::ProblemDescT<float>> hf(n);
      for (int k = 0; k < n; k++) {
         spx::convert_problem(hd[k], hf[k]);
         apply_grid(c, hf[k]);
      }
      SPX_CUDA(cudaMemcpy(b_pr.p, hf.data(), sizeof(spx::ProblemDescT<float>) * n, cudaMemcpyHostToDevice));
   }

   // candidates: the persistent work queue at three block sizes and four refill intervals (two of
   // each for FP64, whose samples take longer); the plain grid as well for FP64, the drop-in's
   // own schedule
   std::vector<spx_tuning> cands;
   if (f64) {
      for (int bs : {128, 64})
         for (int sps : {4, 16}) cands.push_back(spx_tuning{bs, 0, sps, 1});
      cands.push_back(spx_tuning{128, 0, 1 << 30, 0});
      cands.push_back(spx_tuning{64, 0, 1 << 30, 0});
   }
   else {
      for (int bs : {128, 64, 32})
         for (int sps : {2, 4, 8, 16}) cands.push_back(spx_tuning{bs, 0, sps, 1});
   }
   double best_rate = -1.0;
   spx_tuning best_tu = cands[0];
   for (spx_tuning tu : cands) {
      int occ = occupancy(c, tu.block_size, slots);
      if (occ <= 0) continue;
      tu.blocks_per_sm = occ;
      int64_t grid = tu.schedule == 1 ? (int64_t)c->sm_count * occ : (first + tu.block_size - 1) / tu.block_size;
      spx::LaunchArgs a;
      a.block = dim3(tu.block_size);
      a.grid = dim3((unsigned)std::max<int64_t>(1, std::min<int64_t>(grid, 0x7fffffff)));
      a.stream = c->stream;
      a.problems_r = b_pr.p;
      a.problems_d = static_cast<const spx::ProblemDesc*>(b_pd.p);
      a.cfg.traj_kind = c->traj;
      a.cfg.time_flow = c->flow;
      a.cfg.rk = c->rk;
      set_rk(c, a.cfg);
      a.cfg.deriv_mode = c->deriv_mode;
      a.cfg.pa_scattering = c->pa_scattering;
      a.cfg.mu_method = c->mu_method;
      a.cfg.perp_method = c->perp_method;
      a.cfg.max_attempts = c->max_attempts;
      a.cfg.steps_per_orbit = c->steps_per_orbit;
      a.cfg.steps_per_orbit_f = (float)c->steps_per_orbit;
      a.cfg.record_final = 0;
      a.cfg.n_problems = n;
      a.cfg.steps_per_sync = tu.steps_per_sync;
      a.cfg.step_cap = 2048;
      a.cfg.total_traj = first;
      a.cfg.run_index = 0;
      a.ctr = static_cast<spx::RunCounters*>(b_ctr.p);
      a.counts = static_cast<int32_t*>(b_counts.p);
      a.sums = static_cast<double*>(b_sums.p);
      a.n_events = static_cast<unsigned long long*>(b_nev.p);
      a.records = nullptr;
      a.queue = tu.schedule;
      a.bnd_slots = slots;
      SPX_CUDA(cudaMemsetAsync(b_ctr.p, 0, sizeof(spx::RunCounters), c->stream));
      SPX_CUDA(cudaEventRecord(c->ev0, c->stream));
      SPX_CUDA(launch(c, a));
      SPX_CUDA(cudaEventRecord(c->ev1, c->stream));
      SPX_CUDA(cudaStreamSynchronize(c->stream));
      float ms = 0.0f;
      SPX_CUDA(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
      spx::RunCounters h;
      SPX_CUDA(cudaMemcpy(&h, b_ctr.p, sizeof h, cudaMemcpyDeviceToHost));
      double rate = ms > 0.0f ? (double)h.steps / ms : 0.0;
      if (rate > best_rate) {
         best_rate = rate;
         best_tu = tu;
      }
   }
   if (best_rate <= 0.0) return SPX_ERR_CUDA;
   c->tuned = best_tu;
   c->has_tuned = true;
   c->launched = false;  // the timing events now describe a sample, not an spx_run
   if (best) *best = best_tu;
   return SPX_OK;
}

int spx_sync(spx_ctx_t c, spx_stats* stats)
{
   if (!valid_ctx(c)) return SPX_ERR_INVALID_ARG;
   if (!c->launched) return SPX_ERR_STATE;
   SPX_CUDA(cudaStreamSynchronize(c->stream));
   spx::RunCounters h;
   SPX_CUDA(cudaMemcpy(&h, c->d_ctr, sizeof h, cudaMemcpyDeviceToHost));
   float ms = 0.0f;
   SPX_CUDA(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
   c->last.kernel_ms = ms;
   c->last.trajectories = (int64_t)h.finished + (int64_t)h.given_up;
   c->last.steps = (int64_t)h.steps;
   c->last.retries = (int64_t)h.retries;
   c->last.given_up = (int64_t)h.given_up;
   c->last.events = (int64_t)h.events;
   if (stats) *stats = c->last;
   if (h.error != 0) return SPX_ERR_DEVICE;
   return SPX_OK;
}

int spx_get_distribution_info(spx_ctx_t c, int problem, int distro, int64_t* n_bins, int* width)
{
   if (!valid_ctx(c) || problem < 0 || problem >= (int)c->problems.size()) return SPX_ERR_INVALID_ARG;
   const spx::ProblemDesc& pd = c->problems[problem].pd;
   if (distro < 0 || distro >= pd.nd) return SPX_ERR_INVALID_ARG;
   if (n_bins) *n_bins = (int64_t)pd.d[distro].n_bins[0] * pd.d[distro].n_bins[1] * pd.d[distro].n_bins[2];
   if (width) *width = pd.d[distro].width;
   return SPX_OK;
}

int spx_get_distribution(spx_ctx_t c, int problem, int distro, int32_t* counts, double* sums, int64_t* n_events)
{
   int64_t nb = 0;
   int w = 0;
   int rc = spx_get_distribution_info(c, problem, distro, &nb, &w);
   if (rc != SPX_OK) return rc;
   if (c->dirty || c->d_counts == nullptr) {
      if (counts) std::memset(counts, 0, sizeof(int32_t) * nb);
      if (sums) std::memset(sums, 0, sizeof(double) * nb * w);
      if (n_events) *n_events = 0;
      return SPX_OK;
   }
   SPX_CUDA(cudaStreamSynchronize(c->stream));
   const spx::DistParams& d = c->problems[problem].pd.d[distro];
   if (counts) SPX_CUDA(cudaMemcpy(counts, c->d_counts + d.offset_counts, sizeof(int32_t) * nb, cudaMemcpyDeviceToHost));
   if (sums) SPX_CUDA(cudaMemcpy(sums, c->d_sums + d.offset_sums, sizeof(double) * nb * w, cudaMemcpyDeviceToHost));
   if (n_events) {
      unsigned long long ne = 0;
      SPX_CUDA(cudaMemcpy(&ne, c->d_nev + (int64_t)problem * spx::kMaxDistro + distro, sizeof ne, cudaMemcpyDeviceToHost));
      *n_events = (int64_t)ne;
   }
   return SPX_OK;
}

int64_t spx_get_records(spx_ctx_t c, int problem, spx_traj_record* out, int64_t max_records)
{
   if (!valid_ctx(c) || problem < 0 || problem >= (int)c->problems.size() || (!out && max_records > 0))
      return SPX_ERR_INVALID_ARG;
   if (!c->record_final || c->d_rec == nullptr || !c->launched) return SPX_ERR_STATE;
   const spx::ProblemDesc& pd = c->problems[problem].pd;
   int64_t n = std::min<int64_t>(max_records, c->problems[problem].n_traj);
   if (n <= 0) return 0;
   cudaError_t e = cudaStreamSynchronize(c->stream);
   if (e == cudaSuccess) e = cudaMemcpy(out, c->d_rec + pd.first, sizeof(spx::TrajRecord) * n, cudaMemcpyDeviceToHost);
   if (e != cudaSuccess) return cuda_err(e);
   return n;
}

int spx_reset_distributions(spx_ctx_t c)
{
   if (!valid_ctx(c)) return SPX_ERR_INVALID_ARG;
   if (c->d_counts == nullptr) return SPX_OK;
   SPX_CUDA(cudaMemsetAsync(c->d_counts, 0, sizeof(int32_t) * std::max<int64_t>(c->n_counts, 1), c->stream));
   SPX_CUDA(cudaMemsetAsync(c->d_sums, 0, sizeof(double) * std::max<int64_t>(c->n_sums, 1), c->stream));
   SPX_CUDA(cudaMemsetAsync(c->d_nev, 0, sizeof(unsigned long long) * c->problems.size() * spx::kMaxDistro, c->stream));
   if (c->d_rn)
      SPX_CUDA(cudaMemsetAsync(c->d_rn, 0, sizeof(unsigned long long) * c->problems.size() * spx::kMaxDistro, c->stream));
   SPX_CUDA(cudaStreamSynchronize(c->stream));
   return SPX_OK;
}

// The records slice of one keep_records distribution: device pointers and the slot count.
static bool record_slice(const spx_ctx* c, int problem, int distro, double** vals, double** wts, unsigned long long** n)
{
   if (c->d_rn == nullptr) return false;
   int64_t rv = 0, rw = 0;
   for (int k = 0; k < (int)c->problems.size(); k++)
      for (int d = 0; d < c->problems[k].pd.nd; d++) {
         const spx::DistParams& dp = c->problems[k].pd.d[d];
         if (!dp.keep_records) continue;
         if (k == problem && d == distro) {
            *vals = c->d_rvals + rv;
            *wts = c->d_rwts + rw;
            *n = c->d_rn + (int64_t)k * spx::kMaxDistro + d;
            return true;
         }
         rv += 3 * c->rec_capacity;
         rw += (int64_t)dp.width * c->rec_capacity;
      }
   return false;
}

int64_t spx_get_distribution_records(spx_ctx_t c, int problem, int distro, double* values, double* weights,
                                     int64_t max_records, int64_t* n_events)
{
   int64_t nb = 0;
   int w = 0;
   int rc = spx_get_distribution_info(c, problem, distro, &nb, &w);
   if (rc != SPX_OK) return rc;
   if (max_records < 0 || (max_records > 0 && (!values || !weights))) return SPX_ERR_INVALID_ARG;
   if (!c->problems[problem].pd.d[distro].keep_records) return SPX_ERR_STATE;
   double *dv = nullptr, *dw = nullptr;
   unsigned long long* dn = nullptr;
   if (c->dirty || !record_slice(c, problem, distro, &dv, &dw, &dn)) {
      if (n_events) *n_events = 0;
      return 0;
   }
   unsigned long long total = 0;
   SPX_CUDA(cudaStreamSynchronize(c->stream));
   SPX_CUDA(cudaMemcpy(&total, dn, sizeof total, cudaMemcpyDeviceToHost));
   if (n_events) *n_events = (int64_t)total;
   const int64_t k = std::min<int64_t>(std::min<int64_t>((int64_t)total, c->rec_capacity), max_records);
   if (k > 0) {
      SPX_CUDA(cudaMemcpy(values, dv, sizeof(double) * 3 * k, cudaMemcpyDeviceToHost));
      SPX_CUDA(cudaMemcpy(weights, dw, sizeof(double) * w * k, cudaMemcpyDeviceToHost));
   }
   return k;
}

// Checkpoint file: "SPXD" u32 version=1, u32 n_problems, i64 run_index, then per problem u32 nd and
// per distribution u64 n_bins, u32 width, i32 counts[n_bins], f64 sums[n_bins*width], i64 n_events.
int spx_dump(spx_ctx_t c, const char* path)
{
   if (!valid_ctx(c) || !path) return SPX_ERR_INVALID_ARG;
   FILE* f = std::fopen(path, "wb");
   if (!f) return SPX_ERR_IO;
   uint32_t hdr[3] = {0x44585053u, 1u, (uint32_t)c->problems.size()};
   bool ok = std::fwrite(hdr, sizeof hdr, 1, f) == 1 && std::fwrite(&c->run_index, 8, 1, f) == 1;
   for (int p = 0; ok && p < (int)c->problems.size(); p++) {
      const spx::ProblemDesc& pd = c->problems[p].pd;
      uint32_t nd = (uint32_t)pd.nd;
      ok = std::fwrite(&nd, 4, 1, f) == 1;
      for (int d = 0; ok && d < pd.nd; d++) {
         int64_t nb = 0;
         int w = 0;
         spx_get_distribution_info(c, p, d, &nb, &w);
         std::vector<int32_t> counts(nb);
         std::vector<double> sums(nb * w);
         int64_t ne = 0;
         if (spx_get_distribution(c, p, d, counts.data(), sums.data(), &ne) != SPX_OK) ok = false;
         uint64_t nbu = (uint64_t)nb;
         uint32_t wu = (uint32_t)w;
         ok = ok && std::fwrite(&nbu, 8, 1, f) == 1 && std::fwrite(&wu, 4, 1, f) == 1 &&
              std::fwrite(counts.data(), 4, nb, f) == (size_t)nb && std::fwrite(sums.data(), 8, nb * w, f) == (size_t)(nb * w) &&
              std::fwrite(&ne, 8, 1, f) == 1;
      }
   }
   ok = (std::fclose(f) == 0) && ok;
   return ok ? SPX_OK : SPX_ERR_IO;
}

int spx_restore(spx_ctx_t c, const char* path)
{
   if (!valid_ctx(c) || !path) return SPX_ERR_INVALID_ARG;
   if (c->problems.empty()) return SPX_ERR_STATE;
   if (c->dirty) {
      int rc = upload(c);
      if (rc != SPX_OK) return rc;
   }
   FILE* f = std::fopen(path, "rb");
   if (!f) return SPX_ERR_IO;
   uint32_t hdr[3];
   int64_t run_index = 0;
   bool ok = std::fread(hdr, sizeof hdr, 1, f) == 1 && hdr[0] == 0x44585053u && hdr[1] == 1u &&
             hdr[2] == c->problems.size() && std::fread(&run_index, 8, 1, f) == 1;
   for (int p = 0; ok && p < (int)c->problems.size(); p++) {
      const spx::ProblemDesc& pd = c->problems[p].pd;
      uint32_t nd = 0;
      ok = std::fread(&nd, 4, 1, f) == 1 && nd == (uint32_t)pd.nd;
      for (int d = 0; ok && d < pd.nd; d++) {
         uint64_t nb = 0;
         uint32_t w = 0;
         ok = std::fread(&nb, 8, 1, f) == 1 && std::fread(&w, 4, 1, f) == 1;
         int64_t nbe = 0;
         int we = 0;
         spx_get_distribution_info(c, p, d, &nbe, &we);
         ok = ok && (int64_t)nb == nbe && (int)w == we;
         if (!ok) break;
         std::vector<int32_t> counts(nb);
         std::vector<double> sums(nb * w);
         int64_t ne = 0;
         ok = std::fread(counts.data(), 4, nb, f) == nb && std::fread(sums.data(), 8, nb * w, f) == nb * w &&
              std::fread(&ne, 8, 1, f) == 1;
         if (!ok) break;
         const spx::DistParams& dp = pd.d[d];
         unsigned long long neu = (unsigned long long)ne;
         ok = cudaMemcpy(c->d_counts + dp.offset_counts, counts.data(), 4 * nb, cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(c->d_sums + dp.offset_sums, sums.data(), 8 * nb * w, cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(c->d_nev + (int64_t)p * spx::kMaxDistro + d, &neu, 8, cudaMemcpyHostToDevice) == cudaSuccess;
      }
   }
   std::fclose(f);
   if (!ok) return SPX_ERR_IO;
   c->run_index = run_index;  // trajectories after a restore continue with new ids
   return SPX_OK;
}

// One distribution in the file layout of DistributionTemplated::Dump (src/distribution_templated.cc:
// 394-425), native little-endian: u32 name length, the class name, one byte of Specie (a class of
// static members only, so sizeof is 1 and the byte is 0), u32 records and u32 bytes of the parameter
// container and its bytes, i32 n_events, i32 counts[bins], the per-bin sums (1, 3 or 9 doubles), then the
// record arrays: u32 n and the values (3 doubles each), u32 n and the weights (width doubles each); both
// are empty unless the distribution keeps records.
int spx_dump_distribution(spx_ctx_t c, int problem, int distro, const char* path)
{
   int64_t nb = 0;
   int w = 0;
   if (!path) return SPX_ERR_INVALID_ARG;
   int rc = spx_get_distribution_info(c, problem, distro, &nb, &w);
   if (rc != SPX_OK) return rc;
   const PluginBlob& pb = c->problems[problem].dist[distro];
   const char* name = distro_class_name(pb.kind);
   if (!name) return SPX_ERR_INVALID_ARG;
   std::vector<int32_t> counts(nb);
   std::vector<double> sums(nb * w);
   int64_t ne = 0;
   rc = spx_get_distribution(c, problem, distro, counts.data(), sums.data(), &ne);
   if (rc != SPX_OK) return rc;
   if (ne > INT32_MAX) return SPX_ERR_LIMIT;  // the file's event count is an int
   std::vector<double> rvals, rwts;
   uint32_t n_kept = 0;
   if (c->problems[problem].pd.d[distro].keep_records) {
      int64_t total = 0;
      int64_t k = spx_get_distribution_records(c, problem, distro, nullptr, nullptr, 0, &total);
      if (k < 0) return (int)k;
      const int64_t stored = std::min<int64_t>(total, c->rec_capacity);
      if (stored > (int64_t)UINT32_MAX) return SPX_ERR_LIMIT;
      rvals.resize(3 * stored);
      rwts.resize((size_t)w * stored);
      k = spx_get_distribution_records(c, problem, distro, rvals.data(), rwts.data(), stored, &total);
      if (k < 0) return (int)k;
      n_kept = (uint32_t)k;
   }
   FILE* f = std::fopen(path, "wb");
   if (!f) return SPX_ERR_IO;
   const uint32_t name_len = (uint32_t)std::strlen(name), n_rec = pb.n_records, blob_len = (uint32_t)pb.blob.size();
   const uint8_t specie = 0;
   const int32_t ne32 = (int32_t)ne;
   bool ok = put(f, &name_len, 1) && put(f, name, name_len) && put(f, &specie, 1) && put(f, &n_rec, 1) &&
             put(f, &blob_len, 1) && put(f, pb.blob.data(), blob_len) && put(f, &ne32, 1) &&
             put(f, counts.data(), (size_t)nb) && put(f, sums.data(), (size_t)(nb * w)) && put(f, &n_kept, 1) &&
             put(f, rvals.data(), 3 * (size_t)n_kept) && put(f, &n_kept, 1) && put(f, rwts.data(), (size_t)w * n_kept);
   ok = (std::fclose(f) == 0) && ok;
   return ok ? SPX_OK : SPX_ERR_IO;
}

// DistributionTemplated::Restore (src/distribution_templated.cc:433-466) for a distribution whose binning
// is already fixed by its problem: the file's class name and parameter container must equal this
// distribution's (else SPX_ERR_MISMATCH, where the reference returns without restoring); its counts,
// sums and event count replace the device histogram, and the file's records the distribution's records
// when it keeps them (SPX_ERR_TOO_LARGE beyond SPX_OPT_RECORD_CAPACITY); otherwise they are read past.
int spx_restore_distribution(spx_ctx_t c, int problem, int distro, const char* path)
{
   int64_t nb = 0;
   int w = 0;
   if (!path) return SPX_ERR_INVALID_ARG;
   int rc = spx_get_distribution_info(c, problem, distro, &nb, &w);
   if (rc != SPX_OK) return rc;
   const PluginBlob& pb = c->problems[problem].dist[distro];
   const char* name = distro_class_name(pb.kind);
   if (!name) return SPX_ERR_INVALID_ARG;
   if (c->dirty) {
      rc = upload(c);
      if (rc != SPX_OK) return rc;
   }
   FILE* f = std::fopen(path, "rb");
   if (!f) return SPX_ERR_IO;
   rc = SPX_OK;
   uint32_t name_len = 0, n_rec = 0, blob_len = 0, n_values = 0, n_weights = 0;
   uint8_t specie = 0;
   int32_t ne = 0;
   std::string file_name;
   std::vector<uint8_t> blob;
   std::vector<int32_t> counts(nb);
   std::vector<double> sums(nb * w);
   if (!get(f, &name_len, 1) || name_len > 4096) rc = SPX_ERR_IO;
   if (rc == SPX_OK) {
      file_name.resize(name_len);
      if (!get(f, file_name.data(), name_len)) rc = SPX_ERR_IO;
      else if (file_name != name) rc = SPX_ERR_MISMATCH;
   }
   if (rc == SPX_OK && !(get(f, &specie, 1) && get(f, &n_rec, 1) && get(f, &blob_len, 1))) rc = SPX_ERR_IO;
   if (rc == SPX_OK && blob_len != pb.blob.size()) rc = SPX_ERR_MISMATCH;
   if (rc == SPX_OK) {
      blob.resize(blob_len);
      if (!get(f, blob.data(), blob_len)) rc = SPX_ERR_IO;
      else if (blob != pb.blob || n_rec != pb.n_records) rc = SPX_ERR_MISMATCH;
   }
   const bool keep = c->problems[problem].pd.d[distro].keep_records != 0;
   std::vector<double> rvals, rwts;
   if (rc == SPX_OK && !(get(f, &ne, 1) && ne >= 0 && get(f, counts.data(), (size_t)nb) &&
                         get(f, sums.data(), (size_t)(nb * w)) && get(f, &n_values, 1)))
      rc = SPX_ERR_IO;
   if (rc == SPX_OK && keep && (int64_t)n_values > c->rec_capacity) rc = SPX_ERR_TOO_LARGE;
   if (rc == SPX_OK) {
      if (keep) {
         rvals.resize(3 * (size_t)n_values);
         if (!get(f, rvals.data(), rvals.size())) rc = SPX_ERR_IO;
      }
      else if (std::fseek(f, (long)n_values * 24, SEEK_CUR) != 0) rc = SPX_ERR_IO;
   }
   if (rc == SPX_OK && !get(f, &n_weights, 1)) rc = SPX_ERR_IO;
   if (rc == SPX_OK && keep) {
      if (n_weights != n_values) rc = SPX_ERR_IO;
      else {
         rwts.resize((size_t)w * n_weights);
         if (!get(f, rwts.data(), rwts.size())) rc = SPX_ERR_IO;
      }
   }
   std::fclose(f);
   if (rc != SPX_OK) return rc;
   if (keep) {
      double *dv = nullptr, *dw = nullptr;
      unsigned long long* dn = nullptr;
      if (!record_slice(c, problem, distro, &dv, &dw, &dn)) return SPX_ERR_STATE;
      const unsigned long long nv = n_values;
      SPX_CUDA(cudaStreamSynchronize(c->stream));
      if (n_values) {
         SPX_CUDA(cudaMemcpy(dv, rvals.data(), sizeof(double) * rvals.size(), cudaMemcpyHostToDevice));
         SPX_CUDA(cudaMemcpy(dw, rwts.data(), sizeof(double) * rwts.size(), cudaMemcpyHostToDevice));
      }
      SPX_CUDA(cudaMemcpy(dn, &nv, sizeof nv, cudaMemcpyHostToDevice));
   }
   const spx::DistParams& dp = c->problems[problem].pd.d[distro];
   const unsigned long long neu = (unsigned long long)ne;
   SPX_CUDA(cudaStreamSynchronize(c->stream));
   SPX_CUDA(cudaMemcpy(c->d_counts + dp.offset_counts, counts.data(), sizeof(int32_t) * nb, cudaMemcpyHostToDevice));
   SPX_CUDA(cudaMemcpy(c->d_sums + dp.offset_sums, sums.data(), sizeof(double) * nb * w, cudaMemcpyHostToDevice));
   SPX_CUDA(cudaMemcpy(c->d_nev + (int64_t)problem * spx::kMaxDistro + distro, &neu, sizeof neu, cudaMemcpyHostToDevice));
   return SPX_OK;
}

const char* spx_strerror(int code)
{
   switch (code) {
   case SPX_OK: return "success";
   case SPX_ERR_INVALID_ARG: return "invalid argument";
   case SPX_ERR_UNKNOWN_PLUGIN: return "unknown plugin kind for this role or trajectory type";
   case SPX_ERR_BAD_BLOB: return "malformed parameter blob";
   case SPX_ERR_INCOMPLETE: return "simulation not ready: background, time/space/momentum initial conditions, a time boundary (and a diffusion model for Parker) are required";
   case SPX_ERR_CUDA: return "CUDA runtime error";
   case SPX_ERR_OUT_OF_MEMORY: return "out of device memory";
   case SPX_ERR_LIMIT: return "capacity exceeded (4 boundaries per class, 4 distributions, 2^32 trajectory ids)";
   case SPX_ERR_STATE: return "call out of order";
   case SPX_ERR_DEVICE: return "the kernel reported an error (distribution action out of range)";
   case SPX_ERR_NO_DEVICE: return "no sm_103 CUDA device";
   case SPX_ERR_IO: return "checkpoint file error";
   case SPX_ERR_TOO_LARGE: return "size beyond a fixed capacity";
   case SPX_ERR_MISMATCH: return "dump file written for another distribution class or parameter set";
   default: return "unknown error";
   }
}

void spx_destroy(spx_ctx_t c)
{
   if (!c) return;
   if (c->stream) cudaStreamSynchronize(c->stream);
   drop_graph(c);
   free_buffers(c);
   cudaFree(c->d_grid64);
   cudaFree(c->d_grid32);
   if (c->ev0) cudaEventDestroy(c->ev0);
   if (c->ev1) cudaEventDestroy(c->ev1);
   if (c->stream) cudaStreamDestroy(c->stream);
   delete c;
}

const char* spx_version(void) { return "spectrum_gb300 0.1 (sm_103a)"; }

}  // extern "C"

// ---- spx_run_static: the same launch with no device allocation ---------------------------------
// For callers that cannot call cudaMalloc: code that runs where the device allocator is off
// limits (inside a host framework that owns all device memory through its own pool, or on a
// latency-critical path where cudaMalloc's implicit device synchronisation is not acceptable).
// Such a caller passes its own device buffers for the outputs; the scratch memory the launch needs
// -- the run counters, whose first word is the work-queue head, and the device copies of the
// problem descriptors -- lives in one fixed array compiled into the library.
//
// Every GPU that loads the library holds this array until the process exits. All calls share it
// and it keeps the last call's contents: each call clears the run counters before its launch and
// overwrites the descriptors. Calls whose launches overlap on the GPU (two host threads, two
// contexts or two streams at once) race on it and give wrong results.
static __device__ __align__(256) unsigned char spx_static_scratch[SPX_STATIC_SCRATCH_BYTES];

namespace {

constexpr size_t kStaticCounterBytes = 256;  // RunCounters, padded to the array's alignment
static_assert(sizeof(spx::RunCounters) <= kStaticCounterBytes, "run counters exceed their slot");

std::mutex g_static_mu;
void* g_static_ptr[256] = {};

// The array's device address on the current device. Looked up once per device, on the first call
// made with that device current (the look-up may load the library's device code on that device).
int static_scratch(int device, unsigned char** out)
{
   if (device < 0 || device >= 256) return SPX_ERR_NO_DEVICE;
   std::lock_guard<std::mutex> lock(g_static_mu);
   if (g_static_ptr[device] == nullptr) {
      void* ptr = nullptr;
      cudaError_t e = cudaGetSymbolAddress((void**)&ptr, spx_static_scratch);
      if (e != cudaSuccess) return cuda_err(e);
      g_static_ptr[device] = ptr;
   }
   *out = static_cast<unsigned char*>(g_static_ptr[device]);
   return SPX_OK;
}

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

}  // namespace

extern "C" {

int spx_run_static(spx_ctx_t c, const spx_tuning* tuning, int32_t* counts, int64_t n_counts, double* sums,
                   int64_t n_sums, unsigned long long* n_events, int64_t n_events_len, spx_traj_record* records,
                   int64_t n_records, spx_stats* stats)
{
   if (!valid_ctx(c)) return SPX_ERR_INVALID_ARG;
   if (c->problems.empty() || grid_missing(c)) return SPX_ERR_STATE;
   const int n = (int)c->problems.size();
   const bool f64 = c->precision == SPX_FP64;

   // the layout of the distributions and trajectories, on copies of the descriptors
   std::vector<spx::ProblemDesc> hd(n);
   int64_t off_c = 0, off_s = 0, total = 0;
   for (int k = 0; k < n; k++) {
      hd[k] = c->problems[k].pd;
      apply_grid(c, hd[k]);
      hd[k].first = total;
      hd[k].n_traj = c->problems[k].n_traj;
      total += hd[k].n_traj;
      for (int d = 0; d < hd[k].nd; d++) {
         int64_t nb = (int64_t)hd[k].d[d].n_bins[0] * hd[k].d[d].n_bins[1] * hd[k].d[d].n_bins[2];
         hd[k].d[d].offset_counts = off_c;
         hd[k].d[d].offset_sums = off_s;
         off_c += nb;
         off_s += nb * hd[k].d[d].width;
      }
   }

   // scratch: [run counters | FP64 descriptors | FP32 descriptors (mixed precision only)]
   const size_t off_pd = kStaticCounterBytes;
   const size_t bytes_pd = sizeof(spx::ProblemDesc) * n;
   const size_t off_pr = f64 ? off_pd : align_up(off_pd + bytes_pd, 256);
   const size_t bytes_pr = f64 ? 0 : sizeof(spx::ProblemDescT<float>) * n;
   const size_t need = f64 ? off_pd + bytes_pd : off_pr + bytes_pr;
   if (need > (size_t)SPX_STATIC_SCRATCH_BYTES) return SPX_ERR_TOO_LARGE;

   // the caller's outputs
   if (!counts || !sums || !n_events) return SPX_ERR_INVALID_ARG;
   if (n_counts < off_c || n_sums < off_s || n_events_len < (int64_t)n * spx::kMaxDistro) return SPX_ERR_INVALID_ARG;
   if (c->record_final && (!records || n_records < total)) return SPX_ERR_INVALID_ARG;
   for (const auto& p : c->problems)
      if ((uint64_t)(c->run_index + 1) * (uint64_t)p.n_traj > 0x100000000ull) return SPX_ERR_LIMIT;

   SPX_CUDA(cudaSetDevice(c->device));
   unsigned char* scratch = nullptr;
   int rc = static_scratch(c->device, &scratch);
   if (rc != SPX_OK) return rc;

   // launch shape: chosen as spx_run chooses it (the caller's, the autotuned one, or the defaults)
   spx_tuning tu;
   const int slots = bnd_slots(c);
   rc = resolve_tuning(c, tuning, slots, tu);
   if (rc != SPX_OK) return rc;
   int64_t grid = tu.schedule == 1 ? (int64_t)c->sm_count * tu.blocks_per_sm : (total + tu.block_size - 1) / tu.block_size;
   grid = std::max<int64_t>(1, std::min<int64_t>(grid, 0x7fffffff));

   // descriptors into the scratch, counters cleared
   std::vector<spx::ProblemDescT<float>> hf;
   SPX_CUDA(cudaMemsetAsync(scratch, 0, kStaticCounterBytes, c->stream));
   SPX_CUDA(cudaMemcpyAsync(scratch + off_pd, hd.data(), bytes_pd, cudaMemcpyHostToDevice, c->stream));
   if (!f64) {
      hf.resize(n);
      for (int k = 0; k < n; k++) {
         spx::convert_problem(hd[k], hf[k]);
         apply_grid(c, hf[k]);
      }
      SPX_CUDA(cudaMemcpyAsync(scratch + off_pr, hf.data(), bytes_pr, cudaMemcpyHostToDevice, c->stream));
   }

   spx::LaunchArgs a;
   a.block = dim3(tu.block_size);
   a.grid = dim3((unsigned)grid);
   a.stream = c->stream;
   a.problems_r = scratch + off_pr;
   a.problems_d = reinterpret_cast<const spx::ProblemDesc*>(scratch + off_pd);
   a.cfg.traj_kind = c->traj;
   a.cfg.time_flow = c->flow;
   a.cfg.rk = c->rk;
   set_rk(c, a.cfg);
   a.cfg.deriv_mode = c->deriv_mode;
   a.cfg.pa_scattering = c->pa_scattering;
   a.cfg.mu_method = c->mu_method;
   a.cfg.perp_method = c->perp_method;
   a.cfg.max_attempts = c->max_attempts;
   a.cfg.steps_per_orbit = c->steps_per_orbit;
   a.cfg.steps_per_orbit_f = (float)c->steps_per_orbit;
   a.cfg.record_final = c->record_final;
   a.cfg.n_problems = n;
   a.cfg.steps_per_sync = tu.steps_per_sync;
   a.cfg.step_cap = c->step_cap;
   a.cfg.total_traj = total;
   a.cfg.run_index = c->run_index;
   a.ctr = reinterpret_cast<spx::RunCounters*>(scratch);
   a.counts = counts;
   a.sums = sums;
   a.n_events = n_events;
   a.records = c->record_final ? reinterpret_cast<spx::TrajRecord*>(records) : nullptr;
   a.queue = tu.schedule;
   a.bnd_slots = slots;
   SPX_CUDA(cudaEventRecord(c->ev0, c->stream));
   SPX_CUDA(launch(c, a));
   SPX_CUDA(cudaEventRecord(c->ev1, c->stream));
   SPX_CUDA(cudaStreamSynchronize(c->stream));
   c->run_index++;

   spx::RunCounters h;
   SPX_CUDA(cudaMemcpy(&h, scratch, sizeof h, cudaMemcpyDeviceToHost));
   if (stats) {
      float ms = 0.0f;
      SPX_CUDA(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
      *stats = spx_stats{};
      stats->kernel_ms = ms;
      stats->trajectories = (int64_t)h.finished + (int64_t)h.given_up;
      stats->steps = (int64_t)h.steps;
      stats->retries = (int64_t)h.retries;
      stats->given_up = (int64_t)h.given_up;
      stats->events = (int64_t)h.events;
      stats->kernel_launches = 1;
      stats->tuning = tu;
   }
   return h.error != 0 ? SPX_ERR_DEVICE : SPX_OK;
}

}  // extern "C"
