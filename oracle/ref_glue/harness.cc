/*
 * harness.cc -- drives the reference's own TrajectoryType as a test oracle (never shipped).
 *
 * The reference's MPI driver (src/simulation.cc) cannot be built without MPI, so this harness
 * repeats what a worker does per trajectory (src/simulation.cc:262-288): SetStart(); Integrate();
 * and on an exception, a retry of the same slot with fresh random numbers. Plugins are created
 * from the reference classes by name and set up from the same DataContainer byte blobs that the
 * CUDA library's C ABI receives (common/data_container.cc:139-224 gives the layout).
 *
 * Input (little-endian, written by spectrum_gb300/problem.py):
 *   "SPXS" u32 version=1, u64 seed, u32 n_traj, u32 problem, u32 normals_per_step,
 *   u32 max_attempts, u32 n_plugins,
 *   per plugin: u32 role, u32 name_len, name, u32 n_records, u32 blob_len, blob
 *   roles: 0 background, 1 diffusion, 2 source, 3 boundary, 4 initial, 5 distribution
 * Output:
 *   "SPXR" u32 n_traj, u32 n_distro,
 *   per trajectory: u32 attempts, u32 status, u64 steps, f64 t, f64 pos[3], f64 mom[3],
 *                   f64 t0, f64 pos0[3], f64 mom0[3], f64 amp, f64 logwgt
 *   per distribution: u32 n_bins, u32 width, i32 counts[n_bins], f64 sums[n_bins*width],
 *                     i32 n_events
 * With a third argument, each distribution is also written by its own Dump() to
 * <dump_prefix><index>.out, and by its Print1D, Print2D and PrintRecords.
 */
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "config.h"
#include "src/traj_config.hh"
#include "src/background_uniform.hh"
#include "src/background_shock.hh"
#include "src/background_smooth_shock.hh"
#include "src/background_discontinuity.hh"
#include "src/background_smooth_discontinuity.hh"
#include "src/background_dipole.hh"
#include "src/background_solarwind.hh"
#include "src/diffusion_other.hh"
#include "src/boundary_time.hh"
#include "src/boundary_space.hh"
#include "src/boundary_momentum.hh"
#include "src/initial_time.hh"
#include "src/initial_space.hh"
#include "src/initial_momentum.hh"
#include "src/distribution_other.hh"
#include "src/source_other.hh"
#include "gsl_standin_ctl.h"

using namespace Spectrum;

namespace {

struct Reader {
   std::vector<uint8_t> buf;
   size_t pos = 0;
   template <typename T> T get()
   {
      if (pos + sizeof(T) > buf.size()) throw std::runtime_error("truncated spec");
      T v;
      std::memcpy(&v, buf.data() + pos, sizeof(T));
      pos += sizeof(T);
      return v;
   }
   std::vector<uint8_t> bytes(size_t n)
   {
      if (pos + n > buf.size()) throw std::runtime_error("truncated spec");
      std::vector<uint8_t> v(buf.begin() + pos, buf.begin() + pos + n);
      pos += n;
      return v;
   }
};

/* Access to the protected state of the reference trajectory after Integrate(). */
struct Probe : public TrajectoryType {
   double T() const { return _t; }
   GeoVector Pos() const { return _pos; }
   GeoVector Mom() const { return _mom; }
   double T0() const { return traj_t[0]; }
   GeoVector Pos0() const { return traj_pos[0]; }
   GeoVector Mom0() const { return traj_mom[0]; }
   double Amp() const { return _amp; }
   double LogWgt() const { return _wgt; }
   uint16_t Status() const { return _status; }
};

DataContainer MakeContainer(const std::vector<uint8_t>& blob, size_t n_records)
{
   DataContainer c;
   c.resize(n_records, blob.size());
   if (!blob.empty()) std::memcpy(c.data(), blob.data(), blob.size());
   c.Reset();
   return c;
}

#define SPX_TRY_BG(T) if (name == #T) { traj.AddBackground(T(), c); return; }
#define SPX_TRY_DIFF(T) if (name == #T) { traj.AddDiffusion(T(), c); return; }
#define SPX_TRY_SRC(T) if (name == #T) { traj.AddSource(T(), c); return; }
#define SPX_TRY_BND(T) if (name == #T) { traj.AddBoundary(T(), c); return; }
#define SPX_TRY_INI(T) if (name == #T) { traj.AddInitial(T(), c); return; }
#define SPX_TRY_DIST(T) if (name == #T) { auto d = std::make_shared<T>(); d->SetupObject(c); traj.ConnectDistribution(d); distros.push_back(d); widths.push_back(W); return; }

void AddPlugin(Probe& traj, uint32_t role, const std::string& name, const DataContainer& c,
               std::vector<std::shared_ptr<DistributionBase>>& distros, std::vector<int>& widths)
{
   if (role == 0) {
      SPX_TRY_BG(BackgroundUniform)
      SPX_TRY_BG(BackgroundShock)
      SPX_TRY_BG(BackgroundSmoothShock)
      SPX_TRY_BG(BackgroundDiscontinuity)
      SPX_TRY_BG(BackgroundSmoothDiscontinuity)
      SPX_TRY_BG(BackgroundDipole)
      SPX_TRY_BG(BackgroundSolarWind)
   }
   else if (role == 1) {
#if (TRAJ_TYPE != TRAJ_PARKER) && (TRAJ_TYPE != TRAJ_PARKER_SOURCE)
      SPX_TRY_DIFF(DiffusionIsotropicConstant)
      SPX_TRY_DIFF(DiffusionQLTConstant)
      SPX_TRY_DIFF(DiffusionWNLTConstant)
      SPX_TRY_DIFF(DiffusionWNLTRampVLISM)
#endif
      SPX_TRY_DIFF(DiffusionParaConstant)
      SPX_TRY_DIFF(DiffusionPerpConstant)
      SPX_TRY_DIFF(DiffusionFullConstant)
      SPX_TRY_DIFF(DiffusionFlowMomentumPowerLaw)
      SPX_TRY_DIFF(DiffusionKineticEnergyRadialDistancePowerLaw)
      SPX_TRY_DIFF(DiffusionRigidityMagneticFieldPowerLaw)
      SPX_TRY_DIFF(DiffusionStraussEtAl2013)
      SPX_TRY_DIFF(DiffusionPotgieterEtAl2015)
      SPX_TRY_DIFF(DiffusionEmpiricalSOQLTandUNLT)
   }
   else if (role == 2) {
      SPX_TRY_SRC(SourceConstant)
      SPX_TRY_SRC(SourceMomentumInjection)
      SPX_TRY_SRC(SourceSphericalShockInjection)
   }
   else if (role == 3) {
      SPX_TRY_BND(BoundaryTimeExpire)
      SPX_TRY_BND(BoundaryTimePass)
      SPX_TRY_BND(BoundaryTimeRecurrent)
      SPX_TRY_BND(BoundaryPlaneAbsorb)
      SPX_TRY_BND(BoundaryPlaneReflect)
      SPX_TRY_BND(BoundaryPlanePass)
      SPX_TRY_BND(BoundaryBoxReflect)
      SPX_TRY_BND(BoundarySphereAbsorb)
      SPX_TRY_BND(BoundarySphereReflect)
      SPX_TRY_BND(BoundaryRankineAbsorb)
      SPX_TRY_BND(BoundaryCylinderAbsorb)
      SPX_TRY_BND(BoundaryRegionAbsorb)
      SPX_TRY_BND(BoundaryMomentumInject)
      SPX_TRY_BND(BoundaryMomentumPass)
      SPX_TRY_BND(BoundaryMomentumInjectRestrictSlab)
      SPX_TRY_BND(BoundaryMomentumInjectRestrictShell)
#if (TRAJ_TYPE != TRAJ_PARKER) && (TRAJ_TYPE != TRAJ_PARKER_SOURCE) && (TRAJ_TYPE != TRAJ_FIELDLINE)
      SPX_TRY_BND(BoundaryMirror)
#endif
   }
   else if (role == 4) {
      SPX_TRY_INI(InitialTimeFixed)
      SPX_TRY_INI(InitialTimeInterval)
      SPX_TRY_INI(InitialSpaceFixed)
      SPX_TRY_INI(InitialSpaceLine)
      SPX_TRY_INI(InitialSpaceCircle)
      SPX_TRY_INI(InitialSpaceBox)
      SPX_TRY_INI(InitialSpaceSphere)
      SPX_TRY_INI(InitialSpaceSphereSector)
      SPX_TRY_INI(InitialSpaceRankineHalfBody)
      SPX_TRY_INI(InitialSpaceCylinder)
      SPX_TRY_INI(InitialSpaceCylinderSector)
#if (TRAJ_TYPE == TRAJ_LORENTZ) || (TRAJ_TYPE == TRAJ_FIELDLINE)
      SPX_TRY_INI(InitialMomentumFixed)
#endif
#if (TRAJ_TYPE != TRAJ_PARKER) && (TRAJ_TYPE != TRAJ_PARKER_SOURCE) && (TRAJ_TYPE != TRAJ_FIELDLINE)
      SPX_TRY_INI(InitialMomentumBeam)
      SPX_TRY_INI(InitialMomentumRing)
#endif
      SPX_TRY_INI(InitialMomentumShell)
      SPX_TRY_INI(InitialMomentumThickShell)
      SPX_TRY_INI(InitialMomentumMaxwell)
   }
   else if (role == 5) {
      int W = 1;
      SPX_TRY_DIST(DistributionTimeUniform)
      SPX_TRY_DIST(DistributionPositionUniform)
      SPX_TRY_DIST(DistributionMomentumUniform)
      SPX_TRY_DIST(DistributionPositionMomentumUniform)
      SPX_TRY_DIST(DistributionSpectrumKineticEnergyPowerLaw)
      SPX_TRY_DIST(DistributionSpectrumKineticEnergyBentPowerLaw)
      SPX_TRY_DIST(DistributionDivergenceFlowPowerLaw)
#if SPX_REF_TRAJ == TRAJ_LORENTZ
      SPX_TRY_DIST(DistributionAnisotropyLISM)
#endif
      W = 3;
      SPX_TRY_DIST(DistributionPositionCumulativeOrder1)
      SPX_TRY_DIST(DistributionLossCone)
      W = 9;
      SPX_TRY_DIST(DistributionPositionCumulativeOrder2)
   }
   throw std::runtime_error("unknown plugin class for this trajectory type: " + name);
}

template <typename T> void Put(FILE* f, const T& v) { std::fwrite(&v, sizeof(T), 1, f); }

void PutVec(FILE* f, const GeoVector& v)
{
   for (int i = 0; i < 3; i++) Put<double>(f, v[i]);
}

}  // namespace

int main(int argc, char** argv)
{
   if (argc < 3) {
      std::fprintf(stderr, "usage: %s spec.bin out.bin [dump_prefix]\n", argv[0]);
      return 2;
   }
   Reader rd;
   {
      FILE* f = std::fopen(argv[1], "rb");
      if (!f) { std::perror(argv[1]); return 2; }
      std::fseek(f, 0, SEEK_END);
      long n = std::ftell(f);
      std::fseek(f, 0, SEEK_SET);
      rd.buf.resize(n);
      if (std::fread(rd.buf.data(), 1, n, f) != (size_t)n) { std::fclose(f); return 2; }
      std::fclose(f);
   }
   try {
      if (std::memcmp(rd.bytes(4).data(), "SPXS", 4) != 0) throw std::runtime_error("bad magic");
      if (rd.get<uint32_t>() != 1) throw std::runtime_error("bad version");
      uint64_t seed = rd.get<uint64_t>();
      uint32_t n_traj = rd.get<uint32_t>();
      uint32_t problem = rd.get<uint32_t>();
      uint32_t nps = rd.get<uint32_t>();
      uint32_t max_attempts = rd.get<uint32_t>();
      uint32_t n_plugins = rd.get<uint32_t>();

      spx_standin_configure(seed, (int)nps);
      auto rng = std::make_shared<RNG>(0);
      auto traj = std::make_unique<Probe>();
      traj->ConnectRNG(rng);
      std::vector<std::shared_ptr<DistributionBase>> distros;
      std::vector<int> widths;
      for (uint32_t p = 0; p < n_plugins; p++) {
         uint32_t role = rd.get<uint32_t>();
         uint32_t nl = rd.get<uint32_t>();
         auto nb = rd.bytes(nl);
         std::string name(nb.begin(), nb.end());
         uint32_t n_records = rd.get<uint32_t>();
         uint32_t bl = rd.get<uint32_t>();
         auto blob = rd.bytes(bl);
         AddPlugin(*traj, role, name, MakeContainer(blob, n_records), distros, widths);
      }

      FILE* out = std::fopen(argv[2], "wb");
      if (!out) { std::perror(argv[2]); return 2; }
      std::fwrite("SPXR", 1, 4, out);
      Put<uint32_t>(out, n_traj);
      Put<uint32_t>(out, (uint32_t)distros.size());
      auto t_start = std::chrono::steady_clock::now();
      uint64_t total_steps = 0;
      for (uint32_t k = 0; k < n_traj; k++) {
         uint32_t attempt = 0;
         bool done = false;
         while (!done && attempt < max_attempts) {
            spx_standin_begin(k, problem, attempt);
            attempt++;
            try {
               traj->SetStart();
               spx_standin_steps();
               traj->Integrate();
               done = true;
            }
            catch (std::exception& e) {
               std::fprintf(stderr, "trajectory %u attempt %u discarded: %s\n", k, attempt, e.what());
            }
         }
         uint64_t steps = (uint64_t)traj->Segments();
         total_steps += steps;
         Put<uint32_t>(out, attempt);
         Put<uint32_t>(out, (uint32_t)traj->Status() | (done ? 0u : 0x10000u));
         Put<uint64_t>(out, steps);
         Put<double>(out, traj->T());
         PutVec(out, traj->Pos());
         PutVec(out, traj->Mom());
         Put<double>(out, traj->T0());
         PutVec(out, traj->Pos0());
         PutVec(out, traj->Mom0());
         Put<double>(out, traj->Amp());
         Put<double>(out, traj->LogWgt());
      }
      double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
      for (size_t d = 0; d < distros.size(); d++) {
         MultiIndex nb = distros[d]->NBins();
         uint32_t nbins = (uint32_t)nb.Prod();
         size_t dsize = 0;
         const double* sums = (const double*)distros[d]->GetDistroAddress(dsize);
         Put<uint32_t>(out, nbins);
         Put<uint32_t>(out, (uint32_t)widths[d]);
         std::fwrite(distros[d]->GetCountsAddress(), sizeof(int), nbins, out);
         std::fwrite(sums, sizeof(double), (size_t)nbins * widths[d], out);
         Put<int32_t>(out, distros[d]->NEvents());
      }
      std::fclose(out);
      // the reference's own dump files, named as its simulation names them (src/simulation.cc:790-793),
      // and its text output of each distribution: Print1D of every axis, Print2D of every pair, PrintRecords,
      // each in code and in physical units (<prefix><d>.p1d<k>[u], .p2d<k1><k2>[u], .prec[u])
      if (argc > 3)
         for (size_t d = 0; d < distros.size(); d++) {
            const std::string base = std::string(argv[3]) + std::to_string(d);
            distros[d]->Dump(base + ".out");
            for (int u = 0; u < 2; u++) {
               const std::string us = u ? "u" : "";
               for (int k = 0; k < 3; k++) distros[d]->Print1D(k, base + ".p1d" + std::to_string(k) + us, u);
               for (int k1 = 0; k1 < 3; k1++)
                  for (int k2 = k1 + 1; k2 < 3; k2++)
                     distros[d]->Print2D(k1, k2, base + ".p2d" + std::to_string(k1) + std::to_string(k2) + us, u);
               distros[d]->PrintRecords(base + ".prec" + us, u);
            }
         }
      std::fprintf(stderr, "harness: %u trajectories, %llu steps, %.3f s\n", n_traj,
                   (unsigned long long)total_steps, secs);
   }
   catch (std::exception& e) {
      std::fprintf(stderr, "harness error: %s\n", e.what());
      return 1;
   }
   return 0;
}
