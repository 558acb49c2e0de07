// gcr_modulation.cc -- a reference-style application on the C++ host mirror: backward-time GCR
// modulation in the Parker spiral, one problem per energy, the LIS-weighted spectrum and the
// exit-time histogram at the boundaries. The set-up follows the order and parameter layout of
// the reference's own modulation run (runs/gcr_modulation_example.cc:76-332); only the includes
// and the simulation object differ.
//
//   build: g++ -std=c++17 -O2 -ffp-contract=off -I include spectrum_gb300/examples/gcr_modulation.cc
//              -L spectrum_gb300/_lib -lspx -Wl,-rpath,$PWD/spectrum_gb300/_lib -o gcr_modulation
//   run:   ./gcr_modulation <n_energies> <trajectories per energy> <years> <precision 0|1> <out prefix>
// Prints one line per energy: problem, kinetic energy (MeV), counts in the spectrum, weighted sum.
// With "--dump" as the only argument it prints the plugin blobs of a 4-energy set-up as hex
// (role, kind, records, bytes) and exits without touching a GPU.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "spx_simulation.hh"

using namespace spx;
using namespace spx::units;

static void boundary_header(DataContainer& c, int max_crossings, const std::vector<int>& actions)
{
   c.Insert(max_crossings);
   c.Insert(actions);
}

// The plugin set-up, in the reference run's order, into any object with the Add* calls.
template <class Sink>
static void set_up(Sink& sim, const std::vector<double>& energies, double t_max)
{
   const int n_energies = (int)energies.size();
   const double one_au = astronomical_unit / unit_length;
   DataContainer container;

   // Background (runs/gcr_modulation_example.cc:40-78)
   container.Clear();
   container.Insert(0.0);
   container.Insert(gv_zeros);
   const double umag = 4.0e7 / unit_velocity;
   container.Insert(GeoVector(umag, 0.0, 0.0));
   const double rs = 6.957e10 / unit_length;
   const double r_ref = 3.0 * rs;
   const double bmag_e = 5.0e-5 / unit_magnetic;
   const double bmag_ref = bmag_e * std::pow(one_au / r_ref, 2.0);
   container.Insert(GeoVector(bmag_ref, 0.0, 0.0));
   container.Insert(one_au);
   const double w0 = 2.0 * M_PI / (25.0 * 24.0 * 3600.0) * unit_time;
   container.Insert(GeoVector(0.0, 0.0, w0));
   container.Insert(r_ref);
   container.Insert(0.1);
   sim.AddBackground(BackgroundSolarWind(), container);

   // Initial time and position
   container.Clear();
   container.Insert(0.0);
   sim.AddInitial(InitialTimeFixed(), container);
   container.Clear();
   container.Insert(GeoVector(one_au, 0.0, 0.0));
   sim.AddInitial(InitialSpaceFixed(), container);
   // Initial momentum of the first energy (the other energies replace it per problem below)
   container.Clear();
   container.Insert(MeVToMom(energies[0]));
   sim.AddInitial(InitialMomentumShell(), container);

   // Boundaries: inner sphere (cold for the spectrum), outer sphere (hot), time limit
   container.Clear();
   boundary_header(container, 1, {1, -1});
   container.Insert(gv_zeros);
   container.Insert(0.05 * one_au);
   sim.AddBoundary(BoundarySphereAbsorb(), container);
   container.Clear();
   boundary_header(container, 1, {0, 0});
   container.Insert(gv_zeros);
   container.Insert(100.0 * one_au);
   sim.AddBoundary(BoundarySphereAbsorb(), container);
   container.Clear();
   boundary_header(container, 1, {-1, -1});
   container.Insert(-t_max);
   sim.AddBoundary(BoundaryTimeExpire(), container);

   // Diffusion: kappa_par = (lam0 v / 3)(R/R0)^0.5 (B/B0)^-1, kappa_perp = 0.02 kappa_par
   container.Clear();
   container.Insert(0.1 * one_au);
   container.Insert(3.33e6 / (unit_energy / unit_charge));
   container.Insert(bmag_e);
   container.Insert(0.5);
   container.Insert(-1.0);
   container.Insert(0.02);
   sim.AddDiffusion(DiffusionRigidityMagneticFieldPowerLaw(), container);

   // Distribution 0: LIS-weighted kinetic-energy spectrum, 4 log bins per energy
   const double unit_distro = 1.0 / (unit_length * unit_length * unit_time * 4.0 * M_PI * unit_energy);
   container.Clear();
   container.Insert(MultiIndex(4 * n_energies, 0, 0));
   container.Insert(GeoVector(EnrKin(MeVToMom(energies.front())) * 0.5, 0.0, 0.0));
   container.Insert(GeoVector(EnrKin(MeVToMom(energies.back())) * 2.0, 0.0, 0.0));
   container.Insert(MultiIndex(1, 0, 0));
   container.Insert(MultiIndex(0, 0, 0));
   container.Insert(unit_distro);
   container.Insert(GeoVector(unit_energy, 1.0, 1.0));
   container.Insert(false);
   container.Insert(1.0 / unit_distro);
   container.Insert(1.0e9 * electron_volt / unit_energy);
   container.Insert(-1.8);
   container.Insert(0.0);
   sim.AddDistribution(DistributionSpectrumKineticEnergyPowerLaw(), container);

   // Distribution 1: exit time, 32 bins from 0 to -t_max, outliers into the end bins
   container.Clear();
   container.Insert(MultiIndex(32, 0, 0));
   container.Insert(GeoVector(0.0, 0.0, 0.0));
   container.Insert(GeoVector(-t_max, 0.0, 0.0));
   container.Insert(MultiIndex(0, 0, 0));
   container.Insert(MultiIndex(1, 0, 0));
   container.Insert(1.0);
   container.Insert(GeoVector(unit_time, 1.0, 1.0));
   container.Insert(false);
   container.Insert(1.0);
   container.Insert(0.0);
   container.Insert(1);
   sim.AddDistribution(DistributionTimeUniform(), container);
}

// Prints each plugin's blob instead of adding it (a check of the byte layout without a GPU).
struct BlobPrinter {
   void print(int role, int kind, const DataContainer& c)
   {
      std::printf("%d %d %zu ", role, kind, c.size());
      for (size_t i = 0; i < c.length(); i++) std::printf("%02x", c.data()[i]);
      std::printf("\n");
   }
   void AddBackground(const BackgroundBase& p, const DataContainer& c) { print(SPX_ROLE_BACKGROUND, p.kind, c); }
   void AddDiffusion(const DiffusionBase& p, const DataContainer& c) { print(SPX_ROLE_DIFFUSION, p.kind, c); }
   void AddBoundary(const BoundaryBase& p, const DataContainer& c) { print(SPX_ROLE_BOUNDARY, p.kind, c); }
   void AddInitial(const InitialBase& p, const DataContainer& c) { print(SPX_ROLE_INITIAL, p.kind, c); }
   void AddDistribution(const DistributionBase& p, const DataContainer& c) { print(SPX_ROLE_DISTRIBUTION, p.kind, c); }
};

static std::vector<double> log_energies(int n)
{
   const double e1 = 10.0, e2 = 1.0e4;
   std::vector<double> e;
   for (int i = 0; i < n; i++) e.push_back(n > 1 ? e1 * std::pow(e2 / e1, (double)i / (n - 1)) : e1);
   return e;
}

int main(int argc, char** argv)
{
   const double years_dump = 1.0;
   if (argc == 2 && std::string(argv[1]) == "--dump") {
      BlobPrinter printer;
      set_up(printer, log_energies(4), years_dump * 365.0 * 24.0 * 3600.0 / unit_time);
      return 0;
   }
   const int n_energies = argc > 1 ? std::atoi(argv[1]) : 32;
   const int n_traj = argc > 2 ? std::atoi(argv[2]) : 1000;
   const double years = argc > 3 ? std::atof(argv[3]) : 1.0;
   const int precision = argc > 4 ? std::atoi(argv[4]) : SPX_MIXED;
   const std::string prefix = argc > 5 ? argv[5] : "gcr_";
   const double t_max = years * 365.0 * 24.0 * 3600.0 / unit_time;
   const std::vector<double> energies = log_energies(n_energies);

   SimulationGPU sim(SPX_TRAJ_PARKER, SPX_BACKWARD, 0, precision, 0x5EED0000u + 4);
   set_up(sim, energies, t_max);

   // One problem per energy: the momentum sampler (initial slot 2) replaced per problem
   for (int k = 0; k < n_energies; k++) {
      DataContainer mom;
      mom.Insert(MeVToMom(energies[k]));
      std::vector<uint8_t> ov;
      auto put32 = [&ov](uint32_t v) { for (int b = 0; b < 4; b++) ov.push_back((uint8_t)(v >> (8 * b))); };
      if (k > 0) {
         put32(SPX_ROLE_INITIAL);
         put32(2);
         put32((uint32_t)InitialMomentumShell().kind);
         put32((uint32_t)mom.size());
         put32((uint32_t)mom.length());
         ov.insert(ov.end(), mom.data(), mom.data() + mom.length());
      }
      int rc = spx_add_problem(sim.context(), n_traj, 0x5EED0000u + 4, ov.data(), ov.size());
      if (rc < 0) {
         std::fprintf(stderr, "spx_add_problem: %s\n", spx_strerror(rc));
         return 1;
      }
   }

   spx_stats st = sim.MainLoop();
   std::fprintf(stderr, "%s: %lld trajectories, %lld steps, %.1f ms\n", sim.GetTrajectoryName().c_str(),
                (long long)st.trajectories, (long long)st.steps, st.kernel_ms);
   for (int k = 0; k < n_energies; k++) {
      int64_t nb = 0;
      int w = 0;
      spx_get_distribution_info(sim.context(), k, 0, &nb, &w);
      std::vector<int32_t> counts(nb);
      std::vector<double> sums(nb * w);
      int64_t nev = 0;
      spx_get_distribution(sim.context(), k, 0, counts.data(), sums.data(), &nev);
      long long c = 0;
      double s = 0.0;
      for (int64_t i = 0; i < nb; i++) { c += counts[i]; s += sums[i * w]; }
      std::printf("%d %.6e %lld %.12e\n", k, energies[k], c, s);
   }
   sim.PrintDistro1D(1, 0, prefix + "exit_time.dat", false, 0);
   return 0;
}
