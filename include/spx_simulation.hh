// spx_simulation.hh -- C++ host mirror of the reference's simulation interface on top of the C ABI
// of spx.h (header only).
//
// A reference application builds DataContainer parameter blobs and hands them, with a prototype
// object, to SimulationWorker::Add{Background,Diffusion,Source,Boundary,Initial,Distribution}, then
// calls SetTasks and MainLoop and prints or restores distributions (src/simulation.hh:93-138). This
// header gives the same calls the same names and arguments:
//   - spx::DataContainer writes the reference's record layout (one size byte, then the payload;
//     common/data_container.cc:139-224), with Insert for double, int, bool, GeoVector, MultiIndex,
//     GeoMatrix and std::vector;
//   - one empty prototype type per plugin class (BackgroundSolarWind(), BoundaryTimeExpire(), ...),
//     carrying the class's role and kind;
//   - spx::SimulationGPU, whose methods forward to spx_add_plugin / spx_add_problem / spx_run /
//     spx_get_distribution.
// An application changes its includes and the CreateSimulation call; everything between stays.
#ifndef SPX_SIMULATION_HH
#define SPX_SIMULATION_HH

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <stdexcept>
#include <string>
#include <vector>

#include "spx.h"

namespace spx {

// ---- code units of the reference (common/specie.hh:30-82, common/physical_constants.hh) ------------
namespace units {
constexpr double speed_of_light = 2.99792458e10;   // cm/s
constexpr double mass_proton = 1.67262192596e-24;  // g
constexpr double electron_charge = 4.8032044e-10;  // Fr
constexpr double electron_volt = 1.602176634e-12;  // erg
constexpr double astronomical_unit = 1.495978707e13;  // cm
constexpr double unit_length = 1.0e10;
constexpr double unit_velocity = 0.1 * speed_of_light;
constexpr double unit_mass = mass_proton;
constexpr double unit_charge = electron_charge;
constexpr double unit_momentum = unit_mass * unit_velocity;
constexpr double unit_energy = unit_mass * unit_velocity * unit_velocity;
constexpr double unit_time = unit_length / unit_velocity;
constexpr double unit_magnetic = unit_momentum / (unit_charge * unit_time);
constexpr double c_code = speed_of_light / unit_velocity;
// proton kinematics in code units (common/physics.hh:274-316)
inline double EnrTot(double p) { return std::sqrt(p * p + c_code * c_code) * c_code; }
inline double EnrKin(double p) { return EnrTot(p) - c_code * c_code; }
inline double Mom(double enr_kin) { return std::sqrt(enr_kin * (enr_kin + 2.0 * c_code * c_code)) / c_code; }
inline double Vel(double p) { return p * c_code * c_code / EnrTot(p); }
inline double MeVToMom(double e_mev) { return Mom(e_mev * (1.0e6 * electron_volt) / unit_energy); }
}  // namespace units

// ---- parameter containers ------------------------------------------------------------------------
struct GeoVector {
   double x[3];
   GeoVector(double a = 0.0, double b = 0.0, double c = 0.0) : x{a, b, c} {}
   double& operator[](int i) { return x[i]; }
   double operator[](int i) const { return x[i]; }
};

struct MultiIndex {
   int i[3];
   MultiIndex(int a = 0, int b = 0, int c = 0) : i{a, b, c} {}
};

struct GeoMatrix {
   GeoVector row[3];
};

const GeoVector gv_zeros(0.0, 0.0, 0.0);
const GeoVector gv_ones(1.0, 1.0, 1.0);
const GeoVector gv_nz(0.0, 0.0, 1.0);

// The reference's positional parameter blob: per Insert one record of [size byte][payload].
class DataContainer {
   std::vector<uint8_t> bytes_;
   size_t records_ = 0;

   void put(const void* p, size_t n)
   {
      if (n > 255) throw std::length_error("a DataContainer record holds at most 255 bytes");
      bytes_.push_back((uint8_t)n);
      const uint8_t* b = static_cast<const uint8_t*>(p);
      bytes_.insert(bytes_.end(), b, b + n);
      records_++;
   }

public:
   void Clear(void) { bytes_.clear(); records_ = 0; }
   void Insert(double v) { put(&v, sizeof v); }
   void Insert(int v) { put(&v, sizeof v); }
   void Insert(bool v) { uint8_t b = v ? 1 : 0; put(&b, 1); }
   void Insert(const GeoVector& v) { put(v.x, sizeof v.x); }
   void Insert(const MultiIndex& v) { put(v.i, sizeof v.i); }
   void Insert(const GeoMatrix& m)
   {
      double a[9];
      for (int r = 0; r < 3; r++)
         for (int c = 0; c < 3; c++) a[3 * r + c] = m.row[r][c];
      put(a, sizeof a);
   }
   template <typename T>
   void Insert(const std::vector<T>& v) { put(v.data(), v.size() * sizeof(T)); }
   const uint8_t* data(void) const { return bytes_.data(); }
   size_t length(void) const { return bytes_.size(); }
   size_t size(void) const { return records_; }
};

// ---- plugin prototypes ---------------------------------------------------------------------------
struct BackgroundBase { int kind; };
struct DiffusionBase { int kind; };
struct SourceBase { int kind; };
struct BoundaryBase { int kind; };
struct InitialBase { int kind; };
struct DistributionBase { int kind; };

#define SPX_PROTOTYPE(name, base, k) \
   struct name : base {              \
      name() : base{k} {}            \
   };
SPX_PROTOTYPE(BackgroundUniform, BackgroundBase, 1)
SPX_PROTOTYPE(BackgroundShock, BackgroundBase, 2)
SPX_PROTOTYPE(BackgroundSmoothShock, BackgroundBase, 3)
SPX_PROTOTYPE(BackgroundDipole, BackgroundBase, 4)
SPX_PROTOTYPE(BackgroundSolarWind, BackgroundBase, 5)
SPX_PROTOTYPE(BackgroundServerCartesian, BackgroundBase, 6)
SPX_PROTOTYPE(BackgroundDiscontinuity, BackgroundBase, 7)
SPX_PROTOTYPE(BackgroundSmoothDiscontinuity, BackgroundBase, 8)
SPX_PROTOTYPE(DiffusionIsotropicConstant, DiffusionBase, 1)
SPX_PROTOTYPE(DiffusionQLTConstant, DiffusionBase, 2)
SPX_PROTOTYPE(DiffusionParaConstant, DiffusionBase, 3)
SPX_PROTOTYPE(DiffusionPerpConstant, DiffusionBase, 4)
SPX_PROTOTYPE(DiffusionFullConstant, DiffusionBase, 5)
SPX_PROTOTYPE(DiffusionFlowMomentumPowerLaw, DiffusionBase, 6)
SPX_PROTOTYPE(DiffusionKineticEnergyRadialDistancePowerLaw, DiffusionBase, 7)
SPX_PROTOTYPE(DiffusionRigidityMagneticFieldPowerLaw, DiffusionBase, 8)
SPX_PROTOTYPE(DiffusionStraussEtAl2013, DiffusionBase, 9)
SPX_PROTOTYPE(DiffusionPotgieterEtAl2015, DiffusionBase, 10)
SPX_PROTOTYPE(DiffusionEmpiricalSOQLTandUNLT, DiffusionBase, 11)
SPX_PROTOTYPE(DiffusionWNLTConstant, DiffusionBase, 12)
SPX_PROTOTYPE(DiffusionWNLTRampVLISM, DiffusionBase, 13)
SPX_PROTOTYPE(SourceConstant, SourceBase, 1)
SPX_PROTOTYPE(SourceMomentumInjection, SourceBase, 2)
SPX_PROTOTYPE(SourceSphericalShockInjection, SourceBase, 3)
SPX_PROTOTYPE(BoundaryTimeExpire, BoundaryBase, 1)
SPX_PROTOTYPE(BoundaryTimePass, BoundaryBase, 2)
SPX_PROTOTYPE(BoundaryTimeRecurrent, BoundaryBase, 3)
SPX_PROTOTYPE(BoundaryPlaneAbsorb, BoundaryBase, 10)
SPX_PROTOTYPE(BoundaryPlaneReflect, BoundaryBase, 11)
SPX_PROTOTYPE(BoundaryPlanePass, BoundaryBase, 12)
SPX_PROTOTYPE(BoundaryBoxReflect, BoundaryBase, 13)
SPX_PROTOTYPE(BoundarySphereAbsorb, BoundaryBase, 14)
SPX_PROTOTYPE(BoundarySphereReflect, BoundaryBase, 15)
SPX_PROTOTYPE(BoundaryRankineAbsorb, BoundaryBase, 16)
SPX_PROTOTYPE(BoundaryCylinderAbsorb, BoundaryBase, 17)
SPX_PROTOTYPE(BoundaryRegionAbsorb, BoundaryBase, 18)
SPX_PROTOTYPE(BoundarySpherePass, BoundaryBase, 19)  // extension: no reference class
SPX_PROTOTYPE(BoundaryMomentumInject, BoundaryBase, 30)
SPX_PROTOTYPE(BoundaryMomentumPass, BoundaryBase, 31)
SPX_PROTOTYPE(BoundaryMomentumInjectRestrictSlab, BoundaryBase, 32)
SPX_PROTOTYPE(BoundaryMomentumInjectRestrictShell, BoundaryBase, 33)
SPX_PROTOTYPE(BoundaryMirror, BoundaryBase, 34)
SPX_PROTOTYPE(InitialTimeFixed, InitialBase, 1)
SPX_PROTOTYPE(InitialTimeInterval, InitialBase, 2)
SPX_PROTOTYPE(InitialSpaceFixed, InitialBase, 10)
SPX_PROTOTYPE(InitialSpaceLine, InitialBase, 11)
SPX_PROTOTYPE(InitialSpaceCircle, InitialBase, 12)
SPX_PROTOTYPE(InitialSpaceBox, InitialBase, 13)
SPX_PROTOTYPE(InitialSpaceSphere, InitialBase, 14)
SPX_PROTOTYPE(InitialSpaceSphereSector, InitialBase, 15)
SPX_PROTOTYPE(InitialSpaceRankineHalfBody, InitialBase, 16)
SPX_PROTOTYPE(InitialSpaceCylinder, InitialBase, 17)
SPX_PROTOTYPE(InitialSpaceCylinderSector, InitialBase, 18)
SPX_PROTOTYPE(InitialMomentumFixed, InitialBase, 30)
SPX_PROTOTYPE(InitialMomentumBeam, InitialBase, 31)
SPX_PROTOTYPE(InitialMomentumRing, InitialBase, 32)
SPX_PROTOTYPE(InitialMomentumShell, InitialBase, 33)
SPX_PROTOTYPE(InitialMomentumThickShell, InitialBase, 34)
SPX_PROTOTYPE(InitialMomentumMaxwell, InitialBase, 35)
SPX_PROTOTYPE(InitialMomentumLogEnergyPitchBand, InitialBase, 40)  // extension: no reference class
SPX_PROTOTYPE(InitialSpaceEquatorialBand, InitialBase, 41)  // extension: no reference class
SPX_PROTOTYPE(DistributionTimeUniform, DistributionBase, 1)
SPX_PROTOTYPE(DistributionPositionUniform, DistributionBase, 2)
SPX_PROTOTYPE(DistributionMomentumUniform, DistributionBase, 3)
SPX_PROTOTYPE(DistributionPositionMomentumUniform, DistributionBase, 4)
SPX_PROTOTYPE(DistributionSpectrumKineticEnergyPowerLaw, DistributionBase, 5)
SPX_PROTOTYPE(DistributionSpectrumKineticEnergyBentPowerLaw, DistributionBase, 6)
SPX_PROTOTYPE(DistributionPositionCumulativeOrder1, DistributionBase, 7)
SPX_PROTOTYPE(DistributionPositionCumulativeOrder2, DistributionBase, 8)
SPX_PROTOTYPE(DistributionDivergenceFlowPowerLaw, DistributionBase, 9)
SPX_PROTOTYPE(DistributionLossCone, DistributionBase, 10)
SPX_PROTOTYPE(DistributionAnisotropyLISM, DistributionBase, 11)  // Lorentz trajectories only
SPX_PROTOTYPE(DistributionTimeMu, DistributionBase, 20)  // extension: no reference class
#undef SPX_PROTOTYPE

// ---- the data files of the Cartesian server -------------------------------------------------------
// What BackgroundServerCartesian's server reads for the file-name pattern it is given: the reader's blocks
// (4^3 zones of six fluid-unit numbers each, blocks x fastest) from <pattern>.out, and the header from the
// same name with its last four characters replaced by ".info": blocks per axis, domain minimum and
// maximum, variables per zone (ServerCartesianBack::ServerStart, src/server_cartesian.cc:931-933;
// ReadCartesianHeader and ReadCartesianData, src/reader_cartesian.cc:30-133).
struct CartesianData {
   int32_t n_blocks[3] = {0, 0, 0};
   double domain_min[3] = {0, 0, 0}, domain_max[3] = {0, 0, 0};
   std::vector<double> values;

   // false on a missing or short file, or a header that does not give six variables per zone
   bool Read(const std::string& data_file)
   {
      if (data_file.size() < 4) return false;
      std::ifstream header((data_file.substr(0, data_file.size() - 4) + ".info").c_str());
      int nvar = 0;
      header >> n_blocks[0] >> n_blocks[1] >> n_blocks[2] >> domain_min[0] >> domain_min[1] >> domain_min[2] >>
          domain_max[0] >> domain_max[1] >> domain_max[2] >> nvar;
      if (!header || nvar != 6 || n_blocks[0] < 1 || n_blocks[1] < 1 || n_blocks[2] < 1) return false;
      const size_t n = (size_t)n_blocks[0] * n_blocks[1] * n_blocks[2] * 64 * 6;
      values.assign(n, 0.0);
      std::ifstream data(data_file.c_str(), std::ios::binary);
      data.read(reinterpret_cast<char*>(values.data()), (std::streamsize)(n * sizeof(double)));
      return (bool)data;
   }
};

// ---- text output of a distribution ---------------------------------------------------------------
// DistributionTemplated::Print1D, Print2D and PrintRecords (src/distribution_templated.cc:472-686),
// written from a distribution's parameter container, histogram and records. The binning is
// SetupDistribution's (src/distribution_templated.cc:92-137); the files go through an std::ofstream as
// the reference writes them: a comment line, an empty line, then rows of setw(20) columns at 10
// significant digits (PrintRecords keeps the stream's default 6).
struct DistroLayout {
   int n_bins[3] = {1, 1, 1}, log_bins[3] = {0, 0, 0}, width = 1;
   double limits0[3] = {0, 0, 0}, bin_size[3] = {0, 0, 0}, unit_distro[9] = {}, unit_val[3] = {1, 1, 1};

   // From the container's first seven records; false if they are not those of a DistributionTemplated
   // of this width (1, 3 or 9 doubles per bin).
   bool Read(const uint8_t* blob, size_t len, int width_in)
   {
      const size_t expect[7] = {12, 24, 24, 12, 12, 8 * (size_t)width_in, 24};
      const uint8_t* rec[7];
      size_t pos = 0;
      for (int r = 0; r < 7; r++) {
         if (pos >= len || blob[pos] != expect[r] || pos + 1 + blob[pos] > len) return false;
         rec[r] = blob + pos + 1;
         pos += 1 + blob[pos];
      }
      double minval[3], maxval[3];
      width = width_in;
      std::memcpy(n_bins, rec[0], 12);
      std::memcpy(minval, rec[1], 24);
      std::memcpy(maxval, rec[2], 24);
      std::memcpy(log_bins, rec[3], 12);
      std::memcpy(unit_distro, rec[5], 8 * (size_t)width);
      std::memcpy(unit_val, rec[6], 24);
      for (int k = 0; k < 3; k++) {
         n_bins[k] = std::max(n_bins[k], 1);
         const double lo = log_bins[k] ? std::log10(minval[k]) : minval[k];
         const double hi = log_bins[k] ? std::log10(maxval[k]) : maxval[k];
         limits0[k] = lo;
         bin_size[k] = (hi - lo) / n_bins[k];
      }
      return true;
   }

   // DistributionBase::BinCent (src/distribution_base.hh:267-272)
   double BinCent(int ijk, int bin) const
   {
      if (bin < 0 || bin >= n_bins[ijk]) return 0.0;
      const double x = limits0[ijk] + (bin + 0.5) * bin_size[ijk];
      return log_bins[ijk] ? std::pow(10.0, x) : x;
   }

   long Lin(const int b[3]) const { return ((long)b[0] * n_bins[1] + b[1]) * n_bins[2] + b[2]; }

   // PrintSumDistro (src/distribution_templated.cc:472-535): the mean and the sum of the weights
   void SumColumns(std::ofstream& f, long n, const double* s, bool phys) const
   {
      if (width == 1) {
         f << std::setw(20) << (n ? s[0] / n : 0.0) * (phys ? unit_distro[0] : 1.0) << std::setw(20)
           << s[0] * (phys ? unit_distro[0] : 1.0);
      }
      else if (n) {
         for (int i = 0; i < width; i++) f << std::setw(20) << (phys ? s[i] / n * unit_distro[i] : s[i] / n);
         for (int i = 0; i < width; i++) f << std::setw(20) << (phys ? s[i] * unit_distro[i] : s[i]);
      }
      else
         for (int i = 0; i < 2 * width; i++) f << std::setw(20) << 0.0;
   }

   // Print1D: axis ijk, the other two collapsed
   void Print1D(const std::string& path, const int32_t* counts, const double* sums, long long n_events, int ijk,
                bool phys) const
   {
      if (ijk < 0 || ijk >= 3) return;
      const int i1 = (ijk + 1) % 3, i2 = (ijk + 2) % 3;
      std::ofstream f(path.c_str());
      f << "# Total number of events: " << n_events << std::endl << std::endl;
      f << std::setprecision(10);
      int b[3];
      for (b[ijk] = 0; b[ijk] < n_bins[ijk]; b[ijk]++) {
         long n = 0;
         double s[9] = {};
         for (b[i1] = 0; b[i1] < n_bins[i1]; b[i1]++)
            for (b[i2] = 0; b[i2] < n_bins[i2]; b[i2]++) {
               const long k = Lin(b);
               n += counts[k];
               for (int w = 0; w < width; w++) s[w] += sums[k * width + w];
            }
         f << std::setw(20) << BinCent(ijk, b[ijk]) * (phys ? unit_val[ijk] : 1.0);
         SumColumns(f, n, s, phys);
         f << std::setw(20) << n << std::endl;
      }
   }

   // Print2D: axes ijk1 and ijk2, the third collapsed; Print1D for equal axes
   void Print2D(const std::string& path, const int32_t* counts, const double* sums, long long n_events, int ijk1,
                int ijk2, bool phys) const
   {
      if (ijk1 < 0 || ijk1 >= 3 || ijk2 < 0 || ijk2 >= 3) return;
      if (ijk1 == ijk2) {
         Print1D(path, counts, sums, n_events, ijk1, phys);
         return;
      }
      const int ijk = 3 - ijk1 - ijk2;
      std::ofstream f(path.c_str());
      f << "# Total number of events: " << n_events << std::endl << std::endl;
      f << std::setprecision(10);
      int b[3];
      for (b[ijk1] = 0; b[ijk1] < n_bins[ijk1]; b[ijk1]++)
         for (b[ijk2] = 0; b[ijk2] < n_bins[ijk2]; b[ijk2]++) {
            long n = 0;
            double s[9] = {};
            for (b[ijk] = 0; b[ijk] < n_bins[ijk]; b[ijk]++) {
               const long k = Lin(b);
               n += counts[k];
               for (int w = 0; w < width; w++) s[w] += sums[k * width + w];
            }
            f << std::setw(20) << BinCent(ijk1, b[ijk1]) * (phys ? unit_val[ijk1] : 1.0) << std::setw(20)
              << BinCent(ijk2, b[ijk2]) * (phys ? unit_val[ijk2] : 1.0);
            SumColumns(f, n, s, phys);
            f << std::setw(20) << n << std::endl;
         }
   }

   // PrintRecords with PrintWeight (src/distribution_templated.cc:643-682): three values, the weight(s)
   void PrintRecords(const std::string& path, const double* values, const double* weights, size_t n, bool phys) const
   {
      std::ofstream f(path.c_str());
      f << "# Total number of records: " << n << std::endl << std::endl;
      for (size_t i = 0; i < n; i++) {
         for (int j = 0; j < 3; j++) f << std::setw(20) << values[3 * i + j] * (phys ? unit_val[j] : 1.0);
         for (int w = 0; w < width; w++) f << std::setw(20) << weights[i * width + w] * (phys ? unit_distro[w] : 1.0);
         f << std::endl;
      }
   }
};

// ---- the simulation object -----------------------------------------------------------------------
class SimulationGPU {
   spx_ctx_t ctx_ = nullptr;
   int traj_;
   uint64_t seed_;
   std::string prefix_;
   std::vector<std::string> distro_names_;

   void check(int rc, const char* what) const
   {
      if (rc < 0) throw std::runtime_error(std::string(what) + ": " + spx_strerror(rc));
   }
   void add(int role, int kind, const DataContainer& c, const char* what)
   {
      check(spx_add_plugin(ctx_, role, kind, c.data(), c.length(), c.size()), what);
   }

public:
   // traj_kind, time_flow and rk are the reference's configure-time TRAJ_TYPE, TRAJ_TIME_FLOW and
   // RK_INTEGRATOR_TYPE (configure.ac:236-295); precision is SPX_FP64 or SPX_MIXED.
   SimulationGPU(int traj_kind, int time_flow, int rk, int precision, uint64_t seed = 0x5EED0000u)
      : traj_(traj_kind), seed_(seed)
   {
      check(spx_create(&ctx_, traj_kind, time_flow, rk, precision), "spx_create");
   }
   ~SimulationGPU() { if (ctx_) spx_destroy(ctx_); }
   SimulationGPU(const SimulationGPU&) = delete;
   SimulationGPU& operator=(const SimulationGPU&) = delete;

   spx_ctx_t context(void) const { return ctx_; }
   void SetOption(int option, double value) { check(spx_set_option(ctx_, option, value), "spx_set_option"); }

   // src/simulation.hh:105-123. With a file-name pattern a BackgroundServerCartesian reads its data as the
   // reference's server does (CartesianData); ghost_cells stands for the build's SERVER_NUM_GHOST_CELLS.
   void AddBackground(const BackgroundBase& p, const DataContainer& c, const std::string& fname_pattern = "",
                      int ghost_cells = 0)
   {
      add(SPX_ROLE_BACKGROUND, p.kind, c, "AddBackground");
      if (!fname_pattern.empty() && p.kind == BackgroundServerCartesian().kind) {
         CartesianData d;
         if (!d.Read(fname_pattern + ".out")) throw std::runtime_error("AddBackground: cannot read " + fname_pattern + ".out");
         SetBackgroundBlocks(d.n_blocks, d.domain_min, d.domain_max, ghost_cells, d.values.data());
      }
   }
   // The reader's blocks of a BackgroundServerCartesian background (spx_set_background_blocks).
   void SetBackgroundBlocks(const int32_t n_blocks[3], const double domain_min[3], const double domain_max[3],
                            int ghost_cells, const double* values)
   {
      check(spx_set_background_blocks(ctx_, n_blocks, domain_min, domain_max, ghost_cells, values), "SetBackgroundBlocks");
   }
   // The block of a BackgroundServerCartesian background (six values per node: U, B; x fastest),
   // in place of the data files the reference's server reads.
   void SetBackgroundGrid(const int64_t n[3], const double cent_min[3], const double zone_length[3], const double* values)
   {
      check(spx_set_background_grid(ctx_, n, cent_min, zone_length, values), "SetBackgroundGrid");
   }
   void AddDiffusion(const DiffusionBase& p, const DataContainer& c) { add(SPX_ROLE_DIFFUSION, p.kind, c, "AddDiffusion"); }
   void AddSource(const SourceBase& p, const DataContainer& c) { add(SPX_ROLE_SOURCE, p.kind, c, "AddSource"); }
   void AddBoundary(const BoundaryBase& p, const DataContainer& c) { add(SPX_ROLE_BOUNDARY, p.kind, c, "AddBoundary"); }
   void AddInitial(const InitialBase& p, const DataContainer& c) { add(SPX_ROLE_INITIAL, p.kind, c, "AddInitial"); }
   void AddDistribution(const DistributionBase& p, const DataContainer& c)
   {
      add(SPX_ROLE_DISTRIBUTION, p.kind, c, "AddDistribution");
      distro_names_.push_back(std::to_string(p.kind));
      distro_blobs_.emplace_back(c.data(), c.data() + c.length());
   }

   // src/simulation.hh:96-97: one problem of n_traj trajectories (the batch sizes of the MPI farm
   // have no meaning on the device and are ignored). Returns the problem index.
   int SetTasks(int n_traj, int = 0, int = 0)
   {
      check(spx_add_problem(ctx_, n_traj, seed_, nullptr, 0), "SetTasks");
      return n_problems_++;
   }

   std::string GetTrajectoryName(void) const
   {
      switch (traj_) {
      case SPX_TRAJ_FIELDLINE: return "TrajectoryFieldline";
      case SPX_TRAJ_LORENTZ: return "TrajectoryLorentz";
      case SPX_TRAJ_GUIDING: return "TrajectoryGuiding";
      case SPX_TRAJ_GUIDING_SCATT: return "TrajectoryGuidingScatt";
      case SPX_TRAJ_GUIDING_DIFF: return "TrajectoryGuidingDiff";
      case SPX_TRAJ_GUIDING_DIFF_SCATT: return "TrajectoryGuidingDiffScatt";
      case SPX_TRAJ_FOCUSED: return "TrajectoryFocused";
      case SPX_TRAJ_PARKER: return "TrajectoryParker";
      case SPX_TRAJ_PARKER_SOURCE: return "TrajectoryParkerSource";
      default: return "Trajectory";
      }
   }

   // Prefix of the dump files: distribution d of the first problem is <prefix><d>.out, the reference's
   // name (src/simulation.cc:790-793); of problem p > 0, <prefix><d>_problem<p>.out.
   void DistroFileName(const std::string& file_name) { prefix_ = file_name; }
   std::string DistroPath(int distro, int problem = 0) const
   {
      return prefix_ + std::to_string(distro) + (problem ? "_problem" + std::to_string(problem) : std::string()) + ".out";
   }

   // src/simulation.cc:705-793: restore the flagged distributions, every trajectory of every problem,
   // wait, and dump every distribution when a file name was given.
   spx_stats MainLoop(void)
   {
      for (int d : restore_)
         for (int p = 0; p < n_problems_; p++) {
            int rc = spx_restore_distribution(ctx_, p, d, DistroPath(d, p).c_str());
            // DistributionTemplated::Restore returns quietly on a missing file or another class
            if (rc != SPX_OK && rc != SPX_ERR_IO && rc != SPX_ERR_MISMATCH) check(rc, "RestoreDistro");
         }
      check(spx_run(ctx_, nullptr), "spx_run");
      spx_stats st;
      check(spx_sync(ctx_, &st), "spx_sync");
      if (!prefix_.empty()) DumpDistro();
      return st;
   }

   // SimulationMaster::RestoreDistro (src/simulation.cc:714-720): restore distribution d from its dump
   // file when MainLoop starts.
   void RestoreDistro(int distro) { restore_.push_back(distro); }

   // Every distribution of every problem in the reference's dump-file layout (DistributionTemplated::Dump).
   void DumpDistro(void)
   {
      for (int p = 0; p < n_problems_; p++)
         for (int d = 0; d < (int)distro_names_.size(); d++)
            check(spx_dump_distribution(ctx_, p, d, DistroPath(d, p).c_str()), "DumpDistro");
   }

   // The records of a distribution whose container set keep_records (DistributionTemplated::AddRecord):
   // values (3 per event) and weights (width per event), at most SPX_OPT_RECORD_CAPACITY of them.
   int64_t DistributionRecords(int distro, std::vector<double>& values, std::vector<double>& weights, int problem = 0) const
   {
      int64_t nb = 0, total = 0;
      int w = 0;
      check(spx_get_distribution_info(ctx_, problem, distro, &nb, &w), "DistributionRecords");
      int64_t k = spx_get_distribution_records(ctx_, problem, distro, nullptr, nullptr, 0, &total);
      if (k < 0) check((int)k, "DistributionRecords");
      values.assign(3 * (size_t)total, 0.0);
      weights.assign((size_t)w * total, 0.0);
      k = spx_get_distribution_records(ctx_, problem, distro, values.data(), weights.data(), total, &total);
      if (k < 0) check((int)k, "DistributionRecords");
      values.resize(3 * (size_t)k);
      weights.resize((size_t)w * k);
      return k;
   }

   // SimulationMaster::PrintDistro1D / PrintDistro2D / PrintRecords (src/simulation.cc:856-886): the
   // distribution of one problem in the reference's text layout (DistroLayout).
   void PrintDistro1D(int distro, int ijk, const std::string& file_name, bool phys_units, int problem = 0) const
   {
      std::vector<int32_t> counts;
      std::vector<double> sums;
      int64_t nev = 0;
      const DistroLayout L = histogram(distro, problem, counts, sums, nev, "PrintDistro1D");
      L.Print1D(file_name, counts.data(), sums.data(), nev, ijk, phys_units);
   }
   void PrintDistro2D(int distro, int ijk1, int ijk2, const std::string& file_name, bool phys_units, int problem = 0) const
   {
      std::vector<int32_t> counts;
      std::vector<double> sums;
      int64_t nev = 0;
      const DistroLayout L = histogram(distro, problem, counts, sums, nev, "PrintDistro2D");
      L.Print2D(file_name, counts.data(), sums.data(), nev, ijk1, ijk2, phys_units);
   }
   // The device appends records in completion order, the reference in trajectory order.
   void PrintRecords(int distro, const std::string& file_name, bool phys_units, int problem = 0) const
   {
      std::vector<double> values, weights;
      const int64_t n = DistributionRecords(distro, values, weights, problem);
      layout(distro, (int)(n ? weights.size() / n : width(distro, problem)), "PrintRecords")
          .PrintRecords(file_name, values.data(), weights.data(), (size_t)n, phys_units);
   }

private:
   int n_problems_ = 0;
   std::vector<int> restore_;
   std::vector<std::vector<uint8_t>> distro_blobs_;

   int width(int distro, int problem) const
   {
      int64_t nb = 0;
      int w = 0;
      check(spx_get_distribution_info(ctx_, problem, distro, &nb, &w), "spx_get_distribution_info");
      return w;
   }
   DistroLayout layout(int distro, int w, const char* what) const
   {
      DistroLayout L;
      if (distro < 0 || distro >= (int)distro_blobs_.size() ||
          !L.Read(distro_blobs_[distro].data(), distro_blobs_[distro].size(), w))
         throw std::runtime_error(std::string(what) + ": not a distribution of this simulation");
      return L;
   }
   DistroLayout histogram(int distro, int problem, std::vector<int32_t>& counts, std::vector<double>& sums, int64_t& nev,
                          const char* what) const
   {
      int64_t nb = 0;
      int w = 0;
      check(spx_get_distribution_info(ctx_, problem, distro, &nb, &w), what);
      counts.assign((size_t)nb, 0);
      sums.assign((size_t)nb * w, 0.0);
      check(spx_get_distribution(ctx_, problem, distro, counts.data(), sums.data(), &nev), what);
      return layout(distro, w, what);
   }
};

}  // namespace spx

#endif
