// Test oracle only: drives the reference's Cartesian data server -- the reader
// (src/reader_cartesian.cc), the blocks (src/block_base.cc, src/block_cartesian.cc) and the
// front end's GetVariables / GetGradients with first-order interpolation
// (src/server_cartesian.cc:549-865) -- on one process. Every block of the data file is loaded the
// way the back end serves it (SetNode, LoadDimensions(Fluid::unit_length), LoadNeighbors,
// LoadVariables) and put into the front end's cache, so that RequestBlock finds every block there
// and never sends a message (the MPI calls resolve to oracle/ref_glue/mpi/mpi.h).
//
// stdin:  "units" (prints the unit ratios and exits), or <data file (.dat, its .info beside it)> <dmax0>
//         then one position per line: x y z (code units)
// stdout, per position, with SERVER_NUM_GHOST_CELLS 0:
//         status U[3] B[3] Bmag E[3] dmax gradU[9] gradB[9] gradBmag[3]   (%.17g)
//         (SERVER_INTERP_ORDER 0 and -1: |B| of the converted B, as the background's EvaluateBmag forms it;
//         order -1 prints zero gradients, the background takes numerical ones)
//         with SERVER_NUM_GHOST_CELLS 1 (the reader fills no ghost zones, so only the geometry):
//         node cent_min[3] zone_length[3] zone[3] offset[3] weights[8] derivatives[24]
// "ERR" for a position whose evaluation throws.
#include <cstdio>
#include <iostream>
#include <memory>
#include <string>
#include <vector>

#include "src/server_cartesian.hh"
#include "src/block_cartesian.hh"
#include "src/reader_cartesian.hh"
#include "common/spatial_data.hh"

namespace Spectrum {
extern ReaderCartesian CartData;  // the reader's data (defined in src/reader_cartesian.cc, not declared in its header)
}

using namespace Spectrum;

struct Probe : public ServerCartesianFront {
   std::vector<BlockPtrType> blocks;

   void Start(const GeoVector& dmin, const GeoVector& dmax)
   {
      domain_min = dmin;
      domain_max = dmax;
      ServerStart();
   }

   void LoadAll(int n_nodes)
   {
      for (int n = 0; n < n_nodes; n++) {
         BlockPtrType b;
         MakeSharedBlock(b);
#if SERVER_NUM_GHOST_CELLS > 0
         b->SetGhostCells(SERVER_NUM_GHOST_CELLS);
#endif
         b->SetNode(n);
         b->LoadDimensions(Fluid::unit_length);
         b->LoadNeighbors();
         b->LoadVariables();
         b->ConfigureProperties();
         cache_line.AddBlock(b);
         blocks.push_back(b);
      }
   }

   int Status(void) const { return stencil_status; }

   // the stencil of the primary block of "pos", as BuildInterpolationStencil forms it
   void Geometry(const GeoVector& pos)
   {
      int node = cache_line.PosOwner(pos);
      if (node < 0) {
         std::printf("ERR\n");
         return;
      }
      BlockPtrType b = cache_line[node];
      MultiIndex zone_lo, zone_hi;
      GeoVector offset_lo, offset_hi, delta = b->GetZoneLength();
      b->GetZoneOffset(pos, zone_lo, offset_lo);
      offset_hi = 1.0 - offset_lo;
      zone_hi = zone_lo + 1;
      InteriorInterpolationStencil(zone_lo, zone_hi, offset_lo, offset_hi, delta);
      GeoVector cmin = b->GetFaceMin() + 0.5 * delta;
      std::printf("%d", node);
      for (int k = 0; k < 3; k++) std::printf(" %.17g", cmin[k]);
      for (int k = 0; k < 3; k++) std::printf(" %.17g", delta[k]);
      for (int k = 0; k < 3; k++) std::printf(" %d", zone_lo[k]);
      for (int k = 0; k < 3; k++) std::printf(" %.17g", offset_lo[k]);
      for (int c = 0; c < 8; c++) std::printf(" %.17g", stencil.weights[c]);
      for (int c = 0; c < 24; c++) std::printf(" %.17g", stencil.derivatives[c]);
      std::printf("\n");
   }
};

// SERVER_INTERP_ORDER -1: the front end asks the boss for the variables at a position (GetVariablesFromReader,
// src/server_cartesian.cc:381-447); the boss answers with the reader's interpolation at the position scaled back
// to file units (ServerCartesianBack, :1015-1017). Played here in process through the stand-in MPI header.
static int boss_answer(int tag, void* buf, int count)
{
   if (tag != tag_sendvars) return MPI_ERR_OTHER;
   const Inquiry* inq = static_cast<const Inquiry*>(spx_mpi_last_send());
   GeoVector pos_cart = inq->pos / Fluid::unit_length * Particle::unit_length;
   int found = 0;
   ReadCartesianGetBlockData(pos_cart.Data(), static_cast<double*>(buf), &found);
   (void)count;
   return MPI_SUCCESS;
}

int main(void)
{
   spx_mpi_recv_hook() = boss_answer;
   std::string path;
   double dmax0;
   if (!(std::cin >> path)) return 2;
   // "units": the Fluid-to-Particle ratios the front end applies, and the fluid speed of light
   if (path == "units") {
      std::printf("%.17g %.17g %.17g %.17g\n", Fluid::unit_length / Particle::unit_length,
                  Fluid::unit_velocity / Particle::unit_velocity, Fluid::unit_magnetic / Particle::unit_magnetic,
                  Fluid::c_code);
      return 0;
   }
   if (!(std::cin >> dmax0)) return 2;
   ReadCartesianData(path.c_str(), (int)path.size(), 1, 0);
   GeoVector dmin, dmax;
   ReadCartesianGetDomain(dmin.Data(), dmax.Data());
   dmin *= Fluid::unit_length / Particle::unit_length;
   dmax *= Fluid::unit_length / Particle::unit_length;
   Probe srv;
   srv.Start(dmin, dmax);
   srv.LoadAll(CartData.Nblocks.Prod());
   double x, y, z;
   while (std::cin >> x >> y >> z) {
      GeoVector pos(x, y, z);
#if SERVER_NUM_GHOST_CELLS > 0
      srv.Geometry(pos);
#else
      SpatialData sp;
      sp._mask = BACKGROUND_ALL;
      sp.dmax = dmax0;
      try {
         srv.GetVariables(0.0, pos, sp);
#if SERVER_INTERP_ORDER <= 0
         // the background's EvaluateBmag at these orders (src/background_base.cc:388-391)
         sp.Bmag = sp.Bvec.Norm();
#endif
#if SERVER_INTERP_ORDER == -1
         // GetGradients only flags the numerical derivatives the background then takes: none here
         sp.gradUvec = gm_zeros;
         sp.gradBvec = gm_zeros;
         sp.gradBmag = gv_zeros;
#else
         srv.GetGradients(sp);
#endif
      }
      catch (...) {
         std::printf("ERR\n");
         continue;
      }
      std::printf("%d", srv.Status());
      for (int k = 0; k < 3; k++) std::printf(" %.17g", sp.Uvec[k]);
      for (int k = 0; k < 3; k++) std::printf(" %.17g", sp.Bvec[k]);
      std::printf(" %.17g", sp.Bmag);
      for (int k = 0; k < 3; k++) std::printf(" %.17g", sp.Evec[k]);
      std::printf(" %.17g", sp.dmax);
      for (int a = 0; a < 3; a++)
         for (int b = 0; b < 3; b++) std::printf(" %.17g", sp.gradUvec[a][b]);
      for (int a = 0; a < 3; a++)
         for (int b = 0; b < 3; b++) std::printf(" %.17g", sp.gradBvec[a][b]);
      for (int k = 0; k < 3; k++) std::printf(" %.17g", sp.gradBmag[k]);
      std::printf("\n");
#endif
   }
   return 0;
}
