// Prints the reference's Butcher table for the RK_INTEGRATOR_TYPE this unit is compiled with, as
// exact hexadecimal doubles (test oracle only: it pins the tables of this library to the
// reference's common/rk_config.hh). One line: number, stages, order, adaptive, then a[stages],
// b[stages][stages] row by row, v[stages], w[stages].
#include <cstdio>

#include "common/rk_config.hh"

int main()
{
   using namespace Spectrum;
   const int s = RK_Table.stages;
   std::printf("%d %d %d %d", SPX_REF_RK, s, (int)RK_Table.order, RK_Table.adaptive ? 1 : 0);
   for (int i = 0; i < s; i++) std::printf(" %a", RK_Table.a[i]);
   for (int i = 0; i < s; i++)
      for (int j = 0; j < s; j++) std::printf(" %a", RK_Table.b[i][j]);
   for (int i = 0; i < s; i++) std::printf(" %a", RK_Table.v[i]);
   for (int i = 0; i < s; i++) std::printf(" %a", RK_Table.w[i]);
   std::printf("\n");
   return 0;
}
