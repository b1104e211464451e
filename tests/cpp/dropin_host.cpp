// Compiles against include/rt_tilings.hpp as a reference user would (the reference's
// Examples/*.cpp shape) and exercises the host utilities; prints the checked values.
#include <cstdio>

#include "rt_tilings.hpp"

int main() {
  rt::domain d = rt::DominoTiler::AztecDiamond(5);
  rt::tiling tmax = rt::DominoTiler::MaxTiling(d);
  rt::tiling tmin = rt::DominoTiler::MinTiling(d);
  rt::heightfunc h = rt::DominoTiler::TilingToHeightfunc(tmax, d);
  rt::tiling back = rt::DominoTiler::HeightfuncToTiling(h, d);
  long sum_max = 0, sum_min = 0;
  for (int v : tmax) sum_max += v;
  for (int v : tmin) sum_min += v;
  std::printf("side %d max %ld min %ld roundtrip %d\n", rt::side_of(tmax), sum_max, sum_min, back == tmax ? 1 : 0);
  try {
    rt::DominoTiler::MaxTiling(rt::DominoTiler::Rectangle(3, 3));
    std::printf("untileable not detected\n");
  } catch (const rt::Error& e) {
    std::printf("untileable status %d\n", e.status);
  }
  // the other models' host utilities, as the reference's MinimalLozenge / RectTriangle /
  // TriangleDimer examples call them
  rt::domain hexd = rt::LozengeTiler::AlmostHexDomain(4, 0);
  rt::tiling lmax = rt::LozengeTiler::MaxTiling(hexd);
  rt::tiling rmax = rt::RectTriangleTiler::maxHex(5);
  rt::tiling cone = rt::TriangleDimerTiler::IceCreamCone(6, 0);
  rt::domain coned = rt::TriangleDimerTiler::TilingToDomain(cone);
  rt::heightfunc smin = rt::SixVertexTiler::MinHeight(5);
  std::vector<int> asmx = rt::SixVertexTiler::HeightToASM(smin);
  long cone_cells = 0, asm_sum = 0;
  for (int v : coned) cone_cells += v;
  for (int v : asmx) asm_sum += v;
  std::printf("lozenge %d recttri %d cone %d cells %ld asm %ld\n", rt::side_of(lmax), rt::side_of(rmax),
              rt::side_of(cone), cone_cells, asm_sum);
  return 0;
}
