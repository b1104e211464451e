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
  return 0;
}
