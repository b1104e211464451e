// The shape of the reference's CUDA examples (Examples/MinimalDominoEx.cpp: construct the
// tiler, LoadMTGP, Walk(T, 100, 34893)) against include/rt_tilings.hpp; prints the tiling
// after the walk, one value per line.  Argument: the Aztec diamond order of the start tiling.
#include <cstdio>
#include <cstdlib>

#include "rt_tilings.hpp"

int main(int argc, char** argv) {
  const int order = argc > 1 ? std::atoi(argv[1]) : 4;
  rt::tiling T = rt::DominoTiler::MaxTiling(rt::DominoTiler::AztecDiamond(order));
  rt::DominoTiler D;
  D.LoadMTGP();
  D.Walk(T, 100, 34893);
  for (int v : T) std::printf("%d\n", v);
  return 0;
}
