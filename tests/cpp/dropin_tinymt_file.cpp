// The reference's OpenCL-path usage of a parameter file (construct the tiler,
// LoadTinyMT(file, size), Walk(T, steps, seed)) for the lozenge, rectangle-triangle and
// bibone tilers, against include/rt_tilings.hpp; prints the tiling after the walk, one value
// per line.  Arguments: model (lozenge | recttri | bibone), parameter file, number of
// parameter sets, steps, seed.  Start states: the minimal tiling of the side-5 hexagon,
// minHex(5), IceCreamCone(7, 0).
#include <cstdio>
#include <cstdlib>
#include <string>

#include "rt_tilings.hpp"

int main(int argc, char** argv) {
  if (argc != 6) {
    std::fprintf(stderr, "usage: %s lozenge|recttri|bibone params.txt size steps seed\n", argv[0]);
    return 2;
  }
  const std::string model = argv[1], path = argv[2];
  const int size = std::atoi(argv[3]), steps = std::atoi(argv[4]);
  const long seed = std::atol(argv[5]);
  rt::tiling T;
  if (model == "lozenge") {
    rt::LozengeTiler L;
    T = rt::LozengeTiler::MinTiling(rt::LozengeTiler::Hexagon(5));
    L.LoadTinyMT(path, size);
    L.Walk(T, steps, seed);
  } else if (model == "recttri") {
    rt::RectTriangleTiler R;
    T = rt::RectTriangleTiler::minHex(5);
    R.LoadTinyMT(path, size);
    R.Walk(T, steps, seed);
  } else if (model == "bibone") {
    rt::TriangleDimerTiler B;
    T = rt::TriangleDimerTiler::IceCreamCone(7, 0);
    B.LoadTinyMT(path, size);
    B.Walk(T, steps, seed);
  } else {
    return 2;
  }
  for (int v : T) std::printf("%d\n", v);
  return 0;
}
