// TEST INFRASTRUCTURE ONLY. extern "C" wrapper over the reference's RectTriangleTiler static
// host functions (src/RectTriangle/RectTriangleTiler.cpp:173-600), compiled from the
// reference tree by oracle/Makefile.
#include <cstdlib>
#include <cstring>
#include <cuda_runtime.h>
#include <curand_mtgp32.h>
#include "src/common/common.h"
#include "src/RectTriangle/RectTriangleTiler.h"

// Never called: only the static host utilities are used through this library.
void flipTiles(dim3, dim3, curandStateMtgp32*, int*, const int) { std::abort(); }
void updateTiles1(dim3, dim3, int*, int*, const int, const int) { std::abort(); }
void updateTiles2(dim3, dim3, int*, int*, const int, const int) { std::abort(); }

extern "C" int refh_rt_hex(int n, int which, int* out, long cap) {
  tiling t = which == 0 ? RectTriangleTiler::minHex(n) : which == 1 ? RectTriangleTiler::maxHex(n) : RectTriangleTiler::slopeHex(n);
  if ((long)t.size() > cap) return -1;
  std::memcpy(out, t.data(), t.size() * sizeof(int));
  return (int)std::lround(std::sqrt((double)t.size()));
}

extern "C" int refh_rt_from_lozenge(const int* tl, int n, const int* dl, int m, int* out) {
  tiling tL(tl, tl + (size_t)n * n);
  domain dL(dl, dl + (size_t)2 * m * m);
  tiling t = RectTriangleTiler::LozengeToRectTriangle(tL, dL);
  std::memcpy(out, t.data(), t.size() * sizeof(int));
  return 0;
}
