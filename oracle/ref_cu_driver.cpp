// TEST INFRASTRUCTURE ONLY.  Runs the rotate kernels of the reference's CUDA build, compiled
// as host C++ through ref_cu_shim.h (see the Makefile's ref-cu rules), over an emulated
// launch: the grid and 8 x 8 blocks the reference's Walk launches them with
// (DominoTiler.cpp:55-60, LozengeTiler.cpp:71-76, RectTriangleTiler.cpp:75-80,
// TriangleDimerTiler.cpp:280-285), one thread
// at a time (each thread touches only its own site), with the draws supplied per thread.
#include "ref_cu_shim.h"

namespace ref_cu_plain { void RotateTilesKernel(curandStateMtgp32*, char*, const int, const int); }
namespace ref_cu_CFTP { void RotateTilesKernel(curandStateMtgp32*, char*, const int, const int); }
namespace ref_cu_twoperiodic { void RotateTilesKernel(curandStateMtgp32*, char*, const int, const int); }
namespace ref_cu_CFTPtwoperiodic { void RotateTilesKernel(curandStateMtgp32*, char*, const int, const int); }
namespace ref_cu_lozenge { void RotateTilesKernel(curandStateMtgp32*, char*, const int); }
namespace ref_cu_recttri { void flipTilesKernel(curandStateMtgp32*, int*, const int); }
namespace ref_cu_tdimer {
void RotateLozengesKernel(curandStateMtgp32*, int*, const int, const int, const int);
void RotateTrianglesKernel(curandStateMtgp32*, int*, const int, const int);
void RotateButterflysKernel(curandStateMtgp32*, int*, const int, const int, const int, const int);
}  // namespace ref_cu_tdimer

namespace {

template <class F>
void launch(int gx, int gy, int rows, int cols, const float* draws, F thread_body) {
  refcu::draws = draws;
  refcu::rows = rows;
  refcu::cols = cols;
  refcu::block_dim = dim3(8, 8);
  refcu::grid_dim = dim3(gx, gy);
  for (int bx = 0; bx < gx; ++bx)
    for (int by = 0; by < gy; ++by)
      for (int ty = 0; ty < 8; ++ty)
        for (int tx = 0; tx < 8; ++tx) {
          refcu::block_idx = uint3{(unsigned)bx, (unsigned)by, 0};
          refcu::thread_idx = uint3{(unsigned)tx, (unsigned)ty, 0};
          thread_body();
        }
}

}  // namespace

extern "C" {

// Domino: RotateTilesKernel of dominokernel{,CFTP,twoperiodic,CFTPtwoperiodic}.cu (variant 0-3,
// the library's rule numbering) on one colour array (N rows x N/2 bytes), draws per candidate
// (N-2) x (N/2-2) as rt_domino_mtgp_draws lays them out.
int ref_cu_domino_rotate(int variant, char* colour, int N, int t, const float* draws) {
  const int rows = N - 2, cols = N / 2 - 2;
  curandStateMtgp32 st{};
  auto body = [&]() {
    switch (variant) {
      case 0: ref_cu_plain::RotateTilesKernel(&st, colour, N, t); break;
      case 1: ref_cu_CFTP::RotateTilesKernel(&st, colour, N, t); break;
      case 2: ref_cu_twoperiodic::RotateTilesKernel(&st, colour, N, t); break;
      default: ref_cu_CFTPtwoperiodic::RotateTilesKernel(&st, colour, N, t); break;
    }
  };
  if (variant < 0 || variant > 3) return -1;
  launch((rows + 7) / 8, (cols + 7) / 8, rows, cols, draws, body);
  return 0;
}

// Lozenge: RotateTilesKernel of lozengekernel.cu on one colour array (N rows x N/3 bytes),
// draws per slot N x N/3.
int ref_cu_lozenge_rotate(char* colour, int N, const float* draws) {
  curandStateMtgp32 st{};
  launch((N + 7) / 8, (N / 3 + 7) / 8, N, N / 3, draws, [&]() { ref_cu_lozenge::RotateTilesKernel(&st, colour, N); });
  return 0;
}

// Rectangle-triangle: flipTilesKernel of recttrianglekernel.cu (unit weights, as compiled
// there) on one colour array (N rows x N/3 ints), draws per slot N x N/3.
int ref_cu_recttri_flip(int* colour, int N, const float* draws) {
  curandStateMtgp32 st{};
  launch((N + 7) / 8, (N / 3 + 7) / 8, N, N / 3, draws, [&]() { ref_cu_recttri::flipTilesKernel(&st, colour, N); });
  return 0;
}

// Bibone: the rotate kernel of move type 0 / 1 / 2 (RotateLozengesKernel,
// RotateTrianglesKernel, RotateButterflysKernel of triangledimerkernel.cu) on one M x M state
// array, with the class arguments Walk passes (TriangleDimerTiler.cpp:346, 420, 499: r1, r2,
// p1, p2), draws per site M x M.
int ref_cu_td_rotate(int type, int* states, int M, int r1, int r2, int p1, int p2, const float* draws) {
  curandStateMtgp32 st{};
  if (type < 0 || type > 2) return -1;
  launch((M + 7) / 8, (M + 7) / 8, M, M, draws, [&]() {
    if (type == 0) ref_cu_tdimer::RotateLozengesKernel(&st, states, M, r1, r2);
    else if (type == 1) ref_cu_tdimer::RotateTrianglesKernel(&st, states, M, r1);
    else ref_cu_tdimer::RotateButterflysKernel(&st, states, M, r1, p1, p2);
  });
  return 0;
}

}  // extern "C"
