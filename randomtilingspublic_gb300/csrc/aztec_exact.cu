// Exact edge-placement probabilities of the weighted Aztec diamond, computed on the device by
// generalized domino shuffling (J. Propp, "Generalized domino-shuffling", Theoret. Comput.
// Sci. 303 (2003) 267-301).  No counterpart in the reference: it is the exact answer that
// the device-side edge counters (rt_dm_sampler_accumulate_edges, rt_domino_edge_indicators)
// estimate, for the weights of the reference's chains (uniform, dominokernelCFTP.cl, and the
// 2 x 2-periodic a / b rule of dominokernelCFTPtwoperiodic.cl:72-101).
//
// Geometry.  The order-k diamond's cells (the 4-cycles of its dual graph) are its lattice
// points (R, C) with R + C + k odd.  In the rotated coordinates s = R + C, t = R - C they form
// a k x k grid, cell (i, j), and a cell's four domino positions (the grid segments meeting at
// its point) fill a 2 x 2 block of a 2k x 2k array: up (0, 0), left (0, 1), right (1, 0),
// down (1, 1), so that opposite positions sit diagonally opposite.
//
// Weights go down: urban renewal at every cell gives each position its opposite's weight over
// D = w00 w11 + w01 w10, and dropping the array's outer rows and columns leaves the order
// k-1 diamond.  The a / b weights depend on (I mod 4, J mod 4) of the array entry, a property
// both steps keep, so each level is one 4 x 4 tile, computed on the host.
//
// Probabilities go up, the way the shuffling grows a tiling: a domino of the order k-1
// tiling slides across its cell to the opposite position, and the cell's complement (1 minus
// its four order k-1 probabilities, zero outside the smaller array) is filled by a pair, up
// and down in the proportion w00 w11 / D, left and right w01 w10 / D.  The complement is not a
// probability: a cell holding two dominoes (which the shuffling removes) counts twice, so it
// is negative where that is common, and only the final values are clamped at 0 (against
// rounding).  One launch per level, one thread per cell, double precision.  The values keep
// their accuracy at any order (the Kasteleyn inverse, the other exact method, loses all its
// digits beyond order ~50).
#include <cuda_runtime.h>

#include <cmath>
#include <string>
#include <vector>

#include "rt_internal.h"

namespace rt {
namespace {

// pair probability of up + down at level k for cells of parity (i & 1, j & 1); left + right is
// the complement
struct LevelRatio {
  double h[2][2];
};

__global__ void k_shuffle_level(const double* __restrict__ prev, double* __restrict__ cur, int k,
                                const LevelRatio* __restrict__ ratio) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= (int64_t)k * k) return;
  const int i = (int)(c / k), j = (int)(c - (int64_t)i * k);
  const int W = 2 * k, Wp = 2 * k - 2;  // array sides of levels k and k - 1
  // block (i, j) of level k covers entries 2i + dx - 1 .. of the level k - 1 array
  double q[2][2];
#pragma unroll
  for (int dx = 0; dx < 2; ++dx)
#pragma unroll
    for (int dy = 0; dy < 2; ++dy) {
      const int I = 2 * i + dx - 1, J = 2 * j + dy - 1;
      q[dx][dy] = (I >= 0 && J >= 0 && I < Wp && J < Wp) ? prev[(size_t)I * Wp + J] : 0.0;
    }
  // negative where the order k-1 tiling often holds two dominoes in the cell
  const double empty = 1.0 - (q[0][0] + q[0][1] + q[1][0] + q[1][1]);
  const double h = ratio[k - 1].h[i & 1][j & 1];
  const double ph = h * empty, pv = (1.0 - h) * empty;
  double* row0 = cur + (size_t)(2 * i) * W + 2 * j;
  double* row1 = row0 + W;
  row0[0] = q[1][1] + ph;
  row1[1] = q[0][0] + ph;
  row0[1] = q[1][0] + pv;
  row1[0] = q[0][1] + pv;
}

// Level-n array to the [2][N][N] counter layout of the order-n tiling (N = 2n + 6, faces from
// row and column 2): cell (i, j) sits at lattice point R = i + j + 3, C = i - j + n + 2.
__global__ void k_shuffle_layout(const double* __restrict__ P, double* __restrict__ out, int n) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= (int64_t)n * n) return;
  const int i = (int)(c / n), j = (int)(c - (int64_t)i * n);
  const int W = 2 * n, N = 2 * n + 6;
  const int R = i + j + 3, C = i - j + n + 2;
  const double* row0 = P + (size_t)(2 * i) * W + 2 * j;
  const double* row1 = row0 + W;
  const size_t NN = (size_t)N * N;
  out[(size_t)(R - 1) * N + C] = fmax(0.0, row0[0]);    // up: horizontal domino on faces (R-1, C-1), (R-1, C)
  out[(size_t)R * N + C] = fmax(0.0, row1[1]);          // down: faces (R, C-1), (R, C)
  out[NN + (size_t)R * N + C - 1] = fmax(0.0, row0[1]);  // left: vertical domino on faces (R-1, C-1), (R, C-1)
  out[NN + (size_t)R * N + C] = fmax(0.0, row1[0]);      // right: faces (R-1, C), (R, C)
}

// The per-level up + down pair ratios for order n and weights a / b (host; n tiles of 4 x 4).
std::vector<LevelRatio> aztec_level_ratios(int n, double a, double b) {
  std::vector<LevelRatio> out((size_t)n);
  // level-n tile: entry (x, y) = (I mod 4, J mod 4), cell parity (x >> 1, y >> 1), position
  // (x & 1, y & 1); horizontal positions (dx == dy) weigh a when i - j + n is even, vertical
  // ones when i + j is even (the reference's rule on face columns and rows)
  double T[4][4];
  for (int x = 0; x < 4; ++x)
    for (int y = 0; y < 4; ++y) {
      const int pi = x >> 1, pj = y >> 1;
      const bool horizontal = (x & 1) == (y & 1);
      const bool is_a = horizontal ? ((pi - pj + n) % 2 + 2) % 2 == 0 : (pi + pj) % 2 == 0;
      T[x][y] = is_a ? a : b;
    }
  for (int k = n; k >= 1; --k) {
    // the level-k array's blocks start at even entries; tile phase: W_k(I, J) = T[I & 3][J & 3]
    for (int pi = 0; pi < 2; ++pi)
      for (int pj = 0; pj < 2; ++pj) {
        const double w00 = T[2 * pi][2 * pj], w01 = T[2 * pi][2 * pj + 1], w10 = T[2 * pi + 1][2 * pj],
                     w11 = T[2 * pi + 1][2 * pj + 1];
        out[(size_t)k - 1].h[pi][pj] = w00 * w11 / (w00 * w11 + w01 * w10);
      }
    if (k == 1) break;
    double F[4][4];
    for (int x = 0; x < 4; x += 2)
      for (int y = 0; y < 4; y += 2) {
        const double D = T[x][y] * T[x + 1][y + 1] + T[x][y + 1] * T[x + 1][y];
        F[x][y] = T[x + 1][y + 1] / D;
        F[x + 1][y + 1] = T[x][y] / D;
        F[x][y + 1] = T[x + 1][y] / D;
        F[x + 1][y] = T[x][y + 1] / D;
      }
    // dropping the outer rows and columns: W_{k-1}(I, J) = F[(I + 1) & 3][(J + 1) & 3]
    for (int x = 0; x < 4; ++x)
      for (int y = 0; y < 4; ++y) T[x][y] = F[(x + 1) & 3][(y + 1) & 3];
  }
  return out;
}

}  // namespace
}  // namespace rt

using namespace rt;

extern "C" {

RT_API rt_status rt_domino_aztec_edge_probs(int32_t order, double a, double b, double* out, int64_t cap,
                                            void* cuda_stream) {
  clear_error();
  if (order < 1 || order > 16384 || !(a > 0) || !(b > 0) || !std::isfinite(a) || !std::isfinite(b))
    return fail(RT_ERR_INVALID_ARGUMENT, "aztec_edge_probs: order in [1, 16384], finite weights a, b > 0");
  const int n = order, N = 2 * n + 6;
  const size_t outn = (size_t)2 * N * N;
  if (!out || cap < (int64_t)outn) return fail(RT_ERR_BUFFER_TOO_SMALL, "aztec_edge_probs: output holds 2 (2 order + 6)^2 values");
  int devs = 0;
  if (cudaGetDeviceCount(&devs) != cudaSuccess || devs == 0) {
    cudaGetLastError();
    return fail(RT_ERR_CUDA, "no CUDA device: the exact probabilities have no CPU fallback");
  }
  cudaStream_t st = (cudaStream_t)cuda_stream;
  const std::vector<LevelRatio> ratio = aztec_level_ratios(n, a, b);
  const size_t side = (size_t)2 * n;
  double *d_p0 = nullptr, *d_p1 = nullptr, *d_out = nullptr;
  LevelRatio* d_ratio = nullptr;
  // stream-ordered blocks of the library's pool, freed on the stream after the last use
  auto cleanup = [&]() {
    for (void* p : {(void*)d_p0, (void*)d_p1, (void*)d_out, (void*)d_ratio}) dev_free(p, st);
  };
  rt_status as = dev_alloc(&d_p0, side * side * sizeof(double), st);
  if (as == RT_OK) as = dev_alloc(&d_p1, side * side * sizeof(double), st);
  if (as == RT_OK) as = dev_alloc(&d_out, outn * sizeof(double), st);
  if (as == RT_OK) as = dev_alloc(&d_ratio, ratio.size() * sizeof(LevelRatio), st);
  if (as != RT_OK) {
    cleanup();
    return as;
  }
  cudaMemcpyAsync(d_ratio, ratio.data(), ratio.size() * sizeof(LevelRatio), cudaMemcpyHostToDevice, st);
  cudaMemsetAsync(d_out, 0, outn * sizeof(double), st);
  double *prev = d_p0, *cur = d_p1;
  for (int k = 1; k <= n; ++k) {
    const int64_t cells = (int64_t)k * k;
    k_shuffle_level<<<(unsigned)((cells + 255) / 256), 256, 0, st>>>(prev, cur, k, d_ratio);
    std::swap(prev, cur);
  }
  k_shuffle_layout<<<(unsigned)(((int64_t)n * n + 255) / 256), 256, 0, st>>>(prev, d_out, n);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, d_out, outn * sizeof(double), cudaMemcpyDeviceToHost, st);
  cleanup();
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return fail(RT_ERR_CUDA, std::string("aztec_edge_probs: ") + cudaGetErrorString(e));
  return RT_OK;
}

}  // extern "C"
