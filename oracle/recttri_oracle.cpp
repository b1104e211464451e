// TEST INFRASTRUCTURE ONLY - the oracle for the rectangle-triangle path.
//
// CPU restatement of the reference's rectangle-triangle tiler:
//   * maxHex / minHex          src/RectTriangle/RectTriangleTiler.cpp:480-600
//   * Walk :33-171 as the OpenCL path runs it: colours ((i - j) mod 3), generators seeded with
//     the walk seed itself, colours from default_random_engine + uniform_int_distribution(0, 2),
//     flipTiles recttrianglekernel.cl:25-118 (with getWeightRatio :157-160), updateTiles1
//     :120-132, updateTiles2 :134-146
//   * Walk as the CUDA path runs it, given its MTGP32 draws (cuRAND's generator comes in as
//     data): flipTilesKernel recttrianglekernel.cu:31-133 decides as flipTiles does, on every
//     slot of the N x N/3 grid, with the same colour stream and updates
// plus the library's fast mode (colour h mod 3, Philox draws per column quad).  The nine
// weights are runtime arguments here (compile-time #defines at recttrianglekernel.cl:3-11).
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load this.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <vector>

#include "philox_ref.h"
#include "tinymt32_ref.h"

namespace {

// Region codes of the extremal tilings (RectTriangleTiler.cpp:480-600); their change of
// coordinates shears row i by N + 3 - i columns and pads to a multiple of 3.
std::vector<int> shear(const std::vector<int>& t, int N) {
  const int M = 2 * N + 1, M2 = M + 6 + (3 - M % 3) % 3;
  std::vector<int> out((size_t)M2 * M2, 0);
  for (int i = 0; i < M; ++i)
    for (int j = 0; j < M; ++j) {
      const int j2 = j + N + 3 - i;
      if (j2 < M2) out[(size_t)(i + 3) * M2 + j2] = t[(size_t)i * M + j];
    }
  return out;
}

std::vector<int> hex_extremal(int N, bool top) {
  const int M = 2 * N + 1;
  std::vector<int> t((size_t)M * M, 0);
  for (int i = 1; i < M - 1; ++i)
    for (int j = top ? 0 : 1; j < (top ? M : M - 1); ++j) {
      int v = 0;
      if (j - i > N || i - j > N) v = 0;
      else if (top) {
        if (i < N && j < N) v = 0x333333;
        else if (i - j < 0 && j > N) v = 0x111111;
        else if (i > N && i - j > 0) v = 0x222222;
        else if (i == N && j < N) v = 0x333222;
        else if (i < N && j == N) v = 0x331311;
        else if (i - j == 0 && i > N) v = 0x211221;
        else if (i == N && j == N) v = 0x331221;
      } else {
        if (i > N && j > N) v = 0x333333;
        else if (i - j > 0 && j < N) v = 0x111111;
        else if (i < N && i - j < 0) v = 0x222222;
        else if (i == N && j > N) v = 0x222333;
        else if (i > N && j == N) v = 0x113133;
        else if (i - j == 0 && i < N) v = 0x122112;
        else if (i == N && j == N) v = 0x122133;
      }
      t[(size_t)i * M + j] = v;
    }
  if (top) {
    for (int i = 1; i < N; ++i) t[(size_t)i * M] = 0x003033, t[i] = 0x000333;
    for (int i = N + 1; i < M - 1; ++i) t[(size_t)i * M + M - 1] = 0x110100, t[(size_t)(M - 1) * M + i] = 0x222000;
    for (int i = 1; i < N; ++i) t[(size_t)i * M + i + N] = 0x100110, t[(size_t)(i + N) * M + i] = 0x022002;
    t[0] = 0x000033; t[(size_t)N * M] = 0x003002; t[N] = 0x000310;
    t[(size_t)(M - 1) * M + M - 1] = 0x210000; t[(size_t)N * M + M - 1] = 0x100100; t[(size_t)(M - 1) * M + N] = 0x022000;
  } else {
    for (int i = 1; i < N; ++i) t[(size_t)i * M] = 0x001011, t[i] = 0x000222;
    for (int i = N + 1; i < M - 1; ++i) t[(size_t)i * M + M - 1] = 0x330300, t[(size_t)(M - 1) * M + i] = 0x333000;
    for (int i = 1; i < N; ++i) t[(size_t)i * M + i + N] = 0x200220, t[(size_t)(i + N) * M + i] = 0x011001;
    t[0] = 0x000012; t[(size_t)(M - 1) * M + N] = 0x013000; t[(size_t)N * M + M - 1] = 0x200300;
    t[N] = 0x000220; t[(size_t)N * M] = 0x001001; t[(size_t)(M - 1) * M + M - 1] = 0x330000;
  }
  return shear(t, N);
}

struct Weights { float w[16]; };

Weights make_weights(const double* w9) {
  // recttrianglekernel.cl:13: {0, wt1, wt2, wt3, wr1, wr2, wr3, wr1, wr2, wr3, wm1, wm2, wm3, wm1, wm2, wm3}
  // with w9 = {wt1, wt2, wt3, wm1, wm2, wm3, wr1, wr2, wr3}
  Weights W;
  const float wt1 = w9[0], wt2 = w9[1], wt3 = w9[2], wm1 = w9[3], wm2 = w9[4], wm3 = w9[5], wr1 = w9[6], wr2 = w9[7],
              wr3 = w9[8];
  const float tab[16] = {0.0f, wt1, wt2, wt3, wr1, wr2, wr3, wr1, wr2, wr3, wm1, wm2, wm3, wm1, wm2, wm3};
  std::memcpy(W.w, tab, sizeof tab);
  return W;
}

float weight_ratio(const Weights& W, int a, int b) {
  const float* w = W.w;
  return (w[(b & 0xf00000) / 0x100000] * w[(b & 0x0f0000) / 0x010000] * w[(b & 0x00f000) / 0x001000] *
          w[(b & 0x000f00) / 0x000100] * w[(b & 0x0000f0) / 0x000010] * w[(b & 0x00000f)]) /
         (w[(a & 0xf00000) / 0x100000] * w[(a & 0x0f0000) / 0x010000] * w[(a & 0x00f000) / 0x001000] *
          w[(a & 0x000f00) / 0x000100] * w[(a & 0x0000f0) / 0x000010] * w[(a & 0x00000f)]);
}

// flipTiles' decision for one site and one uniform rd in [0, 1).
int flip_site(int hex, float rd, const Weights& W) {
  const float bs = 0.9f;
  if (!(rd < bs)) return hex;
  rd /= bs;
  int next = hex;
  float sc = rd < 0.25f ? 0.0f : (rd < 0.5f ? 0.25f : (rd < 0.75f ? 0.5f : 0.75f));
  // the five hexagons made of triangles or of one rectangle: the quarter of rd picks the
  // target (0x331221, 0x8ebbe8, 0xfc99cf, 0xa7dd7a from the top quarter down), the current
  // state's own target being replaced by 0x122133
  static const int five[5] = {0x122133, 0x331221, 0x8ebbe8, 0xfc99cf, 0xa7dd7a};
  bool in_five = false;
  for (int k = 0; k < 5; ++k) in_five |= hex == five[k];
  if (in_five) {
    int target = (double)rd < 0.25 ? 0xa7dd7a : ((double)rd < 0.5 ? 0xfc99cf : ((double)rd < 0.75 ? 0x8ebbe8 : 0x331221));
    next = target == hex ? 0x122133 : target;
  } else {
    static const int pairs[12][2] = {{0x47d47a, 0xd22a33}, {0xd22a33, 0x47d47a}, {0xa74d74, 0x33a22d}, {0x33a22d, 0xa74d74},
                                     {0x8eb558, 0x331eb1}, {0x331eb1, 0x8eb558}, {0x855be8, 0x1be133}, {0x1be133, 0x855be8},
                                     {0x6699cf, 0xcf1221}, {0xcf1221, 0x6699cf}, {0xfc9966, 0x1221fc}, {0x1221fc, 0xfc9966}};
    for (auto& p : pairs)
      if (hex == p[0]) {
        next = p[1];
        sc = 1.0f;
      }
  }
  const float ratio = weight_ratio(W, hex, next);
  rd = (sc == 1.0f) ? rd : (rd - sc) * 4;
  return ratio >= rd ? next : hex;
}

struct RChain {
  int N, M;
  std::vector<int> X[3];
};

int rcolour(int i, int j) { return ((i - j) % 3 + 3) % 3; }

void rsplit(const int* t, int N, RChain& c) {
  c.N = N;
  c.M = N / 3;
  for (auto& x : c.X) x.assign((size_t)N * c.M, 0);
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) c.X[rcolour(i, j)][(size_t)i * c.M + j / 3] = t[(size_t)i * N + j];
}

void rmerge(const RChain& c, int* t) {
  for (int i = 0; i < c.N; ++i)
    for (int j = 0; j < c.N; ++j) t[(size_t)i * c.N + j] = c.X[rcolour(i, j)][(size_t)i * c.M + j / 3];
}

void rupdate(RChain& c, int r) {
  const int N = c.N, M = c.M, t = r;
  const int* A = c.X[r].data();
  int* T1 = c.X[(r + 1) % 3].data();
  int* T2 = c.X[(r + 2) % 3].data();
  for (int i = 1; i < N - 1; ++i)
    for (int j = 1; j < M - 1; ++j) {
      {
        const int p1 = i % 3 == t, p2 = i % 3 == (t + 1) % 3;
        const int up = A[(size_t)(i - 1) * M + j], same = A[(size_t)i * M + j + p1], dn = A[(size_t)(i + 1) * M + j - p2];
        T1[(size_t)i * M + j] = (up & 0x0000f0) * 0x010000 + (up & 0x00000f) * 0x010000 + (same & 0xf00000) / 0x000100 +
                                (dn & 0x0f0000) / 0x000100 + (dn & 0x00f000) / 0x000100 + (same & 0x000f00) / 0x000100;
      }
      {
        const int p1 = i % 3 == (t + 2) % 3, p2 = i % 3 == (t + 1) % 3;
        const int same = A[(size_t)i * M + j - p1], up = A[(size_t)(i - 1) * M + j + p2], dn = A[(size_t)(i + 1) * M + j];
        T2[(size_t)i * M + j] = (same & 0x00f000) * 0x000100 + (up & 0x000f00) * 0x000100 + (up & 0x0000f0) * 0x000100 +
                                (same & 0x00000f) * 0x000100 + (dn & 0xf00000) / 0x010000 + (dn & 0x0f0000) / 0x010000;
      }
    }
}

}  // namespace

extern "C" {

int orc_rt_hex(int n, int top, int* out, long cap) {
  std::vector<int> t = hex_extremal(n, top != 0);
  const int side = (int)std::lround(std::sqrt((double)t.size()));
  if ((long)t.size() > cap) return -side;
  std::memcpy(out, t.data(), t.size() * sizeof(int));
  return side;
}

// params: nparams triples (mat1, mat2, tmat), triple k for generator k (the reference's
// LoadTinyMT table, RectTriangleTiler.cpp:22-25); generators beyond them keep the jump set.
int orc_rt_walk_tinymt(int* t, int N, long steps, long seed, const double* w9, const uint32_t* params, long nparams) {
  if (N % 3 || N < 9) return -1;
  RChain c;
  rsplit(t, N, c);
  const Weights W = make_weights(w9);
  const int M = c.M;
  std::vector<oracle::TinyMT32> g((size_t)N * M);
  for (size_t k = 0; k < g.size(); ++k) {
    g[k] = oracle::TinyMT32{0, 0, 0, 0, oracle::kTmtMat1, oracle::kTmtMat2, oracle::kTmtTmat};
    if (params && (long)k < nparams) {
      g[k].mat1 = params[3 * k];
      g[k].mat2 = params[3 * k + 1];
      g[k].tmat = params[3 * k + 2];
    }
    oracle::tmt_init(g[k], (uint32_t)seed + (uint32_t)k);
  }
  std::default_random_engine gen;
  std::uniform_int_distribution<int> dist(0, 2);
  gen.seed(seed);
  for (long s = 0; s < steps; ++s) {
    const int r = dist(gen);
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < M; ++j) {
        const float rd = oracle::tmt_u23_to_float(oracle::tmt_next_u23(g[(size_t)i * M + j]));
        int& e = c.X[r][(size_t)i * M + j];
        e = flip_site(e, rd, W);
      }
    rupdate(c, r);
  }
  rmerge(c, t);
  return 0;
}

// RectTriangleTiler::Walk(t, steps, seed), CUDA path (RectTriangleTiler.cpp:75-133), with the
// MTGP32 draws supplied: draws[s][i][j] is the curand_uniform value of slot (i, j) at step s.
int orc_rt_walk_draws(int* t, int N, const float* draws, long steps, long seed, const double* w9) {
  if (N % 3 || N < 9) return -1;
  RChain c;
  rsplit(t, N, c);
  const Weights W = make_weights(w9);
  const int M = c.M;
  std::default_random_engine gen;
  std::uniform_int_distribution<int> dist(0, 2);
  gen.seed(seed);
  for (long s = 0; s < steps; ++s) {
    const int r = dist(gen);
    const float* d = draws + (size_t)s * N * M;
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < M; ++j) {
        int& e = c.X[r][(size_t)i * M + j];
        e = flip_site(e, d[(size_t)i * M + j], W);
      }
    rupdate(c, r);
  }
  rmerge(c, t);
  return 0;
}

// flipTiles on one colour array (N rows x N/3 ints), draws per slot.
void orc_rt_flip_grid(int* colour, int N, const float* draws, const double* w9) {
  const Weights W = make_weights(w9);
  const size_t n = (size_t)N * (N / 3);
  for (size_t k = 0; k < n; ++k) colour[k] = flip_site(colour[k], draws[k], W);
}

// Fast mode: colour h mod 3, draws u32 per site; rd = u * 2^-32 evaluated in float as
// flipTiles does (the library's stated fast-mode rule for this model).
int orc_rt_walk_fast(int* t, int N, long h0, long steps, unsigned long seed, unsigned stream, const double* w9) {
  if (N % 3 || N < 9) return -1;
  RChain c;
  rsplit(t, N, c);
  const Weights W = make_weights(w9);
  const int M = c.M;
  for (long s = 0; s < steps; ++s) {
    const long h = h0 + s;
    const int r = (int)(((h % 3) + 3) % 3);
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < M; ++j) {
        const uint32_t u = oracle::fast_draw(seed, stream, h, (uint32_t)i, (uint32_t)j);
        const float rd = (float)(u >> 8) * (1.0f / 16777216.0f);
        int& e = c.X[r][(size_t)i * M + j];
        e = flip_site(e, rd, W);
      }
    rupdate(c, r);
  }
  rmerge(c, t);
  return 0;
}

}  // extern "C"
