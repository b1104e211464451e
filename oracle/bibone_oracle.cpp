// TEST INFRASTRUCTURE ONLY - the oracle for the bibone (triangular-lattice dimer) path.
//
// CPU restatement of the reference's TriangleDimerTiler (src/TriangleDimer/):
//   * IceCreamCone                      TriangleDimerTiler.cpp:697-793
//   * Walk :101-695 as the OpenCL path runs it: per step a move type, an orientation/kind
//     and a colour (and for butterflies a slice and a parity) from default_random_engine(seed)
//     with uniform_int_distribution(0, 2) / (0, 1), in that order; every one of the M x M
//     TinyMT generators draws once (RotateLozenges :4-22, RotateTriangles :191-211,
//     RotateButterflys :331-353; generator k = row * M + column, seeded seed + k, InitTinyMT
//     :749-756); a site of the chosen class flips when rd < 0.5 and its state is one of the
//     two flippable values (5/10, 45/54, 85/170).
//   * Walk as the CUDA path runs it, given its MTGP32 draws (cuRAND's generator comes in as
//     data): the same step classes, the draw of site (row a, column b) deciding as
//     RotateLozengesKernel / RotateTrianglesKernel / RotateButterflysKernel
//     (triangledimerkernel.cu) do, rd < 0.5
// The reference keeps eight derived state arrays consistent through 30 update kernels; here
// the state is the dimer configuration itself (three edge bits per vertex) and each move is
// the toggle of its alternating cycle, which is what those kernels compute.
// Geometry (vertex (a, b); H(a,b) = (a,b)-(a,b+1), L(a,b) = (a,b)-(a-1,b),
// R(a,b) = (a,b)-(a-1,b+1)); the tiling array t (side N = 2M) holds the lozenge states
//   t[2a][2b+1]   = R(a-1,b) + 2 L(a-1,b+1) + 4 R(a,b) + 8 L(a,b)      (eH)
//   t[2a+1][2b]   = H(a-1,b) + 2 R(a,b)     + 4 H(a,b-1) + 8 R(a,b-1) (eL)
//   t[2a+1][2b+1] = H(a-1,b) + 2 L(a,b+1)   + 4 H(a,b) + 8 L(a,b)     (eR)
// (TriangleDimerTiler.cpp:760-775 with its h array one row down).
// Plus the library's fast mode (schedule and site draws from Philox).
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load this.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <vector>

#include "philox_ref.h"
#include "tinymt32_ref.h"

namespace {

enum { kH = 1, kL = 2, kR = 4 };

struct Edge { int da, db, bit; };
struct Cycle { int n; Edge a[4], b[4]; };  // the two alternating halves (n edges each)

// Cycles by class: lozenge H/L/R (0-2), triangle up/down (3-4), butterfly H/L/R (5-7).
// Half a is the state 5 / 45 / 85 set, half b the 10 / 54 / 170 set.
const Cycle kCycles[8] = {
    {2, {{-1, 0, kR}, {0, 0, kR}}, {{-1, 1, kL}, {0, 0, kL}}},                                   // eH
    {2, {{-1, 0, kH}, {0, -1, kH}}, {{0, 0, kR}, {0, -1, kR}}},                                  // eL
    {2, {{-1, 0, kH}, {0, 0, kH}}, {{0, 1, kL}, {0, 0, kL}}},                                    // eR
    {3, {{-1, 0, kH}, {0, 1, kR}, {1, 0, kL}}, {{0, 0, kL}, {-1, 1, kH}, {1, 0, kR}}},            // tU
    {3, {{0, -1, kH}, {0, 1, kL}, {-1, 0, kR}}, {{0, -1, kR}, {0, 0, kH}, {-1, 1, kL}}},          // tD
    {4, {{-1, 0, kL}, {-2, 1, kH}, {0, 1, kL}, {0, -1, kH}}, {{-2, 0, kH}, {-1, 1, kR}, {0, 0, kH}, {0, -1, kR}}},  // bH
    {4, {{-1, 0, kR}, {0, 1, kL}, {1, -1, kR}, {0, -1, kL}}, {{-1, 1, kL}, {0, 0, kH}, {1, -1, kL}, {-1, -1, kH}}},  // bL
    {4, {{-1, 0, kR}, {-1, 1, kH}, {1, 0, kR}, {0, -1, kH}}, {{-1, 1, kL}, {0, 1, kR}, {1, 0, kL}, {0, -1, kR}}},   // bR
};

struct Dimers {
  int M;
  std::vector<uint8_t> v;  // bits kH | kL | kR per vertex
  uint8_t at(int a, int b) const { return (a >= 0 && b >= 0 && a < M && b < M) ? v[(size_t)a * M + b] : 0; }
};

Dimers from_tiling(const int* t, int N) {
  Dimers d;
  d.M = N / 2;
  d.v.assign((size_t)d.M * d.M, 0);
  for (int a = 0; a < d.M; ++a)
    for (int b = 0; b < d.M; ++b) {
      const int eR = t[(size_t)(2 * a + 1) * N + 2 * b + 1], eH = t[(size_t)(2 * a) * N + 2 * b + 1];
      d.v[(size_t)a * d.M + b] = (uint8_t)(((eR & 4) ? kH : 0) | ((eR & 8) ? kL : 0) | ((eH & 4) ? kR : 0));
    }
  return d;
}

void to_tiling(const Dimers& d, int* t, int N) {
  auto bit = [&](int a, int b, int k) { return (d.at(a, b) & k) ? 1 : 0; };
  for (int a = 0; a < d.M; ++a)
    for (int b = 0; b < d.M; ++b) {
      t[(size_t)(2 * a) * N + 2 * b + 1] = bit(a - 1, b, kR) + 2 * bit(a - 1, b + 1, kL) + 4 * bit(a, b, kR) + 8 * bit(a, b, kL);
      t[(size_t)(2 * a + 1) * N + 2 * b] = bit(a - 1, b, kH) + 2 * bit(a, b, kR) + 4 * bit(a, b - 1, kH) + 8 * bit(a, b - 1, kR);
      t[(size_t)(2 * a + 1) * N + 2 * b + 1] = bit(a - 1, b, kH) + 2 * bit(a, b + 1, kL) + 4 * bit(a, b, kH) + 8 * bit(a, b, kL);
    }
}

// The class predicate of one step at site (a, b).
struct Step { int type, r1, r2, p1, p2; };

int cycle_of(const Step& s) { return s.type == 0 ? s.r1 : s.type == 1 ? (s.r2 == 1 ? 4 : 3) : 5 + s.r1; }

bool in_class(const Step& s, int a, int b) {
  if (s.type == 0) return (((1 - (s.r1 & 1)) * a + ((1 + s.r1) / 2) * b) % 2) == s.r2;
  if (s.type == 1) return (((b - a) % 3 + 3) % 3) == s.r1;
  const int b1 = 1 - (s.r1 & 1), b2 = (1 + s.r1) / 2, b3 = s.r1 & 1;
  return ((b1 * a + b2 * b) % 3) == s.p1 && ((b1 * b + b3 * a) & 1) == s.p2;
}

// Toggles the cycle at (a, b) when one half is fully covered; cycles reaching outside the
// array never move.
void try_flip(Dimers& d, int c, int a, int b) {
  const Cycle& C = kCycles[c];
  bool ha = true, hb = true;
  for (int k = 0; k < C.n; ++k) {
    const Edge* es[2] = {&C.a[k], &C.b[k]};
    for (const Edge* e : es) {
      const int x = a + e->da, y = b + e->db;
      if (x < 0 || y < 0 || x >= d.M || y >= d.M) return;
    }
    ha = ha && (d.at(a + C.a[k].da, b + C.a[k].db) & C.a[k].bit);
    hb = hb && (d.at(a + C.b[k].da, b + C.b[k].db) & C.b[k].bit);
  }
  if (!ha && !hb) return;
  for (int k = 0; k < C.n; ++k) {
    d.v[(size_t)(a + C.a[k].da) * d.M + b + C.a[k].db] ^= (uint8_t)C.a[k].bit;
    d.v[(size_t)(a + C.b[k].da) * d.M + b + C.b[k].db] ^= (uint8_t)C.b[k].bit;
  }
}

// One step on all sites with per-site acceptance `accept(a, b)` (called for every site, as
// every generator draws in the reference).
template <class Accept>
void run_step(Dimers& d, const Step& s, Accept accept) {
  const int c = cycle_of(s);
  std::vector<std::pair<int, int>> flips;
  for (int a = 0; a < d.M; ++a)
    for (int b = 0; b < d.M; ++b)
      if (accept(a, b) && in_class(s, a, b)) flips.push_back({a, b});
  for (auto& f : flips) try_flip(d, c, f.first, f.second);
}

Step fast_step(uint64_t seed, uint32_t stream, int64_t h) {
  oracle::U32x4 c;
  c.v[0] = 0xffffffffu;
  c.v[1] = 0xffffffffu;
  c.v[2] = (uint32_t)(uint64_t)h;
  c.v[3] = ((uint32_t)((uint64_t)h >> 32) & 0xffffu) | (stream << 16);
  const oracle::U32x4 o = oracle::philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  Step s;
  s.type = (int)(o.v[0] % 3u);
  s.r1 = (int)(o.v[1] % 3u);
  s.r2 = (int)(o.v[2] & 1u);
  s.p1 = (int)((o.v[3] >> 1) % 3u);
  s.p2 = (int)(o.v[3] & 1u);
  return s;
}

}  // namespace

extern "C" {

// IceCreamCone(n, m) (TriangleDimerTiler.cpp:697-793): the downward triangle of side n
// with a side-m triangle cut from its top-left corner, as a tiling of side 2 (n + 4).
int orc_td_icecream(int n, int m, int* out, long cap) {
  const int E = n + 4, T = 2 * E, k = ((n + 1) * (n + 2) / 2) % 2;
  if ((long)T * T > cap) return -T;
  std::vector<int> h((size_t)E * E, 0), l((size_t)E * E, 0), r((size_t)E * E, 0);
  for (int i = 2; i < E - 2; ++i)
    for (int j = 2; j < E - i; ++j) {
      if (i < m + 2) {
        if ((i + j) % 2 == m % 2 && (m != 0 && j > m + 3 - i)) h[(size_t)i * E + j] = 1;
        if ((n - m) % 2 == 0 && (i % 2) == 0 && j == E - i - 1) r[(size_t)i * E + j] = 1;
      } else {
        if (j % 2 == 0) h[(size_t)i * E + j] = 1;
        if (i % 4 == (3 + n % 2 + 2 * k) % 4 && j == E - i - 1) h[(size_t)i * E + j] = 0, l[(size_t)i * E + j] = 1;
        if (i % 4 == (2 + n % 2 + 2 * k) % 4 && j == E - i - 1) r[(size_t)i * E + j] = 1;
      }
    }
  // h[i][j] is the horizontal edge of vertex row i - 1 in the geometry above
  Dimers d;
  d.M = E;
  d.v.assign((size_t)E * E, 0);
  for (int a = 0; a < E; ++a)
    for (int b = 0; b < E; ++b)
      d.v[(size_t)a * E + b] = (uint8_t)(((a + 1 < E && h[(size_t)(a + 1) * E + b]) ? kH : 0) |
                                         (l[(size_t)a * E + b] ? kL : 0) | (r[(size_t)a * E + b] ? kR : 0));
  std::vector<int> t((size_t)T * T, 0);
  to_tiling(d, t.data(), T);
  // the reference fills only rows and columns 3 .. T-2 (TriangleDimerTiler.cpp:758-759)
  for (int i = 0; i < T; ++i)
    for (int j = 0; j < T; ++j)
      out[(size_t)i * T + j] = (i >= 3 && j >= 3 && i < T - 1 && j < T - 1) ? t[(size_t)i * T + j] : 0;
  return T;
}

// params: nparams triples (mat1, mat2, tmat), triple k for generator k (the reference's
// LoadTinyMT table, TriangleDimerTiler.cpp:24-27); generators beyond them keep the jump set.
int orc_td_walk_tinymt(int* t, int N, long steps, long seed, const uint32_t* params, long nparams) {
  if (N % 2) return -1;
  Dimers d = from_tiling(t, N);
  const int M = d.M;
  std::vector<oracle::TinyMT32> g((size_t)M * M);
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
  std::uniform_int_distribution<int> d1(0, 2), d2(0, 1);
  gen.seed(seed);
  for (long s = 0; s < steps; ++s) {
    Step st;
    st.type = d1(gen);
    st.r1 = d1(gen);
    st.r2 = d2(gen);
    st.p1 = st.p2 = 0;
    if (st.type == 2) st.p1 = d1(gen), st.p2 = d2(gen);
    run_step(d, st, [&](int a, int b) {
      const float rd = oracle::tmt_u23_to_float(oracle::tmt_next_u23(g[(size_t)a * M + b]));
      return rd < .5;
    });
  }
  to_tiling(d, t, N);
  return 0;
}

// TriangleDimerTiler::Walk(t, steps, seed), CUDA path (TriangleDimerTiler.cpp:279-291), with
// the MTGP32 draws supplied: draws[s][a][b] is the curand_uniform value of site (a, b) at
// step s.
int orc_td_walk_draws(int* t, int N, const float* draws, long steps, long seed) {
  if (N % 2) return -1;
  Dimers d = from_tiling(t, N);
  const int M = d.M;
  std::default_random_engine gen;
  std::uniform_int_distribution<int> d1(0, 2), d2(0, 1);
  gen.seed(seed);
  for (long s = 0; s < steps; ++s) {
    Step st;
    st.type = d1(gen);
    st.r1 = d1(gen);
    st.r2 = d2(gen);
    st.p1 = st.p2 = 0;
    if (st.type == 2) st.p1 = d1(gen), st.p2 = d2(gen);
    const float* dr = draws + (size_t)s * M * M;
    run_step(d, st, [&](int a, int b) { return dr[(size_t)a * M + b] < .5; });
  }
  to_tiling(d, t, N);
  return 0;
}

// The step class test (in_class) for one site: 1 when site (a, b) belongs to the class of
// move type, r1, r2, p1, p2.
int orc_td_in_class(int type, int r1, int r2, int p1, int p2, int a, int b) {
  Step st;
  st.type = type;
  st.r1 = r1;
  st.r2 = r2;
  st.p1 = p1;
  st.p2 = p2;
  return in_class(st, a, b) ? 1 : 0;
}

// Fast mode: step h's class from Philox(ctr = {~0, ~0, lo32(h), hi16(h) | stream << 16});
// site (a, b) accepts when its fast draw (philox_ref.h fast_draw with row a, column b) is
// below 2^31.
int orc_td_walk_fast(int* t, int N, long h0, long steps, unsigned long seed, unsigned stream) {
  if (N % 2) return -1;
  Dimers d = from_tiling(t, N);
  for (long s = 0; s < steps; ++s) {
    const int64_t h = h0 + s;
    const Step st = fast_step(seed, stream, h);
    run_step(d, st, [&](int a, int b) {
      return in_class(st, a, b) && oracle::fast_draw(seed, stream, h, (uint32_t)a, (uint32_t)b) < 0x80000000u;
    });
  }
  to_tiling(d, t, N);
  return 0;
}

void orc_td_fast_step(unsigned long seed, unsigned stream, long h, int* out5) {
  const Step s = fast_step(seed, stream, h);
  out5[0] = s.type, out5[1] = s.r1, out5[2] = s.r2, out5[3] = s.p1, out5[4] = s.p2;
}

}  // extern "C"
