// TEST INFRASTRUCTURE ONLY - the oracle for the lozenge path.
//
// CPU restatement of the reference's lozenge tiler (src/Lozenge/LozengeTiler.cpp):
//   * AlmostHexDomain :422-467, DomainToVertices :483-512, TilingToDomain :514-556
//   * Thurston MinTiling :218-306 / MaxTiling :308-397, HeightfuncToTiling :399-420,
//     TilingToHeightfunc :173-216 (neighbour tables :21-25)
//   * Walk :27-159 as the OpenCL path runs it: three colour arrays by ((j-i) mod 3),
//     generators seeded with the walk seed itself (InitTinyMT, lozengekernel.cl:127-134),
//     colours from std::default_random_engine + uniform_int_distribution(0, 2) seeded with
//     the walk seed, RotateTiles lozengekernel.cl:74-105, UpdateTiles :107-125
//   * Walk as the CUDA path runs it, given its MTGP32 draws (cuRAND's generator is library
//     code and comes in as data): RotateTilesKernel lozengekernel.cu:15-29 on every slot of
//     the N x N/3 grid, the same colour stream and UpdateTiles
// plus the library's fast mode for lozenges (colour h mod 3, Philox draws per column quad).
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load this.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <queue>
#include <random>
#include <utility>
#include <vector>

#include "philox_ref.h"
#include "tinymt32_ref.h"

namespace {

constexpr int kInf = INT_MAX;
const int kNb[6][2] = {{0, 1}, {-1, 1}, {-1, 0}, {0, -1}, {1, -1}, {1, 0}};
const int kDh[6] = {-1, 1, -1, 1, -1, 1};
const int kFace[6][2][2] = {{{0, 0}, {-1, 1}}, {{-1, 1}, {-1, 0}}, {{-1, 0}, {-1, -1}},
                            {{-1, -1}, {0, -2}}, {{0, -2}, {0, -1}}, {{0, -1}, {0, 0}}};
const int kBit[6] = {8, 2, 1, 4, 16, 32};

struct Dom {
  const int* d;
  int M;  // vertex side minus one; the domain holds M rows of 2M triangles
  int face(int i0, int j0, int nb, int which) const {
    return d[(size_t)(i0 + kFace[nb][which][0]) * 2 * M + 2 * j0 + kFace[nb][which][1]];
  }
};

std::vector<int> vertices_of(const int* d, int M) {
  const int N = M + 1;
  std::vector<int> v((size_t)N * N, 0);
  auto F = [&](int r, int c) { return d[(size_t)r * 2 * M + c]; };
  for (int i = 1; i < M; ++i)
    for (int j = 1; j < M; ++j) {
      int f[6] = {F(i, 2 * j), F(i, 2 * j - 1), F(i, 2 * j - 2), F(i - 1, 2 * j), F(i - 1, 2 * j + 1), F(i - 1, 2 * j - 1)};
      bool all = f[0] && f[1] && f[2] && f[3] && f[4] && f[5];
      bool any = f[0] || f[1] || f[2] || f[3] || f[4] || f[5];
      v[(size_t)i * N + j] = all ? 1 : (any ? 2 : 0);
    }
  return v;
}

std::vector<int> hf_to_tiling(const std::vector<int>& hf, const int* d, int N) {
  Dom D{d, N - 1};
  std::vector<int> t((size_t)N * N, 0);
  for (int i0 = 1; i0 < N - 1; ++i0)
    for (int j0 = 1; j0 < N - 1; ++j0)
      for (int nb = 0; nb < 6; ++nb) {
        int i = i0 + kNb[nb][0], j = j0 + kNb[nb][1];
        if (D.face(i0, j0, nb, 0) || D.face(i0, j0, nb, 1)) {
          long long diff = (long long)hf[(size_t)i * N + j] - hf[(size_t)i0 * N + j0];
          if (diff == 2 || diff == -2) t[(size_t)i0 * N + j0] += kBit[nb];
        }
      }
  return t;
}

struct LowFirst {
  bool operator()(const std::pair<std::pair<int, int>, int>& a, const std::pair<std::pair<int, int>, int>& b) const {
    return a.second > b.second;
  }
};
struct HighFirst {
  bool operator()(const std::pair<std::pair<int, int>, int>& a, const std::pair<std::pair<int, int>, int>& b) const {
    return a.second < b.second;
  }
};

// kMax: bulk filled moving only along dh > 0 from the lowest vertex; else dh < 0 from the
// highest.  Returns -1 (and the tiling of the partial heights, as the reference does) when
// a consistency check fails.
template <bool kMax>
int extremal(const int* d, int M, std::vector<int>& out) {
  Dom D{d, M};
  std::vector<int> v = vertices_of(d, M);
  const int N = M + 1;
  std::vector<int> hf((size_t)N * N, kInf);
  std::queue<std::pair<int, int>> q;
  bool found = false;
  for (int i = 0; i < N && !found; ++i)
    for (int j = 0; j < N && !found; ++j)
      if (v[(size_t)i * N + j] == 2) {
        found = true;
        q.push({i, j});
        hf[(size_t)i * N + j] = 0;
      }
  typedef std::pair<std::pair<int, int>, int> E;
  std::priority_queue<E, std::vector<E>, typename std::conditional<kMax, LowFirst, HighFirst>::type> pq;
  int rc = 0;
  while (!q.empty() && rc == 0) {
    auto [i0, j0] = q.front();
    q.pop();
    for (int nb = 0; nb < 6; ++nb) {
      int i = i0 + kNb[nb][0], j = j0 + kNb[nb][1];
      if (v[(size_t)i * N + j] != 2) continue;
      if (!(D.face(i0, j0, nb, 0) ^ D.face(i0, j0, nb, 1))) continue;
      int h = hf[(size_t)i0 * N + j0] + kDh[nb];
      if (hf[(size_t)i * N + j] == kInf) {
        hf[(size_t)i * N + j] = h;
        q.push({i, j});
        pq.push({{i, j}, h});
      } else if (hf[(size_t)i * N + j] != h) {
        rc = -1;
        break;
      }
    }
  }
  if (rc == 0) {
    while (!pq.empty() && rc == 0) {
      E e = pq.top();
      pq.pop();
      int i0 = e.first.first, j0 = e.first.second;
      for (int nb = 0; nb < 6; ++nb) {
        int i = i0 + kNb[nb][0], j = j0 + kNb[nb][1];
        if (v[(size_t)i * N + j] <= 0 || (kMax ? kDh[nb] <= 0 : kDh[nb] >= 0)) continue;
        int h = hf[(size_t)i0 * N + j0] + kDh[nb];
        if (v[(size_t)i * N + j] == 2 && (kMax ? hf[(size_t)i * N + j] > h : hf[(size_t)i * N + j] < h)) {
          rc = -1;
          break;
        }
        if (hf[(size_t)i * N + j] == kInf) {
          hf[(size_t)i * N + j] = h;
          pq.push({{i, j}, h});
        }
      }
    }
    if (rc == 0)
      for (size_t p = 0; p < hf.size(); ++p)
        if (v[p] == 0) hf[p] = kInf;
  }
  out = hf_to_tiling(hf, d, N);
  return rc;
}

// ---- the sweep --------------------------------------------------------------------------
struct LChain {
  int N, M;
  std::vector<uint8_t> X[3];  // colour c: vertices with (j - i) mod 3 == c; [i * M + j / 3]
};

int colour_of(int i, int j) { return ((j - i) % 3 + 3) % 3; }

void lsplit(const int* t, int N, LChain& c) {
  c.N = N;
  c.M = N / 3;
  for (auto& x : c.X) x.assign((size_t)N * c.M, 0);
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) c.X[colour_of(i, j)][(size_t)i * c.M + j / 3] = (uint8_t)t[(size_t)i * N + j];
}

void lmerge(const LChain& c, int* t) {
  for (int i = 0; i < c.N; ++i)
    for (int j = 0; j < c.N; ++j) t[(size_t)i * c.N + j] = c.X[colour_of(i, j)][(size_t)i * c.M + j / 3];
}

// The rotation rule: 0 = lozengekernel.cl:92-96 (up when rd < 0.4, down when 0.4 <= rd < 0.8);
// 1 = qlozengekernel.cl:23-29 with q runtime and its down-move rescaling written as the
// intended (rd - 0.5) / 0.5.  TinyMT: rd = u23 * 2^-23 in the reference's float expressions.
// Fast mode: rule 0 up iff u < ceil(0.4 * 2^32), down iff ceil(0.4 * 2^32) <= u <
// ceil(0.8 * 2^32); rule 1 up iff u < 2^31 and u <= q 2^31, down iff u >= 2^31 and
// u - 2^31 <= 2^31 / q.
int g_lz_rule = 0;
double g_lz_q = 1.0;

inline uint8_t lrotate_cl(uint8_t e, float rd) {
  if (g_lz_rule == 1) {
    if (rd < .5) {
      rd = (float)(rd / .5);
      if (e == 25 && g_lz_q >= rd) return 38;
    } else {
      rd = (float)((rd - .5) / .5);
      if (e == 38 && 1 / g_lz_q >= rd) return 25;
    }
    return e;
  }
  if ((double)rd < .4) {
    if (e == 25) return 38;
  } else if ((double)rd < .8) {
    if (e == 38) return 25;
  }
  return e;
}
inline uint8_t lrotate_fast(uint8_t e, uint32_t u) {
  if (g_lz_rule == 1) {
    if (u < 0x80000000u) return (e == 25 && (double)u <= g_lz_q * 2147483648.0) ? 38 : e;
    return (e == 38 && (double)(u - 0x80000000u) <= 2147483648.0 / g_lz_q) ? 25 : e;
  }
  const uint64_t c4 = (uint64_t)std::ceil(0.4 * 4294967296.0), c8 = (uint64_t)std::ceil(0.8 * 4294967296.0);
  if (u < c4) return e == 25 ? 38 : e;
  if (u < c8) return e == 38 ? 25 : e;
  return e;
}

// lozengekernel.cl:107-125: rebuilds bits of the two passive colours from the active one.
void lupdate(LChain& c, int r) {
  const int N = c.N, M = c.M, t = r;
  const uint8_t* A = c.X[r].data();
  uint8_t* T2 = c.X[(r + 1) % 3].data();
  uint8_t* T3 = c.X[(r + 2) % 3].data();
  for (int i = 1; i < N - 1; ++i)
    for (int j = 1; j < M - 1; ++j) {
      const int p2 = (i % 3 == (2 * t + 1) % 3), p4 = (i % 3 == (2 * t + 2) % 3);
      const int p8 = (i % 3 == (2 * t) % 3), p16 = p2;
      uint8_t& a = T2[(size_t)i * M + j];
      a = (uint8_t)((a & ~(2 | 4 | 32)) + ((A[(size_t)(i - 1) * M + j + p2] & 16) / 8) + ((A[(size_t)i * M + j - p4] & 8) / 2) +
                    ((A[(size_t)(i + 1) * M + j] & 1) * 32));
      uint8_t& b = T3[(size_t)i * M + j];
      b = (uint8_t)((b & ~(1 | 8 | 16)) + ((A[(size_t)(i - 1) * M + j] & 32) / 32) + ((A[(size_t)i * M + j + p8] & 4) * 2) +
                    ((A[(size_t)(i + 1) * M + j - p16] & 2) * 8));
    }
}

void linit(std::vector<oracle::TinyMT32>& g, size_t count, uint32_t seed, const uint32_t* params, long nparams) {
  g.resize(count);
  for (size_t k = 0; k < count; ++k) {
    auto& x = g[k];
    if (params && (long)k < nparams) {
      x.mat1 = params[3 * k]; x.mat2 = params[3 * k + 1]; x.tmat = params[3 * k + 2];
    } else {
      x.mat1 = oracle::kTmtMat1; x.mat2 = oracle::kTmtMat2; x.tmat = oracle::kTmtTmat;
    }
    oracle::tmt_init(x, seed + (uint32_t)k);
  }
}

// One reference Walk(t, steps, seed) on coupled chains sharing the generators.
void lwalk_tinymt(std::vector<LChain*>& chains, long steps, long seed, const uint32_t* params, long nparams) {
  const int N = chains[0]->N, M = chains[0]->M;
  std::vector<oracle::TinyMT32> g;
  linit(g, (size_t)N * M, (uint32_t)seed, params, nparams);
  std::default_random_engine gen;
  std::uniform_int_distribution<int> dist(0, 2);
  gen.seed(seed);
  for (long s = 0; s < steps; ++s) {
    const int r = dist(gen);
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < M; ++j) {
        float rd = oracle::tmt_u23_to_float(oracle::tmt_next_u23(g[(size_t)i * M + j]));
        for (LChain* c : chains) {
          uint8_t& e = c->X[r][(size_t)i * M + j];
          e = lrotate_cl(e, rd);
        }
      }
    for (LChain* c : chains) lupdate(*c, r);
  }
}

// lozengekernel.cu:23-29: up when the float draw is below the double .4, down when it lies in
// [.4, .8).
inline uint8_t lrotate_cu(uint8_t e, float rd) {
  if (rd < .4) return e == 25 ? 38 : e;
  if (rd < .8) return e == 38 ? 25 : e;
  return e;
}

// One reference Walk(t, steps, seed) of the CUDA path with draws[s][i][j] the curand_uniform
// value of slot (i, j) at step s.
void lwalk_draws(std::vector<LChain*>& chains, const float* draws, long steps, long seed) {
  const int N = chains[0]->N, M = chains[0]->M;
  std::default_random_engine gen;
  std::uniform_int_distribution<int> dist(0, 2);
  gen.seed(seed);
  for (long s = 0; s < steps; ++s) {
    const int r = dist(gen);
    const float* d = draws + (size_t)s * N * M;
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < M; ++j)
        for (LChain* c : chains) {
          uint8_t& e = c->X[r][(size_t)i * M + j];
          e = lrotate_cu(e, d[(size_t)i * M + j]);
        }
    for (LChain* c : chains) lupdate(*c, r);
  }
}

inline int fast_colour(long h) { return (int)(((h % 3) + 3) % 3); }

void lwalk_fast(std::vector<LChain*>& chains, long h0, long steps, unsigned long seed, unsigned stream) {
  const int N = chains[0]->N, M = chains[0]->M;
  for (long s = 0; s < steps; ++s) {
    const long h = h0 + s;
    const int r = fast_colour(h);
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < M; ++j) {
        uint32_t u = oracle::fast_draw(seed, stream, h, (uint32_t)i, (uint32_t)j);
        for (LChain* c : chains) {
          uint8_t& e = c->X[r][(size_t)i * M + j];
          e = lrotate_fast(e, u);
        }
      }
    for (LChain* c : chains) lupdate(*c, r);
  }
}

}  // namespace

extern "C" {

// Selects the rotation rule of the walks and CFTP below (0 uniform, 1 q^volume with q).
void orc_lz_set_rule(int rule, double q) {
  g_lz_rule = rule;
  g_lz_q = q;
}

int orc_lz_almost_hex_domain(int n, int m, int* out, long cap) {
  // LozengeTiler.cpp:422-467: a 2n x 4n triangle array of the hexagon of side n with an m x 2m
  // corner removed, padded by 3 rows / 6 columns, then grown so the vertex side is a
  // multiple of 3.  Returns the row count M2 + k (the domain is rows x 2 rows).
  std::vector<int> d((size_t)2 * n * 4 * n, 0);
  const int W2 = 4 * n + 12;
  std::vector<int> d2((size_t)(2 * n + 6) * W2, 0);
  if (m > n) return -1;
  for (int i = 0; i < 2 * n; ++i)
    for (int j = 0; j < 4 * n; ++j) {
      bool in = (i < n) ? (2 * i + j - 1 >= 2 * n - 2) : (2 * i + j <= 6 * n - 2);
      if (in) d[(size_t)i * 4 * n + j] = 1;
    }
  for (int i = 0; i < m; ++i)
    for (int j = 4 * n - 2 * m; j < 4 * n; ++j) d[(size_t)i * 4 * n + j] = 0;
  for (int i = 3; i < 2 * n + 3; ++i)
    for (int j = 6; j < 4 * n + 6; ++j) d2[(size_t)i * W2 + j] = d[(size_t)(i - 3) * 4 * n + j - 6];
  const int M2 = (int)std::lround(std::sqrt((double)d2.size() / 2));
  const int k = (3 - (M2 + 1) % 3) % 3;
  const int R = M2 + k;
  if ((long)R * 2 * R > cap) return -R;
  std::fill(out, out + (size_t)R * 2 * R, 0);
  for (int i = 0; i < M2; ++i)
    for (int j = 0; j < 2 * M2; ++j) out[(size_t)i * 2 * R + j] = d2[(size_t)i * 2 * M2 + j];
  return R;
}

void orc_lz_domain_to_vertices(const int* d, int M, int* out) {
  std::vector<int> v = vertices_of(d, M);
  std::memcpy(out, v.data(), v.size() * sizeof(int));
}

int orc_lz_max_tiling(const int* d, int M, int* out) {
  std::vector<int> t;
  int rc = extremal<true>(d, M, t);
  std::memcpy(out, t.data(), t.size() * sizeof(int));
  return rc;
}

int orc_lz_min_tiling(const int* d, int M, int* out) {
  std::vector<int> t;
  int rc = extremal<false>(d, M, t);
  std::memcpy(out, t.data(), t.size() * sizeof(int));
  return rc;
}

void orc_lz_heightfunc_to_tiling(const int* hf, const int* d, int N, int* out) {
  std::vector<int> h(hf, hf + (size_t)N * N);
  std::vector<int> t = hf_to_tiling(h, d, N);
  std::memcpy(out, t.data(), t.size() * sizeof(int));
}

void orc_lz_tiling_to_heightfunc(const int* t, const int* d, int N, int* out) {
  const int M = N - 1;
  Dom D{d, M};
  std::vector<int> v = vertices_of(d, M);
  std::vector<int> hf((size_t)N * N, kInf);
  std::queue<std::pair<int, int>> q;
  bool found = false;
  for (int i = 0; i < N && !found; ++i)
    for (int j = 0; j < N && !found; ++j)
      if (v[(size_t)i * N + j] == 2) {
        found = true;
        q.push({i, j});
        hf[(size_t)i * N + j] = 0;
      }
  while (!q.empty()) {
    auto [i0, j0] = q.front();
    q.pop();
    for (int nb = 0; nb < 6; ++nb) {
      if (t[(size_t)i0 * N + j0] & kBit[nb]) continue;
      int i = i0 + kNb[nb][0], j = j0 + kNb[nb][1];
      if (v[(size_t)i * N + j] > 0 && hf[(size_t)i * N + j] == kInf && (D.face(i0, j0, nb, 0) || D.face(i0, j0, nb, 1))) {
        hf[(size_t)i * N + j] = hf[(size_t)i0 * N + j0] + kDh[nb];
        q.push({i, j});
      }
    }
  }
  std::memcpy(out, hf.data(), hf.size() * sizeof(int));
}

void orc_lz_tiling_to_domain(const int* t, int N, int* out) {
  const int M = N - 1;
  std::fill(out, out + (size_t)2 * M * M, 0);
  for (int i = 1; i < N - 1; ++i)
    for (int j = 0; j < N - 1; ++j) {
      const int v = t[(size_t)i * N + j];
      if (v & 1) out[(size_t)(i - 1) * 2 * M + 2 * j] = 1, out[(size_t)(i - 1) * 2 * M + 2 * j - 1] = 1;
      if (v & 2) out[(size_t)(i - 1) * 2 * M + 2 * j] = 1, out[(size_t)(i - 1) * 2 * M + 2 * j + 1] = 1;
      if (v & 8) out[(size_t)(i - 1) * 2 * M + 2 * j + 1] = 1, out[(size_t)i * 2 * M + 2 * j] = 1;
    }
}

int orc_lz_walk_tinymt(int* t, int N, long steps, long seed, const uint32_t* params, long nparams) {
  if (N % 3 || N < 6) return -1;
  LChain c;
  lsplit(t, N, c);
  std::vector<LChain*> ch{&c};
  lwalk_tinymt(ch, steps, seed, params, nparams);
  lmerge(c, t);
  return 0;
}

// LozengeTiler::Walk(t, steps, seed), CUDA path, with the MTGP32 draws supplied
// (steps x N x N/3 floats).
int orc_lz_walk_draws(int* t, int N, const float* draws, long steps, long seed) {
  if (N % 3 || N < 6) return -1;
  LChain c;
  lsplit(t, N, c);
  std::vector<LChain*> ch{&c};
  lwalk_draws(ch, draws, steps, seed);
  lmerge(c, t);
  return 0;
}

// The CUDA kernel's rotation of one colour array (N rows x N/3 bytes), draws per slot.
void orc_lz_rotate_cuda_grid(uint8_t* colour, int N, const float* draws) {
  const size_t n = (size_t)N * (N / 3);
  for (size_t k = 0; k < n; ++k) colour[k] = lrotate_cu(colour[k], draws[k]);
}

int orc_lz_walk_fast(int* t, int N, long h0, long steps, unsigned long seed, unsigned stream) {
  if (N % 3 || N < 6) return -1;
  LChain c;
  lsplit(t, N, c);
  std::vector<LChain*> ch{&c};
  lwalk_fast(ch, h0, steps, seed, stream);
  lmerge(c, t);
  return 0;
}

// CFTP with the reference's primitives: each epoch is one Walk(t, steps_k, seed_k) on both
// chains (schedule 0: prepend 2 * steps.back(), 1: 2 * steps.front()); fast mode: attempt j
// runs half-steps [-3T, 0) with T = first * 2^j full sweeps.
int orc_lz_cftp(const int* tmax, const int* tmin, int N, long driver_seed, long first, int schedule, int max_attempts,
                int fast, unsigned stream, int* out, long* total_steps) {
  std::mt19937 drv((uint32_t)driver_seed);
  std::vector<long> steps{first}, seeds{(long)drv()};
  long total = 0, T = first;
  for (int attempt = 1; attempt <= max_attempts; ++attempt) {
    LChain top, bot;
    lsplit(tmax, N, top);
    lsplit(tmin, N, bot);
    std::vector<LChain*> ch{&bot, &top};
    if (fast) {
      lwalk_fast(ch, -3 * T, 3 * T, (unsigned long)driver_seed, stream);
      total += 3 * T;
    } else {
      for (size_t k = 0; k < steps.size(); ++k) {
        lwalk_tinymt(ch, steps[k], seeds[k], nullptr, 0);
        total += steps[k];
      }
    }
    bool same = top.X[0] == bot.X[0] && top.X[1] == bot.X[1] && top.X[2] == bot.X[2];
    if (same) {
      lmerge(top, out);
      if (total_steps) *total_steps = total;
      return attempt;
    }
    if (fast) {
      T *= 2;
    } else {
      long next = schedule == 0 ? steps.back() * 2 : steps.front() * 2;
      steps.insert(steps.begin(), next);
      seeds.insert(seeds.begin(), (long)drv());
    }
  }
  if (total_steps) *total_steps = total;
  return -1;
}

}  // extern "C"
