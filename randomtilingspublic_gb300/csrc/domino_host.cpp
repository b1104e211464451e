// Domino host utilities behind the C ABI: domain constructors, Thurston's extremal
// tilings and height functions.  They run on the host, as in the reference
// (src/Domino/DominoTiler.cpp:249-631); the sweep itself lives in domino_sweep.cu.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <queue>
#include <utility>
#include <vector>

#include "rt_internal.h"

namespace rt {
namespace {

constexpr int32_t kUnset = INT32_MAX;  // "infty" of src/common/common.h:47

// Neighbour (di, dj), the two faces beside the edge toward it, and the indicator bit of
// that edge (DominoTiler.cpp:335-337, in the same order).
struct Dir { int di, dj, fa_i, fa_j, fb_i, fb_j, bit; };
constexpr Dir kDirs[4] = {
    {1, 0, 0, -1, 0, 0, 2},
    {-1, 0, -1, -1, -1, 0, 1},
    {0, 1, -1, 0, 0, 0, 8},
    {0, -1, -1, -1, 0, -1, 4},
};

// Height change when stepping from (i0, j0) along direction nb: +-1 by the colour of the
// vertex and the axis of the step (DominoTiler.cpp:352-363).
inline int height_step(int i0, int j0, int nb) {
  int axis = nb > 1 ? 1 : -1;
  int colour = ((i0 + j0) % 2 == 0) ? 1 : -1;
  return axis * colour;
}

struct Grid {
  const int32_t* d;  // M x M squares
  int M, N;
  int32_t sq(int i, int j) const { return d[(size_t)i * M + j]; }
  bool edge_is_boundary(int i0, int j0, int nb) const {
    const Dir& q = kDirs[nb];
    return (sq(i0 + q.fa_i, j0 + q.fa_j) != 0) != (sq(i0 + q.fb_i, j0 + q.fb_j) != 0);
  }
  bool edge_touches_domain(int i0, int j0, int nb) const {
    const Dir& q = kDirs[nb];
    return sq(i0 + q.fa_i, j0 + q.fa_j) || sq(i0 + q.fb_i, j0 + q.fb_j);
  }
};

// Vertex classes: 0 outside, 1 interior (all four squares in the domain), 2 boundary.
void vertex_classes(const int32_t* d, int M, int32_t* v) {
  const int N = M + 1;
  for (int i = 0; i < N; ++i) {
    for (int j = 0; j < N; ++j) {
      // The four squares around vertex (i, j), clamped into the array at its rim
      // (DominoTiler.cpp:617-620 clamps the same way).
      int lo_i = (i == 0) ? 0 : i - 1, hi_i = (i == M) ? M - 1 : i;
      int lo_j = (j == 0) ? 0 : j - 1, hi_j = (j == M) ? M - 1 : j;
      int s00 = d[(size_t)lo_i * M + lo_j], s01 = d[(size_t)lo_i * M + hi_j];
      int s10 = d[(size_t)hi_i * M + lo_j], s11 = d[(size_t)hi_i * M + hi_j];
      bool rim = (i == 0 || j == 0 || i == M || j == M);
      int32_t cls = 0;
      if (!rim && s00 && s01 && s10 && s11) cls = 1;
      else if (s00 || s01 || s10 || s11) cls = 2;
      v[(size_t)i * N + j] = cls;
    }
  }
}

void hf_to_tiling(const int32_t* hf, const int32_t* d, int N, int32_t* t) {
  const int M = N - 1;
  std::fill(t, t + (size_t)N * N, 0);
  for (int i0 = 0; i0 < N; ++i0) {
    for (int j0 = 0; j0 < N; ++j0) {
      int32_t h0 = hf[(size_t)i0 * N + j0];
      if (h0 == kUnset) continue;
      for (int nb = 0; nb < 4; ++nb) {
        int i = i0 + kDirs[nb].di, j = j0 + kDirs[nb].dj;
        int32_t h1 = hf[(size_t)i * N + j];
        if (h1 == kUnset) continue;
        // The two squares beside the edge (DominoTiler.cpp:545).
        int fa = (i0 - (nb == 1) - (nb > 1)) * M + j0 - (nb <= 1) - (nb == 3);
        int fb = (i0 - (nb == 1)) * M + j0 - (nb == 3);
        if (d[fa] || d[fb]) t[(size_t)i0 * N + j0] += kDirs[nb].bit * std::abs((h1 - h0) / 2);
      }
    }
  }
}

using Entry = std::pair<std::pair<int, int>, int>;
struct LowestFirst {
  bool operator()(const Entry& x, const Entry& y) const { return x.second > y.second; }
};
struct HighestFirst {
  bool operator()(const Entry& x, const Entry& y) const { return x.second < y.second; }
};

// Thurston's algorithm (DominoTiler.cpp:345-531): boundary heights by a walk along the
// boundary edges, then the bulk filled from the extreme boundary vertex inward, moving
// only upward (max) or downward (min).
template <bool kMax>
rt_status thurston(const int32_t* d, int M, int32_t* out) {
  const int N = M + 1;
  std::vector<int32_t> v((size_t)N * N);
  vertex_classes(d, M, v.data());
  std::vector<int32_t> hf((size_t)N * N, kUnset);
  Grid g{d, M, N};

  std::queue<std::pair<int, int>> walk;
  for (size_t p = 0; p < v.size(); ++p) {
    if (v[p] == 2) {
      walk.push({(int)(p / N), (int)(p % N)});
      hf[p] = 0;
      break;
    }
  }
  using PQ = std::priority_queue<Entry, std::vector<Entry>, typename std::conditional<kMax, LowestFirst, HighestFirst>::type>;
  PQ bulk;
  while (!walk.empty()) {
    auto [i0, j0] = walk.front();
    walk.pop();
    for (int nb = 0; nb < 4; ++nb) {
      int i = i0 + kDirs[nb].di, j = j0 + kDirs[nb].dj;
      if (v[(size_t)i * N + j] != 2 || !g.edge_is_boundary(i0, j0, nb)) continue;
      int32_t h = hf[(size_t)i0 * N + j0] + height_step(i0, j0, nb);
      int32_t& slot = hf[(size_t)i * N + j];
      if (slot == kUnset) {
        slot = h;
        walk.push({i, j});
        bulk.push({{i, j}, h});
      } else if (slot != h) {
        set_error("domain is not tileable (boundary height mismatch)");
        return RT_ERR_NOT_TILEABLE;
      }
    }
  }
  while (!bulk.empty()) {
    Entry e = bulk.top();
    bulk.pop();
    int i0 = e.first.first, j0 = e.first.second;
    int32_t here = hf[(size_t)i0 * N + j0];
    for (int nb = 0; nb < 4; ++nb) {
      int i = i0 + kDirs[nb].di, j = j0 + kDirs[nb].dj;
      if (i < 0 || j < 0 || i >= N || j >= N || v[(size_t)i * N + j] == 0) continue;
      int dir = height_step(i0, j0, nb);
      if (kMax ? dir <= 0 : dir >= 0) continue;
      int32_t& slot = hf[(size_t)i * N + j];
      bool bad = kMax ? (v[(size_t)i * N + j] == 2 && slot > here + 1 && v[(size_t)i0 * N + j0] != 2)
                      // DominoTiler.cpp:519 tests the height, not the vertex class, against 2.
                      : (v[(size_t)i * N + j] == 2 && slot < here - 1 && here != 2);
      if (bad) {
        set_error("domain is not tileable (bulk height mismatch)");
        return RT_ERR_NOT_TILEABLE;
      }
      if (slot == kUnset) {
        slot = kMax ? here + 1 : here - 1;
        bulk.push({{i, j}, slot});
      }
    }
  }
  hf_to_tiling(hf.data(), d, N, out);
  return RT_OK;
}

}  // namespace

void domino_vertex_classes(const int32_t* d, int M, int32_t* v) { vertex_classes(d, M, v); }

int64_t domino_count_interior_from_tiling(const int32_t* t, int N) {
  // TilingToDomain (DominoTiler.cpp:595-609) followed by the interior test of
  // DomainToVertices: a vertex is interior when its four squares are covered.
  const int M = N - 1;
  std::vector<uint8_t> sq((size_t)M * M);
  for (int i = 0; i < M; ++i)
    for (int j = 0; j < M; ++j)
      sq[(size_t)i * M + j] = ((t[(size_t)i * N + j] & 10) != 0) || ((t[(size_t)(i + 1) * N + j + 1] & 5) != 0);
  int64_t count = 0;
  for (int i = 1; i < M; ++i)
    for (int j = 1; j < M; ++j)
      count += sq[(size_t)(i - 1) * M + j - 1] && sq[(size_t)(i - 1) * M + j] && sq[(size_t)i * M + j - 1] &&
               sq[(size_t)i * M + j];
  return count;
}

}  // namespace rt

using namespace rt;

extern "C" {

RT_API rt_status rt_domino_aztec_rectangle(int32_t n, const int32_t* remove, int32_t n_remove, int32_t* out,
                                           int64_t cap, int32_t* side) {
  clear_error();
  if (n < 1 || n_remove < 0 || n_remove >= 2 * n || (n_remove > 0 && !remove) || !side)
    return fail(RT_ERR_INVALID_ARGUMENT, "aztec_rectangle: need n >= 1, 0 <= n_remove < 2n");
  const int k = n_remove, M = 2 * n - k;
  const int M2 = M + 4 + (1 - M % 2);  // padded, odd (DominoTiler.cpp:315)
  *side = M2;
  if (!out || cap < (int64_t)M2 * M2) return fail(RT_ERR_BUFFER_TOO_SMALL, "aztec_rectangle: output too small");
  std::fill(out, out + (size_t)M2 * M2, 0);
  // Row r of the M x M diamond spans a run of squares that widens by one on each side per
  // row down to row n-k, stays at full width, then narrows (DominoTiler.cpp:273-296).
  for (int r = 0; r < M; ++r) {
    int lo, hi;
    if (r == 0 || r == M - 1) {
      int c = (n - k) + (r == M - 1 ? k : 0);
      lo = c - 1;
      hi = c;
    } else if (r < n - k) {
      lo = n - k - r - 1;
      hi = n - k + r;
    } else if (r > n - 1) {
      lo = r - n + k;
      hi = 3 * n - k - r - 1;
    } else {
      lo = r - (n - k);
      hi = r + (n - k);
    }
    lo = std::max(lo, 0);
    hi = std::min(hi, M - 1);
    for (int c = lo; c <= hi; ++c) out[(size_t)(r + 2) * M2 + c + 2] = 1;
  }
  for (int q = 0; q < k; ++q) {
    int r = n - k + remove[q], c = remove[q];
    if (r >= 0 && r < M && c >= 0 && c < M) out[(size_t)(r + 2) * M2 + c + 2] = 0;
  }
  return RT_OK;
}

RT_API rt_status rt_domino_aztec_diamond(int32_t n, int32_t* out, int64_t cap, int32_t* side) {
  return rt_domino_aztec_rectangle(n, nullptr, 0, out, cap, side);
}

RT_API rt_status rt_domino_rectangle(int32_t rows, int32_t cols, int32_t* out, int64_t cap, int32_t* side) {
  clear_error();
  if (rows < 1 || cols < 1 || !side) return fail(RT_ERR_INVALID_ARGUMENT, "rectangle: rows, cols >= 1");
  int dim = std::max(rows, cols) + 4;
  if (dim % 2 == 0) dim++;
  *side = dim;
  if (!out || cap < (int64_t)dim * dim) return fail(RT_ERR_BUFFER_TOO_SMALL, "rectangle: output too small");
  std::fill(out, out + (size_t)dim * dim, 0);
  for (int r = 0; r < rows; ++r)
    for (int c = 0; c < cols; ++c) out[(size_t)(r + 2) * dim + c + 2] = 1;
  return RT_OK;
}

RT_API rt_status rt_domino_domain_to_vertices(const int32_t* domain, int32_t m_side, int32_t* out) {
  clear_error();
  if (!domain || !out || m_side < 2) return fail(RT_ERR_INVALID_ARGUMENT, "domain_to_vertices: bad arguments");
  vertex_classes(domain, m_side, out);
  return RT_OK;
}

static rt_status check_padded_domain(const int32_t* domain, int32_t m_side) {
  if (!domain || m_side < 5) return fail(RT_ERR_INVALID_ARGUMENT, "domain must be at least 5 x 5");
  for (int i = 0; i < m_side; ++i)
    for (int j = 0; j < m_side; ++j)
      if ((i < 1 || j < 1 || i >= m_side - 1 || j >= m_side - 1) && domain[(size_t)i * m_side + j])
        return fail(RT_ERR_INVALID_ARGUMENT, "domain must have an empty outer ring of squares");
  return RT_OK;
}

RT_API rt_status rt_domino_max_tiling(const int32_t* domain, int32_t m_side, int32_t* out) {
  clear_error();
  if (rt_status s = check_padded_domain(domain, m_side)) return s;
  if (!out) return fail(RT_ERR_INVALID_ARGUMENT, "max_tiling: out is NULL");
  return thurston<true>(domain, m_side, out);
}

RT_API rt_status rt_domino_min_tiling(const int32_t* domain, int32_t m_side, int32_t* out) {
  clear_error();
  if (rt_status s = check_padded_domain(domain, m_side)) return s;
  if (!out) return fail(RT_ERR_INVALID_ARGUMENT, "min_tiling: out is NULL");
  return thurston<false>(domain, m_side, out);
}

RT_API rt_status rt_domino_heightfunc_to_tiling(const int32_t* hf, const int32_t* domain, int32_t n_side,
                                                int32_t* out) {
  clear_error();
  if (!hf || !domain || !out || n_side < 3) return fail(RT_ERR_INVALID_ARGUMENT, "heightfunc_to_tiling: bad arguments");
  for (int i = 0; i < n_side; ++i)
    for (int j = 0; j < n_side; ++j)
      if ((i == 0 || j == 0 || i == n_side - 1 || j == n_side - 1) && hf[(size_t)i * n_side + j] != kUnset)
        return fail(RT_ERR_INVALID_ARGUMENT, "heightfunc_to_tiling: heights must be unset on the array rim");
  hf_to_tiling(hf, domain, n_side, out);
  return RT_OK;
}

RT_API rt_status rt_domino_tiling_to_heightfunc(const int32_t* t, const int32_t* domain, int32_t n_side,
                                                int32_t* out) {
  clear_error();
  if (!t || !domain || !out || n_side < 3) return fail(RT_ERR_INVALID_ARGUMENT, "tiling_to_heightfunc: bad arguments");
  const int N = n_side, M = N - 1;
  if (rt_status s = check_padded_domain(domain, M)) return s;
  std::vector<int32_t> v((size_t)N * N);
  vertex_classes(domain, M, v.data());
  std::fill(out, out + (size_t)N * N, kUnset);
  Grid g{domain, M, N};
  // Breadth-first from the first boundary vertex, crossing only edges no domino covers
  // (DominoTiler.cpp:555-593).
  std::queue<std::pair<int, int>> q;
  for (size_t p = 0; p < v.size(); ++p) {
    if (v[p] == 2) {
      q.push({(int)(p / N), (int)(p % N)});
      out[p] = 0;
      break;
    }
  }
  while (!q.empty()) {
    auto [i0, j0] = q.front();
    q.pop();
    int32_t mask = t[(size_t)i0 * N + j0];
    for (int nb = 0; nb < 4; ++nb) {
      if (mask & kDirs[nb].bit) continue;
      int i = i0 + kDirs[nb].di, j = j0 + kDirs[nb].dj;
      if (v[(size_t)i * N + j] == 0 || out[(size_t)i * N + j] != kUnset) continue;
      if (!g.edge_touches_domain(i0, j0, nb)) continue;
      out[(size_t)i * N + j] = out[(size_t)i0 * N + j0] + height_step(i0, j0, nb);
      q.push({i, j});
    }
  }
  return RT_OK;
}

RT_API rt_status rt_domino_tiling_to_domain(const int32_t* t, int32_t n_side, int32_t* out) {
  clear_error();
  if (!t || !out || n_side < 2) return fail(RT_ERR_INVALID_ARGUMENT, "tiling_to_domain: bad arguments");
  const int N = n_side, M = N - 1;
  for (int i = 0; i < M; ++i)
    for (int j = 0; j < M; ++j)
      out[(size_t)i * M + j] = ((t[(size_t)i * N + j] & (2 | 8)) != 0) || ((t[(size_t)(i + 1) * N + j + 1] & (1 | 4)) != 0);
  return RT_OK;
}

}  // extern "C"

extern "C" {

// Adds the edge-placement indicators of a tiling to counts ([2][N][N], the layout of
// rt_dm_sampler_accumulate_edges).
RT_API rt_status rt_domino_edge_indicators(const int32_t* tiling, int32_t n_side, uint32_t* counts) {
  rt::clear_error();
  if (!tiling || !counts || n_side < 1) return rt::fail(RT_ERR_INVALID_ARGUMENT, "edge_indicators: bad arguments");
  const size_t nn = (size_t)n_side * n_side;
  for (size_t k = 0; k < nn; ++k) {
    if (tiling[k] & 2) counts[k] += 1u;
    if (tiling[k] & 8) counts[nn + k] += 1u;
  }
  return RT_OK;
}

}  // extern "C"
