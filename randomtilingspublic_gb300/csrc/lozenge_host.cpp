// Lozenge host utilities behind the C ABI: the almost-hexagon domain, Thurston's extremal
// tilings and height functions (src/Lozenge/LozengeTiler.cpp:173-556 of the reference).
//
// Geometry: vertex (i, j) of the triangular lattice, six neighbours (0,+1) (-1,+1) (-1,0)
// (0,-1) (+1,-1) (+1,0) with edge bits 8 2 1 4 16 32 and height steps -1 +1 -1 +1 -1 +1.  A
// domain is an M x 2M array of triangles; the two triangles beside the edge toward
// neighbour nb of vertex (i0, j0) are (i0 + a, 2 j0 + b) for the offsets in kFaces.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <queue>
#include <vector>

#include "rt_internal.h"

namespace rt {
namespace {

constexpr int32_t kUnset = INT32_MAX;

struct Step { int di, dj, dh, bit; int fa_i, fa_j, fb_i, fb_j; };
constexpr Step kSteps[6] = {
    {0, 1, -1, 8, 0, 0, -1, 1},      {-1, 1, 1, 2, -1, 1, -1, 0},   {-1, 0, -1, 1, -1, 0, -1, -1},
    {0, -1, 1, 4, -1, -1, 0, -2},    {1, -1, -1, 16, 0, -2, 0, -1}, {1, 0, 1, 32, 0, -1, 0, 0},
};

struct Tri {
  const int32_t* d;
  int M;
  bool a(int i0, int j0, int nb) const {
    const Step& s = kSteps[nb];
    return d[(size_t)(i0 + s.fa_i) * 2 * M + 2 * j0 + s.fa_j] != 0;
  }
  bool b(int i0, int j0, int nb) const {
    const Step& s = kSteps[nb];
    return d[(size_t)(i0 + s.fb_i) * 2 * M + 2 * j0 + s.fb_j] != 0;
  }
};

// Vertex classes (LozengeTiler.cpp:483-512): interior when all six surrounding triangles lie
// in the domain, boundary when some do; the array's rim is left 0.
void vertex_classes(const int32_t* d, int M, int32_t* v) {
  const int N = M + 1;
  std::fill(v, v + (size_t)N * N, 0);
  for (int i = 1; i < M; ++i)
    for (int j = 1; j < M; ++j) {
      const int32_t* lo = d + (size_t)i * 2 * M;
      const int32_t* up = d + (size_t)(i - 1) * 2 * M;
      const int f[6] = {lo[2 * j], lo[2 * j - 1], lo[2 * j - 2], up[2 * j], up[2 * j + 1], up[2 * j - 1]};
      int n = 0;
      for (int k = 0; k < 6; ++k) n += f[k] != 0;
      v[(size_t)i * N + j] = n == 6 ? 1 : (n > 0 ? 2 : 0);
    }
}

void hf_to_tiling(const int32_t* hf, const int32_t* d, int N, int32_t* t) {
  Tri T{d, N - 1};
  std::fill(t, t + (size_t)N * N, 0);
  for (int i0 = 1; i0 < N - 1; ++i0)
    for (int j0 = 1; j0 < N - 1; ++j0) {
      const int64_t h0 = hf[(size_t)i0 * N + j0];
      for (int nb = 0; nb < 6; ++nb) {
        if (!T.a(i0, j0, nb) && !T.b(i0, j0, nb)) continue;
        const int64_t h1 = hf[(size_t)(i0 + kSteps[nb].di) * N + j0 + kSteps[nb].dj];
        if (h1 - h0 == 2 || h0 - h1 == 2) t[(size_t)i0 * N + j0] += kSteps[nb].bit;  // a lozenge crosses the edge
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

// Thurston (LozengeTiler.cpp:218-397): heights along the boundary edges, then the bulk from
// the extreme boundary vertex, moving only up (max) or only down (min).
template <bool kMax>
rt_status extremal(const int32_t* d, int M, int32_t* out) {
  const int N = M + 1;
  std::vector<int32_t> v((size_t)N * N), hf((size_t)N * N, kUnset);
  vertex_classes(d, M, v.data());
  Tri T{d, M};
  std::queue<std::pair<int, int>> ring;
  for (size_t p = 0; p < v.size(); ++p)
    if (v[p] == 2) {
      ring.push({(int)(p / N), (int)(p % N)});
      hf[p] = 0;
      break;
    }
  std::priority_queue<Entry, std::vector<Entry>, typename std::conditional<kMax, LowestFirst, HighestFirst>::type> bulk;
  while (!ring.empty()) {
    auto [i0, j0] = ring.front();
    ring.pop();
    for (int nb = 0; nb < 6; ++nb) {
      const int i = i0 + kSteps[nb].di, j = j0 + kSteps[nb].dj;
      if (v[(size_t)i * N + j] != 2 || T.a(i0, j0, nb) == T.b(i0, j0, nb)) continue;
      const int32_t h = hf[(size_t)i0 * N + j0] + kSteps[nb].dh;
      int32_t& slot = hf[(size_t)i * N + j];
      if (slot == kUnset) {
        slot = h;
        ring.push({i, j});
        bulk.push({{i, j}, h});
      } else if (slot != h) {
        return fail(RT_ERR_NOT_TILEABLE, "lozenge domain is not tileable (boundary height mismatch)");
      }
    }
  }
  while (!bulk.empty()) {
    const Entry e = bulk.top();
    bulk.pop();
    const int i0 = e.first.first, j0 = e.first.second;
    for (int nb = 0; nb < 6; ++nb) {
      const int dh = kSteps[nb].dh;
      if (kMax ? dh <= 0 : dh >= 0) continue;
      const int i = i0 + kSteps[nb].di, j = j0 + kSteps[nb].dj;
      if (v[(size_t)i * N + j] <= 0) continue;
      const int32_t h = hf[(size_t)i0 * N + j0] + dh;
      int32_t& slot = hf[(size_t)i * N + j];
      if (v[(size_t)i * N + j] == 2 && (kMax ? slot > h : slot < h))
        return fail(RT_ERR_NOT_TILEABLE, "lozenge domain is not tileable (bulk height mismatch)");
      if (slot == kUnset) {
        slot = h;
        bulk.push({{i, j}, h});
      }
    }
  }
  for (size_t p = 0; p < v.size(); ++p)
    if (v[p] == 0) hf[p] = kUnset;
  hf_to_tiling(hf.data(), d, N, out);
  return RT_OK;
}

rt_status check_domain(const int32_t* d, int M) {
  if (!d || M < 4) return fail(RT_ERR_INVALID_ARGUMENT, "lozenge domain must have at least 4 rows");
  for (int i = 0; i < M; ++i)
    for (int j = 0; j < 2 * M; ++j)
      if ((i == 0 || i == M - 1 || j < 2 || j >= 2 * M - 2) && d[(size_t)i * 2 * M + j])
        return fail(RT_ERR_INVALID_ARGUMENT, "lozenge domain must leave its outer rows and two outer columns empty");
  return RT_OK;
}

}  // namespace
}  // namespace rt

using namespace rt;

extern "C" {

RT_API rt_status rt_lozenge_almost_hex_domain(int32_t n, int32_t m, int32_t* out, int64_t cap, int32_t* rows) {
  clear_error();
  if (n < 1 || m < 0 || m > n || !rows) return fail(RT_ERR_INVALID_ARGUMENT, "almost_hex_domain: need 0 <= m <= n, n >= 1");
  // LozengeTiler.cpp:422-467: the 2n x 4n triangle array of the hexagon of side n with an
  // m x 2m block of its top-right corner removed, offset by 3 rows and 6 columns inside a
  // (2n+6) x (4n+12) array, then widened to R rows with R + 1 a multiple of 3.
  const int M2 = 2 * n + 6, k = (3 - (M2 + 1) % 3) % 3, R = M2 + k;
  *rows = R;
  if (!out || cap < (int64_t)R * 2 * R) return fail(RT_ERR_BUFFER_TOO_SMALL, "almost_hex_domain: output too small");
  std::fill(out, out + (size_t)R * 2 * R, 0);
  for (int i = 0; i < 2 * n; ++i)
    for (int j = 0; j < 4 * n; ++j) {
      const bool in = (i < n) ? (2 * i + j - 1 >= 2 * n - 2) : (2 * i + j <= 6 * n - 2);
      const bool cut = (i < m) && (j >= 4 * n - 2 * m);
      if (in && !cut) out[(size_t)(i + 3) * 2 * R + (j + 6)] = 1;
    }
  return RT_OK;
}

RT_API rt_status rt_lozenge_domain_to_vertices(const int32_t* d, int32_t m_rows, int32_t* out) {
  clear_error();
  if (!d || !out || m_rows < 2) return fail(RT_ERR_INVALID_ARGUMENT, "lozenge domain_to_vertices: bad arguments");
  vertex_classes(d, m_rows, out);
  return RT_OK;
}

RT_API rt_status rt_lozenge_max_tiling(const int32_t* d, int32_t m_rows, int32_t* out) {
  clear_error();
  if (rt_status s = check_domain(d, m_rows)) return s;
  if (!out) return fail(RT_ERR_INVALID_ARGUMENT, "lozenge max_tiling: out is NULL");
  return extremal<true>(d, m_rows, out);
}

RT_API rt_status rt_lozenge_min_tiling(const int32_t* d, int32_t m_rows, int32_t* out) {
  clear_error();
  if (rt_status s = check_domain(d, m_rows)) return s;
  if (!out) return fail(RT_ERR_INVALID_ARGUMENT, "lozenge min_tiling: out is NULL");
  return extremal<false>(d, m_rows, out);
}

RT_API rt_status rt_lozenge_heightfunc_to_tiling(const int32_t* hf, const int32_t* d, int32_t n_side, int32_t* out) {
  clear_error();
  if (!hf || !d || !out || n_side < 3) return fail(RT_ERR_INVALID_ARGUMENT, "lozenge heightfunc_to_tiling: bad arguments");
  hf_to_tiling(hf, d, n_side, out);
  return RT_OK;
}

RT_API rt_status rt_lozenge_tiling_to_heightfunc(const int32_t* t, const int32_t* d, int32_t n_side, int32_t* out) {
  clear_error();
  if (!t || !d || !out || n_side < 5) return fail(RT_ERR_INVALID_ARGUMENT, "lozenge tiling_to_heightfunc: bad arguments");
  const int N = n_side, M = N - 1;
  if (rt_status s = check_domain(d, M)) return s;
  std::vector<int32_t> v((size_t)N * N);
  vertex_classes(d, M, v.data());
  Tri T{d, M};
  std::fill(out, out + (size_t)N * N, kUnset);
  // Breadth-first from the first boundary vertex across edges no lozenge covers
  // (LozengeTiler.cpp:173-216).
  std::queue<std::pair<int, int>> q;
  for (size_t p = 0; p < v.size(); ++p)
    if (v[p] == 2) {
      q.push({(int)(p / N), (int)(p % N)});
      out[p] = 0;
      break;
    }
  while (!q.empty()) {
    auto [i0, j0] = q.front();
    q.pop();
    const int32_t mask = t[(size_t)i0 * N + j0];
    for (int nb = 0; nb < 6; ++nb) {
      if (mask & kSteps[nb].bit) continue;
      const int i = i0 + kSteps[nb].di, j = j0 + kSteps[nb].dj;
      if (v[(size_t)i * N + j] <= 0 || out[(size_t)i * N + j] != kUnset) continue;
      if (!T.a(i0, j0, nb) && !T.b(i0, j0, nb)) continue;
      out[(size_t)i * N + j] = out[(size_t)i0 * N + j0] + kSteps[nb].dh;
      q.push({i, j});
    }
  }
  return RT_OK;
}

RT_API rt_status rt_lozenge_tiling_to_domain(const int32_t* t, int32_t n_side, int32_t* out) {
  clear_error();
  if (!t || !out || n_side < 3) return fail(RT_ERR_INVALID_ARGUMENT, "lozenge tiling_to_domain: bad arguments");
  const int N = n_side, M = N - 1;
  std::fill(out, out + (size_t)2 * M * M, 0);
  // A lozenge crossing edge bit 1, 2 or 8 of vertex (i, j) covers the two triangles beside
  // that edge (LozengeTiler.cpp:514-556); row 0 carries no lozenges in a padded tiling.
  for (int i = 1; i < N - 1; ++i)
    for (int j = 0; j < N - 1; ++j) {
      const int32_t x = t[(size_t)i * N + j];
      int32_t* up = out + (size_t)(i - 1) * 2 * M;
      if ((x & 1) && j > 0) up[2 * j] = 1, up[2 * j - 1] = 1;
      if (x & 2) up[2 * j] = 1, up[2 * j + 1] = 1;
      if (x & 8) up[2 * j + 1] = 1, out[(size_t)i * 2 * M + 2 * j] = 1;
    }
  return RT_OK;
}

}  // extern "C"
