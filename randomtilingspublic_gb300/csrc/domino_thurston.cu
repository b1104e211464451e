// Thurston's extremal domino tilings on the device.
//
// The reference (DominoTiler.cpp:345-531) walks the boundary to fix its heights, then fills
// the bulk from a priority queue: the lowest (max tiling) or highest (min tiling) assigned
// vertex expands first, and an unassigned neighbour reached along a +1 (max) / -1 (min) step
// takes that height +-1.  With unit steps that queue computes shortest paths, so the heights
// are the fixed point of h(v) = min over in-neighbours u of h(u) + 1 (max; max and -1 for
// min) from the boundary heights - here found by in-place parallel relaxation sweeps until
// nothing changes.  As in the reference the vertex the boundary walk starts from never
// expands, and its two "not tileable" tests run on the final heights over the same pairs.
// Domains whose boundary walk misses boundary vertices (holes) are refused.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <queue>
#include <unordered_map>
#include <string>
#include <vector>

#include "pdl.cuh"
#include "rt_internal.h"

namespace rt {

void domino_vertex_classes(const int32_t* d, int M, int32_t* v);

namespace {

constexpr int32_t kUnset = INT32_MAX;

struct ThDir {
  int di, dj, fa_i, fa_j, fb_i, fb_j, bit;
};
// Neighbour, the two squares beside the edge toward it, indicator bit (DominoTiler.cpp:335-337).
__constant__ ThDir c_dirs[4] = {
    {1, 0, 0, -1, 0, 0, 2}, {-1, 0, -1, -1, -1, 0, 1}, {0, 1, -1, 0, 0, 0, 8}, {0, -1, -1, -1, 0, -1, 4}};
constexpr ThDir kDirsH[4] = {
    {1, 0, 0, -1, 0, 0, 2}, {-1, 0, -1, -1, -1, 0, 1}, {0, 1, -1, 0, 0, 0, 8}, {0, -1, -1, -1, 0, -1, 4}};

__host__ __device__ inline int th_step(int i0, int j0, int nb) {
  return (nb > 1 ? 1 : -1) * (((i0 + j0) % 2 == 0) ? 1 : -1);
}

struct ThArgs {
  const int32_t* cls;  // vertex classes, N x N
  int32_t* h;          // heights (kUnset: none)
  int N;
  int start;           // index of the walk's start vertex (never expands)
  int kmax;            // 1: max tiling, 0: min tiling
};

// Relaxation of one 32 x 32 tile of vertices in shared memory (its one-vertex halo held fixed)
// until the tile stops changing (at most 2 x 32 x 32 rounds), then written back; changed[0]
// is set when any height of the tile moved.  Only interior vertices (class 1) are relaxed:
// the boundary walk fixed every boundary vertex.
constexpr int kTile = 32;

__global__ void __launch_bounds__(kTile * kTile) k_th_relax_tile(ThArgs a, unsigned* changed) {
  pdl_begin();
  __shared__ int32_t sh[kTile + 2][kTile + 2];
  __shared__ int8_t sc[kTile + 2][kTile + 2];
  const int N = a.N, tx = threadIdx.x, ty = threadIdx.y;
  const int j0 = blockIdx.x * kTile - 1, i0 = blockIdx.y * kTile - 1;
  for (int k = ty * kTile + tx; k < (kTile + 2) * (kTile + 2); k += kTile * kTile) {
    const int r = k / (kTile + 2), c = k % (kTile + 2), i = i0 + r, j = j0 + c;
    const bool in = i >= 0 && j >= 0 && i < N && j < N;
    const int p = i * N + j;
    sh[r][c] = in ? a.h[p] : kUnset;
    // the walk's start vertex never expands: hide it from its neighbours
    sc[r][c] = in ? (p == a.start ? (int8_t)0 : (int8_t)a.cls[p]) : (int8_t)0;
  }
  __syncthreads();
  const int r = ty + 1, c = tx + 1, i = i0 + r, j = j0 + c;
  const bool mine = i < N && j < N && sc[r][c] == 1;
  bool any = false;
  for (int round = 0; round < 2 * kTile * kTile; ++round) {
    int32_t best = sh[r][c];
    if (mine) {
#pragma unroll
      for (int nb = 0; nb < 4; ++nb) {
        const int ur = r - c_dirs[nb].di, uc = c - c_dirs[nb].dj;
        if (sc[ur][uc] == 0) continue;
        const int s = th_step(i - c_dirs[nb].di, j - c_dirs[nb].dj, nb);
        if (a.kmax ? s <= 0 : s >= 0) continue;
        const int32_t hu = sh[ur][uc];
        if (hu == kUnset) continue;
        const int32_t cand = a.kmax ? hu + 1 : hu - 1;
        if (best == kUnset || (a.kmax ? cand < best : cand > best)) best = cand;
      }
    }
    const bool moved = best != sh[r][c];
    __syncthreads();
    if (moved) sh[r][c] = best;
    any = any || moved;
    if (!__syncthreads_or(moved)) break;
  }
  if (mine && i >= 0 && j >= 0) a.h[i * N + j] = sh[r][c];
  if (__syncthreads_or(any) && tx == 0 && ty == 0) *changed = 1u;
}

// Height function of a tiling (TilingToHeightfunc, DominoTiler.cpp:555-593): from the start
// vertex (height 0), heights spread across every edge no domino covers (its bit clear at the
// vertex it leaves) that touches the domain, by +-1 (th_step).  For a tiling the heights do
// not depend on the path, so each unassigned vertex takes the value from its first assigned
// neighbour; one tile at a time in shared memory until the tile stops changing.
__device__ __forceinline__ bool th_touches(const int32_t* dom, int M, int ui, int uj, int nb) {
  const int ai = ui + c_dirs[nb].fa_i, aj = uj + c_dirs[nb].fa_j, bi = ui + c_dirs[nb].fb_i, bj = uj + c_dirs[nb].fb_j;
  const bool fa = ai >= 0 && aj >= 0 && ai < M && aj < M && dom[ai * M + aj];
  const bool fb = bi >= 0 && bj >= 0 && bi < M && bj < M && dom[bi * M + bj];
  return fa || fb;
}

__global__ void __launch_bounds__(kTile * kTile) k_hf_tile(const int32_t* t, const int32_t* cls, const int32_t* dom,
                                                           int32_t* h, int N, unsigned* changed) {
  pdl_begin();
  __shared__ int32_t sh[kTile + 2][kTile + 2];
  __shared__ int8_t st[kTile + 2][kTile + 2];
  __shared__ int8_t sc[kTile + 2][kTile + 2];
  const int M = N - 1, tx = threadIdx.x, ty = threadIdx.y;
  const int j0 = blockIdx.x * kTile - 1, i0 = blockIdx.y * kTile - 1;
  for (int k = ty * kTile + tx; k < (kTile + 2) * (kTile + 2); k += kTile * kTile) {
    const int r = k / (kTile + 2), c = k % (kTile + 2), i = i0 + r, j = j0 + c;
    const bool in = i >= 0 && j >= 0 && i < N && j < N;
    sh[r][c] = in ? h[i * N + j] : kUnset;
    st[r][c] = in ? (int8_t)t[i * N + j] : (int8_t)0;
    sc[r][c] = in ? (int8_t)cls[i * N + j] : (int8_t)0;
  }
  __syncthreads();
  const int r = ty + 1, c = tx + 1, i = i0 + r, j = j0 + c;
  const bool open = i < N && j < N && sc[r][c] > 0;
  constexpr int kOpp[4] = {1, 0, 3, 2};
  bool any = false;
  for (int round = 0; round < 2 * kTile * kTile; ++round) {
    int32_t val = kUnset;
    if (open && sh[r][c] == kUnset) {
#pragma unroll
      for (int nbv = 0; nbv < 4; ++nbv) {
        const int ur = r + c_dirs[nbv].di, uc = c + c_dirs[nbv].dj;
        if (sc[ur][uc] == 0 || sh[ur][uc] == kUnset) continue;
        const int nb = kOpp[nbv];  // the step from u back to v
        if (st[ur][uc] & c_dirs[nb].bit) continue;
        const int ui = i + c_dirs[nbv].di, uj = j + c_dirs[nbv].dj;
        if (!th_touches(dom, M, ui, uj, nb)) continue;
        val = sh[ur][uc] + th_step(ui, uj, nb);
        break;
      }
    }
    const bool moved = val != kUnset;
    __syncthreads();
    if (moved) sh[r][c] = val;
    any = any || moved;
    if (!__syncthreads_or(moved)) break;
  }
  if (open && any) h[i * N + j] = sh[r][c];
  if (__syncthreads_or(any) && tx == 0 && ty == 0) *changed = 1u;
}

__global__ void k_fill_unset(int32_t* h, int64_t nn, int start) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p < nn) h[p] = p == start ? 0 : kUnset;
}

// sums[p] += h[p] for assigned vertices.
__global__ void k_hf_accumulate(const int32_t* h, int64_t nn, long long* sums) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p < nn && h[p] != kUnset) sums[p] += h[p];
}

// Vertex classes of DomainToVertices (DominoTiler.cpp:611-631): 0 outside, 1 interior (four
// squares of the domain around it), 2 boundary; squares clamped into the array at its rim.
__global__ void k_th_classes(const int32_t* d, int M, int32_t* cls, unsigned* boundary) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y, N = M + 1;
  if (j >= N) return;
  const int lo_i = i == 0 ? 0 : i - 1, hi_i = i == M ? M - 1 : i, lo_j = j == 0 ? 0 : j - 1, hi_j = j == M ? M - 1 : j;
  const int s00 = d[lo_i * M + lo_j], s01 = d[lo_i * M + hi_j], s10 = d[hi_i * M + lo_j], s11 = d[hi_i * M + hi_j];
  const bool rim = i == 0 || j == 0 || i == M || j == M;
  int32_t c = 0;
  if (!rim && s00 && s01 && s10 && s11) c = 1;
  else if (s00 || s01 || s10 || s11) c = 2;
  cls[i * N + j] = c;
  if (c == 2) atomicAdd(boundary, 1u);
}

// The reference's bulk tests (DominoTiler.cpp:421-424, 516-520) over every expanding vertex u
// (assigned, not the walk start) and boundary neighbour v along an allowed step.
__global__ void k_th_check(ThArgs a, unsigned* bad) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y, N = a.N;
  if (j >= N) return;
  const int q = i * N + j;
  if (q == a.start || a.cls[q] == 0) return;
  const int32_t here = a.h[q];
  if (here == kUnset) return;
  for (int nb = 0; nb < 4; ++nb) {
    const int vi = i + c_dirs[nb].di, vj = j + c_dirs[nb].dj;
    if (vi < 0 || vj < 0 || vi >= N || vj >= N) continue;
    const int p = vi * N + vj;
    if (a.cls[p] != 2) continue;
    const int s = th_step(i, j, nb);
    if (a.kmax ? s <= 0 : s >= 0) continue;
    const int32_t slot = a.h[p];
    const bool b = a.kmax ? (slot > here + 1 && a.cls[q] != 2) : (slot < here - 1 && here != 2);
    if (b) *bad = 1u;
  }
}

// HeightfuncToTiling (DominoTiler.cpp:534-553): bit of each edge whose height step is 3.
__global__ void k_th_tiling(const int32_t* h, const int32_t* d, int N, int32_t* t) {
  const int j0 = blockIdx.x * blockDim.x + threadIdx.x, i0 = blockIdx.y, M = N - 1;
  if (j0 >= N) return;
  int32_t out = 0;
  const int32_t h0 = h[i0 * N + j0];
  if (h0 != kUnset) {
    for (int nb = 0; nb < 4; ++nb) {
      const int i = i0 + c_dirs[nb].di, j = j0 + c_dirs[nb].dj;
      if (i < 0 || j < 0 || i >= N || j >= N) continue;
      const int32_t h1 = h[i * N + j];
      if (h1 == kUnset) continue;
      const int fa = (i0 - (nb == 1) - (nb > 1)) * M + j0 - (nb <= 1) - (nb == 3);
      const int fb = (i0 - (nb == 1)) * M + j0 - (nb == 3);
      if (d[fa] || d[fb]) out += c_dirs[nb].bit * abs((h1 - h0) / 2);
    }
  }
  t[i0 * N + j0] = out;
}

}  // namespace

// Device height function of the host-layout tiling d_t (N x N) for the domain whose vertex
// classes are d_cls, starting at vertex `start` (height 0).  d_h receives the heights
// (INT32_MAX where unset); d_flags needs 8 words.
rt_status dm_heights_device(const int32_t* d_t, const int32_t* d_cls, const int32_t* d_dom, int N, int start,
                            int32_t* d_h, unsigned* d_flags, cudaStream_t st) {
  const int64_t NN = (int64_t)N * N;
  // every vertex unset, the start vertex at 0
  k_fill_unset<<<(unsigned)((NN + 255) / 256), 256, 0, st>>>(d_h, NN, start);
  constexpr int kBatch = 8;
  const dim3 tgrid((N + kTile - 1) / kTile, (N + kTile - 1) / kTile), tblock(kTile, kTile);
  for (int64_t passes = 0;; passes += kBatch) {
    if (passes > NN + kBatch) return fail(RT_ERR_TIMEOUT, "height function: propagation did not converge");
    cudaMemsetAsync(d_flags, 0, kBatch * sizeof(unsigned), st);
    for (int k = 0; k < kBatch; ++k) pdl_launch(k_hf_tile, tgrid, tblock, st, d_t, d_cls, d_dom, d_h, N, d_flags + k);
    unsigned last = 1;
    cudaMemcpyAsync(&last, d_flags + kBatch - 1, sizeof last, cudaMemcpyDeviceToHost, st);
    const cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail(RT_ERR_CUDA, std::string("height function: ") + cudaGetErrorString(e));
    if (!last) return RT_OK;
  }
}

rt_status dm_heights_accumulate(const int32_t* d_h, int N, long long* sums, cudaStream_t st) {
  const int64_t NN = (int64_t)N * N;
  k_hf_accumulate<<<(unsigned)((NN + 255) / 256), 256, 0, st>>>(d_h, NN, sums);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? RT_OK : fail(RT_ERR_CUDA, std::string("height sums: ") + cudaGetErrorString(e));
}

rt_status dm_classes_device(const int32_t* d_dom, int M, int32_t* d_cls, unsigned* d_count, cudaStream_t st) {
  const int N = M + 1;
  k_th_classes<<<dim3((N + 127) / 128, N), 128, 0, st>>>(d_dom, M, d_cls, d_count);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? RT_OK : fail(RT_ERR_CUDA, std::string("vertex classes: ") + cudaGetErrorString(e));
}

// First boundary vertex in row-major order (the reference's start vertex), or -1.
int dm_first_boundary_vertex(const int32_t* domain, int M) {
  const int N = M + 1;
  for (int p = 0; p < N * N; ++p) {
    const int i = p / N, j = p % N;
    const int lo_i = i == 0 ? 0 : i - 1, hi_i = i == M ? M - 1 : i, lo_j = j == 0 ? 0 : j - 1, hi_j = j == M ? M - 1 : j;
    const bool any = domain[lo_i * M + lo_j] || domain[lo_i * M + hi_j] || domain[hi_i * M + lo_j] || domain[hi_i * M + hi_j];
    const bool rim = i == 0 || j == 0 || i == M || j == M;
    const bool all = domain[lo_i * M + lo_j] && domain[lo_i * M + hi_j] && domain[hi_i * M + lo_j] && domain[hi_i * M + hi_j];
    if (any && (rim || !all)) return p;
  }
  return -1;
}

}  // namespace rt

using namespace rt;

extern "C" {

RT_API rt_status rt_domino_extremal_tiling_device(const int32_t* domain, int32_t m_side, int32_t top, int32_t* out,
                                                  void* cuda_stream) {
  clear_error();
  if (!domain || !out || m_side < 5) return fail(RT_ERR_INVALID_ARGUMENT, "extremal_tiling_device: bad arguments");
  for (int i = 0; i < m_side; ++i)
    for (int j = 0; j < m_side; ++j)
      if ((i < 1 || j < 1 || i >= m_side - 1 || j >= m_side - 1) && domain[(size_t)i * m_side + j])
        return fail(RT_ERR_INVALID_ARGUMENT, "domain must have an empty outer ring of squares");
  const int M = m_side, N = M + 1;
  const size_t NN = (size_t)N * N;
  int devs = 0;
  if (cudaGetDeviceCount(&devs) != cudaSuccess || devs == 0) {
    cudaGetLastError();
    return fail(RT_ERR_CUDA, "no CUDA device: the device Thurston has no CPU fallback");
  }
  cudaStream_t st = (cudaStream_t)cuda_stream;
  int32_t *d_cls = nullptr, *d_h = nullptr, *d_dom = nullptr, *d_t = nullptr;
  unsigned* d_flags = nullptr;
  auto cleanup = [&]() {
    for (void* p : {(void*)d_cls, (void*)d_h, (void*)d_dom, (void*)d_t, (void*)d_flags})
      if (p) cudaFree(p);
  };
  if (cudaMalloc(&d_cls, NN * 4) != cudaSuccess || cudaMalloc(&d_h, NN * 4) != cudaSuccess ||
      cudaMalloc(&d_dom, (size_t)M * M * 4) != cudaSuccess || cudaMalloc(&d_t, NN * 4) != cudaSuccess ||
      cudaMalloc(&d_flags, 64 * sizeof(unsigned)) != cudaSuccess) {
    cudaGetLastError();
    cleanup();
    return fail(RT_ERR_OUT_OF_MEMORY, "extremal_tiling_device: device allocation failed");
  }
  const dim3 grid((N + 127) / 128, N), block(128);
  cudaMemcpyAsync(d_dom, domain, (size_t)M * M * 4, cudaMemcpyHostToDevice, st);
  cudaMemsetAsync(d_flags, 0, 64 * sizeof(unsigned), st);
  k_th_classes<<<grid, block, 0, st>>>(d_dom, M, d_cls, d_flags + 48);
  unsigned boundary = 0;
  cudaMemcpyAsync(&boundary, d_flags + 48, sizeof boundary, cudaMemcpyDeviceToHost, st);
  // Boundary walk (DominoTiler.cpp:358-389 / 452-484) on the host: classes computed as
  // visited, O(perimeter) after the search for the first boundary vertex.
  auto sq = [&](int i, int j) { return domain[(size_t)i * M + j] != 0; };
  auto cls_at = [&](int i, int j) -> int {
    if (i < 0 || j < 0 || i > M || j > M) return 0;
    const int lo_i = i == 0 ? 0 : i - 1, hi_i = i == M ? M - 1 : i, lo_j = j == 0 ? 0 : j - 1, hi_j = j == M ? M - 1 : j;
    const bool s00 = sq(lo_i, lo_j), s01 = sq(lo_i, hi_j), s10 = sq(hi_i, lo_j), s11 = sq(hi_i, hi_j);
    const bool rim = i == 0 || j == 0 || i == M || j == M;
    if (!rim && s00 && s01 && s10 && s11) return 1;
    return (s00 || s01 || s10 || s11) ? 2 : 0;
  };
  std::unordered_map<int, int32_t> hb;  // boundary heights by vertex index
  int start = -1;
  for (int p = 0; p < (int)NN && start < 0; ++p)
    if (cls_at(p / N, p % N) == 2) start = p;
  if (start < 0) {
    cleanup();
    return fail(RT_ERR_INVALID_ARGUMENT, "extremal_tiling_device: empty domain");
  }
  hb[start] = 0;
  std::queue<int> walk;
  walk.push(start);
  while (!walk.empty()) {
    const int p0 = walk.front();
    walk.pop();
    const int i0 = p0 / N, j0 = p0 % N;
    for (int nb = 0; nb < 4; ++nb) {
      const ThDir& q = kDirsH[nb];
      const int i = i0 + q.di, j = j0 + q.dj;
      if (cls_at(i, j) != 2) continue;
      if (sq(i0 + q.fa_i, j0 + q.fa_j) == sq(i0 + q.fb_i, j0 + q.fb_j)) continue;
      const int32_t hv = hb[p0] + th_step(i0, j0, nb);
      auto it = hb.find(i * N + j);
      if (it == hb.end()) {
        hb[i * N + j] = hv;
        walk.push(i * N + j);
      } else if (it->second != hv) {
        cleanup();
        return fail(RT_ERR_NOT_TILEABLE, "domain is not tileable (boundary height mismatch)");
      }
    }
  }
  if (cudaStreamSynchronize(st) != cudaSuccess) {
    cleanup();
    return fail(RT_ERR_CUDA, "extremal_tiling_device: vertex classes failed");
  }
  // Boundary vertices the walk did not reach: a domain with holes, where the reference's
  // answer depends on its queue order; such domains go to rt_domino_max/min_tiling.
  if (hb.size() != boundary) {
    cleanup();
    return fail(RT_ERR_INVALID_ARGUMENT,
                "extremal_tiling_device: the boundary is not one connected walk (use rt_domino_max_tiling / _min_tiling)");
  }
  {
    std::vector<int32_t> h(NN, kUnset);
    for (const auto& kv : hb) h[(size_t)kv.first] = kv.second;
    cudaMemcpyAsync(d_h, h.data(), NN * 4, cudaMemcpyHostToDevice, st);
    cudaStreamSynchronize(st);
  }
  ThArgs a{d_cls, d_h, N, start, top ? 1 : 0};
  // Tile passes in batches of 8, each with its own changed flag; done when the last of a
  // batch changed nothing.  Every pass settles at least one more vertex of each shortest
  // path, so the loop is bounded by N * N passes.
  constexpr int kBatch = 8;
  const dim3 tgrid((N + kTile - 1) / kTile, (N + kTile - 1) / kTile), tblock(kTile, kTile);
  rt_status status = RT_OK;
  for (int64_t passes = 0;; passes += kBatch) {
    if (passes > (int64_t)NN + kBatch) {
      status = fail(RT_ERR_TIMEOUT, "extremal_tiling_device: relaxation did not converge");
      break;
    }
    cudaMemsetAsync(d_flags, 0, kBatch * sizeof(unsigned), st);
    for (int k = 0; k < kBatch; ++k) pdl_launch(k_th_relax_tile, tgrid, tblock, st, a, d_flags + k);
    unsigned last = 1;
    cudaMemcpyAsync(&last, d_flags + kBatch - 1, sizeof last, cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) {
      status = fail(RT_ERR_CUDA, std::string("extremal_tiling_device: ") + cudaGetErrorString(cudaGetLastError()));
      break;
    }
    if (!last) break;
  }
  if (status == RT_OK) {
    unsigned bad = 0;
    cudaMemsetAsync(d_flags + 40, 0, sizeof(unsigned), st);
    k_th_check<<<grid, block, 0, st>>>(a, d_flags + 40);
    k_th_tiling<<<grid, block, 0, st>>>(d_h, d_dom, N, d_t);
    cudaMemcpyAsync(&bad, d_flags + 40, sizeof bad, cudaMemcpyDeviceToHost, st);
    std::vector<int32_t> t(NN);
    cudaMemcpyAsync(t.data(), d_t, NN * 4, cudaMemcpyDeviceToHost, st);
    const cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) status = fail(RT_ERR_CUDA, std::string("extremal_tiling_device: ") + cudaGetErrorString(e));
    else if (bad) status = fail(RT_ERR_NOT_TILEABLE, "domain is not tileable (bulk height mismatch)");
    else std::copy(t.begin(), t.end(), out);  // written only on success, as the host version
  }
  cleanup();
  return status;
}

RT_API rt_status rt_domino_heightfunc_device(const int32_t* tiling, const int32_t* domain, int32_t n_side,
                                             int32_t* out, void* cuda_stream) {
  clear_error();
  if (!tiling || !domain || !out || n_side < 6) return fail(RT_ERR_INVALID_ARGUMENT, "heightfunc_device: bad arguments");
  const int N = n_side, M = N - 1;
  for (int i = 0; i < M; ++i)
    for (int j = 0; j < M; ++j)
      if ((i < 1 || j < 1 || i >= M - 1 || j >= M - 1) && domain[(size_t)i * M + j])
        return fail(RT_ERR_INVALID_ARGUMENT, "domain must have an empty outer ring of squares");
  const int start = dm_first_boundary_vertex(domain, M);
  if (start < 0) return fail(RT_ERR_INVALID_ARGUMENT, "heightfunc_device: empty domain");
  int devs = 0;
  if (cudaGetDeviceCount(&devs) != cudaSuccess || devs == 0) {
    cudaGetLastError();
    return fail(RT_ERR_CUDA, "no CUDA device: the device height function has no CPU fallback");
  }
  cudaStream_t st = (cudaStream_t)cuda_stream;
  const size_t NN = (size_t)N * N;
  int32_t *d_t = nullptr, *d_cls = nullptr, *d_dom = nullptr, *d_h = nullptr;
  unsigned* d_flags = nullptr;
  auto cleanup = [&]() {
    for (void* p : {(void*)d_t, (void*)d_cls, (void*)d_dom, (void*)d_h, (void*)d_flags})
      if (p) cudaFree(p);
  };
  if (cudaMalloc(&d_t, NN * 4) != cudaSuccess || cudaMalloc(&d_cls, NN * 4) != cudaSuccess ||
      cudaMalloc(&d_dom, (size_t)M * M * 4) != cudaSuccess || cudaMalloc(&d_h, NN * 4) != cudaSuccess ||
      cudaMalloc(&d_flags, 16 * sizeof(unsigned)) != cudaSuccess) {
    cudaGetLastError();
    cleanup();
    return fail(RT_ERR_OUT_OF_MEMORY, "heightfunc_device: device allocation failed");
  }
  cudaMemcpyAsync(d_t, tiling, NN * 4, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(d_dom, domain, (size_t)M * M * 4, cudaMemcpyHostToDevice, st);
  cudaMemsetAsync(d_flags, 0, 16 * sizeof(unsigned), st);
  rt_status status = dm_classes_device(d_dom, M, d_cls, d_flags + 8, st);
  if (status == RT_OK) status = dm_heights_device(d_t, d_cls, d_dom, N, start, d_h, d_flags, st);
  if (status == RT_OK) {
    cudaMemcpyAsync(out, d_h, NN * 4, cudaMemcpyDeviceToHost, st);
    const cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) status = fail(RT_ERR_CUDA, std::string("heightfunc_device: ") + cudaGetErrorString(e));
  }
  cleanup();
  return status;
}

}  // extern "C"
