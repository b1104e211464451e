// Batched CFTP for instances too large for one CTA's shared memory: each instance is held by a
// thread-block cluster of C CTAs (C <= 16).  CTA k keeps a strip of about R = rows / C rows
// of both chains, every colour, plus one halo row above and below, in its shared memory.  A
// half-sweep is: flips of the active colour on the strip (a CTA also stores its first and
// last active rows straight into the halo rows of the CTAs above and below, through
// distributed shared memory), one cluster barrier, the rebuild of the passive colour(s) on
// the strip, a CTA barrier.  The halo rows of a colour are written only while that colour is
// active and read only by the rebuild of the same half-sweep, and the colours follow each
// other in a fixed cycle, so the per-colour halo rows double-buffer the exchange without
// further waits.  Coalescence: each CTA counts its differing words, adds them into CTA 0's
// counter for the attempt (a distributed-shared-memory atomic), and every CTA reads the sum
// after a cluster barrier.  A cluster takes instances from a device queue, runs each one's
// attempts in order and writes its result; the draws are the single-instance fast mode's
// (keyed by instance seed, stream, half-sweep, row and column quad), so every sample equals
// the one-CTA batch kernel's and rt_domino_cftp / rt_lozenge_cftp's for the same instance.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <string>

#include "batch_cftp.cuh"

namespace cg = cooperative_groups;

namespace rt {
namespace {

constexpr int kClusterThreads = 1024;
constexpr int kClusterMax = 16;  // non-portable cluster size, enabled per kernel

struct Strip {
  int r0, r1;  // rows this CTA flips
  int s0;      // first row it stores (r0 - 1: the halo above, or row 0)
};

__device__ __forceinline__ Strip strip_of(const DevInstance& in, int R, int rank) {
  const int f0 = flip_row_lo(in), f1 = flip_row_hi(in);
  Strip s;
  s.r0 = min(f1, f0 + rank * R);
  s.r1 = min(f1, s.r0 + R);
  s.s0 = max(0, s.r0 - 1);
  return s;
}

// 16-byte copies of rows [a, b) of the ncol colour arrays of one chain.
__device__ __forceinline__ void copy_rows_in(const RowView& v, int c, int ncol, const uint8_t* g, const DevInstance& in,
                                             int a, int b) {
  const int P = in.P, vec = P / 16;
  const size_t gplane = (size_t)in.N * P;
  const int n = ncol * (b - a) * vec;
  for (int k = threadIdx.x; k < n; k += kClusterThreads) {
    const int x = k % vec, rk = k / vec;
    const int i = a + rk % (b - a), col = rk / (b - a);
    const uint4 w = __ldcg(reinterpret_cast<const uint4*>(g + (size_t)col * gplane + (size_t)i * P) + x);
    reinterpret_cast<uint4*>(v.row(c, ncol, col, i, P))[x] = w;
  }
}

__global__ void __launch_bounds__(kClusterThreads, 1)
    k_batch_cluster(DevInstance* inst, int count, uint8_t* tilings, unsigned* queue, uint32_t c4, uint32_t c8) {
  extern __shared__ __align__(16) uint8_t sm[];
  __shared__ int s_idx;
  __shared__ unsigned s_diff[64];  // CTA 0: differing words of each attempt
  __shared__ uint32_t red[kClusterThreads / 32];
  __shared__ DevInstance s_in;
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank(), C = (int)cluster.num_blocks();
  const int* const idx0 = cluster.map_shared_rank(&s_idx, 0);
  unsigned* const diff0 = cluster.map_shared_rank(s_diff, 0);
  for (;;) {
    if (rank == 0) {
      if (threadIdx.x == 0) s_idx = (int)atomicAdd(queue, 1u);
      if (threadIdx.x < 64) s_diff[threadIdx.x] = 0;
    }
    cluster.sync();
    const int idx = *idx0;
    cluster.sync();  // every CTA has its index before any CTA leaves
    if (idx >= count) break;
    DevInstance* g = &inst[idx];
    if (threadIdx.x == 0) s_in = *g;  // read by every thread from shared memory
    __syncthreads();
    const DevInstance& in = s_in;
    const int ncol = in.model == 0 ? 2 : 3;
    const int R = cluster_rows_per_cta(in, C);
    const size_t plane = cluster_plane_bytes(in, C);
    const int f1 = flip_row_hi(in);
    const Strip me = strip_of(in, R, rank);
    const bool busy = me.r0 < me.r1;             // strips fill from the top; the last may be empty
    const bool has_up = busy && rank > 0;        // the CTA above flips row r0 - 1
    const bool has_dn = busy && me.r1 < f1;      // the CTA below flips row r1
    const RowView mine{sm, plane, me.s0};
    RowView up = mine, dn = mine;
    if (has_up) up = RowView{cluster.map_shared_rank(sm, rank - 1), plane, strip_of(in, R, rank - 1).s0};
    if (has_dn) dn = RowView{cluster.map_shared_rank(sm, rank + 1), plane, strip_of(in, R, rank + 1).s0};
    const int send_up = has_up ? me.r0 : -1, send_dn = has_dn ? me.r1 - 1 : -1;
    // rows this CTA stores, and the rows it owns for the coalescence count and the output
    // (CTA 0 also row 0, the CTA with the last flip row also the rows below it)
    const int st0 = me.s0, st1 = min(in.N, me.r1 + 1);
    const int w0 = rank == 0 ? 0 : me.r0, w1 = me.r1 == f1 ? in.N : me.r1;
    const int b0 = max(me.r0, 1), b1 = min(me.r1, in.N - 1);  // rebuilt rows
    const uint8_t* gmin = tilings + in.off_min;
    const uint8_t* gmax = tilings + in.off_max;
    int attempts = 0;
    int64_t look = 0;
    bool done = false;
    for (int att = 0; att < in.max_attempts && !done; ++att) {
      // chain 0 starts at the min tiling, chain 1 at the max tiling
      if (busy) {
        copy_rows_in(mine, 0, ncol, gmin, in, st0, st1);
        copy_rows_in(mine, 1, ncol, gmax, in, st0, st1);
      }
      cluster.sync();  // no halo row is sent before its CTA has loaded its strip
      look = ncol * (in.first_sweeps << att);
      for (int64_t h = -look; h < 0; ++h) {
        if (in.model == 0) {
          const int t = (h & 1) ? 0 : 1;
          if (busy) dm_flip_rows<kClusterThreads>(mine, in, t, h, me.r0, me.r1, &up, send_up, &dn, send_dn);
          cluster.sync();
          if (busy) dm_rebuild_rows<kClusterThreads>(mine, in, t, b0, b1);
        } else {
          const int r = (int)(((h % 3) + 3) % 3);
          if (busy) lz_rotate_rows<kClusterThreads>(mine, in, r, h, c4, c8, me.r0, me.r1, &up, send_up, &dn, send_dn);
          cluster.sync();
          if (busy) lz_rebuild_rows<kClusterThreads>(mine, in, r, b0, b1);
        }
        __syncthreads();
      }
      uint32_t differ = 0;
      if (busy) {
        const int words = in.P / 4;
        const int n = ncol * (w1 - w0) * words;
        for (int k = threadIdx.x; k < n; k += kClusterThreads) {
          const int x = k % words, rk = k / words;
          const int i = w0 + rk % (w1 - w0), col = rk / (w1 - w0);
          differ += reinterpret_cast<const uint32_t*>(mine.row(0, ncol, col, i, in.P))[x] !=
                    reinterpret_cast<const uint32_t*>(mine.row(1, ncol, col, i, in.P))[x];
        }
      }
      differ = block_sum<kClusterThreads>(differ, red);
      if (threadIdx.x == 0 && differ) atomicAdd(diff0 + att, differ);
      cluster.sync();
      done = *reinterpret_cast<const volatile unsigned*>(diff0 + att) == 0;
      attempts = att + 1;
    }
    // the top chain (from the max tiling) of the last attempt is the sample
    if (busy) {
      const int vec = in.P / 16;
      const size_t gplane = (size_t)in.N * in.P;
      uint8_t* gout = tilings + in.off_out;
      const int n = ncol * (w1 - w0) * vec;
      for (int k = threadIdx.x; k < n; k += kClusterThreads) {
        const int x = k % vec, rk = k / vec;
        const int i = w0 + rk % (w1 - w0), col = rk / (w1 - w0);
        __stcg(reinterpret_cast<uint4*>(gout + (size_t)col * gplane + (size_t)i * in.P) + x,
               reinterpret_cast<const uint4*>(mine.row(1, ncol, col, i, in.P))[x]);
      }
    }
    if (rank == 0 && threadIdx.x == 0) {
      g->attempts = done ? attempts : -attempts;
      g->final_half_sweeps = look;
    }
    cluster.sync();  // every CTA has read the attempt counters before CTA 0 clears them
  }
}

rt_status set_cluster_attrs(size_t smem) {
  if (cudaFuncSetAttribute(k_batch_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess ||
      cudaFuncSetAttribute(k_batch_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
    const cudaError_t e = cudaGetLastError();
    return fail(RT_ERR_CUDA, std::string("cftp_batch: cluster kernel attributes: ") + cudaGetErrorString(e));
  }
  return RT_OK;
}

cudaLaunchConfig_t cluster_config(int C, int clusters, size_t smem, cudaStream_t s, cudaLaunchAttribute* at) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(C * clusters));
  cfg.blockDim = dim3(kClusterThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned)C;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cfg;
}

}  // namespace

int cluster_size_for(const DevInstance& d, size_t smem_limit) {
  for (int C = 2; C <= kClusterMax; ++C)
    if (cluster_smem_bytes(d, C) <= smem_limit) return C;
  return 0;
}

int cluster_capacity(int C, size_t smem) {
  if (set_cluster_attrs(smem) != RT_OK) return 0;
  cudaLaunchAttribute at[1];
  const cudaLaunchConfig_t cfg = cluster_config(C, 1, smem, nullptr, at);
  int clusters = 0;
  if (cudaOccupancyMaxActiveClusters(&clusters, k_batch_cluster, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return clusters;
}

rt_status launch_cluster_group(const ClusterGroup& g, DevInstance* d_inst, int count, uint8_t* d_tilings,
                               unsigned* d_queue, uint32_t lz_c4, uint32_t lz_c8, cudaStream_t s) {
  rt_status st = set_cluster_attrs(g.smem);
  if (st != RT_OK) return st;
  cudaLaunchAttribute at[1];
  const cudaLaunchConfig_t cfg = cluster_config(g.C, g.clusters, g.smem, s, at);
  const cudaError_t e = cudaLaunchKernelEx(&cfg, k_batch_cluster, d_inst, count, d_tilings, d_queue, lz_c4, lz_c8);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(RT_ERR_CUDA, std::string("cftp_batch: cluster launch: ") + cudaGetErrorString(e));
  }
  return RT_OK;
}

}  // namespace rt
