// Device-side state of the domino sweep (see domino_sweep.cu for the layout).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <memory>

#include "domino_bits.h"
#include "domino_persist.h"
#include "domino_runs.h"
#include "domino_rules.h"
#include "rt_internal.h"

namespace rt {

// Plain-data view of a sampler passed to the kernels by value.
struct DmView {
  uint8_t* base;
  int N, P, rows, cols, active;
  size_t chain_stride, colour_stride;
  uint4* tmt;
  const uint4* tmt_params;
  // Colour array t (1 black, 0 white) of chain ch.
  __host__ __device__ uint8_t* colour(int ch, int t) const {
    return base + (size_t)ch * chain_stride + (size_t)t * colour_stride;
  }
};

#ifdef __CUDACC__
// New state of a site in state e for draw u under one case of a rule table: the up move
// 3 -> 12 when u lies in [lo_up, lo_up + w_up), the down move 12 -> 3 in [lo_dn, lo_dn + w_dn).
__device__ __forceinline__ uint8_t dm_flip(uint32_t e, uint32_t u, uint32_t lo_up, uint32_t w_up, uint32_t lo_dn,
                                           uint32_t w_dn) {
  if (e == 3u) return (u - lo_up) < w_up ? 12 : 3;
  if (e == 12u) return (u - lo_dn) < w_dn ? 3 : 12;
  return (uint8_t)e;
}
#endif

// cuRAND MTGP32 mode (domino_mtgp.cu): one half-sweep's rotation of colour t of every active
// chain, on the reference's 8 x 8 block grid over the flip candidates.
rt_status mtgp_rotate(const DmView& v, int t, const DmRule& rule, void* states, cudaStream_t stream);

// Device height functions (domino_thurston.cu).
rt_status dm_heights_device(const int32_t* d_t, const int32_t* d_cls, const int32_t* d_dom, int N, int start,
                            int32_t* d_h, unsigned* d_flags, cudaStream_t st);
rt_status dm_heights_accumulate(const int32_t* d_h, int N, long long* sums, cudaStream_t st);
rt_status dm_classes_device(const int32_t* d_dom, int M, int32_t* d_cls, unsigned* d_count, cudaStream_t st);
int dm_first_boundary_vertex(const int32_t* domain, int M);

struct DmSampler {
  int N = 0, P = 0, n_chains = 0, active = 0;
  size_t chain_stride = 0, colour_stride = 0;
  rt_walk_opts opts{};
  DmRule rule{};
  uint8_t* base = nullptr;
  uint4* tmt = nullptr;
  uint4* tmt_params = nullptr;
  void* mtgp = nullptr;  // RT_RNG_MTGP: the generators of the 8 x 8 blocks (curandStateMtgp32)
  bool mtgp_seeded = false;
  int32_t* scratch = nullptr;
  unsigned long long* counter = nullptr;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  int64_t interior[2] = {0, 0};     // interior vertices of colour 0 (white) and 1 (black)
  int64_t half_sweeps[2] = {0, 0};  // half-sweeps run per colour
  int64_t launches = 0;
  // Persistent engine state: the flip-candidate column range of each colour-array row over
  // all loaded chains (kept on the device by the load scan, fetched when the engine is
  // planned), whether every loaded tiling is consistent, and the engine (re)planned when
  // either changes.
  int* d_cand = nullptr;                 // [2][N]: lowest (INT_MAX: none) and highest column
  unsigned long long* d_scan = nullptr;  // flags, interior count of colour 0, of colour 1
  std::vector<int> cand_lo, cand_hi;     // host copies (-1: no candidate)
  bool any_candidate = false;
  bool consistent = true;
  bool border_candidates = false;  // a candidate borders a cell the reference never rebuilds
  bool plan_dirty = true;
  std::unique_ptr<BitEngine> bits;        // the bit-plane kernel (domino_bits.cu)
  std::unique_ptr<RunEngine> runs;        // the run-resident kernel (domino_runs.cu)
  std::unique_ptr<PersistEngine> persist;  // the per-half-sweep-exchange resident kernel
  int resident = 0;     // the resident kernel the next run uses: 2 run kernel, 3 k_persist,
                        // 4 bit-plane kernel, 0 none
  int last_engine = 0;  // engine of the last run: 1 per-half-sweep kernels, 2-4 as resident
  // Launch shape: an explicit choice (rt_dm_sampler_set_launch; 0 = none), and the shape in
  // force, from that choice, else the autotuner's table, else the defaults (0).
  int launch_engine = 0, launch_bands = 0, launch_threads = 0;
  int eff_bands = 0, eff_threads = 0;
  bool tuned = false;
  // Test hook of the resident engine (rt_dm_sampler_test_silent_band): a band that
  // publishes nothing (-1: none) and the polls after which a wait gives up (0: default).
  int test_silent_band = -1;
  long test_max_spin = 0;

  static rt_status create(int n_side, int n_chains, const rt_walk_opts& o, std::unique_ptr<DmSampler>* out);
  ~DmSampler();
  DmView view() const;
  rt_status check_launch();
  rt_status load(int ch, const int32_t* tiling);
  rt_status fetch_candidates();
  // Device statistics: the domain the height function is taken on, then per-chain heights
  // added to running sums.
  rt_status set_domain(const int32_t* domain, int m_side);
  rt_status accumulate_heights(int ch, long long* sums, int32_t* heights);
  int32_t *d_dom = nullptr, *d_cls = nullptr, *d_h = nullptr;
  unsigned* d_hflags = nullptr;
  int hf_start = -1;
  rt_status store(int ch, int32_t* tiling);
  rt_status copy_chain(int dst, int src);
  // TinyMT: generator k seeded s + k on the device; MTGP: block generator k seeded s + k.
  rt_status seed(int64_t s);
  rt_status run(const uint8_t* colours, int64_t steps);
  rt_status run_fast(uint64_t seed, int64_t h0, int64_t steps);
  rt_status diff(int a, int b, int64_t* ndiff);
  rt_status accumulate_edges(int ch, uint32_t* counts);
  rt_status sync();
  // Picks the engine for the next run: true when a resident kernel (see `resident`) will run it.
  rt_status use_persistent(bool* yes);
  rt_status check_resident_error();
  rt_status launch_resident(const uint8_t* colours, int64_t steps, uint64_t fast_seed, int64_t h0);
};

}  // namespace rt
