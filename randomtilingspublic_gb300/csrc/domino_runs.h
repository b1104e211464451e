// Run-resident engine of the domino sweep (see domino_runs.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "domino_rules.h"
#include "rt_internal.h"

namespace rt {

struct DmSampler;

// One CTA's share: colour-array rows [r0, r1) and the shared-memory column window [wlo, whi)
// (cells, multiples of 16) that holds every cell its quads read.
struct RunBand {
  int r0, r1, wlo, whi;
};

// Bits of a slot's quad descriptor (RunArgs::slot_meta).
constexpr uint32_t kQuadOffMask = 0x3ffffu;  // byte offset of the quad in a colour plane
constexpr uint32_t kQuadOdd = 1u << 18;      // row parity (i & 1)
constexpr int kQuadValidShift = 19;          // 4 bits: cells that draw and may flip
constexpr int kQuadKeepShift = 23;           // 4 bits: cells outside [1, cols], never rebuilt
constexpr uint32_t kQuadHaloUp = 1u << 27;   // the row above comes from the band above
constexpr uint32_t kQuadHaloDn = 1u << 28;   // the row below comes from the band below
constexpr uint32_t kQuadPubUp = 1u << 29;    // published to the band above (band's first row)
constexpr uint32_t kQuadPubDn = 1u << 30;    // published to the band below (band's last row)
constexpr uint32_t kQuadPresent = 1u << 31;

struct RunArgs {
  uint8_t* base;
  int P, cols, nch, nbands, K;
  size_t chain_stride, colour_stride;
  uint4* tmt;
  const uint4* tmt_params;
  const RunBand* bands;
  const uint32_t* slot_meta;   // [band][slot][thread] descriptors (0: empty slot)
  const uint32_t* slot_where;  // [band][slot][thread] (row i << 16) | quad column q
  DmRule rule;
  uint64_t* xbuf;         // [2 parities][band][first, last row][P / 4 quads][nch tagged words]
  int* error;             // set when a wait gave up
  long max_spin;          // polls before a wait gives up
  int silent_band_plus1;  // test hook: 1 + a band that publishes nothing (0: none)
  // TinyMT: runs of equal-colour half-sweeps, (colour << 31) | (epoch start << 30) | length;
  // a run that starts an epoch first seeds every generator from the next epoch seed.
  const uint32_t* runs;
  int64_t nruns;          // runs (TinyMT) or half-sweeps (fast mode) of a plain launch
  int64_t h0;             // fast mode: index of the launch's first half-sweep
  uint64_t fast_seed;
  uint32_t fast_stream;
  // Coupling from the past in one launch (attempts > 0, two chains): before attempt a both
  // chains are reset from the start states at start_base (same layout as base); attempt a
  // runs its segment (TinyMT: attempt_desc[a] = {first run, runs, first epoch seed, 0};
  // fast: the first_half << (attempt0 + a) half-sweeps ending at -1), then counts the bands
  // whose two chains differ into diff[a]; the launch ends at the first attempt with none.
  int attempts;
  int attempt0;  // fast mode: index of the launch's first attempt
  const uint8_t* start_base;
  const int4* attempt_desc;
  const uint32_t* epoch_seeds;
  int64_t first_half;
  unsigned long long* diff;  // [attempts], zeroed
  unsigned* grid_bar;        // zeroed
  int* result;               // {attempts run, coalesced}
};

struct RunPlan {
  bool ok = false;
  std::string why;
  std::vector<RunBand> bands;
  std::vector<uint32_t> meta, where;  // [band][K][threads] (emptied once on the device)
  size_t nslot = 0;                   // entries of meta (and of where)
  int K = 0;
  int threads = 0;                    // threads per band (CTA)
  int64_t quads = 0, draw_cells = 0;  // quads held, cells that draw (flip-candidate generators)
  size_t smem_bytes = 0;
  // From each colour-array row's lowest and highest flip-candidate column (-1: none).
  rt_status build(const std::vector<int>& lo, const std::vector<int>& hi, int N, int P, int mode, int nch, int nbands,
                  size_t smem_limit, int k_max, int threads_per_band);
};

// A plan's device tables (bands, then slot descriptors meta and where), shared by every
// engine whose domain and launch shape give the same plan (domino_runs.cu keeps a small cache).
struct RunDevPlan {
  RunBand* d_bands = nullptr;
  uint32_t* d_meta = nullptr;  // meta then where
  ~RunDevPlan();
};

struct RunEngine {
  RunPlan plan;  // without its slot tables, which live on the device in `dev`
  bool ready = false;
  int nch = 0;
  int bands_asked = 0, threads_asked = 0;  // the sampler's launch shape the plan was made for (0: default)
  void* kernel = nullptr;
  std::shared_ptr<RunDevPlan> dev;
  RunBand* d_bands = nullptr;  // dev's tables
  uint32_t* d_meta = nullptr;
  uint64_t* d_xbuf = nullptr;
  int* d_error = nullptr;
  uint32_t* d_runs = nullptr;
  int64_t runs_cap = 0;
  size_t xbuf_bytes = 0;
  bool pending_error_check = false;
  cudaStream_t stream = nullptr;  // the sampler's: the buffers above are pool blocks ordered on it
  unsigned long long* d_diff = nullptr;  // diff[40], grid barrier, result[2]
  uint32_t* d_epoch = nullptr;           // epoch seeds then attempt descriptors
  size_t epoch_cap = 0;

  ~RunEngine();
  rt_status prepare(DmSampler& s);
  // colours_host: TinyMT colour of each half-sweep; NULL in fast mode (colour from h0 + h).
  rt_status launch(DmSampler& s, const uint8_t* colours_host, int64_t steps, uint64_t fast_seed, int64_t h0);
  // Coupling from the past in one launch on chains 0 (from the min) and 1 (from the max),
  // reset before every attempt from chains 2 and 3.  Attempts [a0, a0 + n): TinyMT attempt
  // a0 + k runs the epochs epochs[k] (seed, colours) in order; fast attempt a runs half-sweeps
  // [-2 first << a, 0) keyed by fast_seed.  Returns the attempts run and whether the last
  // coalesced.
  struct Epoch {
    uint32_t seed;
    const std::vector<uint8_t>* colours;
  };
  rt_status cftp(DmSampler& s, int a0, int n, const std::vector<std::vector<Epoch>>& epochs, int64_t first_sweeps,
                 uint64_t fast_seed, int* attempts_run, bool* coalesced);
  rt_status check_error(DmSampler& s);
};

// Runs of equal colour in colours[0 .. n), appended as (colour << 31) | (epoch << 30) | length,
// the first run flagged as an epoch start when `epoch`.
void append_runs(const uint8_t* colours, int64_t n, bool epoch, std::vector<uint32_t>* runs);

constexpr int kRunThreads = 1024;
// Kernel for (rng mode, quads per thread K, parameter table, chains).
void* dm_runs_kernel_ptr(int mode, int K, bool params, int nch);

}  // namespace rt
