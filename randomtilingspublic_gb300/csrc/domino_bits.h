// Bit-plane engine of the domino sweep (see domino_bits.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "domino_rules.h"
#include "domino_runs.h"
#include "rt_internal.h"

namespace rt {

struct DmSampler;

// One CTA's share: colour-array rows [r0, r1) and the 32-cell words [wlo, whi) that it writes
// back; its shared-memory window holds rows r0-1 .. r1 and words wlo-1 .. whi.  The words of
// the neighbours' boundary rows it reads at the end of a launch are fin[fin0, fin1) (above)
// and fin[fin1, fin2) (below).
struct BitBand {
  int r0, r1, wlo, whi;
  int fin0, fin1, fin2, pad;
};

// A slot is one 32-cell word of one colour-array row, held by the 32 lanes of a warp (lane l:
// cell 32 w + l, with that cell's TinyMT generator).  slot.x = (row << 16) | word; slot.y =
// flags | (first candidate bit << 8) | (last candidate bit << 16).
constexpr uint32_t kSlotPresent = 1u;
constexpr uint32_t kSlotHaloUp = 2u;  // the row above (another band's) has a slot at this word
constexpr uint32_t kSlotHaloDn = 4u;  // the row below (another band's) has a slot at this word
constexpr uint32_t kSlotPubUp = 8u;   // first row of a band with a band above: publishes upward
constexpr uint32_t kSlotPubDn = 16u;  // last row of a band with a band below: publishes downward
constexpr int kBitSlots = 16;         // slots per warp
constexpr int kBitMaxWarps = 16;     // 512 threads: up to 128 registers a thread

struct BitArgs {
  uint8_t* base;
  int N, P, cols, nbands, warps, wn_max;
  size_t chain_stride, colour_stride;
  uint4* tmt;
  const uint4* tmt_params;
  const BitBand* bands;
  const uint2* slots;       // [band][warp][kBitSlots]
  const uint32_t* fin;      // final-read words
  DmRule rule;
  uint64_t* xbuf;           // [2 parities][band][up, down][xwords][2 colours][nch] tagged words
  int xwords;               // words per exchange row
  int* error;
  long max_spin;
  int silent_band_plus1;
  const uint32_t* runs;     // (colour << 31) | (epoch start << 30) | length
  int64_t nruns;
  // Coupling from the past in one launch (attempts > 0, two chains), as in RunArgs.
  int attempts;
  const uint8_t* start_base;
  const int4* attempt_desc;
  const uint32_t* epoch_seeds;
  unsigned long long* diff;
  unsigned* grid_bar;
  int* result;
};

struct BitPlan {
  bool ok = false;
  std::string why;
  std::vector<BitBand> bands;
  std::vector<uint2> slots;    // [band][warp][kBitSlots]
  std::vector<uint32_t> fin;
  int warps = 0;               // warps per band
  int wn_max = 0;              // window words per row, pads included
  int64_t words = 0, draw_cells = 0;
  size_t smem_bytes = 0;
  rt_status build(const std::vector<int>& lo, const std::vector<int>& hi, int N, int P, int nch, int nbands,
                  size_t smem_limit);
};

// A plan's device tables, shared by every engine whose domain and launch shape give the
// same plan (domino_bits.cu keeps a small cache of recent plans).
struct BitDevPlan {
  BitBand* d_bands = nullptr;
  uint2* d_slots = nullptr;
  uint32_t* d_fin = nullptr;
  ~BitDevPlan();
};

struct BitEngine {
  BitPlan plan;  // without its slot and final-read tables, which live on the device in `dev`
  bool ready = false;
  int nch = 0;
  void* kernel = nullptr;
  std::shared_ptr<BitDevPlan> dev;
  BitBand* d_bands = nullptr;  // dev's tables
  uint2* d_slots = nullptr;
  uint32_t* d_fin = nullptr;
  uint64_t* d_xbuf = nullptr;
  int* d_error = nullptr;
  uint32_t* d_runs = nullptr;
  int64_t runs_cap = 0;
  size_t xbuf_bytes = 0;
  int xwords = 0;
  bool pending_error_check = false;
  cudaStream_t stream = nullptr;
  unsigned long long* d_diff = nullptr;
  uint32_t* d_epoch = nullptr;
  size_t epoch_cap = 0;

  ~BitEngine();
  rt_status prepare(DmSampler& s);
  rt_status launch(DmSampler& s, const uint8_t* colours_host, int64_t steps);
  rt_status cftp(DmSampler& s, int n, const std::vector<std::vector<RunEngine::Epoch>>& epochs, int* attempts_run,
                 bool* coalesced);
  rt_status check_error(DmSampler& s);
};

void* dm_bits_kernel_ptr(bool params, int nch);

}  // namespace rt
