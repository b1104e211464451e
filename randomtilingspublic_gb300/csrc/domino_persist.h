// Resident persistent engine of the domino sweep (see domino_persist.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "domino_rules.h"
#include "rt_internal.h"

namespace rt {

struct DmSampler;

// One CTA's share: colour-array rows [r0, r1), shared-memory column window [wlo, whi)
// (cells, multiples of 16), its number of units (flip-candidate sites or quads), and how
// many of them lie in its first row and in its first plus last rows.
struct DmBand {
  int r0, r1, wlo, whi, units, nb_first, nb_boundary, pad;
};

struct PersistArgs {
  uint8_t* base;
  int P, cols, nch, nbands;
  size_t chain_stride, colour_stride;
  uint4* tmt;
  const uint4* tmt_params;
  const DmBand* bands;
  const int* row_lo;      // first unit of each row
  const int* row_prefix;  // unit index of that first unit within the row's band
  DmRule rule;
  uint8_t* xbuf;          // [2 slots][band][first, last row][P x chains / 4 tagged 64-bit words]
  unsigned* flags;        // flags[nbands] is the error word (per-band words unused)
  int* error;
  long max_spin;          // polls before a wait gives up
  int silent_band_plus1;  // test hook: 1 + a band that publishes nothing (0: none)
  int64_t steps, h0;
  uint64_t fast_seed;
  uint32_t fast_stream;
  const uint8_t* colours;
};

struct PersistPlan {
  bool ok = false;
  std::string why;
  std::vector<DmBand> bands;
  std::vector<int> row_lo, row_cnt, row_prefix;
  int max_units = 0, K = 0;
  size_t smem_bytes = 0;
  rt_status build(const std::vector<uint8_t>& candidates, int N, int P, int mode, int nch, int nbands_max,
                  size_t smem_limit);
  // The same from each colour-array row's lowest and highest candidate column (-1: none).
  rt_status build_from_rows(const std::vector<int>& lo, const std::vector<int>& hi, int N, int P, int mode, int nch,
                            int nbands_max, size_t smem_limit);
};

struct PersistEngine {
  PersistPlan plan;
  bool ready = false;
  int nch = 0;
  void* kernel = nullptr;
  DmBand* d_bands = nullptr;
  int* d_rows = nullptr;
  uint8_t* d_xbuf = nullptr;
  unsigned* d_flags = nullptr;
  uint8_t* d_colours = nullptr;
  int64_t colours_cap = 0;
  size_t xbuf_bytes = 0;
  bool pending_error_check = false;
  cudaStream_t stream = nullptr;  // the sampler's: the buffers above are pool blocks ordered on it

  ~PersistEngine();
  rt_status prepare(DmSampler& s);
  rt_status launch(DmSampler& s, const uint8_t* colours_host, int64_t steps, uint64_t fast_seed, int64_t h0);
  rt_status check_error(DmSampler& s);
};

// Threads per CTA of the resident kernel and its entry for (rng mode, units per thread K,
// per-generator parameter table).
constexpr int kPersistThreads = 1024;
// Bytes of the exchange buffer: two slots x bands x two rows x P x nch bytes, each 4 data
// bytes carried in one 8-byte tagged word.
size_t dm_xbuf_bytes(int nbands, int nch, int P);
// nch: swept chains, 1, 2 or 4.  sparse: passive colour kept by per-flip XOR updates
// (consistent tilings only) instead of a full rebuild each half-sweep; params and nch = 4
// exist only with sparse.
void* dm_persist_kernel_ptr(int mode, int K, bool params, int nch, bool sparse);


}  // namespace rt
