// Resident engine of the lozenge sweep (lozenge_resident.cu): one cooperative launch runs
// many steps with every chain held in shared memory, bands of rows exchanging their boundary
// rows through tagged words in global memory.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "rt_internal.h"

namespace rt {

struct LzResidentGeom {
  int N = 0, M = 0, P = 0, nch = 0;
  size_t colour_stride = 0, chain_stride = 0;
};

struct LzResidentRule {
  uint32_t lo_up, w_up, lo_dn, w_dn;
};

// A plan: the band count, threads per band, quads per thread and shared memory per band.
struct LzResidentPlan {
  bool ok = false;
  int bands = 0, threads = 0, K = 0;
  size_t smem = 0;
  int rows_max = 0;  // rows of the largest band
};

// The plan for this geometry and random mode (tinymt: per-vertex generators in registers),
// or ok = false when no cooperative launch holds it.
LzResidentPlan lz_resident_plan(const LzResidentGeom& g, bool tinymt);

struct LzResidentState {
  LzResidentPlan plan;
  uint64_t* xbuf = nullptr;  // tagged boundary words
  int* error = nullptr;
  uint8_t* colours = nullptr;  // TinyMT colour sequence of a launch
  int64_t colours_cap = 0;
  uint32_t tag = 0;  // steps run so far (the next step's tag is tag + 1)
  ~LzResidentState();
};

// Runs `steps` steps on the geometry's chains at base.  TinyMT: colours[s] is step s's colour,
// generators tmt (params: per-generator table or NULL); fast: step h0 + s has colour
// (h0 + s) mod 3 and draws keyed by (seed, stream, h0 + s, row, quad).
rt_status lz_resident_run(LzResidentState& st, const LzResidentGeom& g, uint8_t* base, const LzResidentRule& rule,
                          bool tinymt, uint4* tmt, const uint4* params, const uint8_t* colours_host, int64_t steps,
                          uint64_t fast_seed, uint32_t fast_stream, int64_t h0, cudaStream_t s);

// RT_ERR_TIMEOUT when a band of an earlier launch gave up waiting (synchronises with s).
rt_status lz_resident_error(LzResidentState& st, cudaStream_t s);

}  // namespace rt
