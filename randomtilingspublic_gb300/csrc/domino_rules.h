// Flip rules of the domino sweep as integer acceptance intervals.
//
// Every reference rule (src/Domino/dominokernel*.cl) flips a site whose state is 3 (the
// "up" move, 3 -> 12) or 12 (the "down" move, 12 -> 3) when its uniform draw falls in a set
// that depends only on the row parity of the site and the colour t being rotated.  For all
// four rules that set is one interval of the raw generator output, so the kernels test
// (u - lo) < width on integers.  The host derives the intervals from the reference's own
// float expressions (TinyMT and MTGP modes) or from the fast mode's stated probabilities.
#pragma once
#include <cstdint>

namespace rt {

struct DmRule {
  // Index c = (i & 1) | (t << 1): i the colour-array row, t the rotated colour (1 black).
  uint32_t lo_up[4], w_up[4], lo_dn[4], w_dn[4];
};

// Builds the table; returns false (with a message) for invalid weights.
bool dm_rule_build(int rule, int rng_mode, double a, double b, DmRule* out, const char** err);

// Reference decision for one site (TinyMT scale, u23 in [0, 2^23)); used to derive and to
// check the intervals.  Returns the new state.
uint8_t dm_rule_reference(uint8_t e, uint32_t u23, int rule, int i, int t, double a, double b);

// The same decision as the reference's CUDA kernels make it (src/Domino/dominokernel*.cu,
// float draw rd from cuRAND's MTGP32); it differs from the OpenCL kernels only in the
// two-periodic rule, which divides the draw by the double 0.8 there (by a float 0.8 in the
// .cl kernel), so a threshold can round one ulp apart.
uint8_t dm_rule_reference_cuda(uint8_t e, float rd, int rule, int i, int t, double a, double b);

}  // namespace rt
