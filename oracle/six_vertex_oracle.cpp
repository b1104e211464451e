// TEST INFRASTRUCTURE ONLY - the oracle for the six-vertex path.
//
// The reference has no six-vertex model (it appears only in the library's scope); this is a
// CPU statement of the library's own definition, written independently of the CUDA code,
// against which the kernels are checked.  Parity is "unpinned" by any reference output: the
// model is validated instead by exhaustive enumeration of the domain-wall configurations
// (alternating sign matrices) and by known partition-function values (tests/).
//
// Model.  Vertices of an n x n grid; height points (y, x), 0 <= y, x <= n, at the corners.
// Across a horizontal edge h(below) - h(above) = +1 when its arrow points right; across a
// vertical edge h(right) - h(left) = +1 when its arrow points up.  At a vertex with corner
// heights NW, NE, SW, SE the type is
//   a  (arrows right-right/up-up or left-left/down-down):  NE == SW, NW != SE
//   b  (right-right/down-down or left-left/up-up):          NW == SE, NE != SW
//   c  (the two saddles):                                   NE == SW and NW == SE
// with weights a, b, c.  Domain-wall boundary: h(0, x) = x, h(y, 0) = y, h(n, x) = n - x,
// h(y, n) = n - y.
//
// Sweep.  The height points split into four classes (x mod 2, y mod 2); no two points of a
// class share a vertex.  Sub-sweep s updates class s mod 4 (px = s & 1, py = (s >> 1) & 1):
// every interior point whose four edge neighbours are all equal to h' is set by heat bath to
// h' + 1 with probability P(k1, k2) and to h' - 1 otherwise, where k1 counts the diagonal
// points (-1,-1), (+1,+1) equal to h' + 1 (their shared vertices are a- or c-type) and k2 the
// diagonal points (-1,+1), (+1,-1) equal to h' + 1 (b- or c-type vertices):
//   W+ = c^k1 a^(2-k1) c^k2 b^(2-k2),  W- = c^(2-k1) a^k1 c^(2-k2) b^k2,  P = W+ / (W+ + W-).
// The draw: u < T[3 k1 + k2] with T = min(floor(P 2^32), 2^32 - 1).  The 32 bits of u for
// the point of class row r = (y - py) / 2, bit b of word w (k = (x - px) / 2 = 32 w + b) are
// bit b of 32 random planes; plane 31 - (4 q + t) is word t of
//   Philox4x32-10(ctr = {w | q << 24, r, lo32(s), (hi32(s) & 0xffff) | stream << 16},
//                 key = {lo32(seed), hi32(seed)}),  q = 0..7.
// CFTP: coupled chains from the maximal and minimal height functions, attempt j running
// sub-sweeps [-4 T, 0) with T = first_sweeps * 2^j; exact when c >= max(a, b) (the heat-bath
// update is then monotone in every other point).
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load this.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "philox_ref.h"

namespace {

struct SvThresholds { uint32_t t[9]; };

SvThresholds sv_thresholds(double a, double b, double c) {
  SvThresholds T;
  for (int k1 = 0; k1 < 3; ++k1)
    for (int k2 = 0; k2 < 3; ++k2) {
      double wp = 1.0, wm = 1.0;
      for (int i = 0; i < 2; ++i) {
        wp *= i < k1 ? c : a;
        wm *= i < 2 - k1 ? c : a;
      }
      for (int i = 0; i < 2; ++i) {
        wp *= i < k2 ? c : b;
        wm *= i < 2 - k2 ? c : b;
      }
      const double p = wp / (wp + wm);
      const double s = std::floor(p * 4294967296.0);
      T.t[3 * k1 + k2] = s >= 4294967295.0 ? 0xffffffffu : (uint32_t)s;
    }
  return T;
}

uint32_t sv_draw(uint64_t seed, uint32_t stream, int64_t s, uint32_t r, uint32_t k) {
  const uint32_t w = k >> 5, b = k & 31;
  uint32_t u = 0;
  for (uint32_t q = 0; q < 8; ++q) {
    oracle::U32x4 c;
    c.v[0] = w | (q << 24);
    c.v[1] = r;
    c.v[2] = (uint32_t)(uint64_t)s;
    c.v[3] = ((uint32_t)((uint64_t)s >> 32) & 0xffffu) | (stream << 16);
    const oracle::U32x4 o = oracle::philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    for (int t = 0; t < 4; ++t) u |= ((o.v[t] >> b) & 1u) << (31 - (4 * q + t));
  }
  return u;
}

// One sub-sweep s on the (n+1) x (n+1) height array.
void sv_sub_sweep(int* h, int n, int64_t s, uint64_t seed, uint32_t stream, const SvThresholds& T) {
  const int L = n + 1, px = (int)(s & 1), py = (int)((s >> 1) & 1);
  auto H = [&](int y, int x) { return h[(size_t)y * L + x]; };
  for (int y = (py ? 1 : 2); y <= n - 1; y += 2)
    for (int x = (px ? 1 : 2); x <= n - 1; x += 2) {
      const int hp = H(y, x - 1);
      if (H(y, x + 1) != hp || H(y - 1, x) != hp || H(y + 1, x) != hp) continue;
      const int up = hp + 1;
      const int k1 = (H(y - 1, x - 1) == up) + (H(y + 1, x + 1) == up);
      const int k2 = (H(y - 1, x + 1) == up) + (H(y + 1, x - 1) == up);
      const uint32_t u = sv_draw(seed, stream, s, (uint32_t)((y - py) / 2), (uint32_t)((x - px) / 2));
      h[(size_t)y * L + x] = u < T.t[3 * k1 + k2] ? up : hp - 1;
    }
}

void sv_dwbc(int n, bool top, int* out) {
  const int L = n + 1;
  for (int y = 0; y <= n; ++y)
    for (int x = 0; x <= n; ++x)
      out[(size_t)y * L + x] = top ? std::min(x + y, 2 * n - x - y) : std::abs(x - y);
}

}  // namespace

extern "C" {

void orc_sv_thresholds(double a, double b, double c, unsigned* out9) {
  const SvThresholds T = sv_thresholds(a, b, c);
  std::memcpy(out9, T.t, sizeof T.t);
}

void orc_sv_dwbc(int n, int top, int* out) { sv_dwbc(n, top != 0, out); }

unsigned orc_sv_draw(unsigned long seed, unsigned stream, long s, unsigned r, unsigned k) {
  return sv_draw(seed, stream, s, r, k);
}

// Sub-sweeps [s0, s0 + count) on h ((n+1)^2 heights, updated in place).
int orc_sv_walk(int* h, int n, long s0, long count, unsigned long seed, unsigned stream, double a, double b, double c) {
  if (n < 2) return -1;
  const SvThresholds T = sv_thresholds(a, b, c);
  for (long s = s0; s < s0 + count; ++s) sv_sub_sweep(h, n, s, seed, stream, T);
  return 0;
}

// Returns the attempt that coalesced (1-based) or -1; *sweeps_used = its look-back T.
int orc_sv_cftp(const int* hmax, const int* hmin, int n, unsigned long seed, unsigned stream, long first_sweeps,
                int max_attempts, double a, double b, double c, int* out, long* sweeps_used) {
  const size_t L2 = (size_t)(n + 1) * (n + 1);
  const SvThresholds T = sv_thresholds(a, b, c);
  long Tsw = first_sweeps;
  for (int attempt = 1; attempt <= max_attempts; ++attempt, Tsw *= 2) {
    std::vector<int> top(hmax, hmax + L2), bot(hmin, hmin + L2);
    for (long s = -4 * Tsw; s < 0; ++s) {
      sv_sub_sweep(top.data(), n, s, seed, stream, T);
      sv_sub_sweep(bot.data(), n, s, seed, stream, T);
    }
    if (top == bot) {
      std::memcpy(out, top.data(), L2 * sizeof(int));
      if (sweeps_used) *sweeps_used = Tsw;
      return attempt;
    }
  }
  return -1;
}

}  // extern "C"
