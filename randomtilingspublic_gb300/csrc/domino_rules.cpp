#include "domino_rules.h"

#include <algorithm>
#include <cmath>
#include <cstring>

#include "../../include/rt_tilings.h"

namespace rt {
namespace {

float u23_to_float(uint32_t u23) {
  uint32_t bits = u23 | 0x3f800000u;
  float f;
  std::memcpy(&f, &bits, sizeof f);
  return f - 1.0f;  // exact: u23 * 2^-23
}

// Metropolis ratio of the 2x2-periodic weights for the up / down move at row parity ip and
// colour t, evaluated as the reference kernels do: the weights in double, stored to float,
// the ratio a float division (dominokerneltwoperiodic.cl:22-30).
float ratio_up(int i, int t, double a, double b) {
  float w_init = b * b * ((i + t + 1) % 2) + a * a * ((i + t) % 2);
  float w_fin = a * a * (i % 2) + b * b * ((i + 1) % 2);
  return w_fin / w_init;
}
float ratio_dn(int i, int t, double a, double b) {
  float w_init = a * a * (i % 2) + b * b * ((i + 1) % 2);
  float w_fin = b * b * ((i + t + 1) % 2) + a * a * ((i + t) % 2);
  return w_fin / w_init;
}

uint32_t ceil_scaled(double p, double scale) {
  double x = std::ceil(p * scale);
  if (x < 0) x = 0;
  if (x > 4294967295.0) x = 4294967295.0;
  return (uint32_t)x;
}

// Smallest u in [lo, hi) with accept(u) false, given accept is true on a prefix of [lo, hi).
template <class F>
uint32_t first_reject(uint32_t lo, uint32_t hi, F accept) {
  while (lo < hi) {
    uint32_t mid = lo + (hi - lo) / 2;
    if (accept(mid)) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

}  // namespace

uint8_t dm_rule_reference(uint8_t e, uint32_t u23, int rule, int i, int t, double a, double b) {
  const float rd = u23_to_float(u23);
  switch (rule) {
    case RT_DOMINO_PLAIN:  // dominokernel.cl:14-17
      if ((double)rd < .8) return e == 3 ? 12 : (e == 12 ? 3 : e);
      return e;
    case RT_DOMINO_CFTP:  // dominokernelCFTP.cl:65-69
      if ((double)rd < 0.5) return e == 3 ? 12 : e;
      return e == 12 ? 3 : e;
    case RT_DOMINO_TWOPERIODIC: {  // dominokerneltwoperiodic.cl:17-32
      const float propose = 0.8;
      if (rd < propose) {
        float threshold = rd / propose;
        if (e == 3) return ratio_up(i, t, a, b) > threshold ? 12 : 3;
        if (e == 12) return ratio_dn(i, t, a, b) > threshold ? 3 : 12;
      }
      return e;
    }
    case RT_DOMINO_CFTP_TWOPERIODIC: {  // dominokernelCFTPtwoperiodic.cl:84-99
      if ((double)rd < 0.5) {
        float threshold = (double)rd / 0.5;
        if (e == 3) return ratio_up(i, t, a, b) > threshold ? 12 : 3;
      } else {
        float threshold = ((double)rd - 0.5) / 0.5;
        if (e == 12) return ratio_dn(i, t, a, b) > threshold ? 3 : 12;
      }
      return e;
    }
  }
  return e;
}

uint8_t dm_rule_reference_cuda(uint8_t e, float rd, int rule, int i, int t, double a, double b) {
  switch (rule) {
    case RT_DOMINO_PLAIN:  // dominokernel.cu:19-22 (PROB_PROPOSE 0.8, a double)
      if ((double)rd < .8) return e == 3 ? 12 : (e == 12 ? 3 : e);
      return e;
    case RT_DOMINO_CFTP:  // dominokernelCFTP.cu:26-31
      if ((double)rd < 0.5) return e == 3 ? 12 : e;
      return e == 12 ? 3 : e;
    case RT_DOMINO_TWOPERIODIC: {  // dominokerneltwoperiodic.cu:23-40: compare and divide in double
      if ((double)rd < .8) {
        float threshold = (double)rd / .8;
        if (e == 3) return ratio_up(i, t, a, b) > threshold ? 12 : 3;
        if (e == 12) return ratio_dn(i, t, a, b) > threshold ? 3 : 12;
      }
      return e;
    }
    case RT_DOMINO_CFTP_TWOPERIODIC: {  // dominokernelCFTPtwoperiodic.cu:30-46
      if ((double)rd < 0.5) {
        float threshold = (double)rd / 0.5;
        if (e == 3) return ratio_up(i, t, a, b) > threshold ? 12 : 3;
      } else {
        float threshold = ((double)rd - 0.5) / 0.5;
        if (e == 12) return ratio_dn(i, t, a, b) > threshold ? 3 : 12;
      }
      return e;
    }
  }
  return e;
}

bool dm_rule_build(int rule, int rng_mode, double a, double b, DmRule* out, const char** err) {
  if (rule < RT_DOMINO_PLAIN || rule > RT_DOMINO_CFTP_TWOPERIODIC) {
    *err = "unknown domino rule";
    return false;
  }
  if (rng_mode != RT_RNG_TINYMT && rng_mode != RT_RNG_FAST && rng_mode != RT_RNG_MTGP) {
    *err = "unknown rng mode";
    return false;
  }
  const bool weighted = (rule == RT_DOMINO_TWOPERIODIC || rule == RT_DOMINO_CFTP_TWOPERIODIC);
  if (weighted && !(a > 0.0 && b > 0.0 && std::isfinite(a) && std::isfinite(b))) {
    *err = "two-periodic weights must be finite and > 0";
    return false;
  }
  const bool monotone = (rule == RT_DOMINO_CFTP || rule == RT_DOMINO_CFTP_TWOPERIODIC);
  for (int c = 0; c < 4; ++c) {
    const int ip = c & 1, t = c >> 1;
    const int i = 2 + ip;  // any row of that parity
    uint32_t lo_up = 0, w_up, lo_dn, w_dn;
    if (rng_mode == RT_RNG_MTGP) {
      // MTGP mode: u is the bit pattern of the float draw in (0, 1], and positive floats
      // order as their bit patterns, so each move's set of draws is again an interval (a
      // prefix of [0, 1], or of [0.5, 1] for the down move of the monotone rules).
      const uint32_t U = 0x3f800001u, half = 0x3f000000u;  // bits of 1.0f plus one; of 0.5f
      auto rd_of = [](uint32_t u) {
        float f;
        std::memcpy(&f, &u, sizeof f);
        return f;
      };
      w_up = first_reject(0, U, [&](uint32_t u) { return dm_rule_reference_cuda(3, rd_of(u), rule, i, t, a, b) == 12; });
      lo_dn = monotone ? half : 0;
      w_dn = first_reject(lo_dn, U, [&](uint32_t u) { return dm_rule_reference_cuda(12, rd_of(u), rule, i, t, a, b) == 3; }) -
             lo_dn;
    } else if (rng_mode == RT_RNG_TINYMT) {
      const uint32_t U = 1u << 23, half = 1u << 22;
      w_up = first_reject(0, U, [&](uint32_t u) { return dm_rule_reference(3, u, rule, i, t, a, b) == 12; });
      lo_dn = monotone ? half : 0;
      w_dn = first_reject(lo_dn, U, [&](uint32_t u) { return dm_rule_reference(12, u, rule, i, t, a, b) == 3; }) - lo_dn;
    } else {
      // Fast mode: the reference's move probabilities resolved on a 32-bit draw u.
      // Proposal rules accept when u < ceil(p * 2^32); the monotone rules split u at 2^31
      // into an up half and a down half, each accepting ceil(min(1, ratio) * 2^31) values.
      const double P32 = 4294967296.0, P31 = 2147483648.0;
      switch (rule) {
        case RT_DOMINO_PLAIN:
          w_up = w_dn = ceil_scaled(0.8, P32);
          lo_dn = 0;
          break;
        case RT_DOMINO_CFTP:
          w_up = w_dn = 0x80000000u;
          lo_dn = 0x80000000u;
          break;
        case RT_DOMINO_TWOPERIODIC:
          w_up = ceil_scaled(0.8 * std::min(1.0, (double)ratio_up(i, t, a, b)), P32);
          w_dn = ceil_scaled(0.8 * std::min(1.0, (double)ratio_dn(i, t, a, b)), P32);
          lo_dn = 0;
          break;
        default:  // RT_DOMINO_CFTP_TWOPERIODIC
          w_up = ceil_scaled(std::min(1.0, (double)ratio_up(i, t, a, b)), P31);
          w_dn = ceil_scaled(std::min(1.0, (double)ratio_dn(i, t, a, b)), P31);
          lo_dn = 0x80000000u;
          break;
      }
    }
    out->lo_up[c] = lo_up;
    out->w_up[c] = w_up;
    out->lo_dn[c] = lo_dn;
    out->w_dn[c] = w_dn;
  }
  return true;
}

}  // namespace rt
