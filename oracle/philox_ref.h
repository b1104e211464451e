// TEST INFRASTRUCTURE ONLY. CPU statement of Philox4x32-10 (Salmon, Moraes, Dror, Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC'11), the counter-based generator of the
// library's fast RNG mode.  It is the checker for the CUDA implementation, never called by it.
#pragma once
#include <cstdint>

namespace oracle {

struct U32x4 { uint32_t v[4]; };

inline U32x4 philox4x32_10(U32x4 ctr, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)M0 * ctr.v[0];
    uint64_t p1 = (uint64_t)M1 * ctr.v[2];
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    U32x4 n;
    n.v[0] = hi1 ^ ctr.v[1] ^ k0;
    n.v[1] = lo1;
    n.v[2] = hi0 ^ ctr.v[3] ^ k1;
    n.v[3] = lo0;
    ctr = n;
    k0 += W0;
    k1 += W1;
  }
  return ctr;
}

// Library fast-mode draw for the site in colour-array row i, column m at half-sweep h of
// stream s (s < 2^16, |h| < 2^47): word (m & 3) of
// Philox4x32-10(ctr = {m >> 2, i, lo32(h), (hi32(h) & 0xffff) | (s << 16)},
//               key = {lo32(seed), hi32(seed)}).
inline uint32_t fast_draw(uint64_t seed, uint32_t stream, int64_t h, uint32_t i, uint32_t m) {
  U32x4 c;
  c.v[0] = m >> 2;
  c.v[1] = i;
  c.v[2] = (uint32_t)(uint64_t)h;
  c.v[3] = ((uint32_t)((uint64_t)h >> 32) & 0xffffu) | (stream << 16);
  U32x4 o = philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  return o.v[m & 3];
}

}  // namespace oracle
