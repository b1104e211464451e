// TEST INFRASTRUCTURE ONLY. CPU restatement of TinyMT32 (Saito & Matsumoto, 2011) as the
// reference uses it on its OpenCL path: src/TinyMT/tinymt32.clh:40-129 (next_state, temper,
// single01) and :183-203 (init with one 32-bit seed).  Only tests/, __graft_entry__.smoke()
// and bench.py's CPU baseline may use anything under oracle/.
#pragma once
#include <cstdint>
#include <cstring>

namespace oracle {

struct TinyMT32 {
  uint32_t s0, s1, s2, s3;
  uint32_t mat1, mat2, tmat;
};

// tinymt32.clh:40-55 - one step of the 127-bit linear recurrence.
inline void tmt_next_state(TinyMT32& g) {
  uint32_t x = (g.s0 & 0x7fffffffu) ^ g.s1 ^ g.s2;
  uint32_t y = g.s3;
  x ^= x << 1;
  y ^= (y >> 1) ^ x;
  g.s0 = g.s1;
  g.s1 = g.s2;
  g.s2 = x ^ (y << 10);
  g.s3 = y;
  if (y & 1u) {
    g.s1 ^= g.mat1;
    g.s2 ^= g.mat2;
  }
}

// tinymt32.clh:63-73 - tempering of the current state.
inline uint32_t tmt_temper(const TinyMT32& g) {
  uint32_t t0 = g.s3;
  uint32_t t1 = g.s0 + (g.s2 >> 8);
  t0 ^= t1;
  if (t1 & 1u) t0 ^= g.tmat;
  return t0;
}

// tinymt32.clh:81-129: single01 = as_float((temper >> 9) | 0x3f800000) - 1.0f, which is
// exactly (temper >> 9) * 2^-23.  The sweep only needs the 23-bit integer.
inline uint32_t tmt_next_u23(TinyMT32& g) {
  tmt_next_state(g);
  return tmt_temper(g) >> 9;
}

inline float tmt_u23_to_float(uint32_t u23) {
  uint32_t bits = u23 | 0x3f800000u;
  float f;
  std::memcpy(&f, &bits, 4);
  return f - 1.0f;
}

// tinymt32.clh:183-203 - seeding from one 32-bit value, parameters taken from the table.
inline void tmt_init(TinyMT32& g, uint32_t seed) {
  uint32_t st[4] = {seed, g.mat1, g.mat2, g.tmat};
  for (int i = 1; i < 8; ++i) {
    uint32_t prev = st[(i - 1) & 3];
    st[i & 3] ^= (uint32_t)i + 1812433253u * (prev ^ (prev >> 30));
  }
  g.s0 = st[0]; g.s1 = st[1]; g.s2 = st[2]; g.s3 = st[3];
  // tinymt32.clh:162-174 period certification
  if ((g.s0 & 0x7fffffffu) == 0 && g.s1 == 0 && g.s2 == 0 && g.s3 == 0) {
    g.s0 = 'T'; g.s1 = 'I'; g.s2 = 'N'; g.s3 = 'Y';
  }
  for (int i = 0; i < 8; ++i) tmt_next_state(g);
}

// Default parameter set used for every generator when no parameter table is supplied:
// the TinyMT32 jump parameters of src/TinyMT/tinymt32def.h:48-50.  The reference's
// per-generator table (src/TinyMT/tinymt32dc.0.1048576.txt) is absent from its tree.
constexpr uint32_t kTmtMat1 = 0x8f7011eeu;
constexpr uint32_t kTmtMat2 = 0xfc78ff1fu;
constexpr uint32_t kTmtTmat = 0x3793fdffu;

}  // namespace oracle
