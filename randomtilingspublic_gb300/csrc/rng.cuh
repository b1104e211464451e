// Device random-number generators of the sweep.
//
// TinyMT32 (Saito & Matsumoto): the generator of the reference's OpenCL path
// (src/TinyMT/tinymt32.clh:40-73 step and tempering, :183-203 seeding).  One 127-bit state
// per site, uint4 {s0, s1, s2, s3}; the draw the sweep uses is temper >> 9, the 23-bit
// integer behind tinymt32_single01 (tinymt32.clh:81-129), whose float value is exactly
// u23 * 2^-23.
//
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): the counter-based generator of the
// fast mode; keyed per (seed), counter (column quad, row, half-sweep, stream).
#pragma once
#include <cstdint>

namespace rt {

struct TmtParams {
  uint32_t mat1, mat2, tmat;
};

// Default per-generator parameters: the TinyMT32 jump set (src/TinyMT/tinymt32def.h:48-50).
constexpr uint32_t kTmtMat1 = 0x8f7011eeu;
constexpr uint32_t kTmtMat2 = 0xfc78ff1fu;
constexpr uint32_t kTmtTmat = 0x3793fdffu;

// One generator step followed by tempering; returns the 23-bit draw.
__device__ __forceinline__ uint32_t tmt_next_u23(uint4& s, uint32_t mat1, uint32_t mat2, uint32_t tmat) {
  uint32_t x = (s.x & 0x7fffffffu) ^ s.y ^ s.z;
  uint32_t y = s.w;
  x ^= x << 1;
  y ^= (y >> 1) ^ x;
  const uint32_t odd = 0u - (y & 1u);
  s.x = s.y;
  s.y = s.z ^ (mat1 & odd);
  s.z = (x ^ (y << 10)) ^ (mat2 & odd);
  s.w = y;
  uint32_t t1 = s.x + (s.z >> 8);
  uint32_t t0 = s.w ^ t1;
  t0 ^= tmat & (0u - (t1 & 1u));
  return t0 >> 9;
}

// The same step and tempering with the work spread over both integer pipes: the constant
// shifts are multiplies by powers of two (x << k = x * 2^k, x >> k = the high word of
// x * 2^(32-k)) and the parameter masks are multiplies by the parity bit, which run on the
// multiply-add pipe, leaving the three-input logic ops to the ALU.  Identical results.
__device__ __forceinline__ uint32_t mul_lo(uint32_t a, uint32_t b) {
  uint32_t d;
  asm("mul.lo.u32 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
  return d;
}
__device__ __forceinline__ uint32_t mul_hi(uint32_t a, uint32_t b) {
  uint32_t d;
  asm("mul.hi.u32 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
  return d;
}
__device__ __forceinline__ uint32_t mad_hi(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t d;
  asm("mad.hi.u32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
  return d;
}
__device__ __forceinline__ uint32_t tmt_next_u23_mad(uint4& s, uint32_t mat1, uint32_t mat2, uint32_t tmat) {
  uint32_t x = (s.x & 0x7fffffffu) ^ s.y ^ s.z;
  uint32_t y = s.w;
  x ^= mul_lo(x, 2u);                   // x << 1
  y ^= mul_hi(y, 0x80000000u) ^ x;      // y >> 1
  const uint32_t odd = y & 1u;
  s.x = s.y;
  s.y = s.z ^ mul_lo(mat1, odd);
  s.z = x ^ mul_lo(y, 1024u) ^ mul_lo(mat2, odd);  // y << 10
  s.w = y;
  const uint32_t t1 = mad_hi(s.z, 1u << 24, s.x);  // s.x + (s.z >> 8)
  const uint32_t t0 = s.w ^ t1 ^ mul_lo(tmat, t1 & 1u);
  return mul_hi(t0, 1u << 23);                     // t0 >> 9
}

// The same step returning the whole tempered word t0; the draw is t0 >> 9, so a test
// (u - lo) < w on the draw is mad_hi(t0, 2^23, -lo) < w, one multiply-add.
__device__ __forceinline__ uint32_t tmt_next_t0_mad(uint4& s, uint32_t mat1, uint32_t mat2, uint32_t tmat) {
  uint32_t x = (s.x & 0x7fffffffu) ^ s.y ^ s.z;
  uint32_t y = s.w;
  x ^= mul_lo(x, 2u);
  y ^= mul_hi(y, 0x80000000u) ^ x;
  const uint32_t odd = y & 1u;
  s.x = s.y;
  s.y = s.z ^ mul_lo(mat1, odd);
  s.z = x ^ mul_lo(y, 1024u) ^ mul_lo(mat2, odd);
  s.w = y;
  const uint32_t t1 = mad_hi(s.z, 1u << 24, s.x);
  return s.w ^ t1 ^ mul_lo(tmat, t1 & 1u);
}

__device__ __forceinline__ void tmt_plain_step(uint4& s, uint32_t mat1, uint32_t mat2) {
  uint32_t x = (s.x & 0x7fffffffu) ^ s.y ^ s.z;
  uint32_t y = s.w;
  x ^= x << 1;
  y ^= (y >> 1) ^ x;
  const uint32_t odd = 0u - (y & 1u);
  s.x = s.y;
  s.y = s.z ^ (mat1 & odd);
  s.z = (x ^ (y << 10)) ^ (mat2 & odd);
  s.w = y;
}

// Seeding from one 32-bit value (tinymt32.clh:183-203).
__device__ __forceinline__ uint4 tmt_seed(uint32_t seed, uint32_t mat1, uint32_t mat2, uint32_t tmat) {
  uint32_t st[4] = {seed, mat1, mat2, tmat};
#pragma unroll
  for (int i = 1; i < 8; ++i) {
    uint32_t p = st[(i - 1) & 3];
    st[i & 3] ^= (uint32_t)i + 1812433253u * (p ^ (p >> 30));
  }
  uint4 s = make_uint4(st[0], st[1], st[2], st[3]);
  if ((s.x & 0x7fffffffu) == 0 && s.y == 0 && s.z == 0 && s.w == 0) s = make_uint4('T', 'I', 'N', 'Y');
#pragma unroll
  for (int i = 0; i < 8; ++i) tmt_plain_step(s, mat1, mat2);
  return s;
}

// Philox4x32-10.  ctr = {c0, c1, c2, c3}, key = {k0, k1}.
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
    const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
    c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

// Fast-mode draws for the four sites of column quad q (columns 4q .. 4q+3) of colour-array
// row i at half-sweep h of stream s.
__device__ __forceinline__ uint4 fast_quad(uint64_t seed, uint32_t stream, int64_t h, uint32_t i, uint32_t q) {
  const uint64_t hu = (uint64_t)h;
  uint4 c = make_uint4(q, i, (uint32_t)hu, ((uint32_t)(hu >> 32) & 0xffffu) | (stream << 16));
  return philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
}

}  // namespace rt
