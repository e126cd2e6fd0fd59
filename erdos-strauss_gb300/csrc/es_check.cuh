// es_check.cuh -- the engine re-derives every certificate it emits, on the device, in exact
// fixed-width arithmetic (the gate of sieve/verify_covers.py:246-275, restated so that it
// needs no rationals):
//
//   RUNG p A r u:  with q = pA, x = (q + u)/r, y = qx/u,
//                  1/A + 1/x + 1/y = 1/A + (q + u)/(qx) = 1/A + r/q = (p + r)/(pA),
//                  so 4/p = 1/A + 1/x + 1/y holds exactly iff p + r = 4A, r | q + u and
//                  u | qx (x, y >= 1 integers). q < 2^126, x < 2^127, qx < 2^253.
//   SOLVED p a c d k:  with m = 4acd - 1, e = ck - a, the three fractions
//                  1/(ade) + 1/(acdp) + 1/(cdep) = (cp + e + a)/(acdep), and cp + e + a =
//                  4acde iff cp = em - a = c(mk - 4a^2 d), so 4/p holds exactly iff
//                  e >= 1 and p = mk - 4a^2 d.
//
// A certificate that fails is never emitted: the kernel sets ST_CERT_BAD and the host turns
// it into ES_ERR_DEVICE_STATUS.
#pragma once
#include "es_arith.cuh"

namespace es {

struct U256 { u64 w[4]; };                      // little-endian 64-bit words

__device__ __forceinline__ U256 mul128(U128 a, U128 b) {       // full 256-bit product
  U256 r{{0, 0, 0, 0}};
  const u64 aw[2] = {a.lo, a.hi}, bw[2] = {b.lo, b.hi};
  #pragma unroll
  for (int i = 0; i < 2; ++i) {
    u64 carry = 0;
    #pragma unroll
    for (int j = 0; j < 2; ++j) {
      const u64 lo = aw[i] * bw[j], hi = __umul64hi(aw[i], bw[j]);
      u64 t = r.w[i + j] + lo;
      u64 c1 = t < lo;
      u64 t2 = t + carry;
      c1 += t2 < t;
      r.w[i + j] = t2;
      carry = hi + c1;                               // hi <= 2^64 - 2: no overflow
    }
    r.w[i + 2] += carry;
  }
  return r;
}

// x mod d for a 256-bit x and a nonzero 128-bit d: restoring division one bit at a time,
// from x's top set bit (at most 256 steps).
__device__ inline U128 mod256(const U256 &x, U128 d) {
  int top = 255;
  while (top >= 0 && !((x.w[top >> 6] >> (top & 63)) & 1)) --top;
  U128 rem{0, 0};
  for (int i = top; i >= 0; --i) {
    const u64 bit = (x.w[i >> 6] >> (i & 63)) & 1;
    const u64 carry = rem.hi >> 63;                  // the bit shifted out: rem < 2d <= 2^129
    rem.hi = (rem.hi << 1) | (rem.lo >> 63);
    rem.lo = (rem.lo << 1) | bit;
    if (carry || !lt128(rem, d)) {
      const u64 lo = rem.lo - d.lo;
      rem.hi = rem.hi - d.hi - (rem.lo < d.lo ? 1 : 0);
      rem.lo = lo;
    }
  }
  return rem;
}

// 128-bit by 32-bit division, four 32-bit digits at a time.
__device__ __forceinline__ U128 div128_32(U128 x, u32 r, u32 &rem) {
  u64 carry = 0;
  u32 dig[4] = {(u32)(x.hi >> 32), (u32)x.hi, (u32)(x.lo >> 32), (u32)x.lo};
  #pragma unroll
  for (int i = 0; i < 4; ++i) {
    const u64 cur = (carry << 32) | dig[i];
    dig[i] = (u32)(cur / r);
    carry = cur % r;
  }
  rem = (u32)carry;
  return U128{((u64)dig[2] << 32) | dig[3], ((u64)dig[0] << 32) | dig[1]};
}

__device__ inline bool check_rung_cert(u64 p, u64 A, u64 r, U128 u) {
  if (r == 0 || r > 0xFFFFFFFFull || (u.lo == 0 && u.hi == 0) || (u.hi >> 62)) return false;
  const u64 four_a_lo = A << 2, four_a_hi = A >> 62;     // 4A as 128 bits
  const u64 pr_lo = p + r, pr_hi = pr_lo < p ? 1 : 0;     // p + r as 128 bits
  if (four_a_lo != pr_lo || four_a_hi != pr_hi) return false;
  const U128 q{p * A, __umul64hi(p, A)};
  U128 s{q.lo + u.lo, q.hi + u.hi};
  if (s.lo < q.lo) ++s.hi;                                // q + u < 2^127: no overflow
  u32 rem;
  const U128 x = div128_32(s, (u32)r, rem);
  if (rem != 0 || (x.lo == 0 && x.hi == 0)) return false;
  const U128 m = mod256(mul128(q, x), u);
  return m.lo == 0 && m.hi == 0;
}

__device__ inline bool check_solved_cert(u64 p, u64 a, u64 c, u64 d, u64 k) {
  if (!a || !c || !d || !k || a > 0xFFFFFFFFull || d > 0xFFFFFFFFull) return false;
  // m = 4acd - 1 (as 128 bits; a, d < 2^32 so ad < 2^64)
  const u64 ad = a * d;
  U128 m{ad * c, __umul64hi(ad, c)};
  if (m.hi >> 61) return false;                           // keep 4acd below 2^127
  m.hi = (m.hi << 2) | (m.lo >> 62);
  m.lo <<= 2;
  if (m.lo == 0) --m.hi;
  --m.lo;
  // e = ck - a >= 1
  const U128 ck{c * k, __umul64hi(c, k)};
  if (ck.hi == 0 && ck.lo <= a) return false;
  // p + 4a^2 d == m k (4a^2 d < 2^98; m k < 2^191)
  const U256 mk = mul128(m, U128{k, 0});
  const u64 aa = a * a;                                   // < 2^64
  U128 t{aa * d, __umul64hi(aa, d)};                      // a^2 d < 2^96
  t.hi = (t.hi << 2) | (t.lo >> 62);
  t.lo <<= 2;
  U128 sum{t.lo + p, t.hi};
  if (sum.lo < p) ++sum.hi;
  return mk.w[3] == 0 && mk.w[2] == 0 && mk.w[1] == sum.hi && mk.w[0] == sum.lo;
}

}  // namespace es
