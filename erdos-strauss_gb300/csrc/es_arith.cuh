// es_arith.cuh -- exact 64/128-bit integer arithmetic for the survivor tail, on the device.
//
// Everything here is exact integer arithmetic: Montgomery multiplication valid for every
// odd modulus below 2^64 (the two-word reduction keeps the (t + m*n)/2^64 sum in 65 bits,
// the same care sieve/rung_scan3.cpp:256-282 takes), the 12-base deterministic
// Miller-Rabin of census/rung_scan.cpp:76-92, trial division by multiplicative inverses
// (an odd prime d divides n iff n * d^-1 mod 2^64 <= floor((2^64-1)/d)), Brent's rho
// (census/rung_scan.cpp:94-128, sieve/rung_scan3.cpp:333-369), the rung DP
// (sieve/rung_scan3.cpp:544-565) and the direct search (:607-647).
//
// A factorization is unique, so any exact method gives the reference's certificates:
// the DP takes a minimum over divisors and the direct search a minimum over divisors too.
// Every loop here is bounded. A loop that reaches its bound sets a bit in the engine's
// device status word and returns "not found"; the host turns the bit into
// ES_ERR_DEVICE_STATUS. Nothing traps.
#pragma once
#include <cstdint>

namespace es {

typedef unsigned long long u64;
typedef unsigned int u32;
typedef unsigned short u16;

// Device status bits (written with atomicOr, read by the host after each run).
enum : u32 {
  ST_SURV_OVERFLOW = 1u << 0,   // survivor list longer than its buffer (host re-runs bigger)
  ST_PRIME_OVERFLOW = 1u << 1,
  ST_RHO_BUDGET = 1u << 2,      // Brent's rho exceeded its iteration budget
  ST_FAC_OVERFLOW = 1u << 3,    // more than 16 distinct primes (impossible below 2^64)
  ST_STACK_OVERFLOW = 1u << 4,  // composite stack of the hard factorization overflowed
  ST_QUEUE_TIMEOUT = 1u << 5,   // a work-queue wait gave up
  ST_BAD_INPUT = 1u << 6,       // an argument outside the documented domain reached a kernel
  ST_CERT_BAD = 1u << 7,        // a certificate failed its exact re-derivation (es_check.cuh)
};

constexpr int MAXF = 16;                       // census/rung_scan.cpp:147
constexpr u32 RCAP = 255;                      // census/rung_scan.cpp:64
constexpr u64 DIRECT_NMAX = 18446744065119617025ull;   // (2^32-1)^2, sieve/rung_scan3.cpp:42
constexpr int NTD = 6541;                      // odd primes below 65536 (3 .. 65521)
constexpr u64 RHO_BUDGET = 1ull << 28;         // total rho steps per hard factorization

struct Fac {
  u64 pr[MAXF];
  unsigned char ex[MAXF];
  int k;
};

// Trial-division table: for each odd prime d < 2^16, d^-1 mod 2^64 and floor((2^64-1)/d).
struct TdEntry { u64 inv, lim; };

__device__ __forceinline__ void fac_add(Fac &f, u64 p, int e, u32 *status) {
  for (int i = 0; i < f.k; ++i)
    if (f.pr[i] == p) { f.ex[i] = (unsigned char)(f.ex[i] + e); return; }
  if (f.k >= MAXF) { atomicOr(status, ST_FAC_OVERFLOW); return; }
  f.pr[f.k] = p; f.ex[f.k] = (unsigned char)e; ++f.k;
}

// ---------------------------------------------------------------- Montgomery, n odd
struct Mont {
  u64 n, ninv, one, r2;   // ninv = -n^-1 mod 2^64; one = 2^64 mod n; r2 = 2^128 mod n
};

__device__ __forceinline__ u64 inv_pow2(u64 a) {   // a odd: a^-1 mod 2^64 by Newton
  u64 x = a;                                         // correct to 3 bits
  #pragma unroll
  for (int i = 0; i < 5; ++i) x *= 2 - a * x;        // 6, 12, 24, 48, 96 bits
  return x;
}

__device__ __forceinline__ u64 addmod(u64 a, u64 b, u64 n) {   // a, b < n
  const u64 s = a + b;
  return (s < a || s >= n) ? s - n : s;
}

__device__ __forceinline__ Mont mont_init(u64 n) {
  Mont m;
  m.n = n;
  m.ninv = 0 - inv_pow2(n);
  m.one = (0 - n) % n;                               // 2^64 mod n
  u64 x = m.one;                                     // double 64 times: 2^128 mod n
  for (int i = 0; i < 64; ++i) x = addmod(x, x, n);
  m.r2 = x;
  return m;
}

// (hi:lo) * 2^-64 mod n for (hi:lo) < n * 2^64. The sum t + m*n is a multiple of 2^64
// below 2n * 2^64; its high word can carry out of 64 bits when n >= 2^63, and that carry
// is folded back by the final subtraction.
__device__ __forceinline__ u64 redc(u64 hi, u64 lo, const Mont &M) {
  const u64 m = lo * M.ninv;
  const u64 mnhi = __umul64hi(m, M.n);
  const u64 carry = lo != 0;                          // lo + low64(m*n) is 0 or 2^64
  const u64 s = hi + mnhi;
  const bool c1 = s < hi;
  const u64 s2 = s + carry;
  const bool c2 = s2 < s;
  return (c1 || c2 || s2 >= M.n) ? s2 - M.n : s2;
}
__device__ __forceinline__ u64 mmul(u64 a, u64 b, const Mont &M) {
  return redc(__umul64hi(a, b), a * b, M);
}
__device__ __forceinline__ u64 to_mont(u64 a, const Mont &M) { return mmul(a % M.n, M.r2, M); }

// Two arithmetic policies over a Mont modulus for the hard-cofactor searches (rho, ECM):
// Exact keeps every residue in [0, n) for any odd n < 2^64. Lazy is for odd n < 2^62 and keeps
// residues in [0, 2n), each standing for its class mod n: the product of two such values is
// below 4n^2 < n 2^64, so (T + m n) / 2^64 is already below 2n and the reduction needs no
// final comparison and subtraction (measured on GB300: 86 instead of 119 cycles for one
// dependent Montgomery multiply). gcd(x, n) and x mod p for p | n do not depend on which
// representative x is, so a search that only ever takes gcds with n, as rho and ECM do, finds
// the same divisors either way; norm() gives the representative in [0, n) where a value must
// be exact (a modular inverse).
struct ExactArith {
  static __device__ __forceinline__ u64 mul(u64 a, u64 b, const Mont &M) { return mmul(a, b, M); }
  static __device__ __forceinline__ u64 add(u64 a, u64 b, const Mont &M) { return addmod(a, b, M.n); }
  static __device__ __forceinline__ u64 sub(u64 a, u64 b, const Mont &M) { return a >= b ? a - b : a + (M.n - b); }
  static __device__ __forceinline__ u64 norm(u64 a, const Mont &) { return a; }
};
struct LazyArith {
  static constexpr u64 NMAX = 1ull << 62;            // n must be below this
  static __device__ __forceinline__ u64 mul(u64 a, u64 b, const Mont &M) {
    const u64 lo = a * b, m = lo * M.ninv;
    return __umul64hi(a, b) + __umul64hi(m, M.n) + (lo != 0);   // lo + low64(m n) is 0 or 2^64
  }
  static __device__ __forceinline__ u64 add(u64 a, u64 b, const Mont &M) {
    const u64 s = a + b, n2 = M.n << 1;
    return s >= n2 ? s - n2 : s;
  }
  static __device__ __forceinline__ u64 sub(u64 a, u64 b, const Mont &M) { return a >= b ? a - b : a + ((M.n << 1) - b); }
  static __device__ __forceinline__ u64 norm(u64 a, const Mont &M) { return a >= M.n ? a - M.n : a; }
};

// ---------------------------------------------------------------- Miller-Rabin
// One strong-probable-prime round, base already in Montgomery form; d odd, n-1 = d 2^s.
__device__ __forceinline__ bool sprp_mont(u64 bm, u64 d, int s, const Mont &M) {
  const u64 mone = M.n - M.one;                       // Montgomery form of n-1
  u64 x = M.one, b = bm, e = d;
  while (e) {
    if (e & 1) x = mmul(x, b, M);
    b = mmul(b, b, M);
    e >>= 1;
  }
  if (x == M.one || x == mone) return true;
  for (int i = 1; i < s; ++i) {
    x = mmul(x, x, M);
    if (x == mone) return true;
  }
  return false;
}

// The same round in an arithmetic policy (LazyArith needs n < 2^62): the comparisons take the
// exact representative.
template <class Ar>
__device__ __forceinline__ bool sprp_ar(u64 bm, u64 d, int s, const Mont &M) {
  const u64 mone = M.n - M.one;
  u64 x = M.one, b = bm, e = d;
  while (e) {
    if (e & 1) x = Ar::mul(x, b, M);
    b = Ar::mul(b, b, M);
    e >>= 1;
  }
  x = Ar::norm(x, M);
  if (x == M.one || x == mone) return true;
  for (int i = 1; i < s; ++i) {
    x = Ar::norm(Ar::mul(x, x, M), M);
    if (x == mone) return true;
  }
  return false;
}

// The base-2 round by left-to-right square-and-double: 2^d with a squaring per bit of d and,
// for each set bit, a multiplication by the base that is a modular doubling, so only the
// squarings take Montgomery multiplies (about 63 instead of about 95 for right-to-left binary
// exponentiation). The same x comes out: Ar::norm gives its exact representative.
template <class Ar>
__device__ __forceinline__ bool sprp2_ar(u64 d, int s, const Mont &M) {
  const u64 mone = M.n - M.one;
  u64 x = Ar::add(M.one, M.one, M);                  // 2: the top bit of d (d >= 1)
  for (int i = 62 - __clzll((long long)d); i >= 0; --i) {
    x = Ar::mul(x, x, M);
    if ((d >> i) & 1) x = Ar::add(x, x, M);
  }
  x = Ar::norm(x, M);
  if (x == M.one || x == mone) return true;
  for (int i = 1; i < s; ++i) {
    x = Ar::norm(Ar::mul(x, x, M), M);
    if (x == mone) return true;
  }
  return false;
}
__device__ __forceinline__ bool sprp2_mont(u64 d, int s, const Mont &M) {
  const u64 mone = M.n - M.one;
  u64 x = addmod(M.one, M.one, M.n);
  for (int i = 62 - __clzll((long long)d); i >= 0; --i) {
    x = mmul(x, x, M);
    if ((d >> i) & 1) x = addmod(x, x, M.n);
  }
  if (x == M.one || x == mone) return true;
  for (int i = 1; i < s; ++i) {
    x = mmul(x, x, M);
    if (x == mone) return true;
  }
  return false;
}

__constant__ const u64 MR_BASES[12] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37};

// The reference's is_prime: trial division by the 12 bases, then all 12 SPRP rounds
// (census/rung_scan.cpp:76-92). Deterministic for n < 3.3e24.
__device__ inline bool is_prime64(u64 n) {
  if (n < 2) return false;
  #pragma unroll
  for (int i = 0; i < 12; ++i) {
    if (n == MR_BASES[i]) return true;
    if (n % MR_BASES[i] == 0) return false;
  }
  const Mont M = mont_init(n);
  u64 d = n - 1;
  const int s = __ffsll((long long)d) - 1;
  d >>= s;
  for (int i = 0; i < 12; ++i)
    if (!sprp_mont(to_mont(MR_BASES[i], M), d, s, M)) return false;
  return true;
}

// Base-2 SPRP (sieve/rung_scan3.cpp:680-689) on an odd n > 2. The base is 2 = one + one in
// Montgomery form, so r2 (64 doublings) is not needed; below 2^62 the round runs in the lazy
// arithmetic.
__device__ inline bool sprp2_64(u64 n) {
  if (n < 2) return false;
  if (!(n & 1)) return n == 2;
  Mont M;
  M.n = n;
  M.ninv = 0 - inv_pow2(n);
  M.one = (0 - n) % n;
  M.r2 = 0;
  u64 d = n - 1;
  const int s = __ffsll((long long)d) - 1;
  d >>= s;
  return n < LazyArith::NMAX ? sprp2_ar<LazyArith>(d, s, M) : sprp2_mont(d, s, M);
}

// ---------------------------------------------------------------- gcd, isqrt
__device__ __forceinline__ u64 gcd64(u64 a, u64 b) {           // binary gcd
  if (!a) return b;
  if (!b) return a;
  const int sh = __ffsll((long long)(a | b)) - 1;
  a >>= __ffsll((long long)a) - 1;
  do {
    b >>= __ffsll((long long)b) - 1;
    if (a > b) { const u64 t = a; a = b; b = t; }
    b -= a;
  } while (b);
  return a << sh;
}

// floor(sqrt(n)) for every u64: a double estimate corrected by bounded steps. The probe
// (s+1)^2 is clamped below 2^32 so it cannot wrap (the clamp of sieve/rung_scan3.cpp:
// 288-294).
__device__ __forceinline__ u64 isqrt64(u64 n) {
  u64 s = (u64)sqrt((double)n);
  if (s > 0xFFFFFFFFull) s = 0xFFFFFFFFull;
  for (int i = 0; i < 8 && s > 0 && s * s > n; ++i) --s;
  for (int i = 0; i < 8 && s < 0xFFFFFFFFull && (s + 1) * (s + 1) <= n; ++i) ++s;
  return s;
}

// ---------------------------------------------------------------- Brent's rho
// The structure of sieve/rung_scan3.cpp:333-369 in Montgomery form: y -> y^2 + c, products
// of |x - y| batched 128 at a time between gcds, a backtrack when the batch overshoots, and
// the next c when the cycle closes without a split. The step budget is shared across c;
// exhausting it sets ST_RHO_BUDGET and returns 0.
__device__ inline u64 rho_split(u64 n, u64 &budget, u32 *status) {
  if (!(n & 1)) return 2;
  const Mont M = mont_init(n);
  for (u64 c = 1; c < 4096; ++c) {
    const u64 cm = to_mont(c, M);
    u64 y = to_mont(2, M), g = 1, r = 1, q = M.one, x = 0, ys = 0;
    const u64 m = 128;
    while (g == 1) {
      x = y;
      for (u64 i = 0; i < r; ++i) y = addmod(mmul(y, y, M), cm, n);
      for (u64 k = 0; k < r && g == 1; k += m) {
        ys = y;
        const u64 lim = m < r - k ? m : r - k;
        if (budget < lim) { atomicOr(status, ST_RHO_BUDGET); return 0; }
        budget -= lim;
        for (u64 i = 0; i < lim; ++i) {
          y = addmod(mmul(y, y, M), cm, n);
          if (y == x) { g = n; break; }
          q = mmul(q, x > y ? x - y : y - x, M);
        }
        if (g == n) break;
        g = gcd64(q, n);
      }
      r <<= 1;
      if (r > (1ull << 26)) break;
    }
    if (g == n || g == 1) {
      g = 1;
      for (u64 guard = 0; g == 1 && guard <= (1ull << 27); ++guard) {
        ys = addmod(mmul(ys, ys, M), cm, n);
        const u64 diff = x > ys ? x - ys : ys - x;
        g = gcd64(diff ? diff : n, n);
        if (ys == x) break;
      }
    }
    if (g != 1 && g != n) return g;
    if (budget == 0) break;
  }
  atomicOr(status, ST_RHO_BUDGET);
  return 0;
}

// Factor a cofactor n > 2^32 that has no prime factor below 2^16. Such an n has at most
// three prime factors (65537^4 > 2^64), so a stack of four pending composites suffices.
// Returns false if a bound was hit.
__device__ inline bool factor_hard(u64 n, Fac &f, u32 *status) {
  u64 stack[6];
  int sp = 0;
  stack[sp++] = n;
  u64 budget = RHO_BUDGET;
  int guard = 0;
  while (sp > 0) {
    if (++guard > 64) { atomicOr(status, ST_STACK_OVERFLOW); return false; }
    const u64 v = stack[--sp];
    if (v == 1) continue;
    if (v <= 0xFFFFFFFFull || is_prime64(v)) { fac_add(f, v, 1, status); continue; }
    const u64 s = isqrt64(v);
    if (s * s == v) { fac_add(f, s, 2, status); continue; }   // s < 2^32, no factor < 2^16: prime
    const u64 d = rho_split(v, budget, status);
    if (d == 0) return false;
    if (sp + 2 > 6) { atomicOr(status, ST_STACK_OVERFLOW); return false; }
    stack[sp++] = d;
    stack[sp++] = v / d;
  }
  return true;
}

// The complete factorization of n >= 1 (factorA_fast, sieve/rung_scan3.cpp:410-431):
// powers of 2, trial division by the odd primes below 2^16 while d^2 <= n, then the
// cofactor (prime when <= 2^32, else factor_hard). Prime order is left as found.
__device__ inline bool factor64(u64 n, Fac &f, const u32 *__restrict__ tdp,
                         const TdEntry *__restrict__ tde, u32 *status) {
  f.k = 0;
  if (n == 0) return true;
  if (!(n & 1)) {
    const int e = __ffsll((long long)n) - 1;
    n >>= e;
    fac_add(f, 2, e, status);
  }
  for (int i = 0; i < NTD; ++i) {
    const u64 d = tdp[i];
    if (d * d > n) break;
    const TdEntry t = tde[i];
    u64 x = n * t.inv;
    if (x <= t.lim) {
      int e = 0;
      do { n = x; ++e; x = n * t.inv; } while (x <= t.lim);
      fac_add(f, d, e, status);
    }
  }
  if (n > 1) {
    if (n <= 0xFFFFFFFFull) fac_add(f, n, 1, status);
    else return factor_hard(n, f, status);
  }
  return true;
}

// ---------------------------------------------------------------- 128-bit helpers
struct U128 { u64 lo, hi; };
__device__ __forceinline__ bool lt128(U128 a, U128 b) { return a.hi != b.hi ? a.hi < b.hi : a.lo < b.lo; }
__device__ __forceinline__ U128 mul128_64(U128 a, u64 b, bool &over) {   // a*b, flags >= 2^128
  const u64 lo = a.lo * b;
  const u64 c = __umul64hi(a.lo, b);
  const u64 hl = a.hi * b;
  const u64 hh = __umul64hi(a.hi, b);
  const u64 hi = hl + c;
  over = hh != 0 || hi < hl;
  return U128{lo, hi};
}
// a*b <= q for a < 2^128, b < 2^64, q < 2^128: the exact form of `a <= q / b`.
__device__ __forceinline__ bool mul_le(U128 a, u64 b, U128 q) {
  bool over;
  const U128 p = mul128_64(a, b, over);
  return !over && !lt128(q, p);
}

// ---------------------------------------------------------------- stage D
// Smallest divisor u <= q of q^2 with u == target (mod r), q = p*A, or 0 if none
// (min_div_res, sieve/rung_scan3.cpp:544-565). cur[s] is the least divisor built so far in
// residue class s; absorbing a prime power keeps per-residue minima, and a partial product
// above q is never extended (v > q/pr is tested exactly as v*pr > q).
__device__ inline U128 min_div_res(u64 p, const Fac &fA, U128 q, u32 r, u32 target) {
  U128 cur[RCAP + 1], nxt[RCAP + 1];
  const U128 INF{~0ull, ~0ull};
  for (u32 s = 0; s < r; ++s) cur[s] = INF;
  cur[1 % r] = U128{1, 0};
  for (int t = -1; t < fA.k; ++t) {
    const u64 pr = t < 0 ? p : fA.pr[t];
    const int e = t < 0 ? 2 : 2 * fA.ex[t];
    for (u32 s = 0; s < r; ++s) nxt[s] = INF;
    const u32 prm = (u32)(pr % r);
    for (u32 s = 0; s < r; ++s) {
      if (cur[s].lo == ~0ull && cur[s].hi == ~0ull) continue;
      U128 v = cur[s];
      u32 rr = s;
      for (int j = 0;; ++j) {
        if (lt128(v, nxt[rr])) nxt[rr] = v;
        if (j == e || !mul_le(v, pr, q)) break;
        bool over;
        v = mul128_64(v, pr, over);
        rr = (rr * prm) % r;
      }
    }
    for (u32 s = 0; s < r; ++s) cur[s] = nxt[s];
  }
  const U128 u = cur[target];
  return (u.lo == ~0ull && u.hi == ~0ull) ? U128{0, 0} : u;
}

// solve_rung3 (sieve/rung_scan3.cpp:578-603): the smallest rung r == -p (mod 4), r <= 255,
// skipping gcd(q mod r, r) > 1, at which the DP finds a witness. Returns false when no
// rung certifies p (or when a bound was hit: the status word says which).
__device__ inline bool solve_rung(u64 p, u64 &A_out, u32 &r_out, U128 &u_out, const u32 *tdp,
                           const TdEntry *tde, u32 *status) {
  const u32 pm4 = (u32)(p & 3);
  const u32 r0 = (4 - pm4) % 4 ? (4 - pm4) % 4 : 4;
  for (u32 r = r0; r <= RCAP; r += 4) {
    // A = (p + r)/4 without overflow: p + r may exceed 2^64 only for p within 255 of it.
    const u64 A = (p >> 2) + ((u64)(p & 3) + r) / 4;
    if (!A) continue;
    const u32 qm = (u32)(((p % r) * (A % r)) % r);
    if (r > 1 && gcd64(qm, r) != 1) continue;
    const u32 target = qm ? r - qm : 0;
    Fac f;
    if (!factor64(A, f, tdp, tde, status)) return false;
    const U128 q{p * A, __umul64hi(p, A)};
    const U128 u = min_div_res(p, f, q, r, target);
    if (u.lo == 0 && u.hi == 0) continue;
    A_out = A; r_out = r; u_out = u;
    return true;
  }
  return false;
}

// ---------------------------------------------------------------- stage E
// solve_direct3 (sieve/rung_scan3.cpp:607-647): for a, d in 1..8 in that order, the least
// divisor m of n = p + 4a^2 d with m == -1 (mod 4ad), c = (m+1)/(4ad), k = n/m, ck > a.
// The reference sorts the divisors and takes the first hit; the least hit is the same.
__device__ inline bool solve_direct(u64 p, u64 &a_out, u64 &c_out, u64 &d_out, u64 &k_out,
                             const u32 *tdp, const TdEntry *tde, u32 *status) {
  for (u64 a = 1; a <= 8; ++a)
    for (u64 d = 1; d <= 8; ++d) {
      const u64 add = 4 * a * a * d;
      if (p > DIRECT_NMAX - add) continue;          // n > DIRECT_NMAX
      const u64 n = p + add, q4 = 4 * a * d;
      Fac f;
      if (!factor64(n, f, tdp, tde, status)) return false;
      // Walk every divisor with a mixed-radix counter over the exponents.
      int e[MAXF];
      u64 pw[MAXF];
      for (int i = 0; i < f.k; ++i) { e[i] = 0; pw[i] = 1; }
      u64 best = 0;
      u64 m = 1;
      for (u64 guard = 0; guard < 2000000; ++guard) {
        if (m % q4 == q4 - 1) {
          const u64 c = (m + 1) / q4, k = n / m;
          if (c && k && (__umul64hi(c, k) != 0 || c * k > a) && (best == 0 || m < best)) best = m;
        }
        int i = 0;
        for (; i < f.k; ++i) {
          if (e[i] < f.ex[i]) { ++e[i]; pw[i] *= f.pr[i]; m *= f.pr[i]; break; }
          m /= pw[i]; pw[i] = 1; e[i] = 0;
        }
        if (i == f.k) break;
      }
      if (best) {
        a_out = a; c_out = (best + 1) / q4; d_out = d; k_out = n / best;
        return true;
      }
    }
  return false;
}

}  // namespace es
