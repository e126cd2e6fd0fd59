// Host build of the device ECM (erdos-strauss_gb300/csrc/es_ecm.cuh) for the CPU tests: the
// same source compiled by g++ with the four device intrinsics it uses defined on 128-bit host
// integers. Checks the lazy Montgomery multiply against exact residues, the lazy
// strong-probable-prime round against the exact one and the base-2 round by square-and-double
// against the binary one, then runs 32 curves (sigma 6..37, one
// warp's first round) on seeded 62-bit semiprimes with prime factors of 18-31 bits in the lazy
// arithmetic the engine uses and prints the fraction of curves that split each size; the exact
// arithmetic must find the same divisors curve for curve, and every divisor returned must
// divide n properly.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <random>
#define __device__
#define __forceinline__ inline
#define __constant__
static inline unsigned long long __umul64hi(unsigned long long a, unsigned long long b) {
  return (unsigned long long)(((unsigned __int128)a * b) >> 64);
}
static inline int __ffsll(long long x) { return x ? __builtin_ctzll((unsigned long long)x) + 1 : 0; }
static inline int __clzll(long long x) { return x ? __builtin_clzll((unsigned long long)x) : 64; }
static inline unsigned atomicOr(unsigned *p, unsigned v) { const unsigned o = *p; *p |= v; return o; }
#include "es_ecm.cuh"
using namespace es;

static const u64 BASES[12] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37};
static bool is_prime(u64 n) {
  if (n < 2) return false;
  for (u64 b : BASES) if (n % b == 0) return n == b;
  u64 d = n - 1;
  int s = 0;
  while (!(d & 1)) { d >>= 1; ++s; }
  for (u64 a : BASES) {
    unsigned __int128 x = 1, b = a;
    for (u64 e = d; e; e >>= 1) { if (e & 1) x = x * b % n; b = b * b % n; }
    if (x == 1 || x == n - 1) continue;
    bool ok = false;
    for (int i = 1; i < s && !ok; ++i) { x = x * x % n; ok = x == n - 1; }
    if (!ok) return false;
  }
  return true;
}
static u64 random_prime(int bits, std::mt19937_64 &g) {
  for (;;) {
    const u64 p = (g() & ((1ull << bits) - 1)) | (1ull << (bits - 1)) | 1;
    if (is_prime(p)) return p;
  }
}

int main(int argc, char **argv) {
  const int trials = argc > 1 ? atoi(argv[1]) : 40;
  std::mt19937_64 g(0xE52026);
  for (int t = 0; t < 200000; ++t) {
    const u64 n = (g() >> 2) | 1;
    if (n < 3) continue;
    const Mont M = mont_init(n);
    const u64 a = g() % (2 * n), b = g() % (2 * n);
    const u64 r = LazyArith::mul(a, b, M);
    if (r >= 2 * n || r % n != mmul(a % n, b % n, M)) {
      printf("FAIL lazy multiply a=%llu b=%llu n=%llu\n", a, b, n);
      return 1;
    }
  }
  for (int t = 0; t < 20000; ++t) {                     // the lazy strong-probable-prime round
    const u64 n = (t & 1) ? random_prime(40 + t % 22, g) : ((g() >> 2) | 1);
    if (n < 41) continue;
    const Mont M = mont_init(n);
    u64 d = n - 1;
    const int sh = __ffsll((long long)d) - 1;
    d >>= sh;
    for (u64 b : BASES) {
      const u64 bm = to_mont(b, M);
      if (sprp_ar<LazyArith>(bm, d, sh, M) != sprp_mont(bm, d, sh, M)) {
        printf("FAIL lazy sprp n=%llu base=%llu\n", n, b);
        return 1;
      }
    }
    // the base-2 round by square-and-double, in both arithmetics, against the binary one
    const bool two = sprp_mont(to_mont(2, M), d, sh, M);
    if (sprp2_ar<LazyArith>(d, sh, M) != two || sprp2_mont(d, sh, M) != two) {
      printf("FAIL base-2 round n=%llu\n", n);
      return 1;
    }
  }
  for (int bits = 18; bits <= 31; ++bits) {
    int split = 0, curves = 0, warps = 0;
    for (int t = 0; t < trials; ++t) {
      const u64 p = random_prime(bits, g), q = random_prime(62 - bits, g), n = p * q;
      const Mont M = mont_init(n);
      bool any = false;
      for (u64 lane = 0; lane < 32; ++lane, ++curves) {
        const u64 d = ecm_curve<LazyArith>(6 + lane, M, [] { return false; });
        if (d != ecm_curve<ExactArith>(6 + lane, M, [] { return false; })) {
          printf("FAIL lazy and exact curves differ n=%llu sigma=%llu\n", n, 6 + lane);
          return 1;
        }
        if (!d) continue;
        if (d <= 1 || d >= n || n % d) {
          printf("FAIL divisor %llu of %llu\n", d, n);
          return 1;
        }
        ++split;
        any = true;
      }
      warps += any;
    }
    printf("bits %d curves %.3f warps %.3f\n", bits, (double)split / curves, (double)warps / trials);
  }
  return 0;
}
