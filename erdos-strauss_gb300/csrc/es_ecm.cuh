// es_ecm.cuh -- Lenstra's elliptic-curve method, one curve per lane, for the hard cofactors of
// stage D.
//
// A cofactor that reaches this point is an odd composite below 2^64 with every prime factor
// above 2^16, not a square, and Brent's rho has already walked it for a few hundred steps per
// lane without a collision: in practice a product of two primes of 24-31 bits. For those the
// expected rho walk grows like the square root of the smaller prime (about 20 K steps, 40 K
// Montgomery multiplies, for two 31-bit primes, over 32 walks in lockstep), while one ECM
// curve with B1 = 40 and B2 = 1200 costs about 1.25 K multiplies and splits a 31-bit prime
// with a probability of about 0.015, a 24-bit one about 0.12: a round of 32 curves in a warp
// splits a 31-bit pair about a third of the time, a 24-bit one almost always, and block-mates
// add rounds of their own. On GB300 a single warp's multiply chain is latency-bound (about
// 0.1 us per 64-bit Montgomery multiply), so short rounds that fail now and then beat long sure
// ones: measured on the 4096-window batch, stage D took 0.45 ms with B1 = 40, 0.47 with 50,
// 0.48 with 60, 0.55 with 85 and 0.49 with 30, whose 2^34 window at 1.8e19 then needed 2.1 ms
// (too many failed rounds); with B1 = 40 and the curves inversion-free, B2 = 1200 against
// 2000 and 3000: 0.34 against 0.36 and 0.41 ms here, 0.56-0.58 against 0.59-0.60 and
// 0.62-0.63 ms on the batch at 1e19, 0.32 against 0.35-0.36 and 0.39-0.40 ms on that 2^34
// window (B2 = 800 measured within noise of 1200); B1 re-checked with B2 = 1200: 30 lost at 1e19
// (0.69-0.76 against 0.54-0.56 ms), 50 gained there what it lost on the 4096-window batch
// (0.53-0.54 against 0.54-0.56, and 0.35-0.37 against 0.34-0.35 ms). The reference factors
// with rho alone (sieve/rung_scan3.cpp:333-369); the factorization of a number is unique, so
// the method that finds a divisor cannot change any certificate.
//
// Curves: Montgomery form B y^2 = x^3 + A x^2 + x with Suyama's parametrization (sigma ->
// u = sigma^2 - 5, v = 4 sigma, starting point (u^3 : v^3), (A + 2)/4 = (v - u)^3 (3u + v) /
// (16 u^3 v)), whose group orders are divisible by 12. x-only arithmetic in projective
// coordinates (Montgomery 1987): doubling and differential addition, with (A + 2)/4 kept as
// a fraction, so that a curve takes no modular inverse at all (an inverse -- a data-dependent
// binary extended Euclid -- cost about as much as a quarter of a curve here). Stage 1
// multiplies by k = product of the largest powers of the primes p <= B1 that are <= B1, with
// the ladder; stage 2 is the standard baby-step giant-step continuation with D = 60: for every
// prime q in (B1, B2], written q = mD +- j with j coprime to 60, the product accumulates
// X([mD]Q) Z([j]Q) - X([j]Q) Z([mD]Q), and one gcd with n at the end finds the factor.
//
// Everything here is modular arithmetic modulo n in Montgomery form (the lazy representation of
// es_arith.cuh for n < 2^62); a divisor comes only out of gcd(., n), so it always divides n.
// All lanes of a warp run the same sequence of curve operations (k and the stage-2 table are
// the same for every lane), so the warp stays converged apart from the final gcd. Every loop
// is bounded.
#pragma once
#include "es_arith.cuh"

namespace es {

constexpr u32 ECM_B1 = 40;
constexpr u32 ECM_B2 = 1200;
constexpr u32 ECM_D = 60;
// k = lcm(1..40) = prod over primes p <= 40 of p^floor(log_p 40): 53 bits, little-endian words.
constexpr int ECM_K_BITS = 53;
__constant__ const u32 ECM_K[2] = {0x2b8eb920u, 0x0012fb5eu};
// The baby steps: j < D/2 odd and coprime to D.
constexpr int ECM_NJ = 8;
__constant__ const u32 ECM_J[ECM_NJ] = {1, 7, 11, 13, 17, 19, 23, 29};
// Giant steps m = 1 .. ECM_M1 (ECM_M1 = floor((B2 + D/2) / D)); bit i of ECM_PAIRS[m - 1] is set
// when m*D + J[i] or m*D - J[i] is a prime in (B1, B2]. Every prime of (B1, B2] is covered.
constexpr int ECM_M1 = 20;
__constant__ const unsigned char ECM_PAIRS[ECM_M1] = {
    0xff, 0xfe, 0xff, 0xdf, 0xfe, 0xef, 0xed, 0xff, 0xf3, 0xfb, 0xfb, 0xef, 0xf6, 0xfd, 0xfe, 0x7e,
    0xef, 0xfe, 0x5c, 0xaa};
// One round (about 1.25 K Montgomery multiplies: 12 per bit of k, 3 per stage-2 pair, 6 per
// giant step and baby step) in rho steps of two multiplies.
constexpr u64 ECM_ROUND_STEPS = 625;

struct XZ { u64 x, z; };

// The curve operations over an arithmetic policy Ar (ExactArith or LazyArith, es_arith.cuh).
// [2]P with (A + 2)/4 = a24n / a24d: X = t1 t2, Z = t3 (t2 + a24 t3) (t1 = (x + z)^2,
// t2 = (x - z)^2, t3 = t1 - t2) with both coordinates multiplied by a24d, so that no inverse
// of a24d is needed.
template <class Ar>
__device__ __forceinline__ XZ ecm_dbl(XZ P, u64 a24n, u64 a24d, const Mont &M) {
  const u64 s = Ar::add(P.x, P.z, M), d = Ar::sub(P.x, P.z, M);
  const u64 t1 = Ar::mul(s, s, M), t2 = Ar::mul(d, d, M);
  const u64 t3 = Ar::sub(t1, t2, M);                           // 4xz
  const u64 c = Ar::mul(a24d, t2, M);
  return XZ{Ar::mul(t1, c, M), Ar::mul(t3, Ar::add(c, Ar::mul(a24n, t3, M), M), M)};
}
// P + Q given D = P - Q.
template <class Ar>
__device__ __forceinline__ XZ ecm_add(XZ P, XZ Q, XZ D, const Mont &M) {
  const u64 u = Ar::mul(Ar::sub(P.x, P.z, M), Ar::add(Q.x, Q.z, M), M);
  const u64 v = Ar::mul(Ar::add(P.x, P.z, M), Ar::sub(Q.x, Q.z, M), M);
  const u64 s = Ar::add(u, v, M), d = Ar::sub(u, v, M);
  return XZ{Ar::mul(D.z, Ar::mul(s, s, M), M), Ar::mul(D.x, Ar::mul(d, d, M), M)};
}


// Divisor d of n from gcd(g, n), if it is a proper one; else 0.
__device__ __forceinline__ u64 proper_gcd(u64 g, u64 n) {
  const u64 d = gcd64(g, n);
  return (d > 1 && d < n) ? d : 0;
}

// Giant steps between polls in stage 2, ladder bits between polls in stage 1 (a poll that
// answers "stop" ends the curve at once: another walk or curve has split the cofactor).
constexpr int ECM_STAGE2_POLL = 24;
#ifndef ES_ECM_STAGE1_POLL
#define ES_ECM_STAGE1_POLL 13
#endif
constexpr int ECM_STAGE1_POLL = ES_ECM_STAGE1_POLL;

// One ECM curve (Suyama's sigma, 6 <= sigma < n) on the odd composite n > 2^32, in the
// arithmetic Ar (LazyArith needs n < 2^62). Returns a proper divisor of n, or 0 when this curve
// found none. poll() is called at the same points in every lane (every ECM_STAGE1_POLL ladder
// bits, after stage 1 and every ECM_STAGE2_POLL giant steps); when it returns true the curve
// stops early and returns 0. dead
// lanes keep computing (their result is dropped) so that the lanes of a warp stay in step.
template <class Ar, class Poll>
__device__ inline u64 ecm_curve(u64 sigma, const Mont &M, Poll poll) {
  const u64 n = M.n;
  // --- the curve and its starting point, kept projective: (A + 2)/4 = num / den and the point
  // (u^3 : v^3), so that no inverse is taken (a curve that is degenerate modulo a factor of n
  // only makes the final gcd find that factor, or fail)
  const u64 sm = to_mont(sigma, M);
  const u64 five = to_mont(5, M);
  const u64 u = Ar::sub(Ar::mul(sm, sm, M), five, M);
  const u64 v2 = Ar::add(sm, sm, M), v = Ar::add(v2, v2, M);
  const u64 u3 = Ar::mul(Ar::mul(u, u, M), u, M), v3 = Ar::mul(Ar::mul(v, v, M), v, M);
  const u64 vu = Ar::sub(v, u, M);
  const u64 num = Ar::mul(Ar::mul(Ar::mul(vu, vu, M), vu, M), Ar::add(Ar::add(Ar::add(u, u, M), u, M), v, M), M);
  u64 den = Ar::mul(u3, v, M);
  #pragma unroll
  for (int i = 0; i < 4; ++i) den = Ar::add(den, den, M);      // 16 u^3 v
  const XZ P0{u3, v3};
  // --- stage 1: Q = [k]P0, ladder from the top bit of k (the difference of the ladder's two
  // points is always P0)
  XZ R0 = P0, R1 = ecm_dbl<Ar>(R0, num, den, M);
  for (int i = ECM_K_BITS - 2; i >= 0; --i) {
    const bool b = (ECM_K[i >> 5] >> (i & 31)) & 1u;
    if (b) { const XZ t = R0; R0 = R1; R1 = t; }
    R1 = ecm_add<Ar>(R0, R1, P0, M);
    R0 = ecm_dbl<Ar>(R0, num, den, M);
    if (b) { const XZ t = R0; R0 = R1; R1 = t; }
    if (i && i % ECM_STAGE1_POLL == 0 && poll()) return 0;
  }
  const XZ Q = R0;
  if (poll()) return 0;
  // --- stage 2: baby steps [j]Q for odd j <= 31 (kept for j in ECM_J), giant step [60]Q
  const XZ Q2 = ecm_dbl<Ar>(Q, num, den, M);
  u64 bx[ECM_NJ], bz[ECM_NJ];
  bx[0] = Q.x; bz[0] = Q.z;
  XZ prev = Q, cur = ecm_add<Ar>(Q2, Q, Q, M);                 // [1], [3]
  int nb = 1;
  XZ P29{0, 0};
  #pragma unroll
  for (int j = 3; j <= 29; j += 2) {                           // cur = [j]
    if (j % 3 != 0 && j % 5 != 0) { bx[nb] = cur.x; bz[nb] = cur.z; ++nb; }
    if (j == 29) P29 = cur;
    const XZ nxt = ecm_add<Ar>(cur, Q2, prev, M);              // [j + 2]
    prev = cur; cur = nxt;
  }
  const XZ G1 = ecm_add<Ar>(cur, P29, Q2, M);                  // [31] + [29] = [60]
  // giant steps G_m = [60 m]Q, m = 1 .. ECM_M1; for each prime mD +- j of (B1, B2] the
  // product gathers X(G_m) Z(j) - X(j) Z(G_m), zero modulo p when [mD]Q = +-[j]Q there. It
  // starts from Z(Q): a factor stage 1 already found (Q at infinity modulo p) stays in it.
  u64 acc = Q.z;
  XZ Gp = G1, G = G1;
  for (int m = 1; m <= ECM_M1; ++m) {
    if (m == 2) G = ecm_dbl<Ar>(G1, num, den, M);
    else if (m > 2) { const XZ t = ecm_add<Ar>(G, G1, Gp, M); Gp = G; G = t; }
    const u32 mask = ECM_PAIRS[m - 1];
    #pragma unroll
    for (int i = 0; i < ECM_NJ; ++i)
      if (mask & (1u << i)) acc = Ar::mul(acc, Ar::sub(Ar::mul(G.x, bz[i], M), Ar::mul(bx[i], G.z, M), M), M);
    if (m % ECM_STAGE2_POLL == 0 && poll()) return 0;
  }
  return proper_gcd(Ar::norm(acc, M), n);
}
}  // namespace es
