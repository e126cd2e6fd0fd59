/* es_oracle.c -- CPU restatement of the Erdos-Straus verification sieve's per-window
 * funnel, written from the reference algorithm (sieve/rung_scan3.cpp and the frozen
 * arithmetic it borrows from census/rung_scan.cpp).
 *
 * TEST INFRASTRUCTURE ONLY. This file is the checker: the tests, the smoke check and
 * bench.py's CPU-baseline leg are its only callers. The GB300 product never links it.
 *
 * Parity is pinned two ways (tests/test_oracle.py): against the reference's golden
 * vectors (data/rederive/decades/d*.txt, data/rederive/windows/w19_certificates.txt,
 * the self-test constants of sieve/rung_scan3.cpp:845-893, the class tables in
 * tables/), and against the reference scanners compiled from source by
 * oracle/Makefile (oracle/_ref/rung_scan3, oracle/_ref/cover_scan) where the
 * reference tree is present.
 *
 * Built two ways: with -DES_ORACLE_MAIN as a rung_scan3-compatible CLI (es_oracle),
 * and without it as libes_oracle.so, whose es_o_* entry points tests call by ctypes.
 */
#define _GNU_SOURCE
#include <inttypes.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef uint64_t u64;
typedef unsigned __int128 u128;

/* Compile-time constants of the path (sieve/rung_scan3.cpp:23, :42-43;
 * census/rung_scan.cpp:64, :147, :175). */
#define UCERT_RMAX 63u
#define UCERT_UMAX 64u
#define RCAP 255u
#define MAXF 16
#define TD_BOUND 65536ull
static const u64 DIRECT_NMAX = 18446744065119617025ull; /* (2^32-1)^2 */
static __attribute__((unused)) const u64 DIRECT_PMAX = 18446744065119617025ull - 2048 - 1;

/* Class-table pins per modulus (sieve/rung_scan3.cpp:57-67). */
typedef struct { u64 M, fnv64; const char *sha256; } pin_t;
static const pin_t PINS[] = {
  {120120, 0xdbc4ab9b16d73f76ull, "154e82672d9da66cff97d48079047b8b0b0a31fa049ac62fb05b5c82ad540f60"},
  {2042040, 0xb9b5d1408da3428eull, "a77b2187201ff96ff3ecf822150f4152d841941deeb0cf616238bcbb0a648bbc"},
};
static __attribute__((unused)) const pin_t *pin_for(u64 M) {
  for (size_t i = 0; i < sizeof PINS / sizeof PINS[0]; ++i) if (PINS[i].M == M) return &PINS[i];
  return NULL;
}

static void *xmalloc(size_t n) {
  void *p = malloc(n ? n : 1);
  if (!p) { fprintf(stderr, "es_oracle: out of memory\n"); exit(1); }
  return p;
}
static void *xrealloc(void *q, size_t n) {
  void *p = realloc(q, n ? n : 1);
  if (!p) { fprintf(stderr, "es_oracle: out of memory\n"); exit(1); }
  return p;
}

/* ------------------------------------------------------------ frozen arithmetic
 * census/rung_scan.cpp:68-92: mulmod through a 128-bit product, square-and-multiply,
 * and the 12-base deterministic Miller-Rabin with its trial-division prologue. */
static u64 o_gcd(u64 a, u64 b) { while (b) { u64 t = a % b; a = b; b = t; } return a; }
static inline u64 o_mulmod(u64 a, u64 b, u64 m) { return (u64)((u128)a * b % m); }
static u64 o_powmod(u64 b, u64 e, u64 m) {
  u64 r = 1;
  b %= m;
  while (e) { if (e & 1) r = o_mulmod(r, b, m); b = o_mulmod(b, b, m); e >>= 1; }
  return r;
}
static const u64 MR_BASES[12] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37};

int es_o_is_prime(u64 n) {
  if (n < 2) return 0;
  for (int i = 0; i < 12; ++i) {
    if (n == MR_BASES[i]) return 1;
    if (n % MR_BASES[i] == 0) return 0;
  }
  u64 d = n - 1; int s = 0;
  while (!(d & 1)) { d >>= 1; ++s; }
  for (int i = 0; i < 12; ++i) {
    u64 x = o_powmod(MR_BASES[i], d, n);
    if (x == 1 || x == n - 1) continue;
    int composite = 1;
    for (int j = 1; j < s; ++j) { x = o_mulmod(x, x, n); if (x == n - 1) { composite = 0; break; } }
    if (composite) return 0;
  }
  return 1;
}

/* Base-2 strong probable prime (sieve/rung_scan3.cpp:680-689). */
int es_o_sprp2(u64 n) {
  if (n < 2) return 0;
  if (!(n & 1)) return n == 2;
  u64 d = n - 1; int s = 0;
  while (!(d & 1)) { d >>= 1; ++s; }
  u64 x = o_powmod(2, d, n);
  if (x == 1 || x == n - 1) return 1;
  for (int i = 1; i < s; ++i) { x = o_mulmod(x, x, n); if (x == n - 1) return 1; }
  return 0;
}

/* The scan's primality verdict (sprp2 && is_prime, sieve/rung_scan3.cpp:686-689) over an
 * array, threads over values: out[i] = 1 for a prime. */
void es_o_is_prime_batch(const u64 *n, size_t count, uint8_t *out) {
  #pragma omp parallel for schedule(static)
  for (size_t i = 0; i < count; ++i) out[i] = (uint8_t)(es_o_sprp2(n[i]) && es_o_is_prime(n[i]));
}

/* ------------------------------------------------------------ factorization
 * The factorization of n is unique, so any exact method gives the certificate the
 * reference gives: min_div_res takes a minimum over divisors and divisors3 sorts
 * (sieve/rung_scan3.cpp:247-254). This one follows the frozen factorA
 * (census/rung_scan.cpp:194-204): trial division by the primes <= TD_BOUND while
 * sp^2 <= n, a cofactor <= TD_BOUND^2 is prime, else factor_hard (:184-192) with
 * is_prime, the perfect-square test and Brent's rho (:94-128). */
typedef struct { u64 pr[MAXF]; uint8_t ex[MAXF]; int k; } o_fac;

static void fac_add(o_fac *f, u64 p, int e) {
  for (int i = 0; i < f->k; ++i) if (f->pr[i] == p) { f->ex[i] = (uint8_t)(f->ex[i] + e); return; }
  if (f->k >= MAXF) { fprintf(stderr, "FATAL: more than %d distinct prime factors\n", MAXF); abort(); }
  f->pr[f->k] = p; f->ex[f->k] = (uint8_t)e; ++f->k;
}

static u64 *g_tdp; static size_t g_ntdp;   /* primes <= TD_BOUND, ascending, 2 first */
static void td_init(void) {
  if (g_tdp) return;
  uint8_t *c = calloc(TD_BOUND + 1, 1);
  u64 *p = xmalloc(sizeof(u64) * 7000);
  size_t n = 0;
  for (u64 i = 2; i <= TD_BOUND; ++i) {
    if (c[i]) continue;
    p[n++] = i;
    for (u64 j = i * i; j <= TD_BOUND; j += i) c[j] = 1;
  }
  free(c);
  g_ntdp = n;
  g_tdp = p;
}

/* isqrt_u64 (census/rung_scan.cpp:177-182), with the probe clamped so it is safe for
 * every u64 (the same clamp as sieve/rung_scan3.cpp:288-294). */
static u64 o_isqrt(u64 n) {
  u64 s = (u64)sqrtl((long double)n);
  if (s > 0xFFFFFFFFull) s = 0xFFFFFFFFull;
  while (s > 0 && s * s > n) --s;
  while (s < 0xFFFFFFFFull && (s + 1) * (s + 1) <= n) ++s;
  return s;
}

static u64 o_pollard_brent(u64 n) {                     /* census/rung_scan.cpp:94-128 */
  if ((n & 1) == 0) return 2;
  for (u64 c = 1;; ++c) {
    u64 y = 2, m = 128, g = 1, r = 1, qacc = 1, x = 0, ys = 0;
#define F(v) ((o_mulmod((v), (v), n) + c) % n)
    while (g == 1) {
      x = y;
      for (u64 i = 0; i < r; ++i) y = F(y);
      for (u64 k = 0; k < r && g == 1; k += m) {
        ys = y;
        u64 lim = m < r - k ? m : r - k;
        for (u64 i = 0; i < lim; ++i) {
          y = F(y);
          if (y == x) { g = n; break; }
          u64 diff = x > y ? x - y : y - x;
          qacc = o_mulmod(qacc, diff, n);
        }
        if (g == n) break;
        g = o_gcd(qacc, n);
      }
      r <<= 1;
      if (r > (1ull << 26)) break;
    }
    if (g == n || g == 1) {
      g = 1;
      while (g == 1) {
        ys = F(ys);
        u64 diff = x > ys ? x - ys : ys - x;
        g = o_gcd(diff ? diff : n, n);
        if (ys == x) break;
      }
    }
#undef F
    if (g != 1 && g != n) return g;
  }
}

static void o_factor_hard(u64 n, o_fac *f) {           /* census/rung_scan.cpp:184-192 */
  if (n == 1) return;
  if (es_o_is_prime(n)) { fac_add(f, n, 1); return; }
  u64 s = o_isqrt(n);
  if (s * s == n) {
    o_fac g; g.k = 0;
    o_factor_hard(s, &g);
    for (int i = 0; i < g.k; ++i) fac_add(f, g.pr[i], 2 * g.ex[i]);
    return;
  }
  u64 d = o_pollard_brent(n);
  o_factor_hard(d, f);
  o_factor_hard(n / d, f);
}

static void o_factor(u64 n, o_fac *f) {                /* census/rung_scan.cpp:194-204 */
  td_init();
  f->k = 0;
  for (size_t i = 0; i < g_ntdp; ++i) {
    u64 sp = g_tdp[i];
    if (sp * sp > n) break;
    if (n % sp == 0) { int e = 0; while (n % sp == 0) { n /= sp; ++e; } fac_add(f, sp, e); }
  }
  if (n > 1) {
    if (n <= TD_BOUND * TD_BOUND || es_o_is_prime(n)) fac_add(f, n, 1);
    else o_factor_hard(n, f);
  }
}

/* ctypes view: primes and exponents in ascending prime order; returns the count. */
int es_o_factor(u64 n, u64 *pr, int *ex) {
  o_fac f; o_factor(n, &f);
  for (int i = 1; i < f.k; ++i)
    for (int j = i; j > 0 && f.pr[j - 1] > f.pr[j]; --j) {
      u64 t = f.pr[j]; f.pr[j] = f.pr[j - 1]; f.pr[j - 1] = t;
      uint8_t e = f.ex[j]; f.ex[j] = f.ex[j - 1]; f.ex[j - 1] = e;
    }
  for (int i = 0; i < f.k; ++i) { pr[i] = f.pr[i]; ex[i] = f.ex[i]; }
  return f.k;
}

/* ------------------------------------------------------------ stage D
 * min_div_res (sieve/rung_scan3.cpp:544-565): the smallest divisor u <= q of q^2 with
 * u == target (mod r), by a per-residue minimum DP over the prime powers p^2 and
 * pr^(2e) of A; the bound check `v > q / pr` keeps every value below q. */
static u128 o_min_div_res(u64 p, const o_fac *fA, u128 q, u64 r, u64 target) {
  const u128 INF = ~(u128)0;
  u128 cur[RCAP + 1], nxt[RCAP + 1];
  for (u64 s = 0; s < r; ++s) cur[s] = INF;
  cur[1 % r] = 1;
  for (int t = -1; t < fA->k; ++t) {
    const u64 pr = t < 0 ? p : fA->pr[t];
    const int e = t < 0 ? 2 : 2 * fA->ex[t];
    for (u64 s = 0; s < r; ++s) nxt[s] = INF;
    const u64 prm = pr % r;
    for (u64 s = 0; s < r; ++s) {
      if (cur[s] == INF) continue;
      u128 v = cur[s]; u64 rr = s;
      for (int j = 0;; ++j) {
        if (v < nxt[rr]) nxt[rr] = v;
        if (j == e || v > q / pr) break;
        v *= pr; rr = (u64)((u128)rr * prm % r);
      }
    }
    memcpy(cur, nxt, sizeof(u128) * r);
  }
  return cur[target] == INF ? 0 : cur[target];
}

static int u128_dec(char *out, u128 v) {                /* app_u128, :567-572 */
  char buf[48]; int n = 0;
  if (!v) buf[n++] = '0';
  while (v) { buf[n++] = (char)('0' + (int)(v % 10)); v /= 10; }
  for (int i = 0; i < n; ++i) out[i] = buf[n - 1 - i];
  out[n] = 0;
  return n;
}

/* solve_rung3 (sieve/rung_scan3.cpp:578-603): the smallest rung r == -p (mod 4),
 * r <= RCAP, skipping gcd(q mod r, r) > 1, whose DP finds a witness. Writes the
 * certificate line (with newline) into out. */
int es_o_solve_rung(u64 p, char *out, size_t cap) {
  const u64 r0 = (4 - p % 4) % 4 ? (4 - p % 4) % 4 : 4;
  for (u64 r = r0; r <= RCAP; r += 4) {
    const u64 A = (p + r) / 4;
    if (!A) continue;
    const u128 q = (u128)p * A;
    const u64 qm = (u64)(q % r);
    if (r > 1 && o_gcd(qm, r) != 1) continue;
    const u64 target = qm ? r - qm : 0;
    o_fac f; o_factor(A, &f);
    const u128 u = o_min_div_res(p, &f, q, r, target);
    if (!u) continue;
    char ud[48]; u128_dec(ud, u);
    snprintf(out, cap, "RUNG %" PRIu64 " %" PRIu64 " %" PRIu64 " %s\n", p, A, r, ud);
    return 1;
  }
  return 0;
}

/* solve_direct3 (sieve/rung_scan3.cpp:607-647): for a, d in 1..8, factor
 * n = p + 4a^2 d and take the smallest divisor m == -1 (mod 4ad) with ck > a,
 * c = (m+1)/(4ad), k = n/m. divisors3 sorts, so the first hit is the minimum. */
static int cmp_u64(const void *a, const void *b) {
  u64 x = *(const u64 *)a, y = *(const u64 *)b;
  return x < y ? -1 : x > y;
}
int es_o_solve_direct(u64 p, char *out, size_t cap) {
  for (u64 a = 1; a <= 8; ++a)
    for (u64 d = 1; d <= 8; ++d) {
      const u128 nn = (u128)p + (u128)4 * a * a * d;
      if (nn > (u128)DIRECT_NMAX) continue;
      const u64 n = (u64)nn, q4 = 4 * a * d;
      o_fac f; o_factor(n, &f);
      size_t nd = 1;
      for (int i = 0; i < f.k; ++i) nd *= (size_t)(f.ex[i] + 1);
      u64 *ds = xmalloc(sizeof(u64) * nd);
      size_t cnt = 1; ds[0] = 1;
      for (int i = 0; i < f.k; ++i) {
        size_t base = cnt; u64 pe = 1;
        for (int e = 1; e <= f.ex[i]; ++e) { pe *= f.pr[i]; for (size_t j = 0; j < base; ++j) ds[cnt++] = ds[j] * pe; }
      }
      qsort(ds, cnt, sizeof(u64), cmp_u64);
      int hit = 0;
      for (size_t i = 0; i < cnt && !hit; ++i) {
        const u64 m = ds[i];
        if (m % q4 != q4 - 1) continue;
        const u64 c = (m + 1) / q4, k = n / m;
        if (!c || !k || (u128)c * k <= a) continue;
        snprintf(out, cap, "SOLVED %" PRIu64 " %" PRIu64 " %" PRIu64 " %" PRIu64 " %" PRIu64 "\n", p, a, c, d, k);
        hit = 1;
      }
      free(ds);
      if (hit) return 1;
    }
  return 0;
}

/* ------------------------------------------------------------ certificate families */
typedef struct { u64 mod, res, pmin; uint32_t a, c, d; u64 seq; } o_cover;
static size_t o_small_primes(u64 P, u64 M, u64 **out);
typedef struct { u64 mod, res; uint32_t r, u; } o_ucert;

static int cover_cmp(const void *x, const void *y) {
  const o_cover *a = x, *b = y;
  if (a->mod != b->mod) return a->mod < b->mod ? -1 : 1;
  if (a->res != b->res) return a->res < b->res ? -1 : 1;
  if (a->pmin != b->pmin) return a->pmin < b->pmin ? -1 : 1;
  return a->seq < b->seq ? -1 : a->seq > b->seq;
}
/* Dedup by (mod,res) keeping the smallest pmin, the earliest generated on a tie --
 * the reference's `pmin < best.pmin` replacement rule (sieve/rung_scan3.cpp:103-105). */
static size_t cover_dedup(o_cover *v, size_t n) {
  qsort(v, n, sizeof *v, cover_cmp);
  size_t k = 0;
  for (size_t i = 0; i < n; ++i)
    if (!k || v[k - 1].mod != v[i].mod || v[k - 1].res != v[i].res) v[k++] = v[i];
  return k;
}
static void cover_push(o_cover **v, size_t *n, size_t *cap, u64 a, u64 c, u64 d) {
  const u128 mm = (u128)4 * a * c * d - 1, bb = (u128)4 * a * a * d;
  if (*n == *cap) { *cap = *cap ? *cap * 2 : 1024; *v = xrealloc(*v, *cap * sizeof **v); }
  o_cover *f = &(*v)[*n];
  f->mod = (u64)mm;
  f->res = (u64)((mm - bb % mm) % mm);
  f->pmin = (u64)(mm * (a / c + 1) - bb);
  f->a = (uint32_t)a; f->c = (uint32_t)c; f->d = (uint32_t)d; f->seq = *n;
  ++*n;
}

/* gen_covers (sieve/rung_scan3.cpp:93-112): every F1 cover with m = 4acd-1 <= mmax. */
size_t es_o_gen_covers(u64 mmax, o_cover **out) {
  o_cover *v = NULL; size_t n = 0, cap = 0;
  const u64 nmax = (mmax + 1) / 4;
  for (u64 a = 1; a <= nmax; ++a)
    for (u64 d = 1; a * d <= nmax; ++d)
      for (u64 c = 1; a * d * c <= nmax; ++c) cover_push(&v, &n, &cap, a, c, d);
  *out = v;
  return cover_dedup(v, n);
}

/* gen_wheel_covers (sieve/rung_scan3.cpp:126-165): covers whose modulus divides M,
 * enumerated from the divisors m == 3 (mod 4) of M, a | t, c | t/a, t = (m+1)/4. */
size_t es_o_gen_wheel_covers(u64 M, o_cover **out) {
  u64 divs[4096]; size_t nd = 1; divs[0] = 1;
  u64 n = M;
  for (u64 q = 2; q * q <= n; ++q)
    if (n % q == 0) {
      int e = 0;
      while (n % q == 0) { n /= q; ++e; }
      size_t base = nd; u64 pe = 1;
      for (int i = 1; i <= e; ++i) { pe *= q; for (size_t j = 0; j < base; ++j) divs[nd++] = divs[j] * pe; }
    }
  if (n > 1) { size_t base = nd; for (size_t j = 0; j < base; ++j) divs[nd++] = divs[j] * n; }
  qsort(divs, nd, sizeof(u64), cmp_u64);
  o_cover *v = NULL; size_t cnt = 0, cap = 0;
  for (size_t i = 0; i < nd; ++i) {
    const u64 m = divs[i];
    if (m % 4 != 3) continue;
    const u64 t = (m + 1) / 4;
    for (u64 a = 1; a <= t; ++a) {
      if (t % a) continue;
      const u64 ta = t / a;
      for (u64 c = 1; c <= ta; ++c) {
        if (ta % c) continue;
        cover_push(&v, &cnt, &cap, a, c, ta / c);
      }
    }
  }
  *out = v;
  return cover_dedup(v, cnt);
}

static int ucert_cmp(const void *x, const void *y) {
  const o_ucert *a = x, *b = y;
  if (a->mod != b->mod) return a->mod < b->mod ? -1 : 1;
  if (a->res != b->res) return a->res < b->res ? -1 : 1;
  if (a->r != b->r) return a->r < b->r ? -1 : 1;
  return a->u < b->u ? -1 : a->u > b->u;
}
/* gen_ucerts (sieve/rung_scan3.cpp:177-202): uniform rung certificates (r, u) whose
 * conditions u | q^2, u == -q (mod r) are forced by p mod L, L = 4 lcm(r,u); dedup by
 * (L, res) keeping the smallest (r, u). */
size_t es_o_gen_ucerts(uint32_t rmax, uint32_t umax, o_ucert **out) {
  o_ucert *v = NULL; size_t n = 0, cap = 0;
  for (uint32_t r = 1; r <= rmax; ++r)
    for (uint32_t u = 1; u <= umax; ++u) {
      if (o_gcd(u, r) != 1) continue;
      const u64 L = 4ull * ((u64)r * u / o_gcd(r, u));
      for (u64 rho = 0; rho < L; ++rho) {
        if ((rho + r) % 4) continue;
        int ok = 1;
        for (int lift = 0; ok && lift < 2; ++lift) {
          const u64 p = rho + (u64)lift * L, A = (p + r) / 4, q = p * A;
          if ((q % u) * (q % u) % u || (q + u) % r) ok = 0;
        }
        if (!ok) continue;
        if (n == cap) { cap = cap ? cap * 2 : 1024; v = xrealloc(v, cap * sizeof *v); }
        v[n].mod = L; v[n].res = rho; v[n].r = r; v[n].u = u; ++n;
      }
    }
  qsort(v, n, sizeof *v, ucert_cmp);
  size_t k = 0;
  for (size_t i = 0; i < n; ++i)
    if (!k || v[k - 1].mod != v[i].mod || v[k - 1].res != v[i].res) v[k++] = v[i];
  *out = v;
  return k;
}

/* build_wheel (sieve/rung_scan3.cpp:211-226): classes mod M left alive by every F1 cover
 * with m | M and every F2 certificate with L | M, restricted to units. */
typedef struct { u64 *classes; size_t n; u64 max_pmin, n_f1_only; } o_wheel;
static o_wheel o_build_wheel(u64 M, const o_cover *cov, size_t ncov, const o_ucert *uc, size_t nuc) {
  uint8_t *dead = calloc(M, 1);
  o_wheel w; w.max_pmin = 0; w.n_f1_only = 0; w.n = 0;
  for (size_t i = 0; i < ncov; ++i) {
    if (M % cov[i].mod) continue;
    if (cov[i].pmin > w.max_pmin) w.max_pmin = cov[i].pmin;
    for (u64 x = cov[i].res; x < M; x += cov[i].mod) dead[x] = 1;
  }
  for (u64 x = 1; x < M; ++x) if (!dead[x] && o_gcd(x, M) == 1) ++w.n_f1_only;
  for (size_t i = 0; i < nuc; ++i) {
    if (M % uc[i].mod) continue;
    for (u64 x = uc[i].res; x < M; x += uc[i].mod) dead[x] = 1;
  }
  size_t cap = 1024;
  w.classes = xmalloc(cap * sizeof(u64));
  for (u64 x = 1; x < M; ++x)
    if (!dead[x] && o_gcd(x, M) == 1) {
      if (w.n == cap) { cap *= 2; w.classes = xrealloc(w.classes, cap * sizeof(u64)); }
      w.classes[w.n++] = x;
    }
  free(dead);
  return w;
}

/* fnv64_classes (sieve/rung_scan3.cpp:228-236): FNV-1a over "c0,c1,...". */
static u64 o_fnv64_classes(const u64 *cls, size_t n) {
  u64 h = 14695981039346656037ull;
  char buf[32];
  for (size_t i = 0; i < n; ++i) {
    int k = snprintf(buf, sizeof buf, i ? ",%" PRIu64 : "%" PRIu64, cls[i]);
    for (int j = 0; j < k; ++j) { h ^= (unsigned char)buf[j]; h *= 1099511628211ull; }
  }
  return h;
}

/* ctypes: the wheel for M. Returns the class count; writes up to cap classes. */
size_t es_o_wheel(u64 M, u64 *classes, size_t cap, u64 *max_pmin, u64 *fnv, u64 *n_f1_only) {
  o_cover *wc; size_t nwc = es_o_gen_wheel_covers(M, &wc);
  o_ucert *uc; size_t nuc = es_o_gen_ucerts(UCERT_RMAX, UCERT_UMAX, &uc);
  o_wheel w = o_build_wheel(M, wc, nwc, uc, nuc);
  for (size_t i = 0; i < w.n && i < cap; ++i) classes[i] = w.classes[i];
  if (max_pmin) *max_pmin = w.max_pmin;
  if (fnv) *fnv = o_fnv64_classes(w.classes, w.n);
  if (n_f1_only) *n_f1_only = w.n_f1_only;
  size_t n = w.n;
  free(w.classes); free(wc); free(uc);
  return n;
}

/* ctypes: the generated default filter set for (M, mmax) -- covers with m <= mmax and
 * m not dividing M, in (mod, res) order (sieve/rung_scan3.cpp:1098-1102) -- followed by the
 * stage-B' primes <= sieve_p (:1106-1108). Returns the total count; *ncov gets the
 * certified count; *cover_pmax the largest pmin over all covers with m <= mmax. */
size_t es_o_default_filters(u64 M, u64 mmax, u64 sieve_p, u64 *mods, u64 *ress, size_t cap, size_t *ncov,
                            u64 *cover_pmax) {
  o_cover *c; size_t nc = es_o_gen_covers(mmax, &c);
  size_t n = 0; u64 pm = 0;
  for (size_t i = 0; i < nc; ++i) {
    if (c[i].pmin > pm) pm = c[i].pmin;
    if (M % c[i].mod == 0) continue;
    if (n < cap) { mods[n] = c[i].mod; ress[n] = c[i].res; }
    ++n;
  }
  free(c);
  if (ncov) *ncov = n;
  if (cover_pmax) *cover_pmax = pm;
  if (sieve_p) {
    u64 *sp; size_t nsp = o_small_primes(sieve_p, M, &sp);
    for (size_t i = 0; i < nsp; ++i) { if (n < cap) { mods[n] = sp[i]; ress[n] = 0; } ++n; }
    free(sp);
  }
  return n;
}

/* ------------------------------------------------------------ the sweep */
typedef struct { u64 positions, covered, sieved, mr, composite, rung, direct, survivors; } o_stats;

/* A growable text buffer of certificate lines, one per lane. */
typedef struct { char *s; size_t n, cap; } o_text;
static void text_put(o_text *t, const char *line) {
  size_t k = strlen(line);
  if (t->n + k + 1 > t->cap) { t->cap = (t->n + k + 1) * 2; t->s = xrealloc(t->s, t->cap); }
  memcpy(t->s + t->n, line, k + 1);
  t->n += k;
}

/* Modular inverse by extended Euclid (inv3, sieve/rung_scan3.cpp:74-85). */
static u64 o_inv(u64 a, u64 m) {
  if (m == 1) return 0;
  int64_t t = 0, nt = 1, r = (int64_t)m, nr = (int64_t)(a % m);
  while (nr) {
    int64_t q = r / nr, tmp = t - q * nt; t = nt; nt = tmp;
    tmp = r - q * nr; r = nr; nr = tmp;
  }
  if (r != 1) { fprintf(stderr, "FATAL: inv(%" PRIu64 ",%" PRIu64 ") not coprime\n", a, m); abort(); }
  return (u64)(t < 0 ? t + (int64_t)m : t);
}

/* sweep_lane (sieve/rung_scan3.cpp:711-784). Positions of lane rho are p = first + M*J;
 * filter i hits J == off (mod step) with g = gcd(M, mod), step = mod/g, or never when
 * g does not divide the right-hand side. Segments of `seg` positions carry the offsets.
 * Covers [0,ncov) are marked first, the stage-B' primes [ncov,nall) after a popcount, so
 * `covered` and `sieved` stay apart. Survivors go through sprp2 + is_prime, then the
 * rung walk, then the direct search; anything left is a SURVIVOR. */
static void o_sweep_lane(u64 rho, u64 lo, u64 hi, u64 M, const u64 *mods, const u64 *ress,
                         size_t nall, size_t ncov, u64 seg, o_stats *st, o_text *emit) {
  const u64 first = lo + ((rho + M - lo % M) % M);
  if (first >= hi) return;
  const u64 npos = (hi - first + M - 1) / M;
  uint32_t *off = xmalloc(sizeof(uint32_t) * (nall ? nall : 1));
  uint32_t *step = xmalloc(sizeof(uint32_t) * (nall ? nall : 1));
  for (size_t i = 0; i < nall; ++i) {
    const u64 mod = mods[i], g = o_gcd(M, mod);
    const u64 rhs = (ress[i] + mod - first % mod) % mod;
    if (rhs % g) { step[i] = 0; off[i] = 0; continue; }
    const u64 s = mod / g;
    step[i] = (uint32_t)s;
    off[i] = s == 1 ? 0 : (uint32_t)((u128)(rhs / g) * o_inv((M / g) % s, s) % s);
  }
  const size_t nwmax = (size_t)((seg + 63) / 64);
  u64 *bits = xmalloc(sizeof(u64) * nwmax);
  char line[160];
  for (u64 base = 0; base < npos; base += seg) {
    const u64 n = seg < npos - base ? seg : npos - base;
    const size_t nw = (size_t)((n + 63) / 64);
    for (size_t w = 0; w < nw; ++w) bits[w] = ~0ull;
    if (n & 63) bits[nw - 1] = (1ull << (n & 63)) - 1;
    u64 after_covers = 0;
    for (int phase = 0; phase < 2; ++phase) {
      const size_t from = phase ? ncov : 0, to = phase ? nall : ncov;
      for (size_t i = from; i < to; ++i) {
        const uint32_t s = step[i];
        if (!s) continue;
        uint32_t j = off[i];
        for (; j < n; j += s) bits[j >> 6] &= ~(1ull << (j & 63));
        off[i] = (uint32_t)(j - n);
      }
      if (phase == 0 && ncov != nall)
        for (size_t w = 0; w < nw; ++w) after_covers += (u64)__builtin_popcountll(bits[w]);
    }
    u64 nsurv = 0;
    for (size_t w = 0; w < nw; ++w) nsurv += (u64)__builtin_popcountll(bits[w]);
    st->positions += n;
    if (ncov == nall) st->covered += n - nsurv;
    else { st->covered += n - after_covers; st->sieved += after_covers - nsurv; }
    for (size_t w = 0; w < nw; ++w) {
      u64 x = bits[w];
      while (x) {
        const u64 j = w * 64 + (u64)__builtin_ctzll(x);
        x &= x - 1;
        const u64 p = first + M * (base + j);
        ++st->mr;
        if (!es_o_sprp2(p) || !es_o_is_prime(p)) { ++st->composite; continue; }
        if (es_o_solve_rung(p, line, sizeof line)) { ++st->rung; text_put(emit, line); continue; }
        if (es_o_solve_direct(p, line, sizeof line)) { ++st->direct; text_put(emit, line); continue; }
        ++st->survivors;
        snprintf(line, sizeof line, "SURVIVOR %" PRIu64 "\n", p);
        text_put(emit, line);
      }
    }
  }
  free(off); free(step); free(bits);
}

/* small_primes (sieve/rung_scan3.cpp:664-674): primes q <= P with q not dividing M. */
static size_t o_small_primes(u64 P, u64 M, u64 **out) {
  uint8_t *comp = calloc(P + 1, 1);
  u64 *v = xmalloc(sizeof(u64) * (P + 1));
  size_t n = 0;
  for (u64 i = 2; i <= P; ++i)
    if (!comp[i]) {
      if (M % i) v[n++] = i;
      for (u64 j = i * i; j <= P; j += i) comp[j] = 1;
    }
  free(comp);
  *out = v;
  return n;
}

/* ------------------------------------------------------------ a scan, as a library
 * One window [lo, hi) over every lane, merged in lane order: the stream text (SURVIVOR
 * lines included or not) and the counters. Filters are the caller's (mods/ress, ncov
 * certified covers followed by stage-B' primes). Returns the text, malloc'ed. */
char *es_o_scan(u64 lo, u64 hi, u64 M, const u64 *mods, const u64 *ress, size_t nall,
                size_t ncov, u64 seg, int emit_surv, int threads, u64 *counters8) {
  /* The wheel depends only on M: derive it once per M and keep it (the reference's
   * driver derives it once per process, sieve/rung_scan3.cpp:1032-1034). */
  static u64 cached_M = 0;
  static o_wheel w;
  if (cached_M != M) {
    if (cached_M) free(w.classes);
    o_cover *wc; size_t nwc = es_o_gen_wheel_covers(M, &wc);
    o_ucert *uc; size_t nuc = es_o_gen_ucerts(UCERT_RMAX, UCERT_UMAX, &uc);
    w = o_build_wheel(M, wc, nwc, uc, nuc);
    free(wc); free(uc);
    cached_M = M;
  }
  td_init();                       /* once, before the lanes run in parallel */
  o_stats *lst = calloc(w.n, sizeof(o_stats));
  o_text *lem = calloc(w.n, sizeof(o_text));
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#else
  (void)threads;
#endif
#pragma omp parallel for schedule(dynamic, 1)
  for (size_t i = 0; i < w.n; ++i)
    o_sweep_lane(w.classes[i], lo, hi, M, mods, ress, nall, ncov, seg ? seg : 262144, &lst[i], &lem[i]);
  o_stats st; memset(&st, 0, sizeof st);
  o_text out; memset(&out, 0, sizeof out);
  text_put(&out, "");
  for (size_t i = 0; i < w.n; ++i) {
    st.positions += lst[i].positions; st.covered += lst[i].covered; st.sieved += lst[i].sieved;
    st.mr += lst[i].mr; st.composite += lst[i].composite; st.rung += lst[i].rung;
    st.direct += lst[i].direct; st.survivors += lst[i].survivors;
    if (lem[i].s) {
      char *s = lem[i].s;
      while (*s) {
        char *nl = strchr(s, '\n');
        size_t k = nl ? (size_t)(nl - s + 1) : strlen(s);
        if (emit_surv || strncmp(s, "SURVIVOR ", 9) != 0) {
          char save = s[k]; s[k] = 0; text_put(&out, s); s[k] = save;
        }
        s += k;
      }
      free(lem[i].s);
    }
  }
  free(lst); free(lem);
  const u64 c[8] = {st.positions, st.covered, st.sieved, st.mr, st.composite, st.rung, st.direct, st.survivors};
  if (counters8) memcpy(counters8, c, sizeof c);
  return out.s;
}
void es_o_free(void *p) { free(p); }

#ifdef ES_ORACLE_MAIN
/* ------------------------------------------------------------ the CLI
 * rung_scan3's command line (sieve/rung_scan3.cpp:960-1163): the same flags, refusals,
 * exit codes, stderr banner and SUMMARY line, plus the --verify, --dump-classes and
 * --check-direct modes. */
static int self_test(void) {                            /* :821-897 */
  int fails = 0;
#define CHECK(what, got, want) do { u64 g_ = (got), w_ = (want); \
    if (g_ != w_) { printf("  FAIL %-34s got %" PRIu64 " want %" PRIu64 "\n", what, g_, w_); ++fails; } \
    else printf("  ok   %-34s %" PRIu64 "\n", what, g_); } while (0)
  o_cover *all; size_t nall = es_o_gen_covers(120120, &all);
  o_cover *fast; size_t nfast = es_o_gen_wheel_covers(120120, &fast);
  size_t nslow = 0; u64 diff = 0;
  for (size_t i = 0; i < nall; ++i) if (120120 % all[i].mod == 0) {
    if (nslow < nfast) {
      const o_cover *a = &all[i], *b = &fast[nslow];
      if (!(a->mod == b->mod && a->res == b->res && a->pmin == b->pmin && a->a == b->a && a->c == b->c && a->d == b->d)) diff = 1;
    }
    ++nslow;
  }
  if (nslow != nfast) diff = 1;
  CHECK("wheel covers: divisor == full", diff, 0);
  CHECK("wheel covers at 120120", nfast, nslow);
  o_ucert *uc; size_t nuc = es_o_gen_ucerts(UCERT_RMAX, UCERT_UMAX, &uc);
  o_cover *c840; size_t n840 = es_o_gen_covers(840, &c840);
  o_wheel w840 = o_build_wheel(840, c840, n840, uc, nuc);
  CHECK("wheel(840) F1 only", w840.n_f1_only, 24);
  CHECK("wheel(840) classes", w840.n, 6);
  CHECK("wheel(840) max pmin", w840.max_pmin, 34);
  static const u64 REF840[6] = {1, 121, 169, 289, 361, 529};
  int same = w840.n == 6;
  for (int i = 0; same && i < 6; ++i) same = w840.classes[i] == REF840[i];
  if (!same) { printf("  FAIL wheel(840) != {1,121,169,289,361,529}\n"); ++fails; }
  else printf("  ok   wheel(840) == hard classes (DERIVED, not assumed)\n");
  o_wheel w120 = o_build_wheel(120120, all, nall, uc, nuc);
  CHECK("wheel(120120) F1 only", w120.n_f1_only, 920);
  CHECK("wheel(120120) classes", w120.n, 220);
  CHECK("wheel(120120) max pmin", w120.max_pmin, 15014);
  u64 h = o_fnv64_classes(w120.classes, w120.n);
  if (h != pin_for(120120)->fnv64) { printf("  FAIL wheel(120120) fnv64 %016" PRIx64 "\n", h); ++fails; }
  else printf("  ok   wheel(120120) fnv64            dbc4ab9b16d73f76\n");
  o_cover *c204; size_t n204 = es_o_gen_wheel_covers(2042040, &c204);
  o_wheel w204 = o_build_wheel(2042040, c204, n204, uc, nuc);
  CHECK("wheel(2042040) classes", w204.n, 2308);
  u64 h2 = o_fnv64_classes(w204.classes, w204.n);
  if (h2 != pin_for(2042040)->fnv64) { printf("  FAIL wheel(2042040) fnv64 %016" PRIx64 "\n", h2); ++fails; }
  else printf("  ok   wheel(2042040) fnv64           %016" PRIx64 "\n", h2);
  for (int pass = 0; pass < 2; ++pass) {
    const o_wheel *w = pass ? &w120 : &w204;
    u64 strays = 0;
    for (size_t i = 0; i < w->n; ++i) {
      int hard = 0;
      for (int j = 0; j < 6; ++j) if (w->classes[i] % 840 == REF840[j]) hard = 1;
      if (w->classes[i] % 24 != 1 || !hard) ++strays;
    }
    CHECK(pass ? "survivors outside hard class" : "wheel(2042040) outside hard class", strays, 0);
  }
  printf(fails ? "\nSELF-TEST FAILED (%d checks)\n" : "\nSELF-TEST PASSED\n", fails);
#undef CHECK
  return fails ? 1 : 0;
}

static int dump_classes(u64 M) {                       /* :904-953 */
  o_cover *cov; size_t ncov = es_o_gen_wheel_covers(M, &cov);
  o_ucert *uc; size_t nuc = es_o_gen_ucerts(UCERT_RMAX, UCERT_UMAX, &uc);
  o_wheel w = o_build_wheel(M, cov, ncov, uc, nuc);
  u64 ncop = 0;
  for (u64 x = 1; x < M; ++x) if (o_gcd(x, M) == 1) ++ncop;
  const pin_t *pin = pin_for(M);
  printf("# certified class table mod %" PRIu64 ": every unit class is killed by a named\n"
         "# certificate or survives.  F1: covers m=4acd-1 | M, kill rho \xe2\x89\xa1 -4a^2d (mod m).\n"
         "# F2: uniform rung certificates (r,u), r <= %u u <= %u, kill rho \xe2\x89\xa1 res (mod L).\n",
         M, UCERT_RMAX, UCERT_UMAX);
  printf("# unit_classes=%" PRIu64 " classes=%zu kills=%" PRIu64 " fnv64=%016" PRIx64 " sha256=%s\n",
         ncop, w.n, ncop - w.n, o_fnv64_classes(w.classes, w.n), pin ? pin->sha256 : "unpinned");
  for (size_t i = 0; i < w.n; ++i) printf("CLASS %" PRIu64 "\n", w.classes[i]);
  int32_t *who = xmalloc(sizeof(int32_t) * M);
  for (u64 x = 0; x < M; ++x) who[x] = -1;
  for (size_t i = 0; i < ncov; ++i)
    for (u64 x = cov[i].res; x < M; x += cov[i].mod) if (who[x] < 0) who[x] = (int32_t)i;
  const int32_t F2 = (int32_t)ncov;
  for (size_t i = 0; i < nuc; ++i) {
    if (M % uc[i].mod) continue;
    for (u64 x = uc[i].res; x < M; x += uc[i].mod) if (who[x] < 0) who[x] = F2 + (int32_t)i;
  }
  for (u64 rho = 1; rho < M; ++rho) {
    if (o_gcd(rho, M) != 1 || who[rho] < 0) continue;
    if (who[rho] < F2) {
      const o_cover *f = &cov[who[rho]];
      printf("KILL %" PRIu64 " F1 %" PRIu64 " %" PRIu64 " %u %u %u\n", rho, f->mod, f->res, f->a, f->c, f->d);
    } else {
      const o_ucert *c = &uc[who[rho] - F2];
      printf("KILL %" PRIu64 " F2 %" PRIu64 " %" PRIu64 " %u %u\n", rho, c->mod, c->res, c->r, c->u);
    }
  }
  return 0;
}

static int check_direct(u64 lo, u64 N) {                /* :798-817 */
  u64 found = 0, solved = 0;
  char line[160];
  for (u64 p = lo | 1ull; found < N; p += 2) {
    if (!es_o_is_prime(p)) continue;
    ++found;
    if (es_o_solve_direct(p, line, sizeof line)) { ++solved; fputs(line, stdout); }
    else fprintf(stderr, "  stage E DECLINED p=%" PRIu64 "\n", p);
  }
  fprintf(stderr, "%s check-direct %" PRIu64 "/%" PRIu64 " primes at or above %" PRIu64
          " solved by stage E (ceiling %" PRIu64 ")\n", solved == N ? "ok  " : "FAIL", solved, N, lo, DIRECT_PMAX);
  return solved == N ? 0 : 1;
}

int main(int argc, char **argv) {
  if (argc >= 2 && !strcmp(argv[1], "--verify")) return self_test();
  if (argc >= 4 && !strcmp(argv[1], "--check-direct"))
    return check_direct(strtoull(argv[2], 0, 10), strtoull(argv[3], 0, 10));
  if (argc >= 2 && !strcmp(argv[1], "--dump-classes")) {
    u64 dm = 2042040;
    for (int i = 2; i + 1 < argc; ++i) if (!strcmp(argv[i], "--wheel")) dm = strtoull(argv[i + 1], 0, 10);
    return dump_classes(dm);
  }
  if (argc < 3) {
    fprintf(stderr, "usage: %s LO HI [--mmax N] [--wheel M] [--seg N] [--threads N]\n"
                    "                 [--shard i/n] [--progress N] [--filters FILE] [--sieve P]\n"
                    "                 [--no-emit-survivors]\n"
                    "       %s --verify | --dump-classes | --check-direct LO N\n", argv[0], argv[0]);
    return 1;
  }
  u64 lo = strtoull(argv[1], 0, 10), hi = strtoull(argv[2], 0, 10);
  u64 M = 2042040, mmax = 10000, seg = 262144, shard = 0, nshard = 1, sieve_p = 0;
  int threads = 0, emit_surv = 1;
  const char *ffile = NULL;
  for (int i = 3; i < argc; ++i) {
    if (!strcmp(argv[i], "--mmax") && i + 1 < argc) mmax = strtoull(argv[++i], 0, 10);
    else if (!strcmp(argv[i], "--wheel") && i + 1 < argc) M = strtoull(argv[++i], 0, 10);
    else if (!strcmp(argv[i], "--seg") && i + 1 < argc) seg = strtoull(argv[++i], 0, 10);
    else if (!strcmp(argv[i], "--progress") && i + 1 < argc) ++i;
    else if (!strcmp(argv[i], "--threads") && i + 1 < argc) threads = atoi(argv[++i]);
    else if (!strcmp(argv[i], "--filters") && i + 1 < argc) ffile = argv[++i];
    else if (!strcmp(argv[i], "--sieve") && i + 1 < argc) sieve_p = strtoull(argv[++i], 0, 10);
    else if (!strcmp(argv[i], "--shard") && i + 1 < argc) {
      unsigned long long a = 0, b = 1;
      if (sscanf(argv[++i], "%llu/%llu", &a, &b) == 2) { shard = a; nshard = b; }
    } else if (!strcmp(argv[i], "--no-emit-survivors")) emit_surv = 0;
    else { fprintf(stderr, "FATAL: unknown option '%s'\n", argv[i]); return 1; }
  }
  if (!seg) seg = 262144;
  if (nshard == 0) nshard = 1;
  if (nshard > 1) {                                     /* :1022-1027 */
    const u64 span = (hi - lo + nshard - 1) / nshard;
    const u64 a = lo + shard * span, b = hi < a + span ? hi : a + span;
    lo = a; hi = b > a ? b : a;
  }
  o_cover *covers; size_t ncovers = es_o_gen_covers(mmax, &covers);
  o_cover *wc; size_t nwc = es_o_gen_wheel_covers(M, &wc);
  o_ucert *uc; size_t nuc = es_o_gen_ucerts(UCERT_RMAX, UCERT_UMAX, &uc);
  o_wheel w = o_build_wheel(M, wc, nwc, uc, nuc);
  u64 cover_pmax = 0;
  for (size_t i = 0; i < ncovers; ++i) if (covers[i].pmin > cover_pmax) cover_pmax = covers[i].pmin;
  const pin_t *pin = pin_for(M);
  if (pin) {
    if (o_fnv64_classes(w.classes, w.n) != pin->fnv64) {
      fprintf(stderr, "FATAL: class table digest mismatch at M=%" PRIu64 "\n", M);
      return 1;
    }
  } else {
    fprintf(stderr, "[es_oracle] WARNING: no pinned digest for M=%" PRIu64 " -- running UNPINNED\n", M);
  }
  if (hi > DIRECT_PMAX) { fprintf(stderr, "FATAL: HI must not exceed %" PRIu64 ", the stage-E ceiling\n", DIRECT_PMAX); return 1; }
  const u64 floor_ = w.max_pmin > cover_pmax ? w.max_pmin : cover_pmax;
  if (lo <= floor_) { fprintf(stderr, "FATAL: LO must exceed max pmin of the filter table (%" PRIu64 ")\n", floor_); return 1; }
  u64 *mods = NULL, *ress = NULL; size_t nf = 0, capf = 0;
  if (ffile) {
    FILE *fp = fopen(ffile, "r");
    if (!fp) { fprintf(stderr, "FATAL: cannot open %s\n", ffile); return 1; }
    char line[256];
    while (fgets(line, sizeof line, fp)) {
      unsigned long long mod, res;
      if (sscanf(line, "FILTER %llu %llu", &mod, &res) == 2) {
        if (nf == capf) { capf = capf ? capf * 2 : 4096; mods = xrealloc(mods, capf * 8); ress = xrealloc(ress, capf * 8); }
        mods[nf] = mod; ress[nf] = res; ++nf;
      }
    }
    fclose(fp);
    if (!nf) { fprintf(stderr, "FATAL: no FILTER lines in %s\n", ffile); return 1; }
  } else {
    capf = ncovers + 1; mods = xmalloc(capf * 8); ress = xmalloc(capf * 8);
    for (size_t i = 0; i < ncovers; ++i) if (M % covers[i].mod) { mods[nf] = covers[i].mod; ress[nf] = covers[i].res; ++nf; }
  }
  const size_t ncov = nf;
  if (sieve_p) {
    u64 *sp; size_t nsp = o_small_primes(sieve_p, M, &sp);
    mods = xrealloc(mods, (nf + nsp) * 8); ress = xrealloc(ress, (nf + nsp) * 8);
    for (size_t i = 0; i < nsp; ++i) { mods[nf] = sp[i]; ress[nf] = 0; ++nf; }
    free(sp);
  }
  struct timespec t0, t1;
  clock_gettime(CLOCK_MONOTONIC, &t0);
  u64 c[8];
  char *text = es_o_scan(lo, hi, M, mods, ress, nf, ncov, seg, emit_surv, threads, c);
  clock_gettime(CLOCK_MONOTONIC, &t1);
  fputs(text, stdout);
  free(text);
  printf("SUMMARY lo=%" PRIu64 " hi=%" PRIu64 " wheelM=%" PRIu64 " lanes=%zu mmax=%" PRIu64 " ucert_rmax=%u "
         "ucert_umax=%u wheel_pmin=%" PRIu64 " classes_sha256=%s positions=%" PRIu64 " "
         "covered=%" PRIu64 " sieved=%" PRIu64 " mr=%" PRIu64 " composite=%" PRIu64 " rung=%" PRIu64
         " direct=%" PRIu64 " survivors=%" PRIu64 "\n",
         lo, hi, M, w.n, mmax, UCERT_RMAX, UCERT_UMAX, w.max_pmin, pin ? pin->sha256 : "unpinned",
         c[0], c[1], c[2], c[3], c[4], c[5], c[6], c[7]);
  fprintf(stderr, "sweep_seconds=%.6f\n", (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec));
  return c[7] ? 2 : 0;
}
#endif
