// es_wheel.cpp -- the certificate families and the class table, derived on the host.
#include "es_wheel.h"

#include <algorithm>
#include <cinttypes>
#include <cstdio>
#include <cstring>

namespace es {

typedef unsigned __int128 u128;

static const ClassPin PINS[] = {
  {120120, 0xdbc4ab9b16d73f76ull, "154e82672d9da66cff97d48079047b8b0b0a31fa049ac62fb05b5c82ad540f60"},
  {2042040, 0xb9b5d1408da3428eull, "a77b2187201ff96ff3ecf822150f4152d841941deeb0cf616238bcbb0a648bbc"},
};

const ClassPin *class_pin(u64 M) {
  for (const ClassPin &p : PINS) if (p.M == M) return &p;
  return nullptr;
}

u64 gcd_u64(u64 a, u64 b) {
  while (b) { const u64 t = a % b; a = b; b = t; }
  return a;
}

u64 inv_mod(u64 a, u64 m, bool &ok) {
  ok = true;
  if (m == 1) return 0;
  int64_t t = 0, nt = 1, r = (int64_t)m, nr = (int64_t)(a % m);
  while (nr) {
    const int64_t q = r / nr;
    int64_t tmp = t - q * nt; t = nt; nt = tmp;
    tmp = r - q * nr; r = nr; nr = tmp;
  }
  if (r != 1) { ok = false; return 0; }
  return (u64)(t < 0 ? t + (int64_t)m : t);
}

// Cover candidates are collected in full and then reduced to one per (mod, res): the one
// with the smallest pmin, and among equal pmin the smallest a, then the smallest c. Both
// generators below reach a given (mod, res, pmin) first through its smallest a, which is the
// witness the reference keeps (its first-found-wins replacement on pmin), so the rule gives
// the same (a, c, d) for every cover of the class table.
static Cover make_cover(u64 a, u64 c, u64 d) {
  const u128 mm = (u128)4 * a * c * d - 1, bb = (u128)4 * a * a * d;
  Cover f;
  f.mod = (u64)mm;
  f.res = (u64)((mm - bb % mm) % mm);
  f.pmin = (u64)(mm * (a / c + 1) - bb);
  f.a = (unsigned)a; f.c = (unsigned)c; f.d = (unsigned)d;
  return f;
}

static std::vector<Cover> dedup(std::vector<Cover> &v) {
  std::sort(v.begin(), v.end(), [](const Cover &x, const Cover &y) {
    if (x.mod != y.mod) return x.mod < y.mod;
    if (x.res != y.res) return x.res < y.res;
    if (x.pmin != y.pmin) return x.pmin < y.pmin;
    if (x.a != y.a) return x.a < y.a;
    return x.c < y.c;
  });
  std::vector<Cover> out;
  for (const Cover &f : v)
    if (out.empty() || out.back().mod != f.mod || out.back().res != f.res) out.push_back(f);
  return out;
}

std::vector<Cover> gen_covers(u64 mmax) {
  std::vector<Cover> v;
  const u64 nmax = (mmax + 1) / 4;
  for (u64 a = 1; a <= nmax; ++a)
    for (u64 d = 1; a * d <= nmax; ++d)
      for (u64 c = 1; a * d * c <= nmax; ++c) v.push_back(make_cover(a, c, d));
  return dedup(v);
}

// The divisors of n, ascending: each d up to sqrt(n) that divides n pairs with n / d.
static std::vector<u64> divisors_of(u64 n) {
  std::vector<u64> lowers, uppers;
  for (u64 d = 1; d <= n / d; ++d) {
    if (n % d) continue;
    lowers.push_back(d);
    if (d != n / d) uppers.push_back(n / d);
  }
  lowers.insert(lowers.end(), uppers.rbegin(), uppers.rend());
  return lowers;
}

// Covers whose modulus divides M: an F1 modulus is 4acd - 1, so only the divisors m of M
// with m = 3 (mod 4) can carry one, and its triples are the ordered factorizations
// acd = (m + 1) / 4 -- a a divisor of that product, c a divisor of what a leaves.
std::vector<Cover> gen_wheel_covers(u64 M) {
  std::vector<Cover> v;
  for (u64 m : divisors_of(M)) {
    if (m % 4 != 3) continue;
    const u64 acd = (m + 1) / 4;
    for (u64 a : divisors_of(acd))
      for (u64 c : divisors_of(acd / a)) v.push_back(make_cover(a, c, acd / a / c));
  }
  return dedup(v);
}

// F2: rung r with the fixed witness u, gcd(r, u) = 1, L = 4ru. For p = rho (mod L) with
// rho = -r (mod 4), A = (p + r)/4 is determined mod ru and so is q = pA (mod ru): the two
// conditions of the rung certificate, u | q^2 and q = -u (mod r), hold for every such p or
// for none, and one evaluation at p = rho decides them. Kept per (L, rho): the smallest
// (r, u).
std::vector<Ucert> gen_ucerts(unsigned rmax, unsigned umax) {
  std::vector<Ucert> v;
  for (unsigned r = 1; r <= rmax; ++r)
    for (unsigned u = 1; u <= umax; ++u) {
      if (gcd_u64(r, u) != 1) continue;
      const u64 L = 4ull * r * u;
      for (u64 rho = (4 - r % 4) % 4; rho < L; rho += 4) {
        const u64 q = rho * ((rho + r) / 4);
        const u64 qu = q % u;
        if (qu * qu % u == 0 && (q + u) % r == 0) v.push_back({L, rho, r, u});
      }
    }
  std::sort(v.begin(), v.end(), [](const Ucert &x, const Ucert &y) {
    if (x.mod != y.mod) return x.mod < y.mod;
    if (x.res != y.res) return x.res < y.res;
    return x.r != y.r ? x.r < y.r : x.u < y.u;
  });
  std::vector<Ucert> out;
  for (const Ucert &c : v)
    if (out.empty() || out.back().mod != c.mod || out.back().res != c.res) out.push_back(c);
  return out;
}

// The class table: a state per residue mod M -- not a unit, a live unit, or a unit some
// certificate kills. F1 covers with m | M run first (the unit classes they leave are
// n_f1_only), then the F2 certificates with L | M; a certificate whose modulus does not
// divide M would kill only part of a class and is skipped.
Wheel build_wheel(u64 M, const std::vector<Cover> &cov, const std::vector<Ucert> &uc) {
  enum : uint8_t { NONUNIT = 0, LIVE = 1, KILLED = 2 };
  std::vector<uint8_t> state(M);
  for (u64 x = 0; x < M; ++x) state[x] = gcd_u64(x, M) == 1 ? LIVE : NONUNIT;
  auto kill = [&](u64 res, u64 mod) {
    for (u64 x = res; x < M; x += mod)
      if (state[x] == LIVE) state[x] = KILLED;
  };
  auto live = [&]() { return (u64)std::count(state.begin(), state.end(), (uint8_t)LIVE); };
  Wheel w;
  for (const Cover &f : cov)
    if (M % f.mod == 0) {
      kill(f.res, f.mod);
      w.max_pmin = std::max(w.max_pmin, f.pmin);
    }
  w.n_f1_only = live();
  for (const Ucert &c : uc)
    if (M % c.mod == 0) kill(c.res, c.mod);
  w.classes.reserve(live());
  for (u64 x = 0; x < M; ++x)
    if (state[x] == LIVE) w.classes.push_back(x);
  return w;
}

static void fnv_bytes(u64 &h, const char *s, int n) {
  for (int j = 0; j < n; ++j) { h ^= (unsigned char)s[j]; h *= 1099511628211ull; }
}

u64 fnv64_classes(const std::vector<u64> &cls) {
  u64 h = 14695981039346656037ull;
  char buf[32];
  for (size_t i = 0; i < cls.size(); ++i)
    fnv_bytes(h, buf, snprintf(buf, sizeof buf, i ? ",%llu" : "%llu", cls[i]));
  return h;
}

u64 fnv64_filters(const std::vector<u64> &mods, const std::vector<u64> &ress, size_t ncov) {
  u64 h = 14695981039346656037ull;
  char buf[48];
  for (size_t i = 0; i < ncov; ++i) fnv_bytes(h, buf, snprintf(buf, sizeof buf, "%llu,%llu;", mods[i], ress[i]));
  return h;
}

std::vector<u64> small_primes(u64 P, u64 M) {
  std::vector<uint8_t> comp(P + 1, 0);
  std::vector<u64> out;
  for (u64 i = 2; i <= P; ++i)
    if (!comp[i]) {
      if (M % i) out.push_back(i);
      for (u64 j = i * i; j <= P; j += i) comp[j] = 1;
    }
  return out;
}

std::string class_table_text(u64 M) {
  const std::vector<Cover> cov = gen_wheel_covers(M);
  const std::vector<Ucert> uc = gen_ucerts(UCERT_RMAX, UCERT_UMAX);
  const Wheel w = build_wheel(M, cov, uc);
  u64 ncop = 0;
  for (u64 x = 1; x < M; ++x) if (gcd_u64(x, M) == 1) ++ncop;
  std::string out;
  char line[256];
  const ClassPin *pin = class_pin(M);
  snprintf(line, sizeof line,
           "# certified class table mod %llu: every unit class is killed by a named\n"
           "# certificate or survives.  F1: covers m=4acd-1 | M, kill rho \xe2\x89\xa1 -4a^2d (mod m).\n",
           M);
  out += line;
  snprintf(line, sizeof line,
           "# F2: uniform rung certificates (r,u), r <= %u u <= %u, kill rho \xe2\x89\xa1 res (mod L).\n",
           UCERT_RMAX, UCERT_UMAX);
  out += line;
  snprintf(line, sizeof line, "# unit_classes=%llu classes=%zu kills=%llu fnv64=%016llx sha256=%s\n",
           ncop, w.classes.size(), ncop - (u64)w.classes.size(), fnv64_classes(w.classes),
           pin ? pin->sha256 : "unpinned");
  out += line;
  for (u64 c : w.classes) { snprintf(line, sizeof line, "CLASS %llu\n", c); out += line; }
  // The canonical killer is the first certificate in (F1 by (m,res), then F2 by (L,res))
  // order; marking "only where unmarked" in that order finds it.
  std::vector<int32_t> who(M, -1);
  for (size_t i = 0; i < cov.size(); ++i)
    for (u64 x = cov[i].res; x < M; x += cov[i].mod)
      if (who[x] < 0) who[x] = (int32_t)i;
  const int32_t F2 = (int32_t)cov.size();
  for (size_t i = 0; i < uc.size(); ++i) {
    if (M % uc[i].mod) continue;
    for (u64 x = uc[i].res; x < M; x += uc[i].mod)
      if (who[x] < 0) who[x] = F2 + (int32_t)i;
  }
  for (u64 rho = 1; rho < M; ++rho) {
    if (gcd_u64(rho, M) != 1 || who[rho] < 0) continue;
    if (who[rho] < F2) {
      const Cover &f = cov[who[rho]];
      snprintf(line, sizeof line, "KILL %llu F1 %llu %llu %u %u %u\n", rho, f.mod, f.res, f.a, f.c, f.d);
    } else {
      const Ucert &c = uc[who[rho] - F2];
      snprintf(line, sizeof line, "KILL %llu F2 %llu %llu %u %u\n", rho, c.mod, c.res, c.r, c.u);
    }
    out += line;
  }
  return out;
}

// Mordell's hard classes mod 840: the residues no polynomial identity of the F1 kind can
// cover. Every class the derivation keeps must reduce to one of them and be 1 mod 24.
static bool in_hard_class(u64 c) {
  static const u64 HARD840[6] = {1, 121, 169, 289, 361, 529};
  if (c % 24 != 1) return false;
  for (u64 h : HARD840) if (c % 840 == h) return true;
  return false;
}

int wheel_self_test(std::string &log) {
  struct Row { std::string what; u64 got, want; };
  std::vector<Row> rows;
  auto fnv_text = [](u64 h) { char b[24]; snprintf(b, sizeof b, "%016llx", h); return std::string(b); };
  // 1. The divisor-driven generator against the full enumeration, restricted to m | M, at the
  //    largest modulus where the full enumeration is cheap.
  {
    std::vector<Cover> full;
    for (const Cover &f : gen_covers(120120)) if (120120 % f.mod == 0) full.push_back(f);
    const std::vector<Cover> divd = gen_wheel_covers(120120);
    u64 mismatches = full.size() == divd.size() ? 0 : 1;
    for (size_t i = 0; !mismatches && i < full.size(); ++i)
      mismatches += full[i].mod != divd[i].mod || full[i].res != divd[i].res || full[i].pmin != divd[i].pmin ||
                    full[i].a != divd[i].a || full[i].c != divd[i].c || full[i].d != divd[i].d;
    rows.push_back({"120120: divisor covers differing from full", mismatches, 0});
    rows.push_back({"120120: covers with m | M", divd.size(), full.size()});
  }
  const std::vector<Ucert> uc = gen_ucerts(UCERT_RMAX, UCERT_UMAX);
  // 2. M = 840: the derivation must land on exactly Mordell's six hard classes.
  const Wheel w840 = build_wheel(840, gen_covers(840), uc);
  rows.push_back({"840: units left by F1", w840.n_f1_only, 24});
  rows.push_back({"840: classes left by F1+F2", w840.classes.size(), 6});
  rows.push_back({"840: largest pmin of a wheel cover", w840.max_pmin, 34});
  u64 off840 = w840.classes.size() == 6 ? 0 : 1;
  for (u64 c : w840.classes) off840 += !in_hard_class(c);
  rows.push_back({"840: classes that are not hard classes", off840, 0});
  // 3. M = 120120 (full enumeration) and M = 2042040 (divisor covers): counts and pins.
  const Wheel w120 = build_wheel(120120, gen_covers(120120), uc);
  rows.push_back({"120120: units left by F1", w120.n_f1_only, 920});
  rows.push_back({"120120: classes left by F1+F2", w120.classes.size(), 220});
  rows.push_back({"120120: largest pmin of a wheel cover", w120.max_pmin, 15014});
  rows.push_back({"120120: fnv64 " + fnv_text(fnv64_classes(w120.classes)) + " differs from the pin",
                  fnv64_classes(w120.classes) != class_pin(120120)->fnv64, 0});
  const Wheel w204 = build_wheel(2042040, gen_wheel_covers(2042040), uc);
  rows.push_back({"2042040: classes left by F1+F2", w204.classes.size(), 2308});
  rows.push_back({"2042040: fnv64 " + fnv_text(fnv64_classes(w204.classes)) + " differs from the pin",
                  fnv64_classes(w204.classes) != class_pin(2042040)->fnv64, 0});
  // 4. Both larger tables reproduce Mordell: nothing outside the hard classes survives.
  for (const auto &mw : {std::make_pair("120120", &w120), std::make_pair("2042040", &w204)}) {
    u64 off = 0;
    for (u64 c : mw.second->classes) off += !in_hard_class(c);
    rows.push_back({std::string(mw.first) + ": classes outside the hard classes", off, 0});
  }
  int fails = 0;
  char line[200];
  for (const Row &r : rows) {
    const bool ok = r.got == r.want;
    fails += !ok;
    if (ok) snprintf(line, sizeof line, "  pass  %-50s = %llu\n", r.what.c_str(), r.got);
    else snprintf(line, sizeof line, "  FAIL  %-50s = %llu, expected %llu\n", r.what.c_str(), r.got, r.want);
    log += line;
  }
  return fails;
}

}  // namespace es
