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

// A cover candidate tagged with its generation order, so that ties on pmin keep the
// earliest generated witness -- the replacement rule `pmin < best.pmin` of the reference.
struct Tagged { Cover c; size_t seq; };

static Cover make_cover(u64 a, u64 c, u64 d) {
  const u128 mm = (u128)4 * a * c * d - 1, bb = (u128)4 * a * a * d;
  Cover f;
  f.mod = (u64)mm;
  f.res = (u64)((mm - bb % mm) % mm);
  f.pmin = (u64)(mm * (a / c + 1) - bb);
  f.a = (unsigned)a; f.c = (unsigned)c; f.d = (unsigned)d;
  return f;
}

static std::vector<Cover> dedup(std::vector<Tagged> &v) {
  std::sort(v.begin(), v.end(), [](const Tagged &x, const Tagged &y) {
    if (x.c.mod != y.c.mod) return x.c.mod < y.c.mod;
    if (x.c.res != y.c.res) return x.c.res < y.c.res;
    if (x.c.pmin != y.c.pmin) return x.c.pmin < y.c.pmin;
    return x.seq < y.seq;
  });
  std::vector<Cover> out;
  for (const Tagged &t : v)
    if (out.empty() || out.back().mod != t.c.mod || out.back().res != t.c.res) out.push_back(t.c);
  return out;
}

std::vector<Cover> gen_covers(u64 mmax) {
  std::vector<Tagged> v;
  const u64 nmax = (mmax + 1) / 4;
  for (u64 a = 1; a <= nmax; ++a)
    for (u64 d = 1; a * d <= nmax; ++d)
      for (u64 c = 1; a * d * c <= nmax; ++c) v.push_back({make_cover(a, c, d), v.size()});
  return dedup(v);
}

std::vector<Cover> gen_wheel_covers(u64 M) {
  std::vector<u64> divs{1};
  u64 n = M;
  for (u64 q = 2; q * q <= n; ++q)
    if (n % q == 0) {
      int e = 0;
      while (n % q == 0) { n /= q; ++e; }
      const size_t base = divs.size();
      u64 pe = 1;
      for (int i = 1; i <= e; ++i) { pe *= q; for (size_t j = 0; j < base; ++j) divs.push_back(divs[j] * pe); }
    }
  if (n > 1) { const size_t base = divs.size(); for (size_t j = 0; j < base; ++j) divs.push_back(divs[j] * n); }
  std::sort(divs.begin(), divs.end());
  std::vector<Tagged> v;
  for (u64 m : divs) {
    if (m % 4 != 3) continue;                 // F1 moduli are 4N - 1
    const u64 t = (m + 1) / 4;                // acd = t
    for (u64 a = 1; a <= t; ++a) {
      if (t % a) continue;
      const u64 ta = t / a;
      for (u64 c = 1; c <= ta; ++c)
        if (ta % c == 0) v.push_back({make_cover(a, c, ta / c), v.size()});
    }
  }
  return dedup(v);
}

std::vector<Ucert> gen_ucerts(unsigned rmax, unsigned umax) {
  std::vector<Ucert> v;
  for (unsigned r = 1; r <= rmax; ++r)
    for (unsigned u = 1; u <= umax; ++u) {
      if (gcd_u64(u, r) != 1) continue;
      const u64 L = 4ull * ((u64)r * u / gcd_u64(r, u));
      for (u64 rho = 0; rho < L; ++rho) {
        if ((rho + r) % 4) continue;          // A = (p + r)/4 must be integral
        bool ok = true;
        for (int lift = 0; ok && lift < 2; ++lift) {
          const u64 p = rho + (u64)lift * L, A = (p + r) / 4, q = p * A;
          if ((q % u) * (q % u) % u || (q + u) % r) ok = false;
        }
        if (ok) v.push_back({L, rho, r, u});
      }
    }
  // Generation order is (r, u) ascending, so a stable sort on (L, res) followed by keeping
  // the first of each key keeps the smallest (r, u).
  std::stable_sort(v.begin(), v.end(), [](const Ucert &x, const Ucert &y) {
    return x.mod != y.mod ? x.mod < y.mod : x.res < y.res;
  });
  std::vector<Ucert> out;
  for (const Ucert &c : v)
    if (out.empty() || out.back().mod != c.mod || out.back().res != c.res) out.push_back(c);
  return out;
}

Wheel build_wheel(u64 M, const std::vector<Cover> &cov, const std::vector<Ucert> &uc) {
  std::vector<uint8_t> dead(M, 0);
  Wheel w;
  for (const Cover &f : cov) {
    if (M % f.mod) continue;
    w.max_pmin = std::max(w.max_pmin, f.pmin);
    for (u64 x = f.res; x < M; x += f.mod) dead[x] = 1;
  }
  for (u64 x = 1; x < M; ++x) if (!dead[x] && gcd_u64(x, M) == 1) ++w.n_f1_only;
  for (const Ucert &c : uc) {
    if (M % c.mod) continue;
    for (u64 x = c.res; x < M; x += c.mod) dead[x] = 1;
  }
  for (u64 x = 1; x < M; ++x) if (!dead[x] && gcd_u64(x, M) == 1) w.classes.push_back(x);
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

int wheel_self_test(std::string &log) {
  int fails = 0;
  char line[160];
  auto check = [&](const char *what, u64 got, u64 want) {
    if (got != want) { snprintf(line, sizeof line, "  FAIL %-34s got %llu want %llu\n", what, got, want); ++fails; }
    else snprintf(line, sizeof line, "  ok   %-34s %llu\n", what, got);
    log += line;
  };
  {
    std::vector<Cover> slow;
    for (const Cover &f : gen_covers(120120)) if (120120 % f.mod == 0) slow.push_back(f);
    const std::vector<Cover> fast = gen_wheel_covers(120120);
    u64 diff = slow.size() != fast.size();
    for (size_t i = 0; !diff && i < slow.size(); ++i)
      diff = !(slow[i].mod == fast[i].mod && slow[i].res == fast[i].res && slow[i].pmin == fast[i].pmin &&
               slow[i].a == fast[i].a && slow[i].c == fast[i].c && slow[i].d == fast[i].d);
    check("wheel covers: divisor == full", diff, 0);
    check("wheel covers at 120120", fast.size(), slow.size());
  }
  const std::vector<Ucert> uc = gen_ucerts(UCERT_RMAX, UCERT_UMAX);
  const Wheel w840 = build_wheel(840, gen_covers(840), uc);
  check("wheel(840) F1 only", w840.n_f1_only, 24);
  check("wheel(840) classes", w840.classes.size(), 6);
  check("wheel(840) max pmin", w840.max_pmin, 34);
  static const u64 REF840[6] = {1, 121, 169, 289, 361, 529};
  bool same = w840.classes.size() == 6;
  for (int i = 0; same && i < 6; ++i) same = w840.classes[i] == REF840[i];
  log += same ? "  ok   wheel(840) == hard classes (DERIVED, not assumed)\n"
              : "  FAIL wheel(840) != {1,121,169,289,361,529}\n";
  if (!same) ++fails;
  const Wheel w120 = build_wheel(120120, gen_covers(120120), uc);
  check("wheel(120120) F1 only", w120.n_f1_only, 920);
  check("wheel(120120) classes", w120.classes.size(), 220);
  check("wheel(120120) max pmin", w120.max_pmin, 15014);
  const u64 h = fnv64_classes(w120.classes);
  if (h != class_pin(120120)->fnv64) { snprintf(line, sizeof line, "  FAIL wheel(120120) fnv64 %016llx want dbc4ab9b16d73f76\n", h); ++fails; }
  else snprintf(line, sizeof line, "  ok   wheel(120120) fnv64            dbc4ab9b16d73f76\n");
  log += line;
  const Wheel w204 = build_wheel(2042040, gen_wheel_covers(2042040), uc);
  check("wheel(2042040) classes", w204.classes.size(), 2308);
  const u64 h2 = fnv64_classes(w204.classes);
  if (h2 != class_pin(2042040)->fnv64) { snprintf(line, sizeof line, "  FAIL wheel(2042040) fnv64 %016llx want %016llx\n", h2, class_pin(2042040)->fnv64); ++fails; }
  else snprintf(line, sizeof line, "  ok   wheel(2042040) fnv64           %016llx\n", h2);
  log += line;
  auto strays_of = [&](const Wheel &w) {
    u64 strays = 0;
    for (u64 c : w.classes) {
      bool hard = false;
      for (u64 hc : REF840) if (c % 840 == hc) hard = true;
      if (c % 24 != 1 || !hard) ++strays;
    }
    return strays;
  };
  check("wheel(2042040) outside hard class", strays_of(w204), 0);
  check("survivors outside hard class", strays_of(w120), 0);
  return fails;
}

}  // namespace es
