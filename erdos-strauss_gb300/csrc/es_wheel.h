// es_wheel.h -- host-side tables of the verification sieve: the certificate families, the
// class table ("wheel") they leave alive mod M, and the filter set the device marks with.
//
// These run once per engine on the host (tens of milliseconds at M = 2042040); the device
// gets only the flattened results.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace es {

typedef unsigned long long u64;

constexpr unsigned UCERT_RMAX = 63, UCERT_UMAX = 64;          // sieve/rung_scan3.cpp:23
constexpr u64 DIRECT_PMAX = 18446744065119617025ull - 2048 - 1;  // sieve/rung_scan3.cpp:42-43

// F1 cover: every p == res (mod mod), p >= pmin, is solved by the (a,c,d) identity with
// m = 4acd - 1 (sieve/rung_scan3.cpp:89-91).
struct Cover { u64 mod, res, pmin; unsigned a, c, d; };
// F2 uniform rung certificate (r, u) forced by p mod L, L = 4 lcm(r,u) (:169-175).
struct Ucert { u64 mod, res; unsigned r, u; };

struct Wheel {
  std::vector<u64> classes;   // surviving unit classes mod M, ascending
  u64 max_pmin = 0;           // over covers with m | M
  u64 n_f1_only = 0;          // unit classes alive after F1 alone
};

// Pinned class-table digests per modulus (sieve/rung_scan3.cpp:57-67).
struct ClassPin { u64 M, fnv64; const char *sha256; };
const ClassPin *class_pin(u64 M);

std::vector<Cover> gen_covers(u64 mmax);                  // :93-112
std::vector<Cover> gen_wheel_covers(u64 M);               // :126-165
std::vector<Ucert> gen_ucerts(unsigned rmax, unsigned umax);   // :177-202
Wheel build_wheel(u64 M, const std::vector<Cover> &cov, const std::vector<Ucert> &uc);  // :211-226
u64 fnv64_classes(const std::vector<u64> &cls);           // :228-236
u64 fnv64_filters(const std::vector<u64> &mods, const std::vector<u64> &ress, size_t ncov);  // :1113-1118
std::vector<u64> small_primes(u64 P, u64 M);              // :664-674
u64 gcd_u64(u64 a, u64 b);
u64 inv_mod(u64 a, u64 m, bool &ok);                      // extended Euclid (inv3, :74-85)

// The class table artifact (--dump-classes, sieve/rung_scan3.cpp:904-953), as text.
std::string class_table_text(u64 M);
// The --verify self-test: the same constants as sieve/rung_scan3.cpp:821-897 checks (the
// divisor-driven covers against the full enumeration, the 840 / 120120 / 2042040 tables and
// their pins, Mordell's hard classes); one pass/FAIL line per check into `log`; returns the
// failure count.
int wheel_self_test(std::string &log);

}  // namespace es
