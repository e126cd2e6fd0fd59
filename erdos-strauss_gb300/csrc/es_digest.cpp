// es_digest.cpp -- SHA-256 as FIPS 180-4 specifies it: 64-byte blocks, a 64-word message
// schedule, 64 rounds over eight 32-bit working variables, length-padded final block.
#include "es_digest.h"

#include "../../include/es_sieve.h"

#include <dlfcn.h>

#include <cstdlib>
#include <cstring>
#include <mutex>

namespace es {
namespace {
// Round constants: the first 32 bits of the fractional parts of the cube roots of the first
// 64 primes (FIPS 180-4, 4.2.2).
const uint32_t K[64] = {
    0x428a2f98, 0x71374491, 0xb5c0fbcf, 0xe9b5dba5, 0x3956c25b, 0x59f111f1, 0x923f82a4, 0xab1c5ed5,
    0xd807aa98, 0x12835b01, 0x243185be, 0x550c7dc3, 0x72be5d74, 0x80deb1fe, 0x9bdc06a7, 0xc19bf174,
    0xe49b69c1, 0xefbe4786, 0x0fc19dc6, 0x240ca1cc, 0x2de92c6f, 0x4a7484aa, 0x5cb0a9dc, 0x76f988da,
    0x983e5152, 0xa831c66d, 0xb00327c8, 0xbf597fc7, 0xc6e00bf3, 0xd5a79147, 0x06ca6351, 0x14292967,
    0x27b70a85, 0x2e1b2138, 0x4d2c6dfc, 0x53380d13, 0x650a7354, 0x766a0abb, 0x81c2c92e, 0x92722c85,
    0xa2bfe8a1, 0xa81a664b, 0xc24b8b70, 0xc76c51a3, 0xd192e819, 0xd6990624, 0xf40e3585, 0x106aa070,
    0x19a4c116, 0x1e376c08, 0x2748774c, 0x34b0bcb5, 0x391c0cb3, 0x4ed8aa4a, 0x5b9cca4f, 0x682e6ff3,
    0x748f82ee, 0x78a5636f, 0x84c87814, 0x8cc70208, 0x90befffa, 0xa4506ceb, 0xbef9a3f7, 0xc67178f2};

inline uint32_t rotr(uint32_t x, int n) { return (x >> n) | (x << (32 - n)); }

// libcrypto's EVP interface, resolved once at run time (no link-time dependency).
struct Evp {
  void *(*ctx_new)() = nullptr;
  void (*ctx_free)(void *) = nullptr;
  const void *(*sha256)() = nullptr;
  int (*init)(void *, const void *, void *) = nullptr;
  int (*update)(void *, const void *, size_t) = nullptr;
  int (*final)(void *, unsigned char *, unsigned int *) = nullptr;
  bool ok = false;
};

const Evp &evp() {
  static Evp E;
  static std::once_flag once;
  std::call_once(once, [] {
    if (getenv("ES_SHA256_BUILTIN")) return;
    void *h = nullptr;
    for (const char *name : {"libcrypto.so.3", "libcrypto.so.1.1", "libcrypto.so"})
      if ((h = dlopen(name, RTLD_NOW | RTLD_LOCAL))) break;
    if (!h) return;
    E.ctx_new = reinterpret_cast<void *(*)()>(dlsym(h, "EVP_MD_CTX_new"));
    E.ctx_free = reinterpret_cast<void (*)(void *)>(dlsym(h, "EVP_MD_CTX_free"));
    E.sha256 = reinterpret_cast<const void *(*)()>(dlsym(h, "EVP_sha256"));
    E.init = reinterpret_cast<int (*)(void *, const void *, void *)>(dlsym(h, "EVP_DigestInit_ex"));
    E.update = reinterpret_cast<int (*)(void *, const void *, size_t)>(dlsym(h, "EVP_DigestUpdate"));
    E.final = reinterpret_cast<int (*)(void *, unsigned char *, unsigned int *)>(dlsym(h, "EVP_DigestFinal_ex"));
    E.ok = E.ctx_new && E.ctx_free && E.sha256 && E.init && E.update && E.final;
  });
  return E;
}
}  // namespace

const char *Sha256::backend() { return evp().ok ? "libcrypto" : "builtin"; }

Sha256::~Sha256() {
  if (ctx_) evp().ctx_free(ctx_);
}

Sha256::Sha256() {
  const Evp &E = evp();
  if (E.ok && (ctx_ = E.ctx_new()) != nullptr && E.init(ctx_, E.sha256(), nullptr) != 1) {
    E.ctx_free(ctx_);
    ctx_ = nullptr;
  }
  // initial hash: the first 32 bits of the fractional parts of the square roots of the first
  // eight primes (FIPS 180-4, 5.3.3)
  const uint32_t h0[8] = {0x6a09e667, 0xbb67ae85, 0x3c6ef372, 0xa54ff53a,
                          0x510e527f, 0x9b05688c, 0x1f83d9ab, 0x5be0cd19};
  memcpy(h_, h0, sizeof h_);
}

void Sha256::block(const uint8_t *p) {
  // 16-word circular message schedule, eight rounds per step with the working variables
  // renamed instead of shifted
  uint32_t w[16];
  for (int t = 0; t < 16; ++t)
    w[t] = (uint32_t)p[4 * t] << 24 | (uint32_t)p[4 * t + 1] << 16 | (uint32_t)p[4 * t + 2] << 8 | p[4 * t + 3];
  uint32_t a = h_[0], b = h_[1], c = h_[2], d = h_[3], e = h_[4], f = h_[5], g = h_[6], h = h_[7];
#define ES_SHA_ROUND(a, b, c, d, e, f, g, h, t)                                                        \
  {                                                                                                   \
    uint32_t wt;                                                                                      \
    if ((t) < 16) wt = w[(t)];                                                                        \
    else {                                                                                            \
      const uint32_t w15 = w[((t) - 15) & 15], w2 = w[((t) - 2) & 15];                               \
      wt = w[(t) & 15] += (rotr(w15, 7) ^ rotr(w15, 18) ^ (w15 >> 3)) + w[((t) - 7) & 15] +          \
                         (rotr(w2, 17) ^ rotr(w2, 19) ^ (w2 >> 10));                                  \
    }                                                                                                 \
    const uint32_t t1 = h + (rotr(e, 6) ^ rotr(e, 11) ^ rotr(e, 25)) + ((e & f) ^ (~e & g)) + K[(t)] + wt; \
    const uint32_t t2 = (rotr(a, 2) ^ rotr(a, 13) ^ rotr(a, 22)) + ((a & b) ^ (a & c) ^ (b & c));    \
    d += t1;                                                                                          \
    h = t1 + t2;                                                                                      \
  }
  for (int t = 0; t < 64; t += 8) {
    ES_SHA_ROUND(a, b, c, d, e, f, g, h, t + 0)
    ES_SHA_ROUND(h, a, b, c, d, e, f, g, t + 1)
    ES_SHA_ROUND(g, h, a, b, c, d, e, f, t + 2)
    ES_SHA_ROUND(f, g, h, a, b, c, d, e, t + 3)
    ES_SHA_ROUND(e, f, g, h, a, b, c, d, t + 4)
    ES_SHA_ROUND(d, e, f, g, h, a, b, c, t + 5)
    ES_SHA_ROUND(c, d, e, f, g, h, a, b, t + 6)
    ES_SHA_ROUND(b, c, d, e, f, g, h, a, t + 7)
  }
#undef ES_SHA_ROUND
  h_[0] += a; h_[1] += b; h_[2] += c; h_[3] += d; h_[4] += e; h_[5] += f; h_[6] += g; h_[7] += h;
}

void Sha256::update(const void *data, size_t n) {
  if (ctx_) { evp().update(ctx_, data, n); return; }
  const uint8_t *p = static_cast<const uint8_t *>(data);
  total_ += n;
  if (fill_) {
    const size_t take = n < 64 - fill_ ? n : 64 - fill_;
    memcpy(buf_ + fill_, p, take);
    fill_ += take; p += take; n -= take;
    if (fill_ < 64) return;
    block(buf_);
    fill_ = 0;
  }
  for (; n >= 64; p += 64, n -= 64) block(p);
  if (n) { memcpy(buf_, p, n); fill_ = n; }
}

std::string Sha256::hex() {
  static const char *hx = "0123456789abcdef";
  if (ctx_) {
    unsigned char md[32];
    unsigned int len = 0;
    evp().final(ctx_, md, &len);
    std::string out(64, '0');
    for (int i = 0; i < 32; ++i) { out[2 * i] = hx[md[i] >> 4]; out[2 * i + 1] = hx[md[i] & 15]; }
    return out;
  }
  const uint64_t bits = total_ * 8;
  const uint8_t one = 0x80, zero = 0;
  update(&one, 1);
  while (fill_ != 56) update(&zero, 1);
  uint8_t len[8];
  for (int i = 0; i < 8; ++i) len[i] = (uint8_t)(bits >> (56 - 8 * i));
  update(len, 8);
  std::string out(64, '0');
  for (int i = 0; i < 8; ++i)
    for (int j = 0; j < 8; ++j) out[8 * i + j] = hx[(h_[i] >> (28 - 4 * j)) & 15];
  return out;
}

}  // namespace es

extern "C" size_t es_sha256_hex(const void *data, size_t n, char *out, size_t cap) {
  if (!out || cap < 65 || (!data && n)) return 0;
  es::Sha256 h;
  h.update(data, n);
  const std::string s = h.hex();
  memcpy(out, s.c_str(), 65);
  return 64;
}
