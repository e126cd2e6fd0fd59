// es_digest.h -- SHA-256 (FIPS 180-4) on the host, for shard metas: the digest of a
// certificate stream that is hashed as it is produced and never stored
// (tools/run19.sh:70-77 records `grep -v '^SUMMARY ' | sha256sum`).
//
// Two interchangeable backends give the same digest: the system's libcrypto (OpenSSL,
// loaded at run time when present; it uses the CPU's SHA instructions), and the
// implementation in es_digest.cpp, used when libcrypto is absent or when the environment
// variable ES_SHA256_BUILTIN is set.
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>

namespace es {

class Sha256 {
 public:
  Sha256();
  ~Sha256();
  Sha256(const Sha256 &) = delete;
  Sha256 &operator=(const Sha256 &) = delete;
  void update(const void *data, size_t n);
  void update(const std::string &s) { update(s.data(), s.size()); }
  std::string hex();               // finishes the digest; the object is spent afterwards
  static const char *backend();    // "libcrypto" or "builtin"

 private:
  void block(const uint8_t *p);
  void *ctx_ = nullptr;            // libcrypto context, or null for the built-in
  uint32_t h_[8];
  uint8_t buf_[64];
  size_t fill_ = 0;
  uint64_t total_ = 0;
};

}  // namespace es
