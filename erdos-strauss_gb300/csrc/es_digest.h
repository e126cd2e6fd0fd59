// es_digest.h -- SHA-256 (FIPS 180-4) on the host, for shard metas: the digest of a
// certificate stream that is hashed as it is produced and never stored
// (tools/run19.sh:70-77 records `grep -v '^SUMMARY ' | sha256sum`).
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>

namespace es {

class Sha256 {
 public:
  Sha256();
  void update(const void *data, size_t n);
  void update(const std::string &s) { update(s.data(), s.size()); }
  std::string hex();               // finishes the digest; the object is spent afterwards

 private:
  void block(const uint8_t *p);
  uint32_t h_[8];
  uint8_t buf_[64];
  size_t fill_ = 0;
  uint64_t total_ = 0;
};

}  // namespace es
