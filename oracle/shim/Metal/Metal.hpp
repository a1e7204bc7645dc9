/* Shim: the only part of metal-cpp the reference's host codecs touch is a
 * buffer with host-visible contents. This stand-in wraps caller memory.
 * Test infrastructure only (oracle/_ref). */
#pragma once
#include <cstddef>

namespace MTL {
class Buffer {
 public:
  Buffer(void *data, std::size_t bytes) : data_(data), bytes_(bytes) {}
  void *contents() { return data_; }
  const void *contents() const { return data_; }
  std::size_t length() const { return bytes_; }
  void release() {}

 private:
  void *data_;
  std::size_t bytes_;
};
}  // namespace MTL
