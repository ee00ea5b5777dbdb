// Declarations-only stand-in (see zero_copy_stream.h).
#pragma once
#include <istream>
#include <ostream>
#include "google/protobuf/io/zero_copy_stream.h"
namespace google {
namespace protobuf {
namespace io {
class ArrayInputStream : public ZeroCopyInputStream {
 public:
  ArrayInputStream(const void *data, int size, int block_size = -1);
  bool Next(const void **data, int *size) override;
  void BackUp(int count) override;
  bool Skip(int count) override;
  int64_t ByteCount() const override;
};
class IstreamInputStream : public ZeroCopyInputStream {
 public:
  explicit IstreamInputStream(std::istream *stream, int block_size = -1);
  bool Next(const void **data, int *size) override;
  void BackUp(int count) override;
  bool Skip(int count) override;
  int64_t ByteCount() const override;
};
class OstreamOutputStream : public ZeroCopyOutputStream {
 public:
  explicit OstreamOutputStream(std::ostream *stream, int block_size = -1);
  bool Next(void **data, int *size) override;
  void BackUp(int count) override;
  int64_t ByteCount() const override;
};
}  // namespace io
}  // namespace protobuf
}  // namespace google
