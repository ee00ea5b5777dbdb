// Declarations-only stand-in for protobuf's zero-copy stream interface,
// enough for QDng's headers to compile in the module compile check.  Written
// from protobuf's documented public API; nothing is linked or run.
#pragma once
#include <cstdint>
namespace google {
namespace protobuf {
namespace io {
class ZeroCopyInputStream {
 public:
  virtual ~ZeroCopyInputStream() {}
  virtual bool Next(const void **data, int *size) = 0;
  virtual void BackUp(int count) = 0;
  virtual bool Skip(int count) = 0;
  virtual int64_t ByteCount() const = 0;
};
class ZeroCopyOutputStream {
 public:
  virtual ~ZeroCopyOutputStream() {}
  virtual bool Next(void **data, int *size) = 0;
  virtual void BackUp(int count) = 0;
  virtual int64_t ByteCount() const = 0;
};
}  // namespace io
}  // namespace protobuf
}  // namespace google
