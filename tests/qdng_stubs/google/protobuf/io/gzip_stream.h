// Declarations-only stand-in (see zero_copy_stream.h).
#pragma once
#include "google/protobuf/io/zero_copy_stream.h"
namespace google {
namespace protobuf {
namespace io {
class GzipInputStream : public ZeroCopyInputStream {
 public:
  enum Format { AUTO = 0, GZIP = 1, ZLIB = 2 };
  explicit GzipInputStream(ZeroCopyInputStream *sub_stream, Format format = AUTO, int buffer_size = -1);
  const char *ZlibErrorMessage() const;
  int ZlibErrorCode() const;
  bool Next(const void **data, int *size) override;
  void BackUp(int count) override;
  bool Skip(int count) override;
  int64_t ByteCount() const override;
};
class GzipOutputStream : public ZeroCopyOutputStream {
 public:
  enum Format { GZIP = 1, ZLIB = 2 };
  struct Options {
    Format format = GZIP;
    int buffer_size = 65536;
    int compression_level = -1;
    int compression_strategy = 0;
    Options() {}
  };
  explicit GzipOutputStream(ZeroCopyOutputStream *sub_stream);
  GzipOutputStream(ZeroCopyOutputStream *sub_stream, const Options &options);
  bool Close();
  bool Flush();
  const char *ZlibErrorMessage() const;
  int ZlibErrorCode() const;
  bool Next(void **data, int *size) override;
  void BackUp(int count) override;
  int64_t ByteCount() const override;
};
}  // namespace io
}  // namespace protobuf
}  // namespace google
