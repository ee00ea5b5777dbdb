// Declarations-only stand-in for the protoc output of QDng's
// src/tools/FileSingleHeader.proto, written from that schema and the
// accessor names protobuf generates; for the module compile check only.
#pragma once
#include <cstdint>
#include <istream>
#include <ostream>
#include <string>
#include "google/protobuf/io/zero_copy_stream.h"
namespace QDLIB {
enum FileSingleHeader_Compression {
  FileSingleHeader_Compression_UNCOMPRESSED = 0,
  FileSingleHeader_Compression_ZLIB = 1,
  FileSingleHeader_Compression_BZIP = 2
};
class FileSingleHeader {
 public:
  typedef FileSingleHeader_Compression Compression;
  static const Compression UNCOMPRESSED = FileSingleHeader_Compression_UNCOMPRESSED;
  static const Compression ZLIB = FileSingleHeader_Compression_ZLIB;
  static const Compression BZIP = FileSingleHeader_Compression_BZIP;
  void Clear();
  size_t ByteSizeLong() const;
  int ByteSize() const;
  bool IsInitialized() const;
  bool SerializeToOstream(std::ostream *output) const;
  bool ParseFromIstream(std::istream *input);
  bool ParseFromArray(const void *data, int size);
  bool SerializeToArray(void *data, int size) const;
  bool SerializeToString(std::string *output) const;
  bool ParseFromString(const std::string &data);
  bool SerializeToZeroCopyStream(google::protobuf::io::ZeroCopyOutputStream *output) const;
  bool ParseFromZeroCopyStream(google::protobuf::io::ZeroCopyInputStream *input);
  bool more_files_follow() const;
  void set_more_files_follow(bool v);
  const std::string &class_() const;
  void set_class_(const std::string &v);
  bool has_name() const;
  const std::string &name() const;
  void set_name(const std::string &v);
  bool has_sequence_number() const;
  uint32_t sequence_number() const;
  void set_sequence_number(uint32_t v);
  bool has_meta_data() const;
  const std::string &meta_data() const;
  void set_meta_data(const std::string &v);
  uint64_t payload_size() const;
  void set_payload_size(uint64_t v);
  Compression compression() const;
  void set_compression(Compression v);
  bool has_sub_header() const;
  const std::string &sub_header() const;
  void set_sub_header(const std::string &v);
};
class MultiStateIdentifier {
 public:
  int32_t state() const;
  void set_state(int32_t v);
  bool SerializeToString(std::string *output) const;
  bool ParseFromString(const std::string &data);
};
}  // namespace QDLIB
