// Declarations-only stand-in for the protoc output of QDng's
// src/qdlib/GridSystem.proto (message GridSystemHeader), written from that
// schema and protobuf's generated accessor names; module compile check only.
#pragma once
#include <cstdint>
#include <string>
namespace QDLIB {
class GridSystemHeader_dim_description_t {
 public:
  uint32_t size() const;
  void set_size(uint32_t v);
  double xmin() const;
  void set_xmin(double v);
  double xmax() const;
  void set_xmax(double v);
};
class GridSystemHeader {
 public:
  typedef GridSystemHeader_dim_description_t dim_description_t;
  uint32_t dims() const;
  void set_dims(uint32_t v);
  int dim_size() const;
  const dim_description_t &dim(int i) const;
  dim_description_t *mutable_dim(int i);
  dim_description_t *add_dim();
  void clear_dim();
  bool has_data_size() const;
  uint64_t data_size() const;
  void set_data_size(uint64_t v);
  void Clear();
  size_t ByteSizeLong() const;
  bool SerializeToString(std::string *output) const;
  bool ParseFromString(const std::string &data);
};
}  // namespace QDLIB
