// Declarations-only stand-in (see io/zero_copy_stream.h).
#pragma once
#include <string>
namespace google {
namespace protobuf {
class Message;
class TextFormat {
 public:
  static bool PrintToString(const Message &message, std::string *output);
  static bool ParseFromString(const std::string &input, Message *output);
};
}  // namespace protobuf
}  // namespace google
