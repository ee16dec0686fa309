// Stand-in for jsoncpp (test infrastructure only): parsing always fails, so
// the reference's conformal-map angle file path reports an error.
#pragma once
#include <istream>
#include <string>
namespace Json {
class Value {
 public:
  Value operator[](int) const { return Value(); }
  Value operator[](const char*) const { return Value(); }
  Value operator[](const std::string&) const { return Value(); }
  unsigned size() const { return 0; }
  float asFloat() const { return 0.f; }
};
class Reader {
 public:
  bool parse(std::istream&, Value&) { return false; }
  std::string getFormattedErrorMessages() const { return "json parsing is not available in this build"; }
};
}  // namespace Json
