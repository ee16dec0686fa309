// Stand-in for SEP's exception (test infrastructure only).
#pragma once
#include <stdexcept>
#include <string>
namespace SEP {
class SEPException : public std::runtime_error {
 public:
  explicit SEPException(const std::string& m) : std::runtime_error(m) {}
};
}  // namespace SEP
