// Stand-in for sepVector's Vector base (test infrastructure only).
#pragma once
#include <string>
namespace SEP {
class Vector {
 public:
  virtual ~Vector() {}
  bool spaceOnly() const { return _spaceOnly; }
  void setSpace() { _spaceOnly = true; }
  void setNotSpace() { _spaceOnly = false; }

 protected:
  bool _spaceOnly = true;
  std::string _vecType;
};
}  // namespace SEP
