// Stand-in for SEP genericCpp's paramObj (test infrastructure only): a
// key -> string map with typed getters; a missing key without a default
// throws, as SEP's does.
#pragma once
#include <map>
#include <string>
#include "SEPException.h"
#include "json/json.h"
namespace SEP {
class paramObj {
 public:
  paramObj() {}
  explicit paramObj(const std::map<std::string, std::string>& kv) : _kv(kv) {}
  void set(const std::string& k, const std::string& v) { _kv[k] = v; }
  int getInt(const std::string& k) const { return std::stoi(need(k)); }
  int getInt(const std::string& k, const int d) const { return has(k) ? std::stoi(_kv.at(k)) : d; }
  float getFloat(const std::string& k) const { return std::stof(need(k)); }
  float getFloat(const std::string& k, const float d) const { return has(k) ? std::stof(_kv.at(k)) : d; }
  std::string getString(const std::string& k) const { return need(k); }
  std::string getString(const std::string& k, const std::string& d) const { return has(k) ? _kv.at(k) : d; }
  bool getBool(const std::string& k) const { return tobool(need(k)); }
  bool getBool(const std::string& k, const bool d) const { return has(k) ? tobool(_kv.at(k)) : d; }

 private:
  bool has(const std::string& k) const { return _kv.count(k) != 0; }
  const std::string& need(const std::string& k) const {
    if (!has(k)) throw SEPException("parameter " + k + " not found");
    return _kv.at(k);
  }
  static bool tobool(const std::string& v) { return v == "1" || v == "true" || v == "True" || v == "y"; }
  std::map<std::string, std::string> _kv;
};
}  // namespace SEP
