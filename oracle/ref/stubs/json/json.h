// Stand-in for jsoncpp (test infrastructure only): enough of Json::Value and
// Json::Reader for the reference's geometry and rotation-angle files, JSON
// objects whose members are numbers or arrays of numbers
// ({"sx": [..], "sz": [..], "a": [..]}).
#pragma once
#include <cctype>
#include <cstdlib>
#include <istream>
#include <iterator>
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace Json {

class Value {
 public:
  Value() {}
  explicit Value(double v) : _num(v), _isnum(true) {}
  // array element / object member; absent ones are null values
  Value operator[](int i) const { return i >= 0 && i < (int)_arr.size() ? _arr[i] : Value(); }
  Value operator[](unsigned i) const { return (*this)[(int)i]; }
  Value operator[](const char* k) const { return (*this)[std::string(k)]; }
  Value operator[](const std::string& k) const {
    auto it = _obj.find(k);
    return it == _obj.end() ? Value() : it->second;
  }
  unsigned size() const { return (unsigned)(_isarr ? _arr.size() : _obj.size()); }
  float asFloat() const { return (float)_num; }
  double asDouble() const { return _num; }
  int asInt() const { return (int)_num; }

 private:
  friend class Reader;
  double _num = 0.0;
  bool _isnum = false, _isarr = false;
  std::vector<Value> _arr;
  std::map<std::string, Value> _obj;
};

class Reader {
 public:
  bool parse(std::istream& in, Value& root) {
    _s.assign(std::istreambuf_iterator<char>(in), std::istreambuf_iterator<char>());
    _i = 0;
    _err.clear();
    if (!value(root)) return false;
    ws();
    if (_i != _s.size()) return fail("trailing characters");
    return true;
  }
  std::string getFormattedErrorMessages() const { return _err; }

 private:
  std::string _s, _err;
  size_t _i = 0;
  bool fail(const std::string& m) {
    _err = "json: " + m + " at offset " + std::to_string(_i);
    return false;
  }
  void ws() {
    while (_i < _s.size() && std::isspace((unsigned char)_s[_i])) ++_i;
  }
  bool value(Value& v) {
    ws();
    if (_i >= _s.size()) return fail("unexpected end");
    const char c = _s[_i];
    if (c == '{') return object(v);
    if (c == '[') return array(v);
    if (c == '-' || c == '+' || c == '.' || std::isdigit((unsigned char)c)) {
      char* end = nullptr;
      const double d = std::strtod(_s.c_str() + _i, &end);
      if (end == _s.c_str() + _i) return fail("bad number");
      _i = (size_t)(end - _s.c_str());
      v = Value(d);
      return true;
    }
    return fail("unsupported value");
  }
  bool string(std::string& out) {
    ws();
    if (_i >= _s.size() || _s[_i] != '"') return fail("expected a string");
    const size_t e = _s.find('"', _i + 1);
    if (e == std::string::npos) return fail("unterminated string");
    out = _s.substr(_i + 1, e - _i - 1);
    _i = e + 1;
    return true;
  }
  bool array(Value& v) {
    v = Value();
    v._isarr = true;
    ++_i;
    ws();
    if (_i < _s.size() && _s[_i] == ']') { ++_i; return true; }
    for (;;) {
      Value e;
      if (!value(e)) return false;
      v._arr.push_back(e);
      ws();
      if (_i < _s.size() && _s[_i] == ',') { ++_i; continue; }
      if (_i < _s.size() && _s[_i] == ']') { ++_i; return true; }
      return fail("expected , or ]");
    }
  }
  bool object(Value& v) {
    v = Value();
    ++_i;
    ws();
    if (_i < _s.size() && _s[_i] == '}') { ++_i; return true; }
    for (;;) {
      std::string k;
      if (!string(k)) return false;
      ws();
      if (_i >= _s.size() || _s[_i] != ':') return fail("expected :");
      ++_i;
      Value e;
      if (!value(e)) return false;
      v._obj[k] = e;
      ws();
      if (_i < _s.size() && _s[_i] == ',') { ++_i; continue; }
      if (_i < _s.size() && _s[_i] == '}') { ++_i; return true; }
      return fail("expected , or }");
    }
  }
};

}  // namespace Json
