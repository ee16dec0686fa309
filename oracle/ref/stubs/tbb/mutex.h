// Stand-in for TBB (test infrastructure only).
#pragma once
#include <mutex>
namespace tbb {
class mutex {
 public:
  class scoped_lock {
   public:
    scoped_lock() : _m(nullptr) {}
    explicit scoped_lock(mutex& m) : _m(&m) { _m->_m.lock(); }
    void acquire(mutex& m) { _m = &m; _m->_m.lock(); }
    void release() { if (_m) _m->_m.unlock(); _m = nullptr; }
    ~scoped_lock() { release(); }

   private:
    mutex* _m;
  };
  void lock() { _m.lock(); }
  void unlock() { _m.unlock(); }

 private:
  std::mutex _m;
};
}  // namespace tbb
