// Stand-in for TBB (test infrastructure only).
#pragma once
#include <memory>
namespace tbb {
template <class T>
using cache_aligned_allocator = std::allocator<T>;
}  // namespace tbb
