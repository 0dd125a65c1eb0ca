// Shim for oneTBB's blocked_range (only what the reference uses).
#pragma once
#include <cstddef>

namespace tbb {
template <class T>
class blocked_range {
  public:
    blocked_range(T begin, T end, std::size_t grain = 1) : b_(begin), e_(end), g_(grain ? grain : 1) {}
    T begin() const { return b_; }
    T end() const { return e_; }
    std::size_t size() const { return (std::size_t)(e_ - b_); }
    std::size_t grainsize() const { return g_; }
    bool empty() const { return !(b_ < e_); }

  private:
    T b_, e_;
    std::size_t g_;
};
}  // namespace tbb
