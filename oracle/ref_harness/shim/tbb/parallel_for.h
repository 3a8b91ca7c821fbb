/* Minimal serial stand-in for the two oneTBB names the reference's PLOC
 * build uses (blocked_range, parallel_for).  Serial execution gives the same
 * result as any chunking: every cached distance equals the recomputed one. */
#pragma once
#include <cstddef>

namespace tbb {
template <class T>
class blocked_range {
 public:
  blocked_range(T b, T e) : b_(b), e_(e) {}
  T begin() const { return b_; }
  T end() const { return e_; }

 private:
  T b_, e_;
};

template <class Range, class Body>
void parallel_for(const Range& range, const Body& body) {
  Range r = range;
  body(r);
}
}  // namespace tbb
