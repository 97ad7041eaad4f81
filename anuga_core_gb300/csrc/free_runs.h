// free_runs.h -- free extents of a resource (the pool's tiles, boundary
// slots and halo slots), kept as runs so that allocation, release and the
// largest free run do not scan the resource.
#pragma once
#include <algorithm>
#include <cstdint>
#include <iterator>
#include <map>

namespace agx {

// Free extents of one pool resource (tiles, boundary slots, halo slots) as
// start -> length runs, so that allocation (first fit, lowest start), release
// and the largest free run cost O(runs) instead of a scan of the resource.
class FreeRuns {
 public:
  void init(int64_t n) {
    runs_.clear();
    if (n > 0) runs_[0] = n;
    size_ = n;
  }
  // lowest start of a free run of len units, or -1
  int64_t find(int64_t len) const {
    for (const auto& r : runs_)
      if (r.second >= len) return r.first;
    return -1;
  }
  // marks [start, start + len) used; it lies inside one free run (find)
  void take(int64_t start, int64_t len) {
    auto it = runs_.upper_bound(start);
    --it;
    const int64_t s0 = it->first, l0 = it->second;
    runs_.erase(it);
    if (start > s0) runs_[s0] = start - s0;
    if (s0 + l0 > start + len) runs_[start + len] = s0 + l0 - (start + len);
  }
  // marks [start, start + len) free again, merged with its free neighbours
  void give(int64_t start, int64_t len) {
    if (len <= 0) return;
    auto next = runs_.lower_bound(start);
    if (next != runs_.end() && next->first == start + len) {
      len += next->second;
      next = runs_.erase(next);
    }
    if (next != runs_.begin()) {
      auto prev = std::prev(next);
      if (prev->first + prev->second == start) {
        prev->second += len;
        return;
      }
    }
    runs_[start] = len;
  }
  int64_t largest() const {
    int64_t m = 0;
    for (const auto& r : runs_) m = std::max(m, r.second);
    return m;
  }
  // one past the last used unit (0 when all are free)
  int64_t used_end() const {
    if (runs_.empty()) return size_;
    const auto& last = *runs_.rbegin();
    return last.first + last.second == size_ ? last.first : size_;
  }

 private:
  std::map<int64_t, int64_t> runs_;
  int64_t size_ = 0;
};

}  // namespace agx
