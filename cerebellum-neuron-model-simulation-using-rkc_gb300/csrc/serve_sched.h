// Host-side bookkeeping of the request server (server.cpp), free of CUDA so
// that it builds and is tested on any host: the slot arena of one system
// shape, the admission queue, and latency percentiles.
//
// A slot arena is a fixed run of built systems of one shape (one pool run of
// the engine).  Requests take slots as a few runs of consecutive slots --
// one run when a long enough gap exists (first fit), otherwise gaps in
// address order -- so that resetting and reading a request costs a few bulk
// copies per run, not per system.
#pragma once

#include <algorithm>
#include <cmath>
#include <deque>
#include <map>
#include <utility>
#include <vector>

namespace gbrkc {
namespace serve {

using Run = std::pair<int, int>;  // (first slot, count)

class SlotArena {
 public:
  explicit SlotArena(int n = 0) : cap_(n), free_count_(n) {
    if (n > 0) free_[0] = n;
  }
  int capacity() const { return cap_; }
  int free_slots() const { return free_count_; }
  int gaps() const { return (int)free_.size(); }

  // Take n slots; false (and nothing taken) if fewer are free.
  bool alloc(int n, std::vector<Run> &runs) {
    runs.clear();
    if (n <= 0 || n > free_count_) return false;
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= n) {  // first fit in one run
        take(it, n, runs);
        return true;
      }
    }
    int left = n;
    while (left > 0) {  // gaps in address order
      auto it = free_.begin();
      const int k = std::min(left, it->second);
      take(it, k, runs);
      left -= k;
    }
    return true;
  }

  // Return runs taken by alloc (merging neighbouring gaps).
  void release(const std::vector<Run> &runs) {
    for (const Run &r : runs) {
      int first = r.first, len = r.second;
      auto next = free_.lower_bound(first);
      if (next != free_.begin()) {
        auto prev = std::prev(next);
        if (prev->first + prev->second == first) {
          first = prev->first;
          len += prev->second;
          free_.erase(prev);
        }
      }
      next = free_.lower_bound(first);
      if (next != free_.end() && next->first == first + len) {
        len += next->second;
        free_.erase(next);
      }
      free_[first] = len;
      free_count_ += r.second;
    }
  }

 private:
  void take(std::map<int, int>::iterator it, int k, std::vector<Run> &runs) {
    const int first = it->first, len = it->second;
    free_.erase(it);
    if (len > k) free_[first + k] = len - k;
    runs.push_back({first, k});
    free_count_ -= k;
  }
  int cap_;
  int free_count_;
  std::map<int, int> free_;  // gap start -> length
};

// Admission order within one arena: first come, first served, with
// backfilling -- a later request that fits may go ahead of a head that does
// not, until the head has been passed over max_bypass times; from then on
// nothing overtakes it (no starvation of large requests).
class Admission {
 public:
  explicit Admission(int max_bypass = 8) : max_bypass_(max_bypass) {}
  void push(int req) { q_.push_back({req, 0}); }
  bool empty() const { return q_.empty(); }
  int size() const { return (int)q_.size(); }
  bool remove(int req) {
    for (auto it = q_.begin(); it != q_.end(); ++it)
      if (it->first == req) {
        q_.erase(it);
        return true;
      }
    return false;
  }

  // Admit what fits, in order: fits(req) takes the slots and says whether
  // it did.  Returns the admitted requests.
  template <class Fits>
  std::vector<int> admit(Fits fits) {
    std::vector<int> out;
    while (!q_.empty() && fits(q_.front().first)) {
      out.push_back(q_.front().first);
      q_.pop_front();
    }
    if (q_.empty() || q_.front().second >= max_bypass_) return out;
    bool passed = false;
    for (auto it = std::next(q_.begin()); it != q_.end();) {
      if (fits(it->first)) {
        out.push_back(it->first);
        it = q_.erase(it);
        passed = true;
      } else {
        ++it;
      }
    }
    if (passed) q_.front().second++;
    return out;
  }

 private:
  int max_bypass_;
  std::deque<std::pair<int, int>> q_;  // (request, times the head was passed over)
};

// Nearest-rank percentile (p in [0, 100]) of a sample; 0 for an empty one.
inline double percentile(std::vector<double> v, double p) {
  if (v.empty()) return 0.0;
  std::sort(v.begin(), v.end());
  const double r = std::ceil(p / 100.0 * (double)v.size());
  const long k = std::min<long>((long)v.size() - 1, std::max<long>(0, (long)r - 1));
  return v[k];
}

}  // namespace serve
}  // namespace gbrkc
