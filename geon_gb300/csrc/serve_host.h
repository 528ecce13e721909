// Host-side parts of the serving engine that need no GPU (plain C++; the CPU
// tests compile this header with g++): the first-fit arena bookkeeping, the
// bisection round's speculative tree, and the shortest-remaining-first claim
// order of each ray class.
#pragma once
#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <iterator>
#include <map>
#include <vector>

namespace geon {
namespace serve_host {

constexpr size_t ALIGN = 256;
inline size_t rup(size_t n) { return (n + ALIGN - 1) & ~(ALIGN - 1); }

// First-fit allocator over the device arena (host bookkeeping only).
class Arena {
 public:
  void init(size_t n) {
    free_.clear();
    free_[0] = n;
  }
  bool alloc(size_t n, size_t* off) {
    n = rup(n ? n : 1);
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= n) {
        const size_t o = it->first, rem = it->second - n;
        free_.erase(it);
        if (rem) free_[o + n] = rem;
        *off = o;
        return true;
      }
    }
    return false;
  }
  void release(size_t off, size_t n) {
    n = rup(n ? n : 1);
    auto it = free_.emplace(off, n).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }

 private:
  std::map<size_t, size_t> free_;
};

// One job of the claim order: its ray class, rays not yet claimed, arrival id
// (the tie-break) and job slot.
struct ClaimEntry {
  int cls;
  int64_t left;
  uint64_t id;
  int slot;
};

// The claim order of every class for the next launch: jobs with unclaimed
// rays, fewest unclaimed first (arrival order on ties), so a small request is
// not queued behind a large one; rays already in flight continue first. Writes
// class c's slots to out[c * stride ...] and their number to counts[c].
inline void claim_order(const std::vector<ClaimEntry>& entries, int nclasses, size_t stride, int* out,
                        unsigned* counts) {
  std::vector<std::vector<std::pair<std::pair<int64_t, uint64_t>, int>>> order((size_t)nclasses);
  for (const ClaimEntry& e : entries)
    if (e.left > 0 && e.cls >= 0 && e.cls < nclasses) order[(size_t)e.cls].push_back({{e.left, e.id}, e.slot});
  for (int c = 0; c < nclasses; ++c) {
    auto& o = order[(size_t)c];
    std::sort(o.begin(), o.end());
    const size_t n = std::min(o.size(), stride);
    for (size_t i = 0; i < n; ++i) out[(size_t)c * stride + i] = o[i].second;
    counts[c] = (unsigned)n;
  }
}

// Midpoints of the next `levels` halvings of [lo, hi] in heap order (node i at
// index i-1, children 2i = [lo, mid] and 2i+1 = [mid, hi]), each 0.5*(lo+hi)
// exactly as the sequential loop forms it.
inline void bisect_tree(double lo, double hi, int levels, std::vector<double>& a) {
  const int64_t per = ((int64_t)1 << levels) - 1;
  a.assign(per, 0.0);
  std::vector<double> nl(per), nh(per);
  nl[0] = lo;
  nh[0] = hi;
  for (int64_t i = 1; i <= per; ++i) {
    const double l = nl[i - 1], h = nh[i - 1], mid = 0.5 * (l + h);
    a[i - 1] = mid;
    if (2 * i <= per) {
      nl[2 * i - 1] = l;
      nh[2 * i - 1] = mid;
    }
    if (2 * i + 1 <= per) {
      nl[2 * i] = mid;
      nh[2 * i] = h;
    }
  }
}

}  // namespace serve_host
}  // namespace geon
