// Front storage in the arena with contribution blocks given back.
//
// A front is m x m column-major (leading dimension ld) while it is
// assembled and factorized; afterwards only its first nelim columns (the
// factor, read by the solves) must stay, and its trailing columns (the
// contribution block, rows and columns >= nelim) are needed only until the
// parent's extend-add has read them.  Giving those columns back to a free
// list once the parent's level has run keeps the arena near the live size
// of the factorization instead of the sum of all fronts -- the reference
// allocates a front's contribution blocks from a pool and frees them when
// the node is terminated after its parent's assembly
// (src/NumericFront.hxx:299-390 alloc_contrib_blocks / free_contrib_blocks,
// src/kernels/assemble.hxx:216-223 fini_node).
//
// Host-side bookkeeping only: best fit over coalesced free intervals (the
// shortest that fits, the lowest address among equals), then the top of the
// used region.  The free intervals are kept by address (for coalescing) and
// by length (for the fit), so each call costs O(log #intervals): the LDL^T
// factorization places its fronts level by level at factor time, and a
// linear scan over thousands of holes cost milliseconds per factorization.
// All sizes and addresses are in elements, multiples of 64 (every front
// starts on a 64-element boundary).
#pragma once

#include <cstdint>
#include <iterator>
#include <map>
#include <set>
#include <utility>

namespace sylver_gb300 {

class ArenaAlloc {
 public:
  static int64_t round64(int64_t v) { return (v + 63) / 64 * 64; }
  void reset() {
    free_.clear();
    bylen_.clear();
    top_ = 0;
    high_ = 0;
  }
  // start of a block of `size` elements
  int64_t alloc(int64_t size) {
    size = round64(size);
    auto best = bylen_.lower_bound({size, INT64_MIN});
    if (best != bylen_.end()) {
      const int64_t a = best->second, b = a + best->first;
      bylen_.erase(best);
      free_.erase(a);
      if (b > a + size) add(a + size, b);
      return a;
    }
    const int64_t a = top_;
    top_ += size;
    if (top_ > high_) high_ = top_;
    return a;
  }
  // give back [a, b) (a, b multiples of 64); merges with free neighbours
  // and lowers the top when the block ends there
  void release(int64_t a, int64_t b) {
    if (b <= a) return;
    auto next = free_.lower_bound(a);
    if (next != free_.end() && next->first == b) {
      b = next->second;
      bylen_.erase({next->second - next->first, next->first});
      next = free_.erase(next);
    }
    if (next != free_.begin()) {
      auto prev = std::prev(next);
      if (prev->second == a) {
        a = prev->first;
        bylen_.erase({prev->second - prev->first, prev->first});
        free_.erase(prev);
      }
    }
    if (b == top_) {
      top_ = a;
    } else {
      add(a, b);
    }
  }
  int64_t top() const { return top_; }
  int64_t high_water() const { return high_; }

 private:
  void add(int64_t a, int64_t b) {
    free_[a] = b;
    bylen_.insert({b - a, a});
  }
  std::map<int64_t, int64_t> free_;           // start -> end
  std::set<std::pair<int64_t, int64_t>> bylen_;  // (length, start)
  int64_t top_ = 0, high_ = 0;
};

// The part of a front's block given back after its parent's assembly:
// columns [nelim, m) (rounded in to 64-element boundaries).
inline void cb_span(int64_t off, int64_t ld, int64_t m, int64_t nelim, int64_t* a, int64_t* b) {
  *a = ArenaAlloc::round64(off + nelim * ld);
  *b = off + ArenaAlloc::round64(ld * m);
}

}  // namespace sylver_gb300
