"""The front-block allocator (sylver_gb300/csrc/arena_alloc.hpp), host only:
random sequences of allocations and releases of contribution-block tails,
checked by a small C++ driver compiled here against the header -- blocks
never overlap, released space is reused (best fit), neighbours coalesce and
the top comes back down when the last block is released."""
import os
import subprocess
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
HDR = os.path.join(HERE, "..", "sylver_gb300", "csrc")

DRIVER = r"""
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>
#include "arena_alloc.hpp"
using namespace sylver_gb300;
struct Blk { int64_t a, b; bool live; };
int main() {
  std::mt19937 g(7);
  ArenaAlloc al;
  std::vector<Blk> blks;
  int64_t reused = 0;
  for (int it = 0; it < 20000; ++it) {
    if (blks.empty() || g() % 3 != 0) {
      int64_t sz = 64 * (1 + g() % 200);
      int64_t top0 = al.top();
      int64_t a = al.alloc(sz);
      if (a % 64) { printf("misaligned\n"); return 1; }
      if (a + sz <= top0) reused++;
      for (const Blk& q : blks)
        if (q.live && a < q.b && q.a < a + sz) { printf("overlap\n"); return 1; }
      blks.push_back({a, a + sz, true});
    } else {
      Blk& q = blks[g() % blks.size()];
      if (!q.live) continue;
      // give back a tail (the contribution block) or the whole block
      int64_t keep = 64 * (g() % ((q.b - q.a) / 64 + 1));
      al.release(q.a + keep, q.b);
      if (keep == 0) q.live = false; else q.b = q.a + keep;
    }
  }
  // release everything: the top must return to zero
  for (Blk& q : blks) if (q.live) al.release(q.a, q.b);
  if (al.top() != 0) { printf("top %lld\n", (long long)al.top()); return 1; }
  printf("ok %lld %lld\n", (long long)reused, (long long)al.high_water());
  return reused > 0 ? 0 : 1;
}
"""


def test_arena_alloc_random_sequences():
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "t.cpp")
        open(src, "w").write(DRIVER)
        exe = os.path.join(d, "t")
        subprocess.run(["g++", "-std=c++17", "-O1", "-I", HDR, src, "-o", exe], check=True)
        r = subprocess.run([exe], capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
        assert r.stdout.startswith("ok")
