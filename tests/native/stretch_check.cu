// Host-only check of the tensor-core half-step's work partition
// (tc_stretch_begin / tc_cta_of in wotg_onthefly.cuh): for many grid shapes,
// replays the kernel's walk over (row tile, column tile) pairs and the
// combine's lookup, and checks that every (CTA, row tile) partial slot is
// unique and inside the (CTAs + row tiles) x 128 buffer, and that the merge
// of each row tile reads exactly the CTAs that wrote a partial for it. The
// in-kernel finish (CombineFin) counts 2 x (hi - lo + 1) partials per lane
// quarter of a row tile (two column-half warps per covering CTA), so check 5
// below is also the check of its expected count. Runs on the CPU; launches
// nothing.
#include <cstdio>
#include <set>
#include <vector>

#include "wotg_onthefly.cuh"

using wotg::tc_cta_of;
using wotg::tc_stretch_begin;

static int check(int64_t n_pt, int64_t nq, int64_t ctas) {
  const int64_t total = n_pt * nq;
  std::vector<std::set<int64_t>> writers(n_pt);
  std::set<int64_t> slots;
  for (int64_t c = 0; c < ctas; ++c) {
    const int64_t f0 = tc_stretch_begin(c, total, ctas), f1 = tc_stretch_begin(c + 1, total, ctas);
    const int64_t n = f1 - f0;
    if (n < 1) return 1;                                   // every CTA has work when ctas <= total
    int64_t t = f0 / nq, q = f0 % nq;
    for (int64_t j = 0; j < n; ++j) {                      // the epilogue's walk
      if (++q == nq || j == n - 1) {
        const int64_t slot = c + t;
        if (slot < 0 || slot >= ctas + n_pt) return 2;     // buffer bound
        if (!slots.insert(slot).second) return 3;         // no two (CTA, tile) share a slot
        if (!writers[t].insert(c).second) return 4;        // one partial per (CTA, tile)
        if (q == nq) {
          q = 0;
          ++t;
        }
      }
    }
  }
  std::set<int64_t> used;
  for (int64_t t = 0; t < n_pt; ++t) {                     // the combine's lookup
    const int64_t lo = tc_cta_of(t * nq, total, ctas), hi = tc_cta_of((t + 1) * nq - 1, total, ctas);
    if ((int64_t)writers[t].size() != hi - lo + 1) return 5;
    for (int64_t c = lo; c <= hi; ++c) {
      if (!writers[t].count(c)) return 6;
      if (!used.insert(c + t).second) return 7;            // slots of different tiles never alias
    }
  }
  return 0;
}

int main() {
  const int64_t shapes[][2] = {{1, 1}, {1, 7}, {7, 1}, {3, 5}, {157, 196}, {196, 157}, {469, 469},
                               {63, 79}, {2, 300}, {300, 2}, {40, 40}};
  const int64_t grids[] = {1, 2, 3, 151, 152, 303, 304, 608, 1000};
  int cases = 0;
  for (const auto& s : shapes)
    for (int64_t g : grids) {
      const int64_t ctas = g < s[0] * s[1] ? g : s[0] * s[1];
      const int r = check(s[0], s[1], ctas);
      ++cases;
      if (r) {
        std::printf("FAIL n_pt=%lld nq=%lld ctas=%lld code=%d\n", (long long)s[0], (long long)s[1],
                    (long long)ctas, r);
        return 1;
      }
    }
  std::printf("ok %d\n", cases);
  return 0;
}
