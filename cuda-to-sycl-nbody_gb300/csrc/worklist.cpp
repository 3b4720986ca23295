// Stream-K work-list planner.
//
// The unit of work is one (system, i-tile, j-tile) block of bi x |j-tile| pair
// interactions.  Units are laid out in (system, i-tile, j-tile) order and each
// is charged its j-tile length.  CTA k receives the units whose starting charge
// c satisfies floor(c * grid / total) == k, i.e. one contiguous run of the
// sequence with total / grid charge (+- one tile).  A run that covers only part
// of an i-tile's j-range becomes a "part" of a fixup record: the kernel sums the
// parts in j order once the last one has arrived.
#include "worklist.hpp"

#include <algorithm>

namespace nbg {

WorkListHost plan_worklist(const SystemDesc* sys, int32_t first, int32_t count, int32_t bi,
                           int32_t bj, int32_t max_grid) {
  WorkListHost wl;
  int64_t total = 0, tiles = 0;
  for (int32_t s = first; s < first + count; ++s) {
    const int64_t nit = (sys[s].n + bi - 1) / bi;
    const int64_t njt = (sys[s].npad + bj - 1) / bj;
    total += nit * sys[s].npad;
    tiles += nit * njt;
  }
  const int64_t grid = std::max<int64_t>(1, std::min<int64_t>(max_grid, tiles));
  wl.grid = static_cast<int32_t>(grid);
  wl.seg_begin.assign(grid + 1, 0);

  // CTA owning the unit whose charge starts at c.
  auto owner = [&](int64_t c) { return std::min<int64_t>(grid - 1, (c * grid) / total); };

  int64_t c0 = 0;          // charge before the current i-tile
  int64_t next_cta = 0;    // first CTA whose seg_begin is not yet set
  for (int32_t s = first; s < first + count; ++s) {
    const int32_t nit = (sys[s].n + bi - 1) / bi;
    const int32_t njt = (sys[s].npad + bj - 1) / bj;
    for (int32_t it = 0; it < nit; ++it) {
      const size_t seg_first = wl.segs.size();
      int32_t t = 0;
      while (t < njt) {
        const int64_t k = owner(c0 + static_cast<int64_t>(t) * bj);
        // First tile owned by a later CTA: smallest t' with (c0 + t' bj) grid >= (k+1) total.
        int64_t t_end = njt;
        if (k + 1 < grid) {
          const int64_t need = (k + 1) * total - c0 * grid;  // > t*bj*grid
          t_end = (need + static_cast<int64_t>(bj) * grid - 1) / (static_cast<int64_t>(bj) * grid);
          t_end = std::min<int64_t>(std::max<int64_t>(t_end, t + 1), njt);
        }
        while (next_cta <= k) wl.seg_begin[next_cta++] = static_cast<int32_t>(wl.segs.size());
        wl.segs.push_back(Segment{s, it, t, static_cast<int32_t>(t_end), -1, 0});
        t = static_cast<int32_t>(t_end);
      }
      const size_t nparts = wl.segs.size() - seg_first;
      if (nparts > 1) {
        const int32_t fix_id = static_cast<int32_t>(wl.fix.size());
        wl.fix.push_back(Fixup{static_cast<int32_t>(nparts), wl.slots});
        for (size_t p = 0; p < nparts; ++p) {
          wl.segs[seg_first + p].fix = fix_id;
          wl.segs[seg_first + p].part = static_cast<int32_t>(p);
        }
        wl.slots += static_cast<int32_t>(nparts);
        ++wl.split_tiles;
      }
      c0 += sys[s].npad;
    }
  }
  while (next_cta <= grid) wl.seg_begin[next_cta++] = static_cast<int32_t>(wl.segs.size());
  return wl;
}

}  // namespace nbg
