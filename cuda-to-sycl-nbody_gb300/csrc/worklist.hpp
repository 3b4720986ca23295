// Stream-K work-list planner for the persistent force kernel (host only).
//
// The unit of work is one (system, i-tile, j-tile) block of bi x |j-tile| pair
// interactions; a system's i-tiles cover its shard (SystemDesc::shard_first ..
// shard_end), its j-tiles all of it.  Units are laid out in (system, i-tile, j-tile) order and each
// is charged its j-tile length.  CTA k receives the units whose starting charge
// c satisfies floor(c * grid / total) == k, i.e. one contiguous run of the
// sequence with total / grid charge (+- one tile).  A run that covers only part
// of an i-tile's j-range becomes a "part" of a fixup record: the kernel sums the
// parts in j order once the last one has arrived.
//
// Sizes of a plan over i-tiles `nit` (all systems) on `grid` CTAs: every CTA
// boundary that falls inside an i-tile adds one segment, so
//   segments <= nit + grid - 1,   partial-sum slots <= segments,
//   fixups   <= min(nit, grid - 1).
#pragma once

#include <algorithm>
#include <cstdint>
#include <vector>

#include "nb_internal.hpp"

namespace nbg {

struct WorkListHost {
  std::vector<Segment> segs;
  std::vector<int32_t> seg_begin;  // grid + 1 entries
  std::vector<Fixup> fix;
  int32_t slots = 0;               // partial-sum slots (sum of nparts over fixups)
  int32_t grid = 0;
  int32_t split_tiles = 0;         // number of i-tiles with nparts > 1
};

// The planner itself, writing through `out`, so that growable tables
// (plan_worklist) and fixed ones (nb_accelerations_noalloc) follow one rule.
// Out provides:
//   bool set_grid(int64_t grid)                 false: the grid does not fit
//   bool add_segment(const Segment&)            false: no room
//   Segment& segment(int64_t index)
//   int64_t num_segments() const
//   void set_begin(int64_t cta, int64_t first_segment)
//   bool add_fixup(const Fixup&)                false: no room
//   int64_t num_fixups() const
// Returns false when `out` ran out of room; slots and split tiles go to *slots_out
// and *split_out.
template <class Out>
bool plan_work_into(const SystemDesc* sys, int32_t first, int32_t count, int32_t bi, int32_t bj,
                    int32_t max_grid, Out& out, int32_t* slots_out, int32_t* split_out) {
  int64_t total = 0, tiles = 0;
  for (int32_t s = first; s < first + count; ++s) {
    const int64_t nit = (shard_end(sys[s]) - sys[s].shard_first + bi - 1) / bi;
    const int64_t njt = (sys[s].npad + bj - 1) / bj;
    total += nit * sys[s].npad;
    tiles += nit * njt;
  }
  const int64_t grid = std::max<int64_t>(1, std::min<int64_t>(max_grid, tiles));
  if (!out.set_grid(grid)) return false;

  // CTA owning the unit whose charge starts at c.
  auto owner = [&](int64_t c) { return std::min<int64_t>(grid - 1, (c * grid) / total); };

  int64_t c0 = 0;          // charge before the current i-tile
  int64_t next_cta = 0;    // first CTA whose seg_begin is not yet set
  int32_t slots = 0, split = 0;
  for (int32_t s = first; s < first + count; ++s) {
    const int32_t nit = (shard_end(sys[s]) - sys[s].shard_first + bi - 1) / bi;
    const int32_t njt = (sys[s].npad + bj - 1) / bj;
    for (int32_t it = 0; it < nit; ++it) {
      const int64_t seg_first = out.num_segments();
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
        while (next_cta <= k) out.set_begin(next_cta++, out.num_segments());
        if (!out.add_segment(Segment{s, it, t, static_cast<int32_t>(t_end), -1, 0})) return false;
        t = static_cast<int32_t>(t_end);
      }
      const int64_t nparts = out.num_segments() - seg_first;
      if (nparts > 1) {
        const int32_t fix_id = static_cast<int32_t>(out.num_fixups());
        if (!out.add_fixup(Fixup{static_cast<int32_t>(nparts), slots})) return false;
        for (int64_t p = 0; p < nparts; ++p) {
          out.segment(seg_first + p).fix = fix_id;
          out.segment(seg_first + p).part = static_cast<int32_t>(p);
        }
        slots += static_cast<int32_t>(nparts);
        ++split;
      }
      c0 += sys[s].npad;
    }
  }
  while (next_cta <= grid) out.set_begin(next_cta++, out.num_segments());
  *slots_out = slots;
  *split_out = split;
  return true;
}

// Plan the work of systems [first, first + count) of `sys` for a kernel with
// i-tiles of `bi` particles and j-tiles of `bj` particles on at most `max_grid`
// CTAs.  Every (system, i-tile, j-tile) unit is assigned to exactly one CTA, in
// (system, i-tile, j-tile) order, so that each CTA's share of j-particles is the
// same to within one tile.  Segments reference systems by their index in `sys`.
WorkListHost plan_worklist(const SystemDesc* sys, int32_t first, int32_t count, int32_t bi,
                           int32_t bj, int32_t max_grid);

}  // namespace nbg
