// Stream-K work-list planner for the persistent force kernel (host only).
//
// The unit of work is one (system, i-tile, j-tile) block of bi x |j-tile| pair
// interactions; a system's i-tiles cover its shard (SystemDesc::shard_first ..
// shard_end), its j-tiles all of it.  Units are laid out in (system, i-tile, j-tile)
// order and each is charged bj times the i-tile's weight: the register slots the
// force kernel runs for it (live_slots: fewer than r only in a system's last,
// partly filled i-tile), or 1 for kernels that run every slot.  CTA k receives the
// units whose starting charge c satisfies floor(c * grid / total) == k, i.e. one
// contiguous run of the sequence with total / grid charge (+- one unit).  A run that covers only part
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
// `threads` and `r`: the force kernel's i-particles per thread (r, at stride
// threads), for the weights; threads = 0 weighs every i-tile 1.  Charges times the
// grid can pass 2^63 for the largest systems, so those products are 128-bit.
template <class Out>
bool plan_work_into(const SystemDesc* sys, int32_t first, int32_t count, int32_t bi, int32_t bj,
                    int32_t max_grid, Out& out, int32_t* slots_out, int32_t* split_out,
                    int32_t threads = 0, int32_t r = 1) {
  using wide = __int128;
  auto weight = [&](int32_t rows) -> int64_t {
    return threads > 0 ? live_slots(rows, threads, r) : 1;
  };
  wide total = 0;
  int64_t tiles = 0;
  for (int32_t s = first; s < first + count; ++s) {
    const int32_t rows = shard_end(sys[s]) - sys[s].shard_first;
    const int64_t nit = (rows + bi - 1) / bi;
    const int64_t njt = (sys[s].npad + bj - 1) / bj;
    const int64_t w = static_cast<int64_t>(rows / bi) * weight(bi) +
                      (rows % bi ? weight(rows % bi) : 0);
    total += static_cast<wide>(w) * sys[s].npad;
    tiles += nit * njt;
  }
  if (total == 0) total = 1;
  const int64_t grid = std::max<int64_t>(1, std::min<int64_t>(max_grid, tiles));
  if (!out.set_grid(grid)) return false;

  // CTA owning the unit whose charge starts at c.
  auto owner = [&](wide c) {
    return std::min<int64_t>(grid - 1, static_cast<int64_t>((c * grid) / total));
  };

  wide c0 = 0;             // charge before the current i-tile
  int64_t next_cta = 0;    // first CTA whose seg_begin is not yet set
  int32_t slots = 0, split = 0;
  for (int32_t s = first; s < first + count; ++s) {
    const int32_t rows = shard_end(sys[s]) - sys[s].shard_first;
    const int32_t nit = (rows + bi - 1) / bi;
    const int32_t njt = (sys[s].npad + bj - 1) / bj;
    for (int32_t it = 0; it < nit; ++it) {
      const int64_t seg_first = out.num_segments();
      const wide unit = static_cast<wide>(bj) * weight(rows - it * bi);  // charge of one j-tile
      int32_t t = 0;
      while (t < njt) {
        const int64_t k = owner(c0 + t * unit);
        // First tile owned by a later CTA: smallest t' with (c0 + t' unit) grid >= (k+1) total.
        int64_t t_end = njt;
        if (k + 1 < grid) {
          const wide need = (k + 1) * total - c0 * grid;  // > t*unit*grid
          t_end = static_cast<int64_t>((need + unit * grid - 1) / (unit * grid));
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
      c0 += static_cast<wide>(sys[s].npad) * weight(rows - it * bi);
    }
  }
  while (next_cta <= grid) out.set_begin(next_cta++, out.num_segments());
  *slots_out = slots;
  *split_out = split;
  return true;
}

// Whether the force kernel's live-slot variant pays for systems [first, first +
// count) with i-tiles of threads x r particles: its weighted work is below 99 % of
// every slot's (it carries extra loop variants, and the full loop is allocated
// differently with them, so it is kept for work lists with many part-filled tiles).
inline bool live_slots_pay(const SystemDesc* sys, int32_t first, int32_t count, int32_t threads,
                           int32_t r) {
  const int32_t bi = threads * r;
  double all = 0, live = 0;
  for (int32_t s = first; s < first + count; ++s) {
    const int32_t rows = shard_end(sys[s]) - sys[s].shard_first;
    const double full = rows / bi, rem = rows % bi;
    all += sys[s].npad * (static_cast<double>(r) * (full + (rem > 0 ? 1 : 0)));
    live += sys[s].npad * (r * full + (rem > 0 ? live_slots(rows % bi, threads, r) : 0));
  }
  return live < 0.99 * all;
}

// Plan the work of systems [first, first + count) of `sys` for a kernel with
// i-tiles of `bi` particles and j-tiles of `bj` particles on at most `max_grid`
// CTAs.  Every (system, i-tile, j-tile) unit is assigned to exactly one CTA, in
// (system, i-tile, j-tile) order, so that each CTA's share of weighted j-particles
// is the same to within one unit.  Segments reference systems by their index in
// `sys`.  threads, r: as for plan_work_into (the force kernel's shape; 0 for the
// reference-order kernel, which runs every slot).
WorkListHost plan_worklist(const SystemDesc* sys, int32_t first, int32_t count, int32_t bi,
                           int32_t bj, int32_t max_grid, int32_t threads = 0, int32_t r = 1);

}  // namespace nbg
