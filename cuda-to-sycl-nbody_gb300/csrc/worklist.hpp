// Stream-K work-list planner for the persistent force kernel (host only).
#pragma once

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

// Plan the work of systems [first, first + count) of `sys` for a kernel with
// i-tiles of `bi` particles and j-tiles of `bj` particles on at most `max_grid`
// CTAs.  Every (system, i-tile, j-tile) unit is assigned to exactly one CTA, in
// (system, i-tile, j-tile) order, so that each CTA's share of j-particles is the
// same to within one tile.  Segments reference systems by their index in `sys`.
WorkListHost plan_worklist(const SystemDesc* sys, int32_t first, int32_t count, int32_t bi,
                           int32_t bj, int32_t max_grid);

}  // namespace nbg
