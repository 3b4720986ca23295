// Stream-K work-list planner (the rule is plan_work_into in worklist.hpp).
#include "worklist.hpp"

namespace nbg {

namespace {

// Growable tables for plan_work_into.
struct VectorTables {
  WorkListHost& wl;
  bool set_grid(int64_t grid) {
    wl.grid = static_cast<int32_t>(grid);
    wl.seg_begin.assign(grid + 1, 0);
    return true;
  }
  bool add_segment(const Segment& s) {
    wl.segs.push_back(s);
    return true;
  }
  Segment& segment(int64_t i) { return wl.segs[i]; }
  int64_t num_segments() const { return static_cast<int64_t>(wl.segs.size()); }
  void set_begin(int64_t cta, int64_t first) { wl.seg_begin[cta] = static_cast<int32_t>(first); }
  bool add_fixup(const Fixup& f) {
    wl.fix.push_back(f);
    return true;
  }
  int64_t num_fixups() const { return static_cast<int64_t>(wl.fix.size()); }
};

}  // namespace

WorkListHost plan_worklist(const SystemDesc* sys, int32_t first, int32_t count, int32_t bi,
                           int32_t bj, int32_t max_grid, int32_t threads, int32_t r) {
  WorkListHost wl;
  VectorTables out{wl};
  plan_work_into(sys, first, count, bi, bj, max_grid, out, &wl.slots, &wl.split_tiles, threads,
                 r);
  return wl;
}

}  // namespace nbg
