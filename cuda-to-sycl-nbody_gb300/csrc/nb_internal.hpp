// Internal types shared by the CUDA kernels and the host runtime.
//
// Device layout of one simulation (all systems concatenated, each system padded
// to a multiple of kPadQuantum particles):
//
//   pos[2]  "pair layout": particles 2p and 2p+1 share 32 bytes
//           { x0, x1, y0, y1, z0, z1, m0, m1 }.  A j-tile of the force kernel is
//           a contiguous byte range of this array, so one bulk copy stages it in
//           shared memory, and each 16-byte shared load yields (x0,x1),(y0,y1) or
//           (z0,z1),(m0,m1) register pairs for the packed FP32x2 pipe.
//           Double-buffered like the reference's pos_d / pos_next_d
//           (src/simulator.cuh:152-153).
//   vel     float4 (vx, vy, vz, 0) per particle, updated in place like pVel
//           (src/simulator.cu:214-220).
//
// Padding particles sit at kFarAway with zero mass: every pair term against them
// is exactly zero (d2^3 overflows to +inf, rsqrt(+inf) = 0), so j-tiles never need
// a bounds mask.
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

namespace nbg {

constexpr int kPadQuantum = 16;        // particles; every system's padded size is a multiple
constexpr float kFarAway = 1.0e18f;    // coordinate of padding particles

// Index of component c (0=x,1=y,2=z,3=m) of particle i in the pair layout (floats).
__host__ __device__ inline int64_t pair_index(int64_t i, int c) {
  return (i >> 1) * 8 + c * 2 + (i & 1);
}

struct SystemDesc {
  int64_t offset;  // first particle (even; multiple of kPadQuantum)
  int32_t n;       // real particles
  int32_t npad;    // padded particles, multiple of kPadQuantum
  float gscale;    // G (per-pair masses) or G * m (equal masses, m folded out of the pair loop)
  float mass;      // the common mass when the system is equal-mass, else 0
  int32_t equal_mass;
  // The particles a force pass integrates (a shard, nb_sim_set_shard): i in
  // [shard_first, shard_first + shard_count), each against all n; shard_count 0
  // means to the end of the system.  shard_first is a multiple of kPadQuantum.
  int32_t shard_first;
  int32_t shard_count;
  int32_t pad_;
};

// One past the last i-particle a force pass integrates in system `d`.
__host__ __device__ inline int32_t shard_end(const SystemDesc& d) {
  return d.shard_count ? d.shard_first + d.shard_count : d.n;
}

// Register slots of a force-kernel thread (r i-particles at stride `threads`) that
// hold a particle in an i-tile with `rows` particles to integrate: ceil(rows /
// threads), capped at r, and raised to r when above 4 (the kernel has loop variants
// for 1-4 slots and for all r).  The work-list planner charges an i-tile by it.
__host__ __device__ inline int32_t live_slots(int32_t rows, int32_t threads, int32_t r) {
  const int32_t live = rows <= threads ? 1 : (rows + threads - 1) / threads;
  return live >= r ? r : (live <= 4 ? live : r);
}

// One entry of a CTA's work list: i-tile `itile` of system `sys` against j-tiles
// [jt0, jt1).  `fix` >= 0 when the i-tile's j-range is split over several CTAs:
// this entry is part `part` of fixup record `fix`.
struct Segment {
  int32_t sys;
  int32_t itile;
  int32_t jt0;
  int32_t jt1;
  int32_t fix;
  int32_t part;
};

struct Fixup {
  int32_t nparts;
  int32_t slot0;  // first partial-sum slot (BI records per slot)
};

// Arguments of one force launch (passed by value).
struct ForceArgs {
  const float* pos;         // pair layout, current positions (j and i source)
  float* pos_next;          // pair layout, next positions (integrate mode)
  float4* vel;              // in/out (integrate mode)
  float4* accel_out;        // non-null: write G * sum instead of integrating
  const SystemDesc* sys;
  const Segment* segs;
  const int32_t* seg_begin; // [grid + 1]
  const Fixup* fix;
  float4* partials;         // [slots][BI] (plain) or [slots][BI][2] (compensated)
  int32_t* counters;        // [fixups], zero between launches
  int32_t* err;             // device error word (bit 0: bounded wait timed out)
  float eps2;
  float dt;
  float damping;
  int32_t mask_self;        // 1: exclude j == i explicitly (eps2^3 underflows)
  int32_t inject;           // failure-detection test hook (kInject*), 0 normally
};

// Failure-detection test hooks (ForceArgs::inject), one launch each; neither
// faults anything, each makes a bounded device-side wait run out.
constexpr int32_t kInjectSkipFirstTile = 1;     // no CTA copies its first j-tile
constexpr int32_t kInjectWithholdHandOver = 2;  // sequential-order kernel: no CTA hands
                                                // its running sums over

// Host description of one kernel shape.
struct KernelShape {
  int threads;
  int r;       // i-particles per thread
  int bj;      // j-tile size in particles
  int stages;
  int bi() const { return threads * r; }
};

}  // namespace nbg
