/*
 * nbody_gb300.h -- C ABI of the GB300 (sm_103a) all-pairs softened-gravity step.
 *
 * This is the drop-in boundary for the reference's simulator layer
 * (codeplaysoftware/cuda-to-sycl-nbody):
 *   - `simulation::Simulator` / `DiskGalaxySimulator`  src/simulator.cuh:107-160
 *   - `SimParam` and its argv parser                   src/sim_param.hpp:16-40,
 *                                                       src/sim_param.cpp:12-67
 *   - the force + integrate kernel `particle_interaction`
 *                                                       src/simulator.cu:186-229
 *
 * Conventions
 *   - Every entry point returns an `nb_status` (0 = NB_OK).  No exception and no
 *     exit() crosses this boundary (the reference aborts through gpuErrchk,
 *     src/simulator.cuh:22-31).  `nb_last_error()` returns a thread-local message
 *     describing the last failure on the calling thread.
 *   - Host particle arrays are structure-of-arrays float32, like the reference's
 *     `ParticleData` (src/simulator.cuh:75-84).  Arrays of several systems are
 *     concatenated in system order.
 *   - Pointers are plain host pointers unless a name ends in `_device`.
 *   - `stream` arguments are `cudaStream_t` values passed as `void*`
 *     (NULL = the legacy default stream).
 *   - A simulation object is not thread-safe: one host thread at a time.
 */
#ifndef NBODY_GB300_H
#define NBODY_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NB_ABI_VERSION 1

typedef enum nb_status {
  NB_OK = 0,
  NB_ERR_INVALID_ARGUMENT = 1, /* bad size, NULL pointer, unknown enum value   */
  NB_ERR_CUDA = 2,             /* a CUDA runtime call failed                   */
  NB_ERR_OUT_OF_MEMORY = 3,    /* device or pinned-host allocation failed      */
  NB_ERR_NO_DEVICE = 4,        /* no CUDA device, or not an sm_103 device      */
  NB_ERR_DEVICE_TIMEOUT = 5,   /* a bounded device-side wait gave up           */
  NB_ERR_STATE = 6             /* call not valid in the object's current state */
} nb_status;

/* Kernel variant of the reference (sim_param.hpp:8-11).  PREDICATED reproduces
 * the reference as shipped: its pair term is multiplied by (j == i), so the
 * force is zero except where a pair term is not finite (simulator.cu:208-209).  It
 * runs the reference-order kernel's tiling with that pair term for equal masses,
 * and one thread per particle for per-particle masses; the results are the
 * reference kernel's, bit for bit. */
typedef enum nb_calc_method { NB_BRANCH = 0, NB_PREDICATED = 1 } nb_calc_method;

/* Per-particle force accumulator; the pair arithmetic is FP32 in every mode.
 * PLAIN and COMPENSATED run the tuned kernel, which sums each particle's terms in
 * its own order (COMPENSATED keeps a Kahan-compensated FP32 running sum).
 * REFERENCE_ORDER sums them the way particle_interaction<BRANCH> does
 * (simulator.cu:196-207: one FP32 running sum over j in index order, the same
 * contracted operations), so on the same GPU its results are bit-identical to the
 * reference kernel's; it needs equal masses within each system (the reference has
 * unit masses) and does not use the kernel shapes or the autotuner.
 * nb_params_default selects COMPENSATED: at the tuned kernel's default shape it is
 * both faster than PLAIN and far more accurate. */
typedef enum nb_accumulator {
  NB_ACC_PLAIN = 0,
  NB_ACC_COMPENSATED = 1,
  NB_ACC_REFERENCE_ORDER = 2
} nb_accumulator;

/* Mirror of SimParam (sim_param.hpp:30-39), plus the accumulator mode.
 * `dist_eps` is the softening added to r^2 (the reference's distEps). */
typedef struct nb_params {
  float G;
  float dt;
  float damping;
  float dist_eps;
  uint64_t num_particles;
  uint64_t num_frames;
  int32_t iters_per_frame; /* simIterationsPerFrame */
  int32_t gw_size;         /* reported by nb_sim_gw_size(); the tuned kernel picks its own block */
  int32_t calc_method;     /* nb_calc_method */
  int32_t accumulator;     /* nb_accumulator */
} nb_params;

/* Energy and momentum of one system (or all), reduced in FP64 on the GPU.
 * potential = -G * sum_{i<j} m_i m_j / sqrt(|x_i - x_j|^2 + dist_eps). */
typedef struct nb_diagnostics {
  double kinetic;
  double potential;
  double total;
  double momentum[3];
  double angular_momentum[3];
  double mass;
} nb_diagnostics;

/* Kernel shape selected for a simulation (see nb_sim_autotune). */
/* For NB_ACC_REFERENCE_ORDER, config_index is -1 - (reference-order shape) and the
 * fields describe the reference-order kernel (segments = its i-tiles, no split
 * tiles). */
typedef struct nb_kernel_info {
  int32_t config_index;
  int32_t threads_per_block;
  int32_t particles_per_thread; /* i-particles held in registers per thread */
  int32_t j_tile;               /* j-particles per shared-memory tile       */
  int32_t stages;               /* depth of the shared-memory tile ring     */
  int32_t grid;                 /* persistent CTAs per launch               */
  int32_t segments;             /* work-list entries                        */
  int32_t split_tiles;          /* i-tiles whose j-range spans several CTAs */
  int32_t live_slots;           /* 1: the variant that skips the register slots
                                   past the end of a system in its last i-tile,
                                   with a work list weighted by live slots     */
} nb_kernel_info;

/* One entry of the persistent force kernel's work list: i-tile `i_tile` of
 * system `system` against j-tiles [j_tile_begin, j_tile_end).  `fixup` >= 0 when
 * the i-tile's j-range is split over several CTAs (this entry is part `part`). */
typedef struct nb_segment {
  int32_t system;
  int32_t i_tile;
  int32_t j_tile_begin;
  int32_t j_tile_end;
  int32_t fixup;
  int32_t part;
} nb_segment;

typedef struct nb_sim nb_sim; /* opaque */

/* ---- errors --------------------------------------------------------------- */
/* Replace gpuErrchk's print-and-exit (simulator.cuh:22-31): the message of the
 * calling thread's last failed call, the name of a status code, and the ABI
 * version (no reference counterpart). */
const char* nb_last_error(void);
const char* nb_status_string(int status);
int nb_abi_version(void);

/* ---- parameters: SimParam::SimParam / SimParam::parseArgs ------------------- */
/* Defaults of SimParam::SimParam (sim_param.cpp:12-22). */
void nb_params_default(nb_params* p);
/* Positional argv as SimParam::parseArgs (sim_param.cpp:40-67):
 *   nBatches(x256) iters damping dt distEps G numFrames gwSize calcMethod
 * A calcMethod other than BRANCH/PREDICATED returns NB_ERR_INVALID_ARGUMENT
 * (the reference throws std::invalid_argument, sim_param.cpp:36). */
int nb_params_parse_args(nb_params* p, int argc, const char* const* argv);

/* ---- device ------------------------------------------------------------------ */
/* Name of device 0, as DiskGalaxySimulator::getDeviceName (simulator.cu:36-45). */
int nb_device_name(char* buf, size_t len);
/* Nominal FP32 peak of device 0 in TFLOP/s: SMs x 128 lanes x 2 x max SM clock. */
int nb_device_fp32_peak_tflops(double* tflops);
/* Measured FP32 throughput of the current device in TFLOP/s: the best of 20
 * timed launches, after about 50 ms of warm-up, of a loop of independent packed
 * FP32x2 fused multiply-adds (FFMA2) over every SM, about 65 ms in all.  A measured denominator for the
 * force kernel's efficiency, beside the nominal figure above.  No reference
 * counterpart. */
int nb_measure_fp32_peak_tflops(double* tflops);

/* ---- simulation: DiskGalaxySimulator ---------------------------------------- */
/* Constructor + sendToDevice (simulator.cu:24-34, 79-103) from caller-provided
 * state.  `mass` may be NULL: unit masses, the reference's assumption
 * ("assume uniform unit mass", simulator.cu:204). */
int nb_sim_create(const nb_params* p, const float* x, const float* y, const float* z,
                  const float* vx, const float* vy, const float* vz, const float* mass,
                  nb_sim** out);
/* Constructor with the reference's own initial conditions: randomParticlePos +
 * initialParticleVel (simulator.cu:131-158), default-seeded std::mt19937. */
int nb_sim_create_disk_galaxy(const nb_params* p, nb_sim** out);
/* An ensemble of independent systems advanced together by one persistent launch
 * per step.  sizes[s] particles for system s, arrays concatenated in system order.
 * No reference counterpart (the reference simulates one system). */
int nb_ensemble_create(const nb_params* p, uint32_t num_systems, const uint32_t* sizes,
                       const float* x, const float* y, const float* z, const float* vx,
                       const float* vy, const float* vz, const float* mass, nb_sim** out);
int nb_sim_destroy(nb_sim* s);

/* stepSim (simulator.cu:47-75): iters_per_frame force+integrate iterations, a
 * device synchronize, and the elapsed time recorded with CUDA events.  Unlike the
 * reference it does not copy the state back; call nb_sim_get_state for that. */
int nb_sim_step(nb_sim* s);
/* Enqueue `iterations` iterations on the simulation's stream; returns without
 * waiting. */
int nb_sim_advance(nb_sim* s, int32_t iterations);
/* Baseline for ensembles: the same iterations issued as one launch per system,
 * the way the reference's stepSim launches one grid for its one system
 * (simulator.cu:49-63).  Each system's launch is planned with the kernel shape it
 * would get as a simulation of its own. */
int nb_sim_advance_per_system(nb_sim* s, int32_t iterations);
/* Failure-detection test hook (one shot): the next force launch leaves the
 * first shared-memory tile of every CTA uncopied, so each CTA's bounded wait
 * (2 s) runs out; the launch writes no results, and the next
 * nb_sim_synchronize / nb_sim_get_state returns NB_ERR_DEVICE_TIMEOUT.  No
 * memory is faulted and nothing hangs; the simulation stays usable.  BRANCH
 * method only (NB_ERR_STATE otherwise).  Same as
 * nb_sim_inject_failure(s, NB_INJECT_TILE_NEVER_COPIED). */
int nb_sim_inject_wait_timeout(nb_sim* s);
/* Failure-detection test hooks (one shot, the next force launch), each making one
 * kind of bounded device-side wait run out without faulting anything:
 *   NB_INJECT_TILE_NEVER_COPIED   as nb_sim_inject_wait_timeout;
 *   NB_INJECT_HAND_OVER_WITHHELD  NB_ACC_REFERENCE_ORDER only: no CTA hands the
 *                                 running sums of a split i-tile over, so the CTA
 *                                 that continues it gives up after 2 s.
 * The next nb_sim_synchronize / nb_sim_get_state returns NB_ERR_DEVICE_TIMEOUT and
 * the simulation stays usable.  No reference counterpart (the reference exits on
 * any CUDA error, simulator.cuh:22-31). */
typedef enum nb_inject_kind {
  NB_INJECT_TILE_NEVER_COPIED = 1,
  NB_INJECT_HAND_OVER_WITHHELD = 2
} nb_inject_kind;
int nb_sim_inject_failure(nb_sim* s, int32_t kind);
/* Failure-detection test hook, host side only: the `nth` device allocation the
 * library makes from now on (1 = the next one, in any thread) fails with
 * NB_ERR_OUT_OF_MEMORY without calling cudaMalloc; 0 disarms it.  Lets tests
 * drive every clean-up path.  No reference counterpart (the reference exits on
 * any CUDA error, simulator.cuh:22-31). */
int nb_inject_alloc_failure(int32_t nth);
/* Wait for the stream and report any device-side error (e.g. a wait that timed out). */
int nb_sim_synchronize(nb_sim* s);
/* Run `iterations` iterations bracketed by CUDA events on the simulation's stream
 * and return the device time in milliseconds.  per_system: 0 = one launch over
 * every system; 1 = one launch per system, each with the kernel shape it would get
 * alone (as nb_sim_advance_per_system); 2 = one launch per system, all with the
 * simulation's current shape. */
int nb_sim_time_iterations(nb_sim* s, int32_t iterations, int32_t per_system, float* ms);

/* recvFromDevice (simulator.cu:106-129).  Any output pointer may be NULL. */
int nb_sim_get_state(nb_sim* s, float* x, float* y, float* z, float* vx, float* vy, float* vz);
/* sendToDevice (simulator.cu:79-103).  `mass` NULL keeps the current masses. */
int nb_sim_set_state(nb_sim* s, const float* x, const float* y, const float* z,
                     const float* vx, const float* vy, const float* vz, const float* mass);
/* Accelerations at the current positions, G * sum_j m_j r_ij / (|r_ij|^2 + eps)^(3/2),
 * the force sum of particle_interaction (simulator.cu:193-211) scaled by G.
 * Does not change the state. */
int nb_sim_accelerations(nb_sim* s, float* ax, float* ay, float* az);

/* getNumParticles / getLastStepTime / getGwSize / getCM (simulator.cuh:134-140). */
int nb_sim_num_particles(const nb_sim* s, uint64_t* n);
int nb_sim_num_systems(const nb_sim* s, uint32_t* n);
int nb_sim_last_step_ms(const nb_sim* s, float* ms);
int nb_sim_gw_size(const nb_sim* s, int32_t* gw);
int nb_sim_calc_method(const nb_sim* s, int32_t* method);

/* Use `stream` for all later work of this simulation (NULL = legacy default).  The
 * reference always uses the default stream (simulator.cu:67, 80, 107). */
int nb_sim_set_stream(nb_sim* s, void* stream);
/* Device hand-off replacing the per-frame host copy to the renderer
 * (RendererGL::updateParticles, renderer_gl.cpp:111-114, 156-172): writes the
 * current positions as float4 (x, y, z, mass) into caller device memory, and
 * velocities as float4 (vx, vy, vz, 0) when vel_xyzw_device is not NULL.
 * Stream-ordered on the simulation's stream. */
int nb_sim_export_device(nb_sim* s, float* pos_xyzm_device, float* vel_xyzw_device);

/* ---- one system split over several GPUs or processes ---------------------------- */
/* No reference counterpart: the reference runs its one system on device 0
 * (simulator.cu:40, launches :59-63).  A system of n particles splits into shards,
 * one per GPU (or process): every shard owner keeps a whole copy of the system,
 * integrates only its own particles, each against all n, and between steps the
 * owners exchange the position blocks of their shards (an all-gather of
 * nb_sim_copy_state_block / nb_sim_load_state_block, for instance over NCCL).
 * The Python ShardedSimulation (nbody_gb300.shard) does exactly that. */
typedef enum nb_block_kind { NB_BLOCK_POSITIONS = 1, NB_BLOCK_VELOCITIES = 2 } nb_block_kind;
/* From now on this one-system simulation's force passes integrate only particles
 * [first, first + count): their next positions and velocities are written, the
 * others' are not.  first is a multiple of 16, and so is count unless the shard
 * ends the system; count = 0 restores the whole system.  Drops any captured graph;
 * the adjoint needs the whole system.  nb_sim_accelerations then computes only the
 * shard's rows (the other rows it returns are unspecified).  BRANCH method only. */
int nb_sim_set_shard(nb_sim* s, uint64_t first, uint64_t count);
/* Size in bytes of the state block of particles [first, first + count) (16 bytes per
 * particle; a block that ends the system is padded to a multiple of 16 particles). */
int nb_sim_state_block_bytes(const nb_sim* s, uint64_t first, uint64_t count, int32_t what,
                             uint64_t* bytes);
/* Copy the current positions (what = NB_BLOCK_POSITIONS) or velocities of particles
 * [first, first + count) to, or from, device memory, in the library's own layout:
 * the bytes are only for another simulation of the same system (another shard's
 * owner).  Same rules for first and count as nb_sim_set_shard.  Stream-ordered on
 * the simulation's stream. */
int nb_sim_copy_state_block(nb_sim* s, uint64_t first, uint64_t count, int32_t what,
                            void* dst_device);
int nb_sim_load_state_block(nb_sim* s, uint64_t first, uint64_t count, int32_t what,
                            const void* src_device);

/* ---- kernel selection ---------------------------------------------------------- */
/* The compiled shapes of the tuned kernel (index 0 .. nb_num_kernel_configs() - 1);
 * nb_kernel_config_info and nb_plan_work also take -1 - k for shape k of the
 * reference-order kernel.  No reference counterpart: the reference launches
 * ceil(N / gwSize) blocks of gwSize threads (simulator.cu:49-50), and gwSize is only
 * reported here (nb_sim_gw_size). */
int nb_num_kernel_configs(void);
int nb_kernel_config_info(int32_t index, nb_kernel_info* info);
/* Select a kernel shape by index (-1 = the built-in default for this size).  With
 * NB_ACC_REFERENCE_ORDER the index selects one of the reference-order kernel's
 * shapes (0 = the largest i-tiles; nb_sim_kernel_info reports it as -1 - index). */
int nb_sim_set_kernel_config(nb_sim* s, int32_t index);
int nb_sim_kernel_info(const nb_sim* s, nb_kernel_info* info);
/* Time every kernel shape on this simulation's data (accelerations only, the
 * state is not advanced) and keep the fastest; `chosen` may be NULL.  With
 * NB_ACC_REFERENCE_ORDER it times that kernel's shapes (all give the same bits)
 * and reports -1 - shape; a no-op for NB_PREDICATED (it keeps its default shape,
 * reported as -1 - shape). */
int nb_sim_autotune(nb_sim* s, int32_t* chosen);

/* Plan the work list of kernel shape `config_index` for systems of the given
 * sizes on at most `max_grid` CTAs (host only; needs no GPU).  Every
 * (system, i-tile, j-tile) block is assigned to exactly one CTA and each CTA
 * gets the same work to within one block.  A block of the tuned kernel costs its
 * j-tile length times the register slots it runs (the i-particles per thread, fewer
 * only in a system's last, partly filled i-tile); a block of the reference-order
 * kernel costs its j-tile length.  `segments`
 * (capacity max_segments) and `seg_begin` (capacity max_grid + 1) may be NULL to
 * query the counts only.  No reference counterpart (the reference launches one
 * thread per particle, simulator.cu:49-50). */
int nb_plan_work(uint32_t num_systems, const uint32_t* sizes, int32_t config_index,
                 int32_t max_grid, nb_segment* segments, int32_t max_segments,
                 int32_t* seg_begin, int32_t* grid, int32_t* num_segments, int32_t* num_fixups,
                 int32_t* num_partial_slots);

/* ---- CUDA graphs ------------------------------------------------------------------ */
/* No reference counterpart: stepSim launches every iteration itself
 * (simulator.cu:57-66). */
/* Capture `iterations` iterations into a CUDA graph (replacing any earlier one).
 * The graph holds the current work list's device addresses: choosing another
 * kernel shape (nb_sim_set_kernel_config, nb_sim_autotune) or shard drops it, and
 * nb_sim_graph_launch then returns NB_ERR_STATE until the next capture. */
int nb_sim_graph_capture(nb_sim* s, int32_t iterations);
/* Launch the captured graph once on the simulation's stream. */
int nb_sim_graph_launch(nb_sim* s);

/* ---- FP64 diagnostics ---------------------------------------------------------- */
/* No reference counterpart: the reference reports only kernel times
 * (nbody.cpp:108-123). */
/* Energy and momenta of system `system` (-1 = all systems together, without the
 * cross-system potential).  FP64 pair arithmetic and reductions on the GPU. */
int nb_sim_diagnostics(nb_sim* s, int32_t system, nb_diagnostics* out);
/* FP64 accelerations for `count` particle indices (global, system-concatenated),
 * computed on the GPU against all particles of each row's system. */
int nb_sim_fp64_accelerations(nb_sim* s, const uint64_t* rows, uint64_t count,
                              double* ax, double* ay, double* az);

/* ---- adjoint ----------------------------------------------------------------------- */
/* No reference counterpart: gradients of the reference's T-iteration map
 * (simulator.cu:186-229 applied T times) with respect to the initial state. */
/* Run T iterations forward from the current state, keeping a checkpoint of
 * (x, v) every `checkpoint_every` iterations for nb_sim_adjoint_backward. */
int nb_sim_adjoint_forward(nb_sim* s, int32_t T, int32_t checkpoint_every);
/* Vector-Jacobian product of the T-step map recorded by nb_sim_adjoint_forward:
 * given dL/dx_T and dL/dv_T (xyz-interleaved, n x 3 floats; dL/dv_T may be NULL
 * for zero), return dL/dx_0 and dL/dv_0 (n x 3).  Recomputes the states between
 * checkpoints; leaves the simulation at its state after the forward run. */
int nb_sim_adjoint_backward(nb_sim* s, const float* gx_T, const float* gv_T,
                            float* gx_0, float* gv_0);
/* nb_sim_adjoint_backward on device arrays (n x 3 floats each, xyz-interleaved;
 * gv_T_device may be NULL), enqueued on the simulation's stream without waiting:
 * for callers whose loss and optimiser live on the GPU. */
int nb_sim_adjoint_backward_device(nb_sim* s, const float* gx_T_device,
                                   const float* gv_T_device, float* gx_0_device,
                                   float* gv_0_device);

/* ---- accelerations without allocation ------------------------------------------ */
/* For callers that cannot allocate GPU memory themselves or through this library
 * -- an engine or plugin host that hands out all device memory from its own
 * pools, or a frame loop that must not stall on cudaMalloc.  No counterpart in
 * the reference.  The caller passes n particles as float4 (x, y, z, mass) in
 * `pos_xyzm_device` and receives float4 (ax, ay, az, 0) in `accel_xyzw_device`
 * (both device memory, 16-byte aligned); a = G * sum_{j != i} m_j r_ij /
 * (|r_ij|^2 + dist_eps)^(3/2).  The call allocates no memory: its scratch is one
 * fixed 13 MiB device array inside the library, which limits n to 262,144
 * (larger n: NB_ERR_INVALID_ARGUMENT) and which every GPU that loads the library
 * keeps until the process exits.  The first call on a device looks that array up
 * and should come before any stream capture.  All calls share the array, which
 * keeps the last call's contents (each call clears what must start at zero); calls
 * whose work overlapped on the GPU would race on it, so each call holds a
 * process-wide lock until its work has finished: calls from several threads or
 * streams of one process run one after another.  Runs on `stream` and waits for
 * it before returning. */
int nb_accelerations_noalloc(const float* pos_xyzm_device, uint64_t n, float G, float dist_eps,
                             float* accel_xyzw_device, void* stream);

/* ---- headless render math ---------------------------------------------------------- */
/* Camera matrices of the reference's orbit camera (Camera::getView / getProj,
 * camera.cpp:38-52): eye at distance `distance` from `look_at` (NULL = origin) at
 * the given azimuth and elevation (radians), z up; infinite perspective, fovy 30
 * degrees, near 1, aspect width / height.  Column-major 4x4, as OpenGL. */
int nb_camera_matrices(float azimuth, float elevation, float distance, const float look_at[3],
                       int32_t width, int32_t height, float view[16], float proj[16]);
/* The renderer's fixed tables: the 13 merged Gaussian blur taps (sigma 10, 25
 * taps; RendererGL::gaussKernel/optimGaussKernel, renderer_gl.cpp:314-368) and the
 * 16 x 16 flare texture (genFlareTex, gen.cpp:36-51). */
int nb_render_tables(float* gauss_offsets, float* gauss_weights, int32_t* taps, float* flare);
/* Render the current state as the reference's OpenGL renderer does
 * (RendererGL::render, renderer_gl.cpp:96-157, and the shaders in shaders/gl): additive
 * velocity-coloured flare sprites into an HDR buffer with a 50-pixel margin,
 * half-resolution separable Gaussian bloom, mean luminance, exposure tonemap and
 * gamma 2.2 -- on the GPU, with no graphics API.  Writes width x height float4
 * RGBA (row 0 at the bottom) to `rgba_device`.  Stream-ordered. */
int nb_sim_render(nb_sim* s, const float view[16], const float proj[16], int32_t width,
                  int32_t height, float* rgba_device);

/* ---- initial conditions on the device ---------------------------------------------- */
typedef enum nb_ic_kind { NB_IC_THIN_DISK = 1, NB_IC_PLUMMER = 2, NB_IC_TWO_DISKS = 3 } nb_ic_kind;
/* Overwrite the state of every system with seeded initial conditions generated on
 * the GPU, directly in the device layout (the reference can only generate on the
 * host and copy, simulator.cu:77-103).  System k uses seed + k and gets the same
 * draws as the host generator below with that seed (values can differ from the
 * host's by one float rounding).  Thin disks use the simulation's dist_eps;
 * NB_IC_TWO_DISKS needs even system sizes.  Masses become 1/n per system (1/(n/2)
 * for two disks). */
int nb_sim_generate(nb_sim* s, int32_t kind, uint64_t seed);

/* ---- initial conditions (host, seeded, deterministic) -------------------------------- */
/* No reference counterpart: the workloads' generators.  The reference's own
 * initial state is nb_ic_reference_disk / nb_sim_create_disk_galaxy. */
/* Thin disk: r = sqrt(u), theta uniform, z ~ N(0, 0.01^2), tangential speed
 * r * sqrt(n m r^2 / (r^2 + eps)^1.5) + N(0, 0.01) per component, m = 1/n. */
int nb_ic_thin_disk(uint64_t seed, uint64_t n, float eps, float* x, float* y, float* z,
                    float* vx, float* vy, float* vz, float* mass);
/* Plummer sphere of scale radius 1 and total mass 1 (Aarseth, Henon & Wielen 1974),
 * velocities by rejection sampling, centre of mass at rest at the origin. */
int nb_ic_plummer(uint64_t seed, uint64_t n, float* x, float* y, float* z, float* vx,
                  float* vy, float* vz, float* mass);
/* Two thin disks of n/2 each, centres +-(2,0,0), bulk velocities -+0.3 in x,
 * the second tilted 30 degrees about the x axis. */
int nb_ic_two_disks(uint64_t seed, uint64_t n, float eps, float* x, float* y, float* z,
                    float* vx, float* vy, float* vz, float* mass);
/* num_systems sizes drawn log-uniform in [lo, hi]. */
int nb_ic_ensemble_sizes(uint64_t seed, uint32_t num_systems, uint32_t lo, uint32_t hi,
                         uint32_t* sizes);
/* The reference's own initial state (simulator.cu:131-158). */
int nb_ic_reference_disk(uint64_t n, float* x, float* y, float* z, float* vx, float* vy,
                         float* vz);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* NBODY_GB300_H */
