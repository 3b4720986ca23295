/*
 * nbody_oracle.c -- CPU oracle for the all-pairs softened-gravity step.
 *
 * TEST INFRASTRUCTURE ONLY.  The tests, the smoke check and the CPU-baseline leg
 * of the benchmark use this file as the checker; the library never calls it.
 *
 * It restates the reference kernel particle_interaction
 * (codeplaysoftware/cuda-to-sycl-nbody, src/simulator.cu:186-229) in FP32 with the
 * same operation order, plus FP64 references for accelerations, energy and
 * momentum.  Compiled with -ffp-contract=off: every fused multiply-add is an
 * explicit fmaf() placed where nvcc contracts the reference's expressions, so
 * results are identical on x86-64 and aarch64 hosts.  rsqrt (a hardware
 * approximation on the GPU, simulator.cu:202) is 1/sqrtf here, correctly rounded.
 *
 * Parity pin: tests compare this restatement with the reference kernel itself,
 * compiled from src/simulator.cu into a cubin (oracle/build_ref.sh) and run on
 * the GPU, and with golden vectors produced from that kernel (tests/golden/).
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#define ORACLE_BRANCH 0
#define ORACLE_PREDICATED 1

/* Force sum of particle_interaction for particle `id` (simulator.cu:193-211),
 * with an optional per-particle mass multiplying each pair term (the reference
 * assumes unit mass, :204). */
static void force_fp32(int64_t n, const float* x, const float* y, const float* z,
                       const float* mass, float eps, int method, int64_t id, float* fx,
                       float* fy, float* fz) {
  const float px = x[id], py = y[id], pz = z[id];
  float ax = 0.0f, ay = 0.0f, az = 0.0f;
  for (int64_t i = 0; i < n; ++i) {
    const float rx = x[i] - px; /* other_pos - pos, :199 */
    const float ry = y[i] - py;
    const float rz = z[i] - pz;
    /* dot(r, r) + distEps (:201), contracted as nvcc does for the reference:
     * fma(r.z, r.z, fma(r.x, r.x, r.y * r.y)) + distEps */
    const float d2 = fmaf(rz, rz, fmaf(rx, rx, ry * ry)) + eps;
    float inv = 1.0f / sqrtf(d2 * d2 * d2); /* rsqrt(d2^3), :202 */
    if (mass) inv *= mass[i];
    if (method == ORACLE_BRANCH) {
      if (i == id) continue; /* :206 */
      ax = fmaf(rx, inv, ax); /* force += r * inv, :207 */
      ay = fmaf(ry, inv, ay);
      az = fmaf(rz, inv, az);
    } else {
      const float m = (i == id) ? 1.0f : 0.0f; /* * (i == id), :209 */
      ax = fmaf(rx * inv, m, ax);
      ay = fmaf(ry * inv, m, ay);
      az = fmaf(rz * inv, m, az);
    }
  }
  *fx = ax;
  *fy = ay;
  *fz = az;
}

/* One iteration: velocities in place, next positions out (simulator.cu:213-228). */
void oracle_step_fp32(int64_t n, const float* x, const float* y, const float* z, float* vx,
                      float* vy, float* vz, float* xn, float* yn, float* zn, const float* mass,
                      float G, float dt, float damping, float eps, int method) {
#pragma omp parallel for schedule(static)
  for (int64_t id = 0; id < n; ++id) {
    float fx, fy, fz;
    force_fp32(n, x, y, z, mass, eps, method, id, &fx, &fy, &fz);
    /* curr_vel *= damping; curr_vel += force * dt * G  (:214-216) */
    const float ux = fmaf(fx * dt, G, vx[id] * damping);
    const float uy = fmaf(fy * dt, G, vy[id] * damping);
    const float uz = fmaf(fz * dt, G, vz[id] * damping);
    vx[id] = ux;
    vy[id] = uy;
    vz[id] = uz;
    /* curr_pos += curr_vel * dt  (:223-228) */
    xn[id] = fmaf(ux, dt, x[id]);
    yn[id] = fmaf(uy, dt, y[id]);
    zn[id] = fmaf(uz, dt, z[id]);
  }
}

/* `iters` iterations with the reference's buffer swap (simulator.cu:57-66);
 * positions and velocities updated in place. */
void oracle_run_fp32(int64_t n, float* x, float* y, float* z, float* vx, float* vy, float* vz,
                     const float* mass, float G, float dt, float damping, float eps, int method,
                     int iters, float* scratch /* 3n */) {
  float* xn = scratch;
  float* yn = scratch + n;
  float* zn = scratch + 2 * n;
  for (int it = 0; it < iters; ++it) {
    oracle_step_fp32(n, x, y, z, vx, vy, vz, xn, yn, zn, mass, G, dt, damping, eps, method);
    memcpy(x, xn, sizeof(float) * n);
    memcpy(y, yn, sizeof(float) * n);
    memcpy(z, zn, sizeof(float) * n);
  }
}

/* G times the FP32 force sum for rows[0..count) (count < 0: all particles). */
void oracle_accel_fp32(int64_t n, const float* x, const float* y, const float* z,
                       const float* mass, float G, float eps, int method, const int64_t* rows,
                       int64_t count, float* ax, float* ay, float* az) {
  const int64_t m = count < 0 ? n : count;
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < m; ++k) {
    const int64_t id = count < 0 ? k : rows[k];
    float fx, fy, fz;
    force_fp32(n, x, y, z, mass, eps, method, id, &fx, &fy, &fz);
    ax[k] = fx * G;
    ay[k] = fy * G;
    az[k] = fz * G;
  }
}

/* FP64 accelerations G * sum_{j != i} m_j r_ij / (|r_ij|^2 + eps)^(3/2). */
void oracle_accel_fp64(int64_t n, const float* x, const float* y, const float* z,
                       const float* mass, double G, double eps, const int64_t* rows, int64_t count,
                       double* ax, double* ay, double* az) {
  const int64_t m = count < 0 ? n : count;
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t k = 0; k < m; ++k) {
    const int64_t id = count < 0 ? k : rows[k];
    const double px = x[id], py = y[id], pz = z[id];
    double sx = 0.0, sy = 0.0, sz = 0.0;
    for (int64_t j = 0; j < n; ++j) {
      if (j == id) continue;
      const double rx = (double)x[j] - px, ry = (double)y[j] - py, rz = (double)z[j] - pz;
      const double d2 = rx * rx + ry * ry + rz * rz + eps;
      const double s = (mass ? (double)mass[j] : 1.0) / (d2 * sqrt(d2));
      sx += rx * s;
      sy += ry * s;
      sz += rz * s;
    }
    ax[k] = G * sx;
    ay[k] = G * sy;
    az[k] = G * sz;
  }
}

/* FP64 energy and momenta: out = {KE, PE, px, py, pz, Lx, Ly, Lz, M}. */
void oracle_energy_fp64(int64_t n, const float* x, const float* y, const float* z,
                        const float* vx, const float* vy, const float* vz, const float* mass,
                        double G, double eps, double* out) {
  double ke = 0, pe = 0, p[3] = {0, 0, 0}, l[3] = {0, 0, 0}, msum = 0;
  for (int64_t i = 0; i < n; ++i) {
    const double m = mass ? mass[i] : 1.0;
    const double ux = vx[i], uy = vy[i], uz = vz[i];
    ke += 0.5 * m * (ux * ux + uy * uy + uz * uz);
    p[0] += m * ux;
    p[1] += m * uy;
    p[2] += m * uz;
    l[0] += m * ((double)y[i] * uz - (double)z[i] * uy);
    l[1] += m * ((double)z[i] * ux - (double)x[i] * uz);
    l[2] += m * ((double)x[i] * uy - (double)y[i] * ux);
    msum += m;
  }
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : pe)
  for (int64_t i = 0; i < n; ++i) {
    const double mi = mass ? mass[i] : 1.0;
    double s = 0.0;
    for (int64_t j = i + 1; j < n; ++j) {
      const double rx = (double)x[j] - x[i], ry = (double)y[j] - y[i], rz = (double)z[j] - z[i];
      s += (mass ? (double)mass[j] : 1.0) / sqrt(rx * rx + ry * ry + rz * rz + eps);
    }
    pe += -G * mi * s;
  }
  out[0] = ke;
  out[1] = pe;
  out[2] = p[0];
  out[3] = p[1];
  out[4] = p[2];
  out[5] = l[0];
  out[6] = l[1];
  out[7] = l[2];
  out[8] = msum;
}

int oracle_num_threads(void) {
#ifdef _OPENMP
  extern int omp_get_max_threads(void);
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* Threads for the parallel loops from now on (OpenMP's omp_set_num_threads); a
 * launcher such as torchrun sets OMP_NUM_THREADS=1, and the CPU baseline wants
 * every core it may use. */
void oracle_set_num_threads(int n) {
#ifdef _OPENMP
  extern void omp_set_num_threads(int);
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}
