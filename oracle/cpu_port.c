/*
 * cpu_port.c -- the reference's force sum as a CPU loop, built for speed: the timed
 * CPU baseline of the benchmark (its cpu_baseline leg and its reference arm).
 *
 * TEST AND BENCHMARK INFRASTRUCTURE ONLY; the library never calls it.
 *
 * The loop body is the reference kernel's (particle_interaction<BRANCH>,
 * codeplaysoftware/cuda-to-sycl-nbody src/simulator.cu:193-211): r = x_j - x_i,
 * d2 = dot(r, r) + distEps, inv = rsqrt(d2^3), the j == i term left out, force +=
 * r * inv; one OpenMP task per i-row.  Unlike the parity oracle (nbody_oracle.c,
 * -ffp-contract=off, correctly rounded 1/sqrtf) it is compiled with
 * -O3 -ffast-math -fopenmp, so the compiler may reassociate the sum and vectorise
 * the j loop across the core's SIMD lanes: the left-out j == i term becomes a
 * select instead of a branch.  Results agree with the oracle to FP32 rounding of a
 * reordered sum (and, where the compiler uses a reciprocal-square-root estimate,
 * to that estimate's accuracy); the tests check 1e-4.  No -march=native: the same
 * source and flags build on the x86-64 and aarch64 hosts.
 */
#include <math.h>
#include <stdint.h>

static void port_row(int64_t n, const float* restrict x, const float* restrict y,
                     const float* restrict z, float eps, int64_t id, float* fx, float* fy,
                     float* fz) {
  const float px = x[id], py = y[id], pz = z[id];
  float ax = 0.0f, ay = 0.0f, az = 0.0f;
  for (int64_t j = 0; j < n; ++j) {
    const float rx = x[j] - px;
    const float ry = y[j] - py;
    const float rz = z[j] - pz;
    const float d2 = rx * rx + ry * ry + rz * rz + eps;
    const float inv = 1.0f / sqrtf(d2 * d2 * d2);
    const float w = (j == id) ? 0.0f : inv;
    ax += rx * w;
    ay += ry * w;
    az += rz * w;
  }
  *fx = ax;
  *fy = ay;
  *fz = az;
}

/* G times the force sum of rows[0..count) (count < 0: all n particles), unit masses
 * (an equal mass is folded into G by the caller). */
void cpu_port_accel(int64_t n, const float* x, const float* y, const float* z, float G,
                    float eps, const int64_t* rows, int64_t count, float* ax, float* ay,
                    float* az) {
  const int64_t m = count < 0 ? n : count;
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t k = 0; k < m; ++k) {
    const int64_t id = count < 0 ? k : rows[k];
    float fx, fy, fz;
    port_row(n, x, y, z, eps, id, &fx, &fy, &fz);
    ax[k] = fx * G;
    ay[k] = fy * G;
    az[k] = fz * G;
  }
}

int cpu_port_num_threads(void) {
#ifdef _OPENMP
  extern int omp_get_max_threads(void);
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void cpu_port_set_num_threads(int n) {
#ifdef _OPENMP
  extern void omp_set_num_threads(int);
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}
