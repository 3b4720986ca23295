/*
 * workload_ic.c -- the benchmark workload's seeded Plummer sphere, restated in C.
 *
 * TEST AND BENCHMARK INFRASTRUCTURE ONLY.  The benchmark's reference arm times the
 * reference's CPU path on the same 1,048,576-particle Plummer sphere as the GPU
 * arm, and makes those inputs here so that it never loads the library under test.
 * A CPU test checks that this file and the library's generator (nb_ic_plummer)
 * give the same floats, bit for bit.
 *
 * The generator: counter-based draws, the SplitMix64 output function (Steele, Lea
 * & Flood, OOPSLA 2014) over (seed, particle, draw index); radius from the
 * cumulative mass fraction X, r = (X^(-2/3) - 1)^(-1/2), X redrawn above 0.999;
 * isotropic directions; speed q * sqrt(2) (1 + r^2)^(-1/4) with q from
 * g(q) = q^2 (1 - q^2)^(7/2) by rejection under 0.1 (Aarseth, Henon & Wielen
 * 1974); centre of mass moved to the origin and at rest; masses 1/n.
 * Compiled with -ffp-contract=off, like the library's host code.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>

static const double kTwoPiW = 6.283185307179586476925286766559;

static uint64_t w_mix(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

/* Uniform in (0, 1) from draw k of particle i: 53 bits, centred in their bin. */
static double w_unit(uint64_t seed, uint64_t i, uint64_t k) {
  const uint64_t d = w_mix(seed * 0x9E3779B97F4A7C15ull + w_mix(i * 0xD1B54A32D192ED03ull + k + 1));
  return ((double)(d >> 11) + 0.5) * 0x1.0p-53;
}

/* Returns 0, or -1 when the scratch allocation fails. */
int workload_plummer(uint64_t seed, uint64_t n, float* x, float* y, float* z, float* vx,
                     float* vy, float* vz, float* mass) {
  double* buf = (double*)malloc(sizeof(double) * 6 * (n ? n : 1));
  if (!buf) return -1;
  double *px = buf, *py = buf + n, *pz = buf + 2 * n;
  double *qx = buf + 3 * n, *qy = buf + 4 * n, *qz = buf + 5 * n;
  double cx = 0, cy = 0, cz = 0, cvx = 0, cvy = 0, cvz = 0;
  for (uint64_t i = 0; i < n; ++i) {
    uint64_t k = 0;
    double X;
    do {
      X = w_unit(seed, i, k++);
    } while (X > 0.999 && k < 64);
    const double r = 1.0 / sqrt(pow(X, -2.0 / 3.0) - 1.0);
    const double ct = 1.0 - 2.0 * w_unit(seed, i, 64);
    const double st = sqrt(fmax(0.0, 1.0 - ct * ct));
    const double ph = kTwoPiW * w_unit(seed, i, 65);
    px[i] = r * st * cos(ph);
    py[i] = r * st * sin(ph);
    pz[i] = r * ct;
    double q = 0.0;
    uint64_t kk = 128;
    for (int it = 0; it < 20000; ++it) {
      q = w_unit(seed, i, kk);
      const double g = 0.1 * w_unit(seed, i, kk + 1);
      kk += 2;
      if (g < q * q * pow(1.0 - q * q, 3.5)) break;
    }
    const double v = q * sqrt(2.0) * pow(1.0 + r * r, -0.25);
    const double cv = 1.0 - 2.0 * w_unit(seed, i, 66);
    const double sv = sqrt(fmax(0.0, 1.0 - cv * cv));
    const double pv = kTwoPiW * w_unit(seed, i, 67);
    qx[i] = v * sv * cos(pv);
    qy[i] = v * sv * sin(pv);
    qz[i] = v * cv;
    cx += px[i];
    cy += py[i];
    cz += pz[i];
    cvx += qx[i];
    cvy += qy[i];
    cvz += qz[i];
  }
  const double inv = 1.0 / (double)n;
  cx *= inv;
  cy *= inv;
  cz *= inv;
  cvx *= inv;
  cvy *= inv;
  cvz *= inv;
  for (uint64_t i = 0; i < n; ++i) {
    x[i] = (float)(px[i] - cx);
    y[i] = (float)(py[i] - cy);
    z[i] = (float)(pz[i] - cz);
    vx[i] = (float)(qx[i] - cvx);
    vy[i] = (float)(qy[i] - cvy);
    vz[i] = (float)(qz[i] - cvz);
    if (mass) mass[i] = (float)inv;
  }
  free(buf);
  return 0;
}
