// Seeded initial conditions (host).  Compiled with -ffp-contract=off so that
// the values are identical on x86-64 and aarch64 hosts.
//
// Random numbers are counter based: draw(seed, particle, k) hashes the triple
// with the SplitMix64 output function (Steele, Lea & Flood, "Fast splittable
// pseudorandom number generators", OOPSLA 2014), so every particle's numbers
// are independent of the order in which particles are generated.
#include <cmath>
#include <cstdint>
#include <random>
#include <vector>

#include "nbody_gb300.h"

namespace {

constexpr double kTwoPi = 6.283185307179586476925286766559;

uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

uint64_t draw(uint64_t seed, uint64_t particle, uint64_t k) {
  return mix64(seed * 0x9E3779B97F4A7C15ull + mix64(particle * 0xD1B54A32D192ED03ull + k + 1));
}

// Uniform in (0, 1): 53 random bits, centred in their bin.
double unit(uint64_t seed, uint64_t particle, uint64_t k) {
  return (static_cast<double>(draw(seed, particle, k) >> 11) + 0.5) * 0x1.0p-53;
}

// Standard normal pair by Box-Muller from draws k, k+1.
void normal2(uint64_t seed, uint64_t particle, uint64_t k, double& a, double& b) {
  const double u = unit(seed, particle, k), v = unit(seed, particle, k + 1);
  const double rad = std::sqrt(-2.0 * std::log(u));
  a = rad * std::cos(kTwoPi * v);
  b = rad * std::sin(kTwoPi * v);
}

// One thin disk of n particles; particle i's random numbers are keyed by (seed, i).
void thin_disk(uint64_t seed, uint64_t n, double eps, float* x, float* y, float* z, float* vx,
               float* vy, float* vz, float* mass) {
  const double m = 1.0 / static_cast<double>(n);
  const double nm = static_cast<double>(n) * m;
  for (uint64_t i = 0; i < n; ++i) {
    const double r = std::sqrt(unit(seed, i, 0));
    const double th = kTwoPi * unit(seed, i, 1);
    double gz, g0, g1, g2;
    normal2(seed, i, 2, gz, g0);
    normal2(seed, i, 4, g1, g2);
    const double r2 = r * r;
    const double vt = r * std::sqrt(nm * r2 / std::pow(r2 + eps, 1.5));
    const double c = std::cos(th), s = std::sin(th);
    x[i] = static_cast<float>(r * c);
    y[i] = static_cast<float>(r * s);
    z[i] = static_cast<float>(0.01 * gz);
    vx[i] = static_cast<float>(-vt * s + 0.01 * g0);
    vy[i] = static_cast<float>(vt * c + 0.01 * g1);
    vz[i] = static_cast<float>(0.01 * g2);
    if (mass) mass[i] = static_cast<float>(m);
  }
}

bool bad_outputs(const void* a, const void* b, const void* c, const void* d, const void* e,
                 const void* f) {
  return !a || !b || !c || !d || !e || !f;
}

}  // namespace

extern "C" int nb_ic_thin_disk(uint64_t seed, uint64_t n, float eps, float* x, float* y,
                               float* z, float* vx, float* vy, float* vz, float* mass) {
  if (n == 0 || bad_outputs(x, y, z, vx, vy, vz) || !(eps >= 0.f)) return NB_ERR_INVALID_ARGUMENT;
  thin_disk(seed, n, eps, x, y, z, vx, vy, vz, mass);
  return NB_OK;
}

// Plummer sphere (Aarseth, Henon & Wielen 1974, A&A 37, 183): radius from the
// cumulative mass fraction X, r = (X^(-2/3) - 1)^(-1/2) (X resampled above 0.999,
// which truncates at r ~ 22.8 scale radii), isotropic direction; speed q * v_esc
// with v_esc = sqrt(2) (1 + r^2)^(-1/4) and q drawn from g(q) = q^2 (1 - q^2)^(7/2)
// by rejection under the bound 0.1.  G = M = a = 1.  The centre of mass is moved
// to the origin and set at rest.
extern "C" int nb_ic_plummer(uint64_t seed, uint64_t n, float* x, float* y, float* z,
                             float* vx, float* vy, float* vz, float* mass) {
  if (n == 0 || bad_outputs(x, y, z, vx, vy, vz)) return NB_ERR_INVALID_ARGUMENT;
  std::vector<double> px(n), py(n), pz(n), qx(n), qy(n), qz(n);
  double cx = 0, cy = 0, cz = 0, cvx = 0, cvy = 0, cvz = 0;
  for (uint64_t i = 0; i < n; ++i) {
    uint64_t k = 0;
    double X;
    do {
      X = unit(seed, i, k++);
    } while (X > 0.999 && k < 64);  // draws 0..63 only (64.. are the angles)
    const double r = 1.0 / std::sqrt(std::pow(X, -2.0 / 3.0) - 1.0);
    const double ct = 1.0 - 2.0 * unit(seed, i, 64);
    const double st = std::sqrt(std::max(0.0, 1.0 - ct * ct));
    const double ph = kTwoPi * unit(seed, i, 65);
    px[i] = r * st * std::cos(ph);
    py[i] = r * st * std::sin(ph);
    pz[i] = r * ct;
    double q;
    uint64_t kk = 128;
    for (int it = 0; it < 20000; ++it) {  // acceptance ~0.4: the bound is never reached
      q = unit(seed, i, kk);
      const double g = 0.1 * unit(seed, i, kk + 1);
      kk += 2;
      if (g < q * q * std::pow(1.0 - q * q, 3.5)) break;
    }
    const double v = q * std::sqrt(2.0) * std::pow(1.0 + r * r, -0.25);
    const double cv = 1.0 - 2.0 * unit(seed, i, 66);
    const double sv = std::sqrt(std::max(0.0, 1.0 - cv * cv));
    const double pv = kTwoPi * unit(seed, i, 67);
    qx[i] = v * sv * std::cos(pv);
    qy[i] = v * sv * std::sin(pv);
    qz[i] = v * cv;
    cx += px[i];
    cy += py[i];
    cz += pz[i];
    cvx += qx[i];
    cvy += qy[i];
    cvz += qz[i];
  }
  const double inv = 1.0 / static_cast<double>(n);
  cx *= inv, cy *= inv, cz *= inv, cvx *= inv, cvy *= inv, cvz *= inv;
  for (uint64_t i = 0; i < n; ++i) {
    x[i] = static_cast<float>(px[i] - cx);
    y[i] = static_cast<float>(py[i] - cy);
    z[i] = static_cast<float>(pz[i] - cz);
    vx[i] = static_cast<float>(qx[i] - cvx);
    vy[i] = static_cast<float>(qy[i] - cvy);
    vz[i] = static_cast<float>(qz[i] - cvz);
    if (mass) mass[i] = static_cast<float>(inv);
  }
  return NB_OK;
}

extern "C" int nb_ic_two_disks(uint64_t seed, uint64_t n, float eps, float* x, float* y,
                               float* z, float* vx, float* vy, float* vz, float* mass) {
  if (n < 2 || (n % 2) != 0 || bad_outputs(x, y, z, vx, vy, vz) || !(eps >= 0.f))
    return NB_ERR_INVALID_ARGUMENT;
  const uint64_t h = n / 2;
  thin_disk(seed, h, eps, x, y, z, vx, vy, vz, mass);
  thin_disk(seed + 0x5bd1e995ull, h, eps, x + h, y + h, z + h, vx + h, vy + h, vz + h,
            mass ? mass + h : nullptr);
  const double ca = std::cos(kTwoPi / 12.0), sa = std::sin(kTwoPi / 12.0);  // 30 degrees
  for (uint64_t i = 0; i < h; ++i) {
    x[i] = static_cast<float>(static_cast<double>(x[i]) - 2.0);
    vx[i] = static_cast<float>(static_cast<double>(vx[i]) + 0.3);
  }
  for (uint64_t i = h; i < n; ++i) {
    const double yy = y[i], zz = z[i], vyy = vy[i], vzz = vz[i];
    y[i] = static_cast<float>(ca * yy - sa * zz);
    z[i] = static_cast<float>(sa * yy + ca * zz);
    vy[i] = static_cast<float>(ca * vyy - sa * vzz);
    vz[i] = static_cast<float>(sa * vyy + ca * vzz);
    x[i] = static_cast<float>(static_cast<double>(x[i]) + 2.0);
    vx[i] = static_cast<float>(static_cast<double>(vx[i]) - 0.3);
  }
  return NB_OK;
}

extern "C" int nb_ic_ensemble_sizes(uint64_t seed, uint32_t num_systems, uint32_t lo,
                                    uint32_t hi, uint32_t* sizes) {
  if (!sizes || lo == 0 || hi < lo) return NB_ERR_INVALID_ARGUMENT;
  const double a = std::log(static_cast<double>(lo)), b = std::log(static_cast<double>(hi));
  for (uint32_t s = 0; s < num_systems; ++s) {
    const double v = std::exp(a + (b - a) * unit(seed, s, 0));
    const double r = std::floor(v + 0.5);
    sizes[s] = static_cast<uint32_t>(std::min<double>(hi, std::max<double>(lo, r)));
  }
  return NB_OK;
}

// DiskGalaxySimulator::randomParticlePos / initialParticleVel
// (simulator.cu:131-158): default-seeded std::mt19937 and
// std::uniform_real_distribution<double>(0, 1); per particle an angle
// t = 2 pi u and a radius s = 100 u (single precision, cos/sin of a float as the
// CUDA host headers resolve them), then z = 4 u for all particles; velocity
// normalize(p x z_hat) * sqrt(2 |p x z_hat|) with |.| evaluated in double
// (std::pow(float, 2) promotes) and rounded to float.
extern "C" int nb_ic_reference_disk(uint64_t n, float* x, float* y, float* z, float* vx,
                                    float* vy, float* vz) {
  if (n == 0 || bad_outputs(x, y, z, vx, vy, vz)) return NB_ERR_INVALID_ARGUMENT;
  const float kPi = 3.14159265358979323846f;
  std::mt19937 gen;
  std::uniform_real_distribution<> dis(0.0, 1.0);
  for (uint64_t i = 0; i < n; ++i) {
    const float t = static_cast<float>(dis(gen) * 2 * kPi);
    const float s = static_cast<float>(dis(gen) * 100);
    x[i] = std::cos(t) * s;
    y[i] = std::sin(t) * s;
  }
  for (uint64_t i = 0; i < n; ++i) z[i] = static_cast<float>(4.0 * dis(gen));
  auto length = [](float a, float b, float c) {
    return static_cast<float>(std::sqrt(std::pow(a, 2) + std::pow(b, 2) + std::pow(c, 2)));
  };
  for (uint64_t i = 0; i < n; ++i) {
    // cross(p, (0, 0, 1)) in float
    const float cx = y[i] * 1.0f - z[i] * 0.0f;
    const float cy = z[i] * 0.0f - x[i] * 1.0f;
    const float cz = x[i] * 0.0f - y[i] * 0.0f;
    const float orbital = static_cast<float>(std::sqrt(2.0 * length(cx, cy, cz)));
    const float len = length(cx, cy, cz);
    vx[i] = (cx / len) * orbital;
    vy[i] = (cy / len) * orbital;
    vz[i] = (cz / len) * orbital;
  }
  return NB_OK;
}
