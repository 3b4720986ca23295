// Headless renderer (host side): camera matrices, the Gaussian and flare tables of
// the reference's renderer, and nb_sim_render.  The image arithmetic is in
// render_kernels.cu.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "nb_render.hpp"
#include "nb_runtime.hpp"
#include "nbody_gb300.h"

namespace nbg {

// RendererGL::gaussKernel + optimGaussKernel (renderer_gl.cpp:314-368): a
// normalised 1-D Gaussian of `halfwidth` taps, then pairs of neighbouring taps
// merged into one bilinear sample at their weighted mean offset.
void render_gauss_tables(float sigma, int halfwidth, float* offsets, float* weights, int* taps) {
  const float pi = 3.14159265358979323846f;
  const float sigma_factor = 1.0f / (sigma * std::sqrt(2 * pi));
  std::vector<float> w(halfwidth);
  for (int n = 0; n < halfwidth; ++n)
    w[n] = static_cast<float>(sigma_factor * std::exp(-std::pow(static_cast<float>(n), 2) /
                                                      (2 * std::pow(sigma, 2))));
  const float halfnorm = static_cast<float>(std::accumulate(w.begin() + 1, w.end(), 0.0));
  const float norm = 2 * halfnorm + w[0];
  for (auto& v : w) v = v / norm;
  const int out = halfwidth / 2 + 1;
  offsets[0] = 0.f;
  weights[0] = w[0];
  for (int i = 1; i < out; ++i) {
    weights[i] = w[2 * i - 1];
    offsets[i] = static_cast<float>(2 * i - 1);
    if (2 * i < halfwidth) {
      weights[i] += w[2 * i];
      offsets[i] = ((2 * i - 1) * w[2 * i - 1] + (2 * i) * w[2 * i]) / weights[i];
    }
  }
  *taps = out;
}

// genFlareTex (gen.cpp:36-51): a gamma-corrected Gaussian, sigma^2 = n / 2.
void render_flare_texture(int n, float* pixels) {
  const float sigma2 = n / 2.0f;
  for (int i = 0; i < n; ++i) {
    const float i1 = static_cast<float>(i - n / 2);
    for (int j = 0; j < n; ++j) {
      const float j1 = static_cast<float>(j - n / 2);
      pixels[i * n + j] = static_cast<float>(
          std::pow(std::exp(-((i1 * i1) / (2 * sigma2) + (j1 * j1) / (2 * sigma2))), 2.2));
    }
  }
}

}  // namespace nbg

using namespace nbg;

namespace {

constexpr int kMargin = 50;     // FBO_MARGIN, renderer_gl.cpp:18
constexpr int kFlareSize = 16;  // texSize, renderer_gl.cpp:54
constexpr int kBlurDownscale = 2;

void mat_mul(const float* a, const float* b, float* c) {  // c = a * b, column-major
  for (int col = 0; col < 4; ++col)
    for (int row = 0; row < 4; ++row) {
      float s = 0.f;
      for (int k = 0; k < 4; ++k) s += a[k * 4 + row] * b[col * 4 + k];
      c[col * 4 + row] = s;
    }
}

void release_render(RenderBuffers& b) {
  dev_free(b.hdr);
  dev_free(b.blur1);
  dev_free(b.blur2);
  dev_free(b.lum);
  dev_free(b.block_sums);
  dev_free(b.mean);
  dev_free(b.flare);
  b = RenderBuffers{};
}

}  // namespace

namespace nbg {
void release_render_buffers(nb_sim* s) { release_render(s->render); }
}  // namespace nbg

extern "C" {

int nb_camera_matrices(float azimuth, float elevation, float distance, const float look_at[3],
                       int32_t width, int32_t height, float view[16], float proj[16]) {
  if (!view || !proj || width <= 0 || height <= 0 || !(distance > 0.f))
    return set_error(NB_ERR_INVALID_ARGUMENT, "bad camera arguments");
  const float at[3] = {look_at ? look_at[0] : 0.f, look_at ? look_at[1] : 0.f,
                       look_at ? look_at[2] : 0.f};
  // Camera::getView (camera.cpp:43-52): polar position around look_at, z up.
  const float eye[3] = {std::cos(azimuth) * std::cos(elevation) * distance + at[0],
                        std::sin(azimuth) * std::cos(elevation) * distance + at[1],
                        std::sin(elevation) * distance + at[2]};
  float f[3] = {at[0] - eye[0], at[1] - eye[1], at[2] - eye[2]};
  float fl = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
  for (float& v : f) v /= fl;
  const float up[3] = {0.f, 0.f, 1.f};
  float sv[3] = {f[1] * up[2] - f[2] * up[1], f[2] * up[0] - f[0] * up[2],
                 f[0] * up[1] - f[1] * up[0]};
  const float sl = std::sqrt(sv[0] * sv[0] + sv[1] * sv[1] + sv[2] * sv[2]);
  if (!(sl > 0.f)) return set_error(NB_ERR_INVALID_ARGUMENT, "view direction parallel to z");
  for (float& v : sv) v /= sl;
  const float uv[3] = {sv[1] * f[2] - sv[2] * f[1], sv[2] * f[0] - sv[0] * f[2],
                       sv[0] * f[1] - sv[1] * f[0]};
  std::memset(view, 0, 16 * sizeof(float));
  for (int k = 0; k < 3; ++k) {  // right-handed look-at, column-major
    view[k * 4 + 0] = sv[k];
    view[k * 4 + 1] = uv[k];
    view[k * 4 + 2] = -f[k];
  }
  view[12] = -(sv[0] * eye[0] + sv[1] * eye[1] + sv[2] * eye[2]);
  view[13] = -(uv[0] * eye[0] + uv[1] * eye[1] + uv[2] * eye[2]);
  view[14] = f[0] * eye[0] + f[1] * eye[1] + f[2] * eye[2];
  view[15] = 1.f;
  // Camera::getProj (camera.cpp:38-41): infinite perspective, fovy 30 deg, near 1.
  const float fovy = 30.f * 3.14159265358979323846f / 180.f, near = 1.f;
  const float aspect = static_cast<float>(width) / static_cast<float>(height);
  const float range = std::tan(fovy / 2.f) * near;
  std::memset(proj, 0, 16 * sizeof(float));
  proj[0] = (2.f * near) / (range * aspect - (-range * aspect));
  proj[5] = (2.f * near) / (range - (-range));
  proj[10] = -1.f;
  proj[11] = -1.f;
  proj[14] = -2.f * near;
  return NB_OK;
}

int nb_render_tables(float* gauss_offsets, float* gauss_weights, int32_t* taps, float* flare) {
  if (!gauss_offsets || !gauss_weights || !taps || !flare)
    return set_error(NB_ERR_INVALID_ARGUMENT, "NULL argument");
  int t = 0;
  render_gauss_tables(10.0f, 25, gauss_offsets, gauss_weights, &t);  // renderer_gl.cpp:86
  *taps = t;
  render_flare_texture(kFlareSize, flare);
  return NB_OK;
}

int nb_sim_render(nb_sim* s, const float view[16], const float proj[16], int32_t width,
                  int32_t height, float* rgba_device) {
  if (!s || !view || !proj || !rgba_device)
    return set_error(NB_ERR_INVALID_ARGUMENT, "NULL argument");
  DeviceGuard dg_(s->device);
  if (width < 16 || height < 16 || width > 16384 || height > 16384)
    return set_error(NB_ERR_INVALID_ARGUMENT, "image size must be in [16, 16384]");
  if (reinterpret_cast<uintptr_t>(rgba_device) & 15)
    return set_error(NB_ERR_INVALID_ARGUMENT, "image buffer must be 16-byte aligned");
  RenderUniforms u{};
  float pv[16];
  mat_mul(proj, view, pv);
  std::memcpy(u.pv, pv, sizeof(pv));
  u.flare_x = kFlareSize / static_cast<float>(2 * width);  // renderer_gl.cpp:79-80
  u.flare_y = kFlareSize / static_cast<float>(2 * height);
  u.width = width;
  u.height = height;
  u.margin = kMargin;
  u.bw = width + 2 * kMargin;
  u.bh = height + 2 * kMargin;
  u.ow = u.bw / kBlurDownscale;
  u.oh = u.bh / kBlurDownscale;
  u.lw = u.bw / 2;
  u.lh = u.bh / 2;
  u.flare_n = kFlareSize;
  u.size_x = static_cast<float>(kBlurDownscale) / width;  // renderer_gl.cpp:82-83
  u.size_y = static_cast<float>(kBlurDownscale) / height;
  int taps = 0;
  render_gauss_tables(10.0f, 25, u.offset, u.weight, &taps);
  u.taps = taps;
  RenderBuffers& b = s->render;
  if (b.width != width || b.height != height) {
    release_render(b);
    NB_TRY(dev_alloc(&b.hdr, static_cast<size_t>(u.bw) * u.bh));
    NB_TRY(dev_alloc(&b.blur1, static_cast<size_t>(u.ow) * u.oh));
    NB_TRY(dev_alloc(&b.blur2, static_cast<size_t>(u.ow) * u.oh));
    NB_TRY(dev_alloc(&b.lum, static_cast<size_t>(u.lw) * u.lh));
    NB_TRY(dev_alloc(&b.block_sums, static_cast<size_t>((u.lw + 15) / 16) * ((u.lh + 15) / 16)));
    NB_TRY(dev_alloc(&b.mean, 1));
    NB_TRY(dev_alloc(&b.flare, kFlareSize * kFlareSize));
    std::vector<float> fl(kFlareSize * kFlareSize);
    render_flare_texture(kFlareSize, fl.data());
    NB_CUDA(cudaMemcpy(b.flare, fl.data(), fl.size() * sizeof(float), cudaMemcpyHostToDevice));
    b.width = width;
    b.height = height;
  }
  NB_CUDA(launch_render(s->pos_d[s->cur], s->vel_d, s->n_pad, u, b,
                        reinterpret_cast<float4*>(rgba_device), s->stream));
  return NB_OK;
}

}  // extern "C"
