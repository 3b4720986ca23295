// Parameters and buffers of the headless renderer (render_kernels.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace nbg {

constexpr int kRenderMaxTaps = 32;

struct RenderUniforms {
  float pv[16];          // proj * view, column-major
  float flare_x;         // sprite half-size in NDC
  float flare_y;
  int32_t width;         // output image
  int32_t height;
  int32_t margin;        // HDR framebuffer margin (FBO_MARGIN)
  int32_t bw, bh;        // HDR framebuffer
  int32_t ow, oh;        // blur targets (downscaled by 2)
  int32_t lw, lh;        // luminance target (half size)
  int32_t flare_n;       // flare texture is flare_n x flare_n
  float size_x, size_y;  // blur sample step (blurDownscale / width, / height)
  int32_t taps;          // Gaussian taps (centre + taps - 1 symmetric pairs)
  float offset[kRenderMaxTaps];
  float weight[kRenderMaxTaps];
};

struct RenderBuffers {
  float4* hdr = nullptr;     // bw x bh
  float4* blur1 = nullptr;   // ow x oh
  float4* blur2 = nullptr;   // ow x oh (bloom)
  float* lum = nullptr;      // lw x lh
  double* block_sums = nullptr;
  float* mean = nullptr;
  float* flare = nullptr;    // flare_n x flare_n
  int32_t width = 0, height = 0;
};

cudaError_t launch_render(const float* pos, const float4* vel, int64_t n_pad,
                          const RenderUniforms& u, const RenderBuffers& b, float4* out,
                          cudaStream_t stream);

// Host tables shared by the renderer and its tests.
void render_gauss_tables(float sigma, int halfwidth, float* offsets, float* weights, int* taps);
void render_flare_texture(int n, float* pixels);

}  // namespace nbg
