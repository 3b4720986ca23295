// Headless render math of the reference's OpenGL renderer, as CUDA kernels.
//
// The reference draws every particle as an additive, velocity-coloured point
// sprite into an HDR framebuffer with a 50-pixel margin
// (src/renderer_gl.cpp:96-111; shaders/gl/main.{vert,geom,frag}).  It then blurs
// a half-resolution copy with a separable Gaussian (renderer_gl.cpp:113-137,
// shaders/gl/blur.frag), reduces luminance over a mip chain (renderer_gl.cpp:139-146,
// shaders/gl/luminance.frag), and tonemaps HDR + bloom with an exposure and
// gamma 2.2 (renderer_gl.cpp:148-156, shaders/gl/tonemap.frag).  Here the same
// arithmetic runs on device buffers: images are row-major float4 with row 0 at
// the bottom (the framebuffer convention), sampling is bilinear with the
// texture's wrap mode, and blending is float atomics (FP32 instead of the
// reference's RGBA16F).
#include <cuda_runtime.h>

#include <cstdint>

#include "nb_internal.hpp"
#include "nb_render.hpp"

namespace nbg {
namespace {

__device__ __forceinline__ float4 f4(float a, float b, float c, float d) {
  return make_float4(a, b, c, d);
}

// Bilinear fetch at normalised coordinates, clamp-to-edge.
__device__ float4 sample_clamp(const float4* img, int w, int h, float s, float t) {
  const float u = s * w - 0.5f, v = t * h - 0.5f;
  const float fu = floorf(u), fv = floorf(v);
  const float a = u - fu, b = v - fv;
  int x0 = static_cast<int>(fu), y0 = static_cast<int>(fv);
  int x1 = x0 + 1, y1 = y0 + 1;
  x0 = min(max(x0, 0), w - 1);
  x1 = min(max(x1, 0), w - 1);
  y0 = min(max(y0, 0), h - 1);
  y1 = min(max(y1, 0), h - 1);
  const float4 p00 = img[y0 * w + x0], p10 = img[y0 * w + x1];
  const float4 p01 = img[y1 * w + x0], p11 = img[y1 * w + x1];
  const float w00 = (1 - a) * (1 - b), w10 = a * (1 - b), w01 = (1 - a) * b, w11 = a * b;
  return f4(p00.x * w00 + p10.x * w10 + p01.x * w01 + p11.x * w11,
            p00.y * w00 + p10.y * w10 + p01.y * w01 + p11.y * w11,
            p00.z * w00 + p10.z * w10 + p01.z * w01 + p11.z * w11,
            p00.w * w00 + p10.w * w10 + p01.w * w01 + p11.w * w11);
}

// Bilinear fetch of the flare texture (one channel), repeat wrap (its sampler
// never sets a wrap mode, renderer_gl.cpp:53-63).
__device__ float sample_flare(const float* tex, int n, float s, float t) {
  const float u = s * n - 0.5f, v = t * n - 0.5f;
  const float fu = floorf(u), fv = floorf(v);
  const float a = u - fu, b = v - fv;
  const int x0 = ((static_cast<int>(fu) % n) + n) % n, y0 = ((static_cast<int>(fv) % n) + n) % n;
  const int x1 = (x0 + 1) % n, y1 = (y0 + 1) % n;
  return tex[y0 * n + x0] * (1 - a) * (1 - b) + tex[y0 * n + x1] * a * (1 - b) +
         tex[y1 * n + x0] * (1 - a) * b + tex[y1 * n + x1] * a * b;
}

// One thread per particle: main.vert (colour), main.geom (screen-aligned quad of
// half-size flare * w in clip space), main.frag (flare alpha), additive blend.
__global__ void splat_kernel(const float* __restrict__ pos, const float4* __restrict__ vel,
                             int64_t n_pad, RenderUniforms u, const float* __restrict__ flare,
                             float4* __restrict__ hdr) {
  for (int64_t g = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; g < n_pad;
       g += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    if (pos[pair_index(g, 3)] == 0.f && pos[pair_index(g, 0)] == kFarAway) continue;  // padding
    const float px = pos[pair_index(g, 0)], py = pos[pair_index(g, 1)], pz = pos[pair_index(g, 2)];
    const float* M = u.pv;  // p * mv, column-major
    const float cx = M[0] * px + M[4] * py + M[8] * pz + M[12];
    const float cy = M[1] * px + M[5] * py + M[9] * pz + M[13];
    const float cz = M[2] * px + M[6] * py + M[10] * pz + M[14];
    const float cw = M[3] * px + M[7] * py + M[11] * pz + M[15];
    if (!(cw > 0.f) || cz < -cw || cz > cw) continue;  // clipped
    // slow -> blue, fast -> purple; the velocity attribute carries w = 1 (renderer_gl.cpp:169)
    const float4 v = vel[g];
    const float t = fminf(fmaxf((v.x * v.x + v.y * v.y + v.z * v.z + 1.f) * 0.0006f, 0.f), 1.f);
    // GLSL mix(x, y, a) = x * (1 - a) + y * a of (0, 0.4, 1) and (1, 0.2, 1)
    const float r = 0.f * (1.f - t) + 1.f * t;
    const float gr = 0.4f * (1.f - t) + 0.2f * t;
    const float b = 1.f * (1.f - t) + 1.f * t;
    const float nx = cx / cw, ny = cy / cw;
    const float x0 = nx - u.flare_x, x1 = nx + u.flare_x;
    const float y0 = ny - u.flare_y, y1 = ny + u.flare_y;
    // pixel centres (k + 0.5) inside [x0, x1) in NDC
    const int kx0 = max(0, static_cast<int>(ceilf((x0 + 1.f) * 0.5f * u.bw - 0.5f)));
    const int kx1 = min(u.bw - 1, static_cast<int>(ceilf((x1 + 1.f) * 0.5f * u.bw - 0.5f)) - 1);
    const int ky0 = max(0, static_cast<int>(ceilf((y0 + 1.f) * 0.5f * u.bh - 0.5f)));
    const int ky1 = min(u.bh - 1, static_cast<int>(ceilf((y1 + 1.f) * 0.5f * u.bh - 0.5f)) - 1);
    for (int ky = ky0; ky <= ky1; ++ky) {
      const float ndy = (ky + 0.5f) / u.bh * 2.f - 1.f;
      const float by = (ndy - y0) / (y1 - y0);
      for (int kx = kx0; kx <= kx1; ++kx) {
        const float ndx = (kx + 0.5f) / u.bw * 2.f - 1.f;
        const float bx = (ndx - x0) / (x1 - x0);
        const float alpha = sample_flare(flare, u.flare_n, bx, by);
        // One 16-byte vector reduction per pixel (sm_90+ global float4 atomicAdd)
        // instead of three scalar ones: the splat is bound by L2 atomic throughput.
        atomicAdd(hdr + static_cast<int64_t>(ky) * u.bw + kx, f4(r * alpha, gr * alpha, b * alpha, 0.f));
      }
    }
  }
}

// One pass of the separable blur (blur.frag) into a (ow x oh) target.
__global__ void blur_kernel(const float4* __restrict__ src, int sw, int sh, float4* __restrict__ dst,
                            int ow, int oh, RenderUniforms u, float mx, float my) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= ow || y >= oh) return;
  const float s = (x + 0.5f) / ow, t = (y + 0.5f) / oh;
  float4 c = sample_clamp(src, sw, sh, s, t);
  float4 acc = f4(c.x * u.weight[0], c.y * u.weight[0], c.z * u.weight[0], c.w * u.weight[0]);
  for (int i = 1; i < u.taps; ++i) {
    const float dx = u.offset[i] * mx * u.size_x, dy = u.offset[i] * my * u.size_y;
    const float4 a = sample_clamp(src, sw, sh, s + dx, t + dy);
    const float4 b = sample_clamp(src, sw, sh, s - dx, t - dy);
    acc.x += (a.x + b.x) * u.weight[i];
    acc.y += (a.y + b.y) * u.weight[i];
    acc.z += (a.z + b.z) * u.weight[i];
    acc.w += (a.w + b.w) * u.weight[i];
  }
  dst[y * ow + x] = acc;
}

// luminance.frag at half resolution; per-block sums for the mean (the top of
// the mip chain the tonemap reads).
__global__ void luminance_kernel(const float4* __restrict__ hdr, RenderUniforms u,
                                 float* __restrict__ lum, double* __restrict__ block_sums) {
  __shared__ double sh[256];
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  double v = 0.0;
  if (x < u.lw && y < u.lh) {
    const float s = (x * 2.f + 0.5f + 1.f) / u.bw;  // (gl_FragCoord * 2 + 0.5) / size
    const float t = (y * 2.f + 0.5f + 1.f) / u.bh;
    const float4 c = sample_clamp(hdr, u.bw, u.bh, s, t);
    const float l = 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z;
    lum[y * u.lw + x] = l;
    v = l;
  }
  sh[tid] = v;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (tid < w) sh[tid] += sh[tid + w];
    __syncthreads();
  }
  if (tid == 0) block_sums[blockIdx.y * gridDim.x + blockIdx.x] = sh[0];
}

// Mean of the luminance blocks' sums: one block of kMeanThreads threads, each
// summing a fixed stride of the blocks, then a fixed tree (deterministic).
constexpr int kMeanThreads = 256;

__global__ void __launch_bounds__(kMeanThreads) mean_kernel(const double* __restrict__ block_sums,
                                                            int count, double inv_pixels,
                                                            float* __restrict__ mean) {
  __shared__ double sh[kMeanThreads];
  double s = 0.0;
  for (int i = threadIdx.x; i < count; i += kMeanThreads) s += block_sums[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = kMeanThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *mean = static_cast<float>(sh[0] * inv_pixels);
}

// tonemap.frag: HDR + bloom, exposure from the mean luminance, gamma 2.2.
__global__ void tonemap_kernel(const float4* __restrict__ hdr, const float4* __restrict__ bloom,
                               const float* __restrict__ mean, RenderUniforms u,
                               float4* __restrict__ out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= u.width || y >= u.height) return;
  const int cx = x + u.margin, cy = y + u.margin;
  const float4 c = hdr[cy * u.bw + cx];
  const float exposure = 1.f / fminf(fmaxf(*mean * 10.f, 0.2f), 1000.f);
  const float4 b = sample_clamp(bloom, u.ow, u.oh, static_cast<float>(cx) / u.bw,
                                static_cast<float>(cy) / u.bh);
  const float r = 1.f - expf(-(c.x + b.x) * exposure);
  const float g = 1.f - expf(-(c.y + b.y) * exposure);
  const float bl = 1.f - expf(-(c.z + b.z) * exposure);
  out[y * u.width + x] = f4(powf(r, 1.f / 2.2f), powf(g, 1.f / 2.2f), powf(bl, 1.f / 2.2f), 1.f);
}

}  // namespace

cudaError_t launch_render(const float* pos, const float4* vel, int64_t n_pad,
                          const RenderUniforms& u, const RenderBuffers& b, float4* out,
                          cudaStream_t stream) {
  cudaError_t e = cudaMemsetAsync(b.hdr, 0, sizeof(float4) * u.bw * u.bh, stream);
  if (e != cudaSuccess) return e;
  const int64_t blocks = (n_pad + 255) / 256;
  splat_kernel<<<static_cast<unsigned>(blocks < 8192 ? blocks : 8192), 256, 0, stream>>>(
      pos, vel, n_pad, u, b.flare, b.hdr);
  const dim3 blk(16, 16);
  const dim3 go((u.ow + 15) / 16, (u.oh + 15) / 16);
  blur_kernel<<<go, blk, 0, stream>>>(b.hdr, u.bw, u.bh, b.blur1, u.ow, u.oh, u, 1.f, 0.f);
  blur_kernel<<<go, blk, 0, stream>>>(b.blur1, u.ow, u.oh, b.blur2, u.ow, u.oh, u, 0.f, 1.f);
  const dim3 gl((u.lw + 15) / 16, (u.lh + 15) / 16);
  luminance_kernel<<<gl, blk, 0, stream>>>(b.hdr, u, b.lum, b.block_sums);
  mean_kernel<<<1, kMeanThreads, 0, stream>>>(b.block_sums, static_cast<int>(gl.x * gl.y),
                                    1.0 / (static_cast<double>(u.lw) * u.lh), b.mean);
  const dim3 gt((u.width + 15) / 16, (u.height + 15) / 16);
  tonemap_kernel<<<gt, blk, 0, stream>>>(b.hdr, b.blur2, b.mean, u, out);
  return cudaGetLastError();
}

}  // namespace nbg
