/*
 * render_oracle.c -- CPU restatement of the reference's render math.
 *
 * TEST INFRASTRUCTURE ONLY: the checker of the library's headless renderer
 * (csrc/render_kernels.cu).  It follows the reference's OpenGL pipeline in plain C,
 * one pixel and one particle at a time:
 *   sprites    shaders/gl/main.vert:15-20, main.geom:15-39, main.frag:11-15,
 *              additive blend (src/renderer_gl.cpp:100-111), FBO margin 50 (:18, :52-53)
 *   bloom      shaders/gl/blur.frag:17-30 at half size, horizontal then vertical
 *              (src/renderer_gl.cpp:116-137)
 *   luminance  shaders/gl/luminance.frag:8-15 at half size, then its mean (the top
 *              of the mip chain read at src/renderer_gl.cpp:146, tonemap.frag:22)
 *   tonemap    shaders/gl/tonemap.frag:16-29
 * The reference's GL output cannot be produced here (no graphics stack), so this
 * restatement is not pinned to reference output.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

static void sample_clamp(const float* img, int w, int h, float s, float t, float* out) {
  const float u = s * w - 0.5f, v = t * h - 0.5f;
  const float fu = floorf(u), fv = floorf(v);
  const float a = u - fu, b = v - fv;
  int x0 = (int)fu, y0 = (int)fv, x1 = x0 + 1, y1 = y0 + 1;
  x0 = x0 < 0 ? 0 : (x0 > w - 1 ? w - 1 : x0);
  x1 = x1 < 0 ? 0 : (x1 > w - 1 ? w - 1 : x1);
  y0 = y0 < 0 ? 0 : (y0 > h - 1 ? h - 1 : y0);
  y1 = y1 < 0 ? 0 : (y1 > h - 1 ? h - 1 : y1);
  const float w00 = (1 - a) * (1 - b), w10 = a * (1 - b), w01 = (1 - a) * b, w11 = a * b;
  for (int c = 0; c < 4; ++c)
    out[c] = img[4 * (y0 * w + x0) + c] * w00 + img[4 * (y0 * w + x1) + c] * w10 +
             img[4 * (y1 * w + x0) + c] * w01 + img[4 * (y1 * w + x1) + c] * w11;
}

static float sample_flare(const float* tex, int n, float s, float t) {
  const float u = s * n - 0.5f, v = t * n - 0.5f;
  const float fu = floorf(u), fv = floorf(v);
  const float a = u - fu, b = v - fv;
  const int x0 = (((int)fu % n) + n) % n, y0 = (((int)fv % n) + n) % n;
  const int x1 = (x0 + 1) % n, y1 = (y0 + 1) % n;
  return tex[y0 * n + x0] * (1 - a) * (1 - b) + tex[y0 * n + x1] * a * (1 - b) +
         tex[y1 * n + x0] * (1 - a) * b + tex[y1 * n + x1] * a * b;
}

static void blur(const float* src, int sw, int sh, float* dst, int ow, int oh, const float* off,
                 const float* wt, int taps, float size_x, float size_y, float mx, float my) {
  for (int y = 0; y < oh; ++y)
    for (int x = 0; x < ow; ++x) {
      const float s = (x + 0.5f) / ow, t = (y + 0.5f) / oh;
      float c[4], a[4], b[4], acc[4];
      sample_clamp(src, sw, sh, s, t, c);
      for (int k = 0; k < 4; ++k) acc[k] = c[k] * wt[0];
      for (int i = 1; i < taps; ++i) {
        const float dx = off[i] * mx * size_x, dy = off[i] * my * size_y;
        sample_clamp(src, sw, sh, s + dx, t + dy, a);
        sample_clamp(src, sw, sh, s - dx, t - dy, b);
        for (int k = 0; k < 4; ++k) acc[k] += (a[k] + b[k]) * wt[i];
      }
      memcpy(dst + 4 * (y * ow + x), acc, sizeof(acc));
    }
}

/* out: width x height x 4 floats (row 0 at the bottom).  pv: proj * view,
 * column-major.  Returns 0, or 1 if memory ran out. */
int oracle_render(int64_t n, const float* px, const float* py, const float* pz, const float* vx,
                  const float* vy, const float* vz, const float* pv, int width, int height,
                  const float* off, const float* wt, int taps, const float* flare, int flare_n,
                  float* out) {
  const int margin = 50, bw = width + 2 * margin, bh = height + 2 * margin;
  const int ow = bw / 2, oh = bh / 2, lw = bw / 2, lh = bh / 2;
  const float fx = flare_n / (float)(2 * width), fy = flare_n / (float)(2 * height);
  const float size_x = 2.0f / width, size_y = 2.0f / height;
  float* hdr = calloc((size_t)bw * bh * 4, sizeof(float));
  float* b1 = calloc((size_t)ow * oh * 4, sizeof(float));
  float* b2 = calloc((size_t)ow * oh * 4, sizeof(float));
  if (!hdr || !b1 || !b2) {
    free(hdr);
    free(b1);
    free(b2);
    return 1;
  }
  for (int64_t i = 0; i < n; ++i) {
    const float X = px[i], Y = py[i], Z = pz[i];
    const float cx = pv[0] * X + pv[4] * Y + pv[8] * Z + pv[12];
    const float cy = pv[1] * X + pv[5] * Y + pv[9] * Z + pv[13];
    const float cz = pv[2] * X + pv[6] * Y + pv[10] * Z + pv[14];
    const float cw = pv[3] * X + pv[7] * Y + pv[11] * Z + pv[15];
    if (!(cw > 0.f) || cz < -cw || cz > cw) continue;
    float t = (vx[i] * vx[i] + vy[i] * vy[i] + vz[i] * vz[i] + 1.f) * 0.0006f;
    t = fminf(fmaxf(t, 0.f), 1.f);
    const float r = 0.f * (1.f - t) + 1.f * t;
    const float g = 0.4f * (1.f - t) + 0.2f * t;
    const float b = 1.f * (1.f - t) + 1.f * t;
    const float nx = cx / cw, ny = cy / cw;
    const float x0 = nx - fx, x1 = nx + fx, y0 = ny - fy, y1 = ny + fy;
    int kx0 = (int)ceilf((x0 + 1.f) * 0.5f * bw - 0.5f);
    int kx1 = (int)ceilf((x1 + 1.f) * 0.5f * bw - 0.5f) - 1;
    int ky0 = (int)ceilf((y0 + 1.f) * 0.5f * bh - 0.5f);
    int ky1 = (int)ceilf((y1 + 1.f) * 0.5f * bh - 0.5f) - 1;
    if (kx0 < 0) kx0 = 0;
    if (ky0 < 0) ky0 = 0;
    if (kx1 > bw - 1) kx1 = bw - 1;
    if (ky1 > bh - 1) ky1 = bh - 1;
    for (int ky = ky0; ky <= ky1; ++ky) {
      const float ndy = (ky + 0.5f) / bh * 2.f - 1.f;
      const float by = (ndy - y0) / (y1 - y0);
      for (int kx = kx0; kx <= kx1; ++kx) {
        const float ndx = (kx + 0.5f) / bw * 2.f - 1.f;
        const float bx = (ndx - x0) / (x1 - x0);
        const float a = sample_flare(flare, flare_n, bx, by);
        float* d = hdr + 4 * ((int64_t)ky * bw + kx);
        d[0] += r * a;
        d[1] += g * a;
        d[2] += b * a;
      }
    }
  }
  blur(hdr, bw, bh, b1, ow, oh, off, wt, taps, size_x, size_y, 1.f, 0.f);
  blur(b1, ow, oh, b2, ow, oh, off, wt, taps, size_x, size_y, 0.f, 1.f);
  double lsum = 0.0;
  for (int y = 0; y < lh; ++y)
    for (int x = 0; x < lw; ++x) {
      float c[4];
      sample_clamp(hdr, bw, bh, (x * 2.f + 0.5f + 1.f) / bw, (y * 2.f + 0.5f + 1.f) / bh, c);
      lsum += 0.2126f * c[0] + 0.7152f * c[1] + 0.0722f * c[2];
    }
  const float mean = (float)(lsum / ((double)lw * lh));
  const float exposure = 1.f / fminf(fmaxf(mean * 10.f, 0.2f), 1000.f);
  for (int y = 0; y < height; ++y)
    for (int x = 0; x < width; ++x) {
      const int cx = x + margin, cy = y + margin;
      const float* c = hdr + 4 * (cy * bw + cx);
      float bl[4];
      sample_clamp(b2, ow, oh, (float)cx / bw, (float)cy / bh, bl);
      float* o = out + 4 * (y * width + x);
      for (int k = 0; k < 3; ++k) o[k] = powf(1.f - expf(-(c[k] + bl[k]) * exposure), 1.f / 2.2f);
      o[3] = 1.f;
    }
  free(hdr);
  free(b1);
  free(b2);
  return 0;
}
