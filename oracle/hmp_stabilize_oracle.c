/*
 * hmp_stabilize_oracle.c -- CPU restatement of hm-cupano's frame stabiliser.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for libhmpano's stabiliser kernels. Only tests/ load it
 * (through oracle/oracle.py); the product never links, loads or calls it.
 *
 * It restates src/cuda/cudaStabilize.cu step by step, in the reference's operation order, FP32,
 * no fused multiply-add (the library is built with -ffp-contract=off):
 *   - Sobel gradients of interior pixels               cudaStabilize.cu:24-37
 *   - Harris response over a 3x3 window, det - k tr^2  cudaStabilize.cu:43-69
 *   - threshold + 3x3 non-maximum suppression, corners
 *     in raster order                                  cudaStabilize.cu:157-204
 *   - sparse Lucas-Kanade, 10 iterations, displacement
 *     rounded to whole pixels for sampling             cudaStabilize.cu:75-132
 *   - global motion = mean flow, translation by the
 *     rounded mean, zero fill                          cudaStabilize.cu:137-150, 243-267
 * Where the reference reads memory it never defines, this restatement fixes a value:
 *   - its gradient buffers are never written outside the interior and its response buffer never
 *     on the image border (cudaMalloc'd, so undefined), yet the Harris window and the
 *     suppression read them there: here they are 0;
 *   - its flow window admits taps in column 0 and row 0, whose central differences read the
 *     pixel before the image (index -1, or the row above row 0): here those taps are skipped;
 *   - with no corners the reference's mean is 0/0: here the motion is 0;
 *   - a displacement is rounded to whole pixels the way the GPU's float-to-int conversion does it
 *     (saturating, NaN to 0), clamped here to +-2^24: any shift that large moves every tap and
 *     every warped pixel off the frame, as the saturated one does (plain C leaves it undefined).
 * Parity unpinned: the reference ships this only as a demo program, with no tests or vectors.
 */
#include <math.h>
#include <stddef.h>

#include "hmp_oracle.h"

static int shift_of(float v) {
  if (!(v == v)) return 0;
  const float r = roundf(v);
  if (r > 16777216.0f) return 16777216;
  if (r < -16777216.0f) return -16777216;
  return (int)r;
}

static void gradients(const float* img, int w, int h, float* gx, float* gy) {
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      float vx = 0.0f, vy = 0.0f;
      if (x > 0 && x < w - 1 && y > 0 && y < h - 1) {
        const float* r0 = img + (size_t)(y - 1) * w;
        const float* r1 = img + (size_t)y * w;
        const float* r2 = img + (size_t)(y + 1) * w;
        vx = r0[x + 1] + 2.0f * r1[x + 1] + r2[x + 1] - r0[x - 1] - 2.0f * r1[x - 1] - r2[x - 1];
        vy = r0[x - 1] + 2.0f * r0[x] + r0[x + 1] - r2[x - 1] - 2.0f * r2[x] - r2[x + 1];
      }
      gx[(size_t)y * w + x] = vx;
      gy[(size_t)y * w + x] = vy;
    }
}

void hmpo_stab_harris(const float* img, int w, int h, float k, float* gx, float* gy, float* resp) {
  gradients(img, w, h, gx, gy);
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      float r = 0.0f;
      if (x > 0 && x < w - 1 && y > 0 && y < h - 1) {
        float sxx = 0.0f, sxy = 0.0f, syy = 0.0f;
        for (int j = -1; j <= 1; ++j)
          for (int i = -1; i <= 1; ++i) {
            const float ix = gx[(size_t)(y + j) * w + (x + i)];
            const float iy = gy[(size_t)(y + j) * w + (x + i)];
            sxx += ix * ix;
            sxy += ix * iy;
            syy += iy * iy;
          }
        const float det = sxx * syy - sxy * sxy;
        const float tr = sxx + syy;
        r = det - k * tr * tr;
      }
      resp[(size_t)y * w + x] = r;
    }
}

int hmpo_stab_corners(const float* resp, int w, int h, float threshold, int* xy, int cap) {
  int n = 0;
  for (int y = 1; y < h - 1; ++y)
    for (int x = 1; x < w - 1; ++x) {
      const float r = resp[(size_t)y * w + x];
      if (!(r > threshold)) continue;
      int is_max = 1;
      for (int j = -1; j <= 1 && is_max; ++j)
        for (int i = -1; i <= 1; ++i)
          if (resp[(size_t)(y + j) * w + (x + i)] > r) {
            is_max = 0;
            break;
          }
      if (!is_max) continue;
      if (n < cap) {
        xy[2 * n] = x;
        xy[2 * n + 1] = y;
      }
      ++n;
    }
  return n;
}

void hmpo_stab_flow(const float* prev, const float* next, const int* xy, int n, int w, int h, int window,
                    float* flow) {
  const int half = window / 2;
  for (int f = 0; f < n; ++f) {
    const int px = xy[2 * f], py = xy[2 * f + 1];
    float dx = 0.0f, dy = 0.0f;
    for (int iter = 0; iter < 10; ++iter) {
      float sxx = 0.0f, syy = 0.0f, sxy = 0.0f, stx = 0.0f, sty = 0.0f;
      const int rdx = shift_of(dx), rdy = shift_of(dy);
      for (int j = -half; j <= half; ++j)
        for (int i = -half; i <= half; ++i) {
          const int x = px + i, y = py + j, xn = x + rdx, yn = y + rdy;
          if (x < 1 || x >= w - 1 || y < 1 || y >= h - 1 || xn < 0 || xn >= w - 1 || yn < 0 || yn >= h - 1) continue;
          const float ix = (prev[(size_t)y * w + (x + 1)] - prev[(size_t)y * w + (x - 1)]) * 0.5f;
          const float iy = (prev[(size_t)(y + 1) * w + x] - prev[(size_t)(y - 1) * w + x]) * 0.5f;
          const float it = next[(size_t)yn * w + xn] - prev[(size_t)y * w + x];
          sxx += ix * ix;
          syy += iy * iy;
          sxy += ix * iy;
          stx += ix * it;
          sty += iy * it;
        }
      const float det = sxx * syy - sxy * sxy;
      if (fabsf(det) < 1e-6f) break;
      const float ddx = (-syy * stx + sxy * sty) / det;
      const float ddy = (sxy * stx - sxx * sty) / det;
      dx += ddx;
      dy += ddy;
      if (sqrtf(ddx * ddx + ddy * ddy) < 0.01f) break;
    }
    flow[2 * f] = dx;
    flow[2 * f + 1] = dy;
  }
}

void hmpo_stab_mean(const float* flow, int n, float* dx, float* dy) {
  float sx = 0.0f, sy = 0.0f;
  for (int f = 0; f < n; ++f) {
    sx += flow[2 * f];
    sy += flow[2 * f + 1];
  }
  *dx = n > 0 ? sx / (float)n : 0.0f;
  *dy = n > 0 ? sy / (float)n : 0.0f;
}

void hmpo_stab_warp(const float* in, int w, int h, float dx, float dy, float* out) {
  const int sx = shift_of(dx), sy = shift_of(dy);
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      const int u = x - sx, v = y - sy;
      out[(size_t)y * w + x] = (u >= 0 && u < w && v >= 0 && v < h) ? in[(size_t)v * w + u] : 0.0f;
    }
}
