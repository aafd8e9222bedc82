/*
 * hmp_oracle_body.h -- precision-generic part of the oracle. Included twice by
 * hmp_oracle.c with REAL = float (SFX = f32) and REAL = double (SFX = f64).
 *
 * TEST INFRASTRUCTURE ONLY (see hmp_oracle.h).
 *
 * Images are RGBA, REAL, row-major [batch][h][w][4]. Masks are [h][w][k].
 */

#define CAT2(a, b) a##_##b
#define CAT(a, b) CAT2(a, b)
#define FN(name) CAT(name, SFX)

/* Alpha-aware 2x2 box downsample of a batch of RGBA images (3-channel pixels: the plain mean).
 * src/cuda/cudaBlend.cu:46-144 (2-image), cudaBlendN.cu:53-113 (N), cudaBlend3.cu:100-215 (3):
 * over in-bounds (2x+dx, 2y+dy), dy outer / dx inner; alpha is max-pooled; rgb is the mean
 * over pixels with alpha != 0 (0 if none). */
static void FN(down_rgba)(const REAL* in, int iw, int ih, REAL* out, int ow, int oh, int batch) {
  for (int b = 0; b < batch; ++b) {
    const REAL* src = in + (size_t)b * iw * ih * 4;
    REAL* dst = out + (size_t)b * ow * oh * 4;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < oh; ++y) {
      for (int x = 0; x < ow; ++x) {
        REAL s0 = 0, s1 = 0, s2 = 0, amax = 0;
        int cnt = 0;
        if (g_ch == 3) { /* no alpha: the mean of the in-bounds pixels */
          for (int dy = 0; dy < 2; ++dy)
            for (int dx = 0; dx < 2; ++dx) {
              const int ix = 2 * x + dx, iy = 2 * y + dy;
              if (ix >= iw || iy >= ih)
                continue;
              const REAL* p = src + ((size_t)iy * iw + ix) * 4;
              s0 += p[0];
              s1 += p[1];
              s2 += p[2];
              ++cnt;
            }
          REAL* o = dst + ((size_t)y * ow + x) * 4;
          o[0] = s0 / (REAL)cnt;
          o[1] = s1 / (REAL)cnt;
          o[2] = s2 / (REAL)cnt;
          o[3] = 0;
          continue;
        }
        for (int dy = 0; dy < 2; ++dy) {
          for (int dx = 0; dx < 2; ++dx) {
            const int ix = 2 * x + dx, iy = 2 * y + dy;
            if (ix >= iw || iy >= ih)
              continue;
            const REAL* p = src + ((size_t)iy * iw + ix) * 4;
            if (p[3] > amax)
              amax = p[3];
            if (p[3] != 0) {
              s0 += p[0];
              s1 += p[1];
              s2 += p[2];
              ++cnt;
            }
          }
        }
        REAL* o = dst + ((size_t)y * ow + x) * 4;
        if (cnt > 0) {
          o[0] = s0 / (REAL)cnt;
          o[1] = s1 / (REAL)cnt;
          o[2] = s2 / (REAL)cnt;
        } else {
          o[0] = o[1] = o[2] = 0;
        }
        o[3] = amax;
      }
    }
  }
}

/* k-channel mask mean over the in-bounds 2x2 block.
 * src/cuda/cudaBlend.cu:268-296, cudaBlendN.cu:19-48, cudaBlend3.cu:220-262. */
static void FN(down_mask)(const REAL* in, int iw, int ih, int k, REAL* out, int ow, int oh) {
#pragma omp parallel for schedule(static)
  for (int y = 0; y < oh; ++y) {
    REAL sums[8];
    for (int x = 0; x < ow; ++x) {
      for (int c = 0; c < k; ++c)
        sums[c] = 0;
      int cnt = 0;
      for (int dy = 0; dy < 2; ++dy)
        for (int dx = 0; dx < 2; ++dx) {
          const int ix = 2 * x + dx, iy = 2 * y + dy;
          if (ix >= iw || iy >= ih)
            continue;
          const REAL* p = in + ((size_t)iy * iw + ix) * k;
          for (int c = 0; c < k; ++c)
            sums[c] += p[c];
          ++cnt;
        }
      for (int c = 0; c < k; ++c)
        out[((size_t)y * ow + x) * k + c] = sums[c] / (REAL)cnt;
    }
  }
}

/* Alpha-aware bilinear upsample sample at high-res (x, y) from low (lw x lh), top-left aligned:
 * gx = x/2, gxi = floor, gxi1 = min(gxi+1, lw-1), taps in order 00,10,01,11, only taps whose
 * alpha != 0 contribute, normalised by their weight sum (0 if none).
 * src/cuda/cudaBlend.cu:389-455 (Laplacian), 581-672 (reconstruct). */
static inline void FN(up_alpha)(const REAL* low, int lw, int lh, int x, int y, REAL out3[3]) {
  const REAL gx = (REAL)x / (REAL)2, gy = (REAL)y / (REAL)2;
  int gxi = x >> 1, gyi = y >> 1;
  if (gxi > lw - 1)
    gxi = lw - 1;
  if (gyi > lh - 1)
    gyi = lh - 1;
  const int gxi1 = gxi + 1 < lw - 1 ? gxi + 1 : lw - 1;
  const int gyi1 = gyi + 1 < lh - 1 ? gyi + 1 : lh - 1;
  const REAL dx = gx - (REAL)gxi, dy = gy - (REAL)gyi;
  const REAL one = 1;
  const REAL w[4] = {(one - dx) * (one - dy), dx * (one - dy), (one - dx) * dy, dx * dy};
  const REAL* p[4] = {low + ((size_t)gyi * lw + gxi) * 4, low + ((size_t)gyi * lw + gxi1) * 4,
                      low + ((size_t)gyi1 * lw + gxi) * 4, low + ((size_t)gyi1 * lw + gxi1) * 4};
  if (g_ch == 3) { /* no alpha: separable bilinear, x then y (cudaBlend.cu:445-448); the
                     * reconstruction uses up_taps3 instead */
    for (int c = 0; c < 3; ++c) {
      const REAL v0 = p[0][c] * (one - dx) + p[1][c] * dx;
      const REAL v1 = p[2][c] * (one - dx) + p[3][c] * dx;
      out3[c] = v0 * (one - dy) + v1 * dy;
    }
    return;
  }
  for (int c = 0; c < 3; ++c) {
    REAL sw = 0, sv = 0;
    for (int t = 0; t < 4; ++t) {
      if (p[t][3] != 0) {
        sw += w[t];
        sv += p[t][c] * w[t];
      }
    }
    out3[c] = sw > 0 ? sv / sw : (REAL)0;
  }
}

/* The reconstruction's upsample of 3-channel pixels: the sequential four-tap sum
 * (((0 + v00 w00) + v10 w10) + v01 w01) + v11 w11 of the reference's reconstructions
 * (cudaBlend.cu:581-672 and cudaBlendN.cu:372-447, whose weight sum is exactly 1 here;
 * cupano/ops.py:514-565). It rounds differently from the separable form of the Laplacian at
 * pixels with odd x and odd y once a level holds blended (non-dyadic) values. */
static inline void FN(up_taps3)(const REAL* low, int lw, int lh, int x, int y, REAL out3[3]) {
  int gxi = x >> 1, gyi = y >> 1;
  if (gxi > lw - 1)
    gxi = lw - 1;
  if (gyi > lh - 1)
    gyi = lh - 1;
  const int gxi1 = gxi + 1 < lw - 1 ? gxi + 1 : lw - 1;
  const int gyi1 = gyi + 1 < lh - 1 ? gyi + 1 : lh - 1;
  const REAL dx = (REAL)x / (REAL)2 - (REAL)gxi, dy = (REAL)y / (REAL)2 - (REAL)gyi, one = 1;
  const REAL w[4] = {(one - dx) * (one - dy), dx * (one - dy), (one - dx) * dy, dx * dy};
  const REAL* p[4] = {low + ((size_t)gyi * lw + gxi) * 4, low + ((size_t)gyi * lw + gxi1) * 4,
                      low + ((size_t)gyi1 * lw + gxi) * 4, low + ((size_t)gyi1 * lw + gxi1) * 4};
  for (int c = 0; c < 3; ++c) {
    REAL sv = 0;
    for (int t = 0; t < 4; ++t)
      sv += p[t][c] * w[t];
    out3[c] = sv;
  }
}

/* lap = high - up_alpha(low) for rgb, lap.a = high.a (cudaBlend.cu:356-456). */
static void FN(laplacian)(const REAL* high, int hw, int hh, const REAL* low, int lw, int lh, REAL* lap, int batch) {
  for (int b = 0; b < batch; ++b) {
    const REAL* H = high + (size_t)b * hw * hh * 4;
    const REAL* L = low + (size_t)b * lw * lh * 4;
    REAL* O = lap + (size_t)b * hw * hh * 4;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < hh; ++y)
      for (int x = 0; x < hw; ++x) {
        REAL up[3];
        FN(up_alpha)(L, lw, lh, x, y, up);
        const REAL* h = H + ((size_t)y * hw + x) * 4;
        REAL* o = O + ((size_t)y * hw + x) * 4;
        o[0] = h[0] - up[0];
        o[1] = h[1] - up[1];
        o[2] = h[2] - up[2];
        o[3] = h[3];
      }
  }
}

/* R_l = up(R_{l+1}) + blend_l (rgb), alpha = blend_l alpha, up = up_alpha for 4 channels and
 * up_taps3 for 3 (cudaBlend.cu:581-672, cudaBlendN.cu:372-447). */
static void FN(reconstruct)(const REAL* low, int lw, int lh, const REAL* lap, int hw, int hh, REAL* out, int batch) {
  for (int b = 0; b < batch; ++b) {
    const REAL* L = low + (size_t)b * lw * lh * 4;
    const REAL* P = lap + (size_t)b * hw * hh * 4;
    REAL* O = out + (size_t)b * hw * hh * 4;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < hh; ++y)
      for (int x = 0; x < hw; ++x) {
        REAL up[3];
        if (g_ch == 3)
          FN(up_taps3)(L, lw, lh, x, y, up);
        else
          FN(up_alpha)(L, lw, lh, x, y, up);
        const REAL* p = P + ((size_t)y * hw + x) * 4;
        REAL* o = O + ((size_t)y * hw + x) * 4;
        o[0] = up[0] + p[0];
        o[1] = up[1] + p[1];
        o[2] = up[2] + p[2];
        o[3] = p[3];
      }
  }
}

/* Two-image blend (cudaBlend.cu:520-576): alpha-0 bypass to the other image, else
 * rgb = m*l1 + (1-m)*l2 and alpha = alpha2. The mask is not batched. */
static void FN(blend_two)(const REAL* l1, const REAL* l2, const REAL* mask, int w, int h, REAL* out, int batch) {
  for (int b = 0; b < batch; ++b) {
    const size_t off = (size_t)b * w * h * 4;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; ++y)
      for (int x = 0; x < w; ++x) {
        const size_t i = ((size_t)y * w + x);
        const REAL* a = l1 + off + i * 4;
        const REAL* c = l2 + off + i * 4;
        REAL* o = out + off + i * 4;
        const REAL m = mask[i];
        const REAL mm1 = (REAL)1 - m;
        if (g_ch == 3) { /* no alpha bypass */
          for (int ch = 0; ch < 3; ++ch) {
            const REAL t1 = m * a[ch];
            const REAL t2 = mm1 * c[ch];
            o[ch] = t1 + t2;
          }
          o[3] = 0;
          continue;
        }
        if (a[3] == 0) {
          o[0] = c[0];
          o[1] = c[1];
          o[2] = c[2];
          o[3] = c[3];
        } else if (c[3] == 0) {
          o[0] = a[0];
          o[1] = a[1];
          o[2] = a[2];
          o[3] = a[3];
        } else {
          for (int ch = 0; ch < 3; ++ch) {
            const REAL t1 = m * a[ch];
            const REAL t2 = mm1 * c[ch];
            o[ch] = t1 + t2;
          }
          o[3] = c[3];
        }
      }
  }
}

/* Three-image blend (cudaBlend3.cu:376-531): mask weights zeroed where alpha == 0 and
 * renormalised by their sum; if none survive, copy the pixel of the strictly highest-alpha
 * contributor (or zeros). rgb = (m1*v1 + m2*v2) + m3*v3, alpha = max over m_i > 0. */
static void FN(blend_three)(const REAL* const* laps, const REAL* mask, int w, int h, REAL* out, int batch) {
  for (int b = 0; b < batch; ++b) {
    const size_t off = (size_t)b * w * h * 4;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; ++y)
      for (int x = 0; x < w; ++x) {
        const size_t i = ((size_t)y * w + x);
        const REAL* L[3] = {laps[0] + off + i * 4, laps[1] + off + i * 4, laps[2] + off + i * 4};
        REAL* o = out + off + i * 4;
        REAL m[3] = {mask[i * 3 + 0], mask[i * 3 + 1], mask[i * 3 + 2]};
        if (g_ch == 3) { /* no alpha: the raw weights, not normalised (cudaBlend3.cu:468-480) */
          for (int c = 0; c < 3; ++c) {
            const REAL t0 = m[0] * L[0][c];
            const REAL t1 = m[1] * L[1][c];
            const REAL t2 = m[2] * L[2][c];
            o[c] = (t0 + t1) + t2;
          }
          o[3] = 0;
          continue;
        }
        for (int k = 0; k < 3; ++k)
          if (L[k][3] == 0)
            m[k] = 0;
        const REAL sum = m[0] + m[1] + m[2];
        if (sum > 0) {
          m[0] /= sum;
          m[1] /= sum;
          m[2] /= sum;
        } else {
          int src = -1;
          REAL amax = 0;
          for (int k = 0; k < 3; ++k)
            if (L[k][3] > amax) {
              amax = L[k][3];
              src = k;
            }
          for (int c = 0; c < 4; ++c)
            o[c] = src < 0 ? (REAL)0 : L[src][c];
          continue;
        }
        for (int c = 0; c < 3; ++c) {
          const REAL t0 = m[0] * L[0][c];
          const REAL t1 = m[1] * L[1][c];
          const REAL t2 = m[2] * L[2][c];
          o[c] = (t0 + t1) + t2;
        }
        REAL aout = 0;
        for (int k = 0; k < 3; ++k)
          if (m[k] > 0 && L[k][3] > aout)
            aout = L[k][3];
        o[3] = aout;
      }
  }
}

/* N-way blend (cudaBlendN.cu:199-288): w_i = mask_i / sum(mask) (if > 0), zeroed where
 * alpha == 0, renormalised; fallback to the first strictly-highest-alpha contributor;
 * rgb = sum_i w_i * lap_i (in order), alpha = max over w_i != 0. */
static void FN(blend_nway)(const REAL* const* laps, int n, const REAL* mask, int w, int h, REAL* out, int batch) {
  for (int b = 0; b < batch; ++b) {
    const size_t off = (size_t)b * w * h * 4;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; ++y)
      for (int x = 0; x < w; ++x) {
        const size_t i = ((size_t)y * w + x);
        REAL wt[8];
        REAL sumw = 0;
        for (int k = 0; k < n; ++k) {
          wt[k] = mask[i * n + k];
          sumw += wt[k];
        }
        if (sumw > 0)
          for (int k = 0; k < n; ++k)
            wt[k] /= sumw;
        if (g_ch == 3) { /* no alpha: the normalised weights as they are */
          REAL* o3 = out + off + i * 4;
          for (int c = 0; c < 3; ++c) {
            REAL acc = 0;
            for (int k = 0; k < n; ++k) {
              const REAL t = wt[k] * laps[k][off + i * 4 + c];
              acc += t;
            }
            o3[c] = acc;
          }
          o3[3] = 0;
          continue;
        }
        REAL sumw2 = 0, amax = 0;
        int aidx = -1;
        for (int k = 0; k < n; ++k) {
          const REAL a = laps[k][off + i * 4 + 3];
          if (a > amax) {
            amax = a;
            aidx = k;
          }
          if (a == 0)
            wt[k] = 0;
          sumw2 += wt[k];
        }
        REAL* o = out + off + i * 4;
        if (sumw2 > 0) {
          for (int k = 0; k < n; ++k)
            wt[k] /= sumw2;
        } else {
          for (int c = 0; c < 4; ++c)
            o[c] = (aidx >= 0 && amax != 0) ? laps[aidx][off + i * 4 + c] : (REAL)0;
          continue;
        }
        for (int c = 0; c < 3; ++c) {
          REAL acc = 0;
          for (int k = 0; k < n; ++k) {
            const REAL t = wt[k] * laps[k][off + i * 4 + c];
            acc += t;
          }
          o[c] = acc;
        }
        REAL aout = 0;
        for (int k = 0; k < n; ++k)
          if (wt[k] != 0 && laps[k][off + i * 4 + 3] > aout)
            aout = laps[k][off + i * 4 + 3];
        o[3] = aout;
      }
  }
}

static void FN(blend_rule)(int rule, const REAL* const* laps, int n, const REAL* mask, int w, int h, REAL* out,
                           int batch) {
  if (rule == RULE_TWO)
    FN(blend_two)(laps[0], laps[1], mask, w, h, out, batch);
  else if (rule == RULE_THREE)
    FN(blend_three)(laps, mask, w, h, out, batch);
  else
    FN(blend_nway)(laps, n, mask, w, h, out, batch);
}

/* ---------------------------------------------------------------------------------------------
 * Binomial5 variant (no reference implementation; parity unpinned). 5-tap [1,4,6,4,1]/16
 * separable, reflect-101 borders, decimate by 2. Alpha validity follows the reference rule:
 * taps whose alpha == 0 are dropped and the remaining weights renormalised; alpha itself is
 * max-pooled over the in-bounds 2x2 block exactly as in the box pyramid.
 * ------------------------------------------------------------------------------------------- */
static void FN(down_rgba_b5)(const REAL* in, int iw, int ih, REAL* out, int ow, int oh, int batch) {
  static const int k5[5] = {1, 4, 6, 4, 1};
  for (int b = 0; b < batch; ++b) {
    const REAL* src = in + (size_t)b * iw * ih * 4;
    REAL* dst = out + (size_t)b * ow * oh * 4;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < oh; ++y)
      for (int x = 0; x < ow; ++x) {
        REAL sw = 0, s[3] = {0, 0, 0};
        for (int j = -2; j <= 2; ++j) {
          const int iy = reflect101(2 * y + j, ih);
          for (int i = -2; i <= 2; ++i) {
            const int ix = reflect101(2 * x + i, iw);
            const REAL* p = src + ((size_t)iy * iw + ix) * 4;
            if (p[3] == 0)
              continue;
            const REAL wgt = (REAL)(k5[i + 2] * k5[j + 2]) / (REAL)256;
            sw += wgt;
            for (int c = 0; c < 3; ++c)
              s[c] += wgt * p[c];
          }
        }
        REAL amax = 0;
        for (int dy = 0; dy < 2; ++dy)
          for (int dx = 0; dx < 2; ++dx) {
            const int ix = 2 * x + dx, iy = 2 * y + dy;
            if (ix < iw && iy < ih && src[((size_t)iy * iw + ix) * 4 + 3] > amax)
              amax = src[((size_t)iy * iw + ix) * 4 + 3];
          }
        REAL* o = dst + ((size_t)y * ow + x) * 4;
        for (int c = 0; c < 3; ++c)
          o[c] = sw > 0 ? s[c] / sw : (REAL)0;
        o[3] = amax;
      }
  }
}

/* Expand (Burt-Adelson): even high-res x uses low taps x/2-1, x/2, x/2+1 with weights 1,6,1;
 * odd x uses (x-1)/2, (x+1)/2 with weights 4,4 (per axis, reflect-101 at the low level).
 * Alpha-aware: taps with alpha == 0 dropped, weights renormalised. */
static inline void FN(up_b5)(const REAL* low, int lw, int lh, int x, int y, REAL out3[3]) {
  int tx[3], ty[3], nx, ny;
  REAL wx[3], wy[3];
  if ((x & 1) == 0) {
    nx = 3;
    tx[0] = reflect101(x / 2 - 1, lw);
    tx[1] = reflect101(x / 2, lw);
    tx[2] = reflect101(x / 2 + 1, lw);
    wx[0] = 1;
    wx[1] = 6;
    wx[2] = 1;
  } else {
    nx = 2;
    tx[0] = reflect101((x - 1) / 2, lw);
    tx[1] = reflect101((x + 1) / 2, lw);
    wx[0] = 4;
    wx[1] = 4;
  }
  if ((y & 1) == 0) {
    ny = 3;
    ty[0] = reflect101(y / 2 - 1, lh);
    ty[1] = reflect101(y / 2, lh);
    ty[2] = reflect101(y / 2 + 1, lh);
    wy[0] = 1;
    wy[1] = 6;
    wy[2] = 1;
  } else {
    ny = 2;
    ty[0] = reflect101((y - 1) / 2, lh);
    ty[1] = reflect101((y + 1) / 2, lh);
    wy[0] = 4;
    wy[1] = 4;
  }
  REAL sw = 0, s[3] = {0, 0, 0};
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      const REAL* p = low + ((size_t)ty[j] * lw + tx[i]) * 4;
      if (p[3] == 0)
        continue;
      const REAL wgt = wx[i] * wy[j] / (REAL)64;
      sw += wgt;
      for (int c = 0; c < 3; ++c)
        s[c] += wgt * p[c];
    }
  for (int c = 0; c < 3; ++c)
    out3[c] = sw > 0 ? s[c] / sw : (REAL)0;
}

static void FN(laplacian_b5)(const REAL* high, int hw, int hh, const REAL* low, int lw, int lh, REAL* lap,
                              int batch) {
  for (int b = 0; b < batch; ++b) {
    const REAL* H = high + (size_t)b * hw * hh * 4;
    const REAL* L = low + (size_t)b * lw * lh * 4;
    REAL* O = lap + (size_t)b * hw * hh * 4;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < hh; ++y)
      for (int x = 0; x < hw; ++x) {
        REAL up[3];
        FN(up_b5)(L, lw, lh, x, y, up);
        const REAL* h = H + ((size_t)y * hw + x) * 4;
        REAL* o = O + ((size_t)y * hw + x) * 4;
        for (int c = 0; c < 3; ++c)
          o[c] = h[c] - up[c];
        o[3] = h[3];
      }
  }
}

static void FN(reconstruct_b5)(const REAL* low, int lw, int lh, const REAL* lap, int hw, int hh, REAL* out,
                                int batch) {
  for (int b = 0; b < batch; ++b) {
    const REAL* L = low + (size_t)b * lw * lh * 4;
    const REAL* P = lap + (size_t)b * hw * hh * 4;
    REAL* O = out + (size_t)b * hw * hh * 4;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < hh; ++y)
      for (int x = 0; x < hw; ++x) {
        REAL up[3];
        FN(up_b5)(L, lw, lh, x, y, up);
        const REAL* p = P + ((size_t)y * hw + x) * 4;
        REAL* o = O + ((size_t)y * hw + x) * 4;
        for (int c = 0; c < 3; ++c)
          o[c] = up[c] + p[c];
        o[3] = p[3];
      }
  }
}

/* Full Laplacian blend of n level-0 buffers (w x h, batch) with a k-channel mask.
 * Mirrors cudaBatchedLaplacianBlendWithContext{,3,N}: Gaussian pyramids, mask pyramid,
 * Laplacians (last level = Gaussian), per-level blend, reconstruction. */
static int FN(laplacian_blend)(const REAL* const* inputs, int n, const REAL* mask, int k, int w, int h, int levels,
                               int rule, int filter, int batch, REAL* out) {
  int lw[32], lh[32];
  lw[0] = w;
  lh[0] = h;
  for (int l = 1; l < levels; ++l) {
    lw[l] = (lw[l - 1] + 1) / 2;
    lh[l] = (lh[l - 1] + 1) / 2;
  }
  REAL* gauss[8][32];
  REAL* laps[8][32];
  REAL* mpyr[32];
  REAL* blend[32];
  memset(gauss, 0, sizeof(gauss));
  memset(laps, 0, sizeof(laps));
  memset(mpyr, 0, sizeof(mpyr));
  memset(blend, 0, sizeof(blend));
  int rc = HMPO_OK;
  for (int l = 0; l < levels && rc == HMPO_OK; ++l) {
    const size_t px = (size_t)lw[l] * lh[l];
    for (int i = 0; i < n; ++i) {
      if (l > 0)
        gauss[i][l] = (REAL*)malloc(px * 4 * batch * sizeof(REAL));
      laps[i][l] = (REAL*)malloc(px * 4 * batch * sizeof(REAL));
      if ((l > 0 && !gauss[i][l]) || !laps[i][l])
        rc = HMPO_ENOMEM;
    }
    if (l > 0)
      mpyr[l] = (REAL*)malloc(px * k * sizeof(REAL));
    blend[l] = (REAL*)malloc(px * 4 * batch * sizeof(REAL));
    if ((l > 0 && !mpyr[l]) || !blend[l])
      rc = HMPO_ENOMEM;
  }
  if (rc == HMPO_OK) {
    for (int i = 0; i < n; ++i)
      gauss[i][0] = (REAL*)inputs[i];
    mpyr[0] = (REAL*)mask;
    for (int l = 0; l + 1 < levels; ++l) {
      for (int i = 0; i < n; ++i) {
        if (filter == HMPO_FILTER_BINOMIAL5)
          FN(down_rgba_b5)(gauss[i][l], lw[l], lh[l], gauss[i][l + 1], lw[l + 1], lh[l + 1], batch);
        else
          FN(down_rgba)(gauss[i][l], lw[l], lh[l], gauss[i][l + 1], lw[l + 1], lh[l + 1], batch);
      }
      FN(down_mask)(mpyr[l], lw[l], lh[l], k, mpyr[l + 1], lw[l + 1], lh[l + 1]);
    }
    for (int l = 0; l + 1 < levels; ++l)
      for (int i = 0; i < n; ++i) {
        if (filter == HMPO_FILTER_BINOMIAL5)
          FN(laplacian_b5)(gauss[i][l], lw[l], lh[l], gauss[i][l + 1], lw[l + 1], lh[l + 1], laps[i][l], batch);
        else
          FN(laplacian)(gauss[i][l], lw[l], lh[l], gauss[i][l + 1], lw[l + 1], lh[l + 1], laps[i][l], batch);
      }
    const int last = levels - 1;
    for (int i = 0; i < n; ++i)
      memcpy(laps[i][last], gauss[i][last], (size_t)lw[last] * lh[last] * 4 * batch * sizeof(REAL));
    for (int l = 0; l < levels; ++l) {
      const REAL* lv[8];
      for (int i = 0; i < n; ++i)
        lv[i] = laps[i][l];
      FN(blend_rule)(rule, lv, n, mpyr[l], lw[l], lh[l], blend[l], batch);
    }
    /* Reconstruct: R_last = blend_last; R_l = up(R_{l+1}) + blend_l. */
    REAL* rec = blend[last];
    REAL* tmp = NULL;
    for (int l = last - 1; l >= 0; --l) {
      REAL* dst = l == 0 ? out : (REAL*)malloc((size_t)lw[l] * lh[l] * 4 * batch * sizeof(REAL));
      if (!dst) {
        rc = HMPO_ENOMEM;
        break;
      }
      if (filter == HMPO_FILTER_BINOMIAL5)
        FN(reconstruct_b5)(rec, lw[l + 1], lh[l + 1], blend[l], lw[l], lh[l], dst, batch);
      else
        FN(reconstruct)(rec, lw[l + 1], lh[l + 1], blend[l], lw[l], lh[l], dst, batch);
      if (tmp)
        free(tmp);
      tmp = l == 0 ? NULL : dst;
      rec = dst;
    }
    if (tmp)
      free(tmp);
    if (last == 0)
      memcpy(out, blend[0], (size_t)w * h * 4 * batch * sizeof(REAL));
  }
  for (int l = 0; l < levels; ++l) {
    for (int i = 0; i < n; ++i) {
      if (l > 0)
        free(gauss[i][l]);
      free(laps[i][l]);
    }
    if (l > 0)
      free(mpyr[l]);
    free(blend[l]);
  }
  return rc;
}

/* Remap one image into a REAL RGBA buffer at (off_x, off_y), restricted to a ROI of the map
 * (cudaRemap.cu:60-198, no_unmapped_write=false): in-range source -> cast; otherwise zero rgb
 * with alpha = (sx == 65535 ? 0 : 255). With skip_invalid (3-image fused remap,
 * cudaFusedKernels3.cu:25-119) invalid pixels are left untouched instead. */
static void FN(remap_into)(const uint8_t* src, int sw, int sh, const uint16_t* mx, const uint16_t* my, int mw, int mh,
                           int roi_x, int roi_y, int roi_w, int roi_h, int off_x, int off_y, REAL* dst, int dw,
                           int dh, int batch, int skip_invalid) {
  for (int b = 0; b < batch; ++b) {
    const uint8_t* S = src + (size_t)b * sw * sh * g_ch;
    REAL* D = dst + (size_t)b * dw * dh * 4;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < roi_h; ++y)
      for (int x = 0; x < roi_w; ++x) {
        const int mxp = roi_x + x, myp = roi_y + y;
        if (mxp < 0 || mxp >= mw || myp < 0 || myp >= mh)
          continue;
        const int dx = off_x + mxp, dy = off_y + myp;
        if (dx < 0 || dx >= dw || dy < 0 || dy >= dh)
          continue;
        const int sx = mx[(size_t)myp * mw + mxp], sy = my[(size_t)myp * mw + mxp];
        REAL* o = D + ((size_t)dy * dw + dx) * 4;
        if (sx < sw && sy < sh) {
          const uint8_t* p = S + ((size_t)sy * sw + sx) * g_ch;
          o[0] = p[0];
          o[1] = p[1];
          o[2] = p[2];
          o[3] = g_ch == 4 ? p[3] : 0;
        } else if (!skip_invalid) {
          o[0] = o[1] = o[2] = 0;
          o[3] = (sx == 65535 || g_ch == 3) ? (REAL)0 : (REAL)255;
        }
      }
  }
}

/* Truncating pack (cudaUtils.cuh:18-28): v <= 0 -> 0, v >= 255 -> 255, else trunc. */
static inline uint8_t FN(pack)(REAL v) {
  if (v <= 0)
    return 0;
  if (v >= 255)
    return 255;
  return (uint8_t)v;
}

/* Paste a REAL RGBA region into the uint8 canvas with the truncating pack
 * (copyRoiKernelBatched, cudaMakeFull.cu:40-69). */
static void FN(paste)(const REAL* src, int sw, int sh, int region_w, int region_h, int src_x, int src_y,
                      uint8_t* canvas, int cw, int ch, int off_x, int off_y, int batch) {
  for (int b = 0; b < batch; ++b) {
    const REAL* S = src + (size_t)b * sw * sh * 4;
    uint8_t* C = canvas + (size_t)b * cw * ch * g_ch;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < region_h; ++y)
      for (int x = 0; x < region_w; ++x) {
        const int sx = src_x + x, sy = src_y + y;
        if (sx < 0 || sy < 0 || sx >= sw || sy >= sh)
          continue;
        const int dx = off_x + x, dy = off_y + y;
        if (dx < 0 || dy < 0 || dx >= cw || dy >= ch)
          continue;
        for (int c = 0; c < g_ch; ++c)
          C[((size_t)dy * cw + dx) * g_ch + c] = FN(pack)(S[((size_t)sy * sw + sx) * 4 + c]);
      }
  }
}

/* The soft-seam stitch (num_levels > 0) for every stitcher kind. When roi_out is non-NULL the
 * blend result of the write ROI is returned unpacked instead of being pasted. */
static int FN(stitch_soft)(const hmpo_config* cfg, const uint8_t* const* inputs, const int* in_w, const int* in_h,
                           uint8_t* canvas, REAL* roi_out) {
  geom_t g;
  int rc = compute_geometry(cfg, &g);
  if (rc != HMPO_OK)
    return rc;
  const int n = cfg->n_images, B = cfg->batch, W = g.canvas_w, H = g.canvas_h;
  const int Wb = g.blend.w, Hb = g.blend.h;
  const size_t fpx = (size_t)Wb * Hb;
  REAL* full[8] = {0};
  REAL* mask = NULL;
  REAL* out = NULL;
  uint8_t* tmp_canvas = NULL;
  for (int i = 0; i < n; ++i) {
    full[i] = (REAL*)calloc(fpx * 4 * B, sizeof(REAL));
    if (!full[i])
      rc = HMPO_ENOMEM;
  }
  mask = (REAL*)calloc(fpx * g.mask_k, sizeof(REAL));
  out = (REAL*)calloc(fpx * 4 * B, sizeof(REAL));
  if (!mask || !out)
    rc = HMPO_ENOMEM;
  if (rc == HMPO_OK) {
    /* Level-0 mask over the blend region. */
    for (int y = 0; y < Hb; ++y)
      for (int x = 0; x < Wb; ++x) {
        const uint8_t v = g.seam[(size_t)(g.blend.y + y) * W + (g.blend.x + x)];
        if (g.mask_k == 1)
          mask[(size_t)y * Wb + x] = (REAL)v;
        else
          for (int c = 0; c < g.mask_k; ++c)
            mask[((size_t)y * Wb + x) * g.mask_k + c] = v == c ? (REAL)1 : (REAL)0;
      }
    if (cfg->kind == HMPO_KIND_PANO2 && g.minimized) {
      /* cudaPano.inl:203-318: remap 1 onto the canvas, copy its blend strip into full1, remap 2
       * onto the canvas, copy its strip into full2. */
      const int x1 = cfg->pos_x[0], y1 = cfg->pos_y[0], x2 = cfg->pos_x[1], y2 = cfg->pos_y[1];
      const int pad = OVERLAP_PAD, ow = cfg->map_w[0] - x2;
      const int rw = ow + pad;
      REAL* cv = (REAL*)calloc((size_t)W * H * 4 * B, sizeof(REAL));
      if (!cv) {
        rc = HMPO_ENOMEM;
      } else {
        FN(remap_into)(inputs[0], in_w[0], in_h[0], cfg->map_x[0], cfg->map_y[0], cfg->map_w[0], cfg->map_h[0], 0, 0,
                       cfg->map_w[0], cfg->map_h[0], x1, y1, cv, W, H, B, 0);
        for (int b = 0; b < B; ++b)
          for (int y = 0; y < Hb; ++y)
            for (int x = 0; x < rw; ++x) {
              const int sx = (x2 - pad - x1) + x, sy = y;
              const int dx = x1 + x, dy = y;
              if (sx < 0 || sx >= W || sy >= H || dx < 0 || dx >= Wb || dy >= Hb)
                continue;
              memcpy(full[0] + ((size_t)b * fpx + (size_t)dy * Wb + dx) * 4,
                     cv + ((size_t)b * W * H + (size_t)sy * W + sx) * 4, 4 * sizeof(REAL));
            }
        FN(remap_into)(inputs[1], in_w[1], in_h[1], cfg->map_x[1], cfg->map_y[1], cfg->map_w[1], cfg->map_h[1], 0, 0,
                       cfg->map_w[1], cfg->map_h[1], x2, y2, cv, W, H, B, 0);
        for (int b = 0; b < B; ++b)
          for (int y = 0; y < Hb; ++y)
            for (int x = 0; x < rw; ++x) {
              const int sx = x2 + x, sy = y;
              const int dx = x1 + pad + x, dy = y;
              if (sx < 0 || sx >= W || sy >= H || dx < 0 || dx >= Wb || dy >= Hb)
                continue;
              memcpy(full[1] + ((size_t)b * fpx + (size_t)dy * Wb + dx) * 4,
                     cv + ((size_t)b * W * H + (size_t)sy * W + sx) * 4, 4 * sizeof(REAL));
            }
        /* Canvas outside the blend strip: image 2 over image 1 (uint8 copies). */
        if (canvas)
          for (size_t p = 0; p < (size_t)W * H * B; ++p)
            for (int c = 0; c < g_ch; ++c)
              canvas[p * g_ch + c] = FN(pack)(cv[p * 4 + c]);
        free(cv);
      }
    } else if (cfg->kind == HMPO_KIND_PANON && g.minimized) {
      /* cudaPanoN.inl:530-621: fused hard seam onto the canvas, then ROI remaps. */
      if (canvas)
        hard_seam(cfg, &g, inputs, in_w, in_h, canvas);
      for (int i = 0; i < n; ++i) {
        if (g.remap_roi[i].w <= 0 || g.remap_roi[i].h <= 0)
          continue;
        FN(remap_into)(inputs[i], in_w[i], in_h[i], cfg->map_x[i], cfg->map_y[i], cfg->map_w[i], cfg->map_h[i],
                       g.remap_roi[i].x, g.remap_roi[i].y, g.remap_roi[i].w, g.remap_roi[i].h,
                       cfg->pos_x[i] - g.blend.x, cfg->pos_y[i] - g.blend.y, full[i], Wb, Hb, B, 0);
      }
    } else {
      /* Full-canvas blend (PANO2/PANON without minimisation, PANO3). */
      if (canvas)
        memset(canvas, 0, (size_t)W * H * g_ch * B);
      const int skip = cfg->kind == HMPO_KIND_PANO3 && cfg->fused3;
      for (int i = 0; i < n; ++i)
        FN(remap_into)(inputs[i], in_w[i], in_h[i], cfg->map_x[i], cfg->map_y[i], cfg->map_w[i], cfg->map_h[i], 0, 0,
                       cfg->map_w[i], cfg->map_h[i], cfg->pos_x[i], cfg->pos_y[i], full[i], Wb, Hb, B, skip);
    }
  }
  if (rc == HMPO_OK) {
    const REAL* ins[8] = {0};
    for (int i = 0; i < n; ++i)
      ins[i] = full[i];
    rc = FN(laplacian_blend)(ins, n, mask, g.mask_k, Wb, Hb, g.levels, g.rule, cfg->filter, B, out);
  }
  if (rc == HMPO_OK) {
    const int srcx = g.write.x - g.blend.x, srcy = g.write.y - g.blend.y;
    if (roi_out) {
      for (int b = 0; b < B; ++b)
        for (int y = 0; y < g.write.h; ++y)
          for (int x = 0; x < g.write.w; ++x)
            for (int c = 0; c < 4; ++c)
              roi_out[(((size_t)b * g.write.h + y) * g.write.w + x) * 4 + c] =
                  out[(((size_t)b * Hb + srcy + y) * Wb + srcx + x) * 4 + c];
    }
    if (canvas)
      FN(paste)(out, Wb, Hb, g.write.w, g.write.h, srcx, srcy, canvas, W, H, g.write.x, g.write.y, B);
  }
  for (int i = 0; i < n; ++i)
    free(full[i]);
  free(mask);
  free(out);
  free(tmp_canvas);
  free_geometry(&g);
  return rc;
}

#undef FN
#undef CAT
#undef CAT2
