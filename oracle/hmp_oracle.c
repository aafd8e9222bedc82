/*
 * hmp_oracle.c -- CPU restatement of hm-cupano's stitching path (TEST INFRASTRUCTURE ONLY).
 * See hmp_oracle.h for what is restated and where it comes from. Build with
 * -ffp-contract=off so that no multiply-add is fused (the reference's Python port and the
 * CUDA kernels under test round every product and sum separately).
 */
#include "hmp_oracle.h"

#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OVERLAP_PAD 128 /* CanvasManager overlap_pad default, src/pano/canvasManager.h:65 */
#define RULE_NWAY 1
#define RULE_TWO 2
#define RULE_THREE 3

typedef struct {
  int x, y, w, h;
} rect_t;

typedef struct {
  int canvas_w, canvas_h;
  uint8_t* seam; /* seam padded (replicate right/bottom) to the canvas, owned */
  int minimized;
  rect_t blend;  /* blend buffer region, canvas coordinates */
  rect_t write;  /* region pasted back onto the canvas */
  rect_t remap_roi[8];
  int levels; /* effective level count */
  int rule;
  int mask_k;
} geom_t;

static int g_threads = 0;
/* Pixel channels of the stitch in progress: 4 (RGBA) or 3 (RGB, no alpha: plain means, plain
 * bilinear upsampling, blends without alpha tests, zero fill for out-of-range entries). The
 * op-level entry points below run with 4, except hmpo_laplacian_blend_ch_f32. */
static int g_ch = 4;

void hmpo_set_threads(int n) {
  g_threads = n;
#ifdef _OPENMP
  if (n > 0)
    omp_set_num_threads(n);
#endif
}

int hmpo_get_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

static inline int imin(int a, int b) { return a < b ? a : b; }
static inline int imax(int a, int b) { return a > b ? a : b; }

static inline int reflect101(int m, int n) {
  if (n == 1)
    return 0;
  while (m < 0 || m >= n) {
    if (m < 0)
      m = -m;
    if (m >= n)
      m = 2 * n - 2 - m;
  }
  return m;
}

static int validate(const hmpo_config* cfg) {
  if (!cfg || cfg->n_images < 2 || cfg->n_images > 8 || cfg->batch < 1 || cfg->num_levels < 0 ||
      cfg->num_levels > 24)
    return HMPO_EINVAL;
  if (cfg->kind == HMPO_KIND_PANO2 && cfg->n_images != 2)
    return HMPO_EINVAL;
  if (cfg->kind == HMPO_KIND_PANO3 && cfg->n_images != 3)
    return HMPO_EINVAL;
  if (cfg->kind != HMPO_KIND_PANO2 && cfg->kind != HMPO_KIND_PANO3 && cfg->kind != HMPO_KIND_PANON)
    return HMPO_EINVAL;
  for (int i = 0; i < cfg->n_images; ++i)
    if (!cfg->map_x[i] || !cfg->map_y[i] || cfg->map_w[i] <= 0 || cfg->map_h[i] <= 0 || cfg->pos_x[i] < 0 ||
        cfg->pos_y[i] < 0)
      return HMPO_EINVAL;
  if (!cfg->seam || cfg->seam_w <= 0 || cfg->seam_h <= 0)
    return HMPO_EINVAL;
  return HMPO_OK;
}

int hmpo_canvas_size(const hmpo_config* cfg, int* width, int* height) {
  int rc = validate(cfg);
  if (rc != HMPO_OK)
    return rc;
  int w = 0, h = 0;
  for (int i = 0; i < cfg->n_images; ++i) {
    w = imax(w, cfg->pos_x[i] + cfg->map_w[i]);
    h = imax(h, cfg->pos_y[i] + cfg->map_h[i]);
  }
  *width = w;
  *height = h;
  return HMPO_OK;
}

/* compute_num_levels (cupano/ops.py:871-881; cudaBlendN.cu:680-688): stop adding levels once a
 * side of the previous level is below 2. */
static int effective_levels(int w, int h, int requested) {
  int levels = requested < 1 ? 1 : requested;
  int cw = w, ch = h, n = 1;
  for (int l = 1; l < levels; ++l) {
    if (cw < 2 || ch < 2)
      break;
    cw = (cw + 1) / 2;
    ch = (ch + 1) / 2;
    ++n;
  }
  return n;
}

/* seam_boundary_bbox (src/pano/cudaPanoN.inl:38-75). */
static rect_t seam_boundary_bbox(const uint8_t* s, int w, int h, int* found) {
  rect_t r = {0, 0, 0, 0};
  *found = 0;
  if (w <= 1 || h <= 1)
    return r;
  int min_x = w, min_y = h, max_x = -1, max_y = -1;
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      const uint8_t v = s[(size_t)y * w + x];
      if (x + 1 < w && v != s[(size_t)y * w + x + 1]) {
        min_x = imin(min_x, x);
        min_y = imin(min_y, y);
        max_x = imax(max_x, x + 1);
        max_y = imax(max_y, y);
      }
      if (y + 1 < h && v != s[(size_t)(y + 1) * w + x]) {
        min_x = imin(min_x, x);
        min_y = imin(min_y, y);
        max_x = imax(max_x, x);
        max_y = imax(max_y, y + 1);
      }
    }
  if (max_x < 0 || max_y < 0)
    return r;
  *found = 1;
  r.x = min_x;
  r.y = min_y;
  r.w = max_x - min_x + 1;
  r.h = max_y - min_y + 1;
  return r;
}

/* expand_and_clamp / align_and_clamp (src/pano/cudaPanoN.inl:77-105). */
static rect_t expand_and_clamp(rect_t r, int pad, int mw, int mh) {
  rect_t o = {0, 0, 0, 0};
  if (r.w <= 0 || r.h <= 0)
    return o;
  const int x0 = imax(0, r.x - pad), y0 = imax(0, r.y - pad);
  const int x1 = imin(mw, r.x + r.w + pad), y1 = imin(mh, r.y + r.h + pad);
  o.x = x0;
  o.y = y0;
  o.w = imax(0, x1 - x0);
  o.h = imax(0, y1 - y0);
  return o;
}

static rect_t align_and_clamp(rect_t r, int align, int mw, int mh) {
  rect_t o = {0, 0, 0, 0};
  if (r.w <= 0 || r.h <= 0)
    return o;
  if (align <= 1)
    return r;
  const int x0 = imax(0, (r.x / align) * align), y0 = imax(0, (r.y / align) * align);
  const int x1 = imin(mw, ((r.x + r.w + align - 1) / align) * align);
  const int y1 = imin(mh, ((r.y + r.h + align - 1) / align) * align);
  o.x = x0;
  o.y = y0;
  o.w = imax(0, x1 - x0);
  o.h = imax(0, y1 - y0);
  return o;
}

static void free_geometry(geom_t* g) {
  free(g->seam);
  g->seam = NULL;
}

static int compute_geometry(const hmpo_config* cfg, geom_t* g) {
  memset(g, 0, sizeof(*g));
  int rc = hmpo_canvas_size(cfg, &g->canvas_w, &g->canvas_h);
  if (rc != HMPO_OK)
    return rc;
  const int W = g->canvas_w, H = g->canvas_h, L = cfg->num_levels, n = cfg->n_images;
  if (cfg->seam_w > W || cfg->seam_h > H)
    return HMPO_EGEOM;
  /* convertMaskMat: replicate-pad the seam to the canvas (canvasManager.cpp:63-101). */
  g->seam = (uint8_t*)malloc((size_t)W * H);
  if (!g->seam)
    return HMPO_ENOMEM;
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x)
      g->seam[(size_t)y * W + x] = cfg->seam[(size_t)imin(y, cfg->seam_h - 1) * cfg->seam_w + imin(x, cfg->seam_w - 1)];
  rect_t full = {0, 0, W, H};
  g->blend = full;
  g->write = full;
  g->mask_k = n;
  g->rule = RULE_NWAY;
  if (cfg->kind == HMPO_KIND_PANO2) {
    g->mask_k = 1;
    g->rule = RULE_TWO;
    /* updateMinimizeBlend (canvasManager.cpp:16-61): the two footprints must overlap. */
    const int overlap = cfg->map_w[0] - cfg->pos_x[1];
    if (overlap <= 0) {
      free_geometry(g);
      return HMPO_EGEOM;
    }
    if (L > 0 && cfg->minimize_blend) {
      const int x_start = cfg->pos_x[1] - OVERLAP_PAD, x_end = cfg->map_w[0] + OVERLAP_PAD;
      if (x_start < 0 || x_end > W || cfg->pos_x[1] - OVERLAP_PAD - cfg->pos_x[0] < 0) {
        free_geometry(g);
        return HMPO_EGEOM;
      }
      g->minimized = 1;
      g->blend.x = x_start;
      g->blend.y = 0;
      g->blend.w = x_end - x_start;
      g->blend.h = H;
      g->write = g->blend;
    }
  } else if (cfg->kind == HMPO_KIND_PANO3) {
    g->mask_k = 3;
    g->rule = RULE_THREE;
  } else if (L > 0 && cfg->minimize_blend) {
    int found = 0;
    rect_t bbox = seam_boundary_bbox(g->seam, W, H, &found);
    if (found) {
      const int margin = 1 << (L < 30 ? L : 30);
      const int align = L <= 1 ? 1 : 1 << (L - 1 < 30 ? L - 1 : 30);
      g->write = expand_and_clamp(bbox, OVERLAP_PAD, W, H);
      g->blend = align_and_clamp(expand_and_clamp(g->write, margin, W, H), align, W, H);
      g->minimized = 1;
      for (int i = 0; i < n; ++i) {
        const int ix0 = imax(cfg->pos_x[i], g->blend.x), iy0 = imax(cfg->pos_y[i], g->blend.y);
        const int ix1 = imin(cfg->pos_x[i] + cfg->map_w[i], g->blend.x + g->blend.w);
        const int iy1 = imin(cfg->pos_y[i] + cfg->map_h[i], g->blend.y + g->blend.h);
        rect_t r = {0, 0, 0, 0};
        if (ix1 > ix0 && iy1 > iy0) {
          r.x = ix0 - cfg->pos_x[i];
          r.y = iy0 - cfg->pos_y[i];
          r.w = ix1 - ix0;
          r.h = iy1 - iy0;
        }
        g->remap_roi[i] = r;
      }
    }
  }
  g->levels = L > 0 ? effective_levels(g->blend.w, g->blend.h, L) : 0;
  return HMPO_OK;
}

int hmpo_blend_geometry(const hmpo_config* cfg, int* out9) {
  geom_t g;
  int rc = compute_geometry(cfg, &g);
  if (rc != HMPO_OK)
    return rc;
  out9[0] = g.blend.x;
  out9[1] = g.blend.y;
  out9[2] = g.blend.w;
  out9[3] = g.blend.h;
  out9[4] = g.write.x;
  out9[5] = g.write.y;
  out9[6] = g.write.w;
  out9[7] = g.write.h;
  out9[8] = g.levels;
  free_geometry(&g);
  return HMPO_OK;
}

/* Hard seam (levels == 0), every kind: a canvas pixel takes the pixel of the image its seam
 * label selects, when inside that image's table and the table entry lies inside the source;
 * everything else stays 0. PANO2: label 1 -> image 1, label 0 -> image 2 (the seam was inverted
 * at load, cudaPano.inl:262-359). PANO3/PANON: label k -> image k (cudaRemap.cu:251-294,
 * cudaFusedKernels3.cu:124-217). */
static void hard_seam(const hmpo_config* cfg, const geom_t* g, const uint8_t* const* inputs, const int* in_w,
                      const int* in_h, uint8_t* canvas) {
  const int W = g->canvas_w, H = g->canvas_h, n = cfg->n_images;
  memset(canvas, 0, (size_t)W * H * g_ch * cfg->batch);
  for (int b = 0; b < cfg->batch; ++b) {
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y)
      for (int x = 0; x < W; ++x) {
        const int label = g->seam[(size_t)y * W + x];
        int o = -1;
        if (cfg->kind == HMPO_KIND_PANO2)
          o = label == 1 ? 0 : (label == 0 ? 1 : -1);
        else if (label < n)
          o = label;
        if (o < 0)
          continue;
        const int rx = x - cfg->pos_x[o], ry = y - cfg->pos_y[o];
        if (rx < 0 || ry < 0 || rx >= cfg->map_w[o] || ry >= cfg->map_h[o])
          continue;
        const int sx = cfg->map_x[o][(size_t)ry * cfg->map_w[o] + rx];
        const int sy = cfg->map_y[o][(size_t)ry * cfg->map_w[o] + rx];
        if (sx < in_w[o] && sy < in_h[o])
          memcpy(canvas + (((size_t)b * H + y) * W + x) * g_ch,
                 inputs[o] + (((size_t)b * in_h[o] + sy) * in_w[o] + sx) * g_ch, g_ch);
      }
  }
}

#define REAL float
#define SFX f32
#include "hmp_oracle_body.h"
#undef REAL
#undef SFX

#define REAL double
#define SFX f64
#include "hmp_oracle_body.h"
#undef REAL
#undef SFX

static int stitch_any_ch(const hmpo_config* cfg, const uint8_t* const* inputs, const int* in_w, const int* in_h,
                         uint8_t* canvas, int dbl) {
  int rc = HMPO_OK;
  for (int i = 0; i < cfg->n_images; ++i)
    if (!inputs[i] || in_w[i] <= 0 || in_h[i] <= 0 || in_w[i] >= 65535)
      return HMPO_EINVAL;
  if (cfg->num_levels == 0) {
    geom_t g;
    rc = compute_geometry(cfg, &g);
    if (rc != HMPO_OK)
      return rc;
    hard_seam(cfg, &g, inputs, in_w, in_h, canvas);
    free_geometry(&g);
    return HMPO_OK;
  }
  return dbl ? stitch_soft_f64(cfg, inputs, in_w, in_h, canvas, NULL)
             : stitch_soft_f32(cfg, inputs, in_w, in_h, canvas, NULL);
}

static int stitch_any(const hmpo_config* cfg, const uint8_t* const* inputs, const int* in_w, const int* in_h,
                      uint8_t* canvas, int dbl) {
  int rc = validate(cfg);
  if (rc != HMPO_OK)
    return rc;
  if (cfg->channels != 0 && cfg->channels != 3 && cfg->channels != 4)
    return HMPO_EINVAL;
  if (cfg->channels == 3 && cfg->filter != HMPO_FILTER_REFBOX)
    return HMPO_EINVAL;
  g_ch = cfg->channels == 3 ? 3 : 4;
  rc = stitch_any_ch(cfg, inputs, in_w, in_h, canvas, dbl);
  g_ch = 4;
  return rc;
}

int hmpo_stitch_f32(const hmpo_config* cfg, const uint8_t* const* inputs, const int* in_w, const int* in_h,
                    uint8_t* canvas) {
  return stitch_any(cfg, inputs, in_w, in_h, canvas, 0);
}

int hmpo_stitch_f64(const hmpo_config* cfg, const uint8_t* const* inputs, const int* in_w, const int* in_h,
                    uint8_t* canvas) {
  return stitch_any(cfg, inputs, in_w, in_h, canvas, 1);
}

int hmpo_stitch_f64_unpacked(const hmpo_config* cfg, const uint8_t* const* inputs, const int* in_w,
                             const int* in_h, double* roi_out) {
  int rc = validate(cfg);
  if (rc != HMPO_OK)
    return rc;
  if (cfg->num_levels == 0)
    return HMPO_EINVAL;
  return stitch_soft_f64(cfg, inputs, in_w, in_h, NULL, roi_out);
}

void hmpo_downsample_rgba_f32(const float* in, int iw, int ih, float* out) {
  down_rgba_f32(in, iw, ih, out, (iw + 1) / 2, (ih + 1) / 2, 1);
}

void hmpo_laplacian_rgba_f32(const float* high, int hw, int hh, const float* low, float* lap) {
  laplacian_f32(high, hw, hh, low, (hw + 1) / 2, (hh + 1) / 2, lap, 1);
}

void hmpo_reconstruct_rgba_f32(const float* low, const float* lap, int hw, int hh, float* out) {
  reconstruct_f32(low, (hw + 1) / 2, (hh + 1) / 2, lap, hw, hh, out, 1);
}

void hmpo_downsample_mask_f32(const float* in, int iw, int ih, int k, float* out) {
  down_mask_f32(in, iw, ih, k, out, (iw + 1) / 2, (ih + 1) / 2);
}

void hmpo_blend_nway_f32(const float* const* laps, int n, const float* mask, int w, int h, float* out) {
  blend_nway_f32(laps, n, mask, w, h, out, 1);
}

void hmpo_blend_two_f32(const float* l1, const float* l2, const float* mask, int w, int h, float* out) {
  blend_two_f32(l1, l2, mask, w, h, out, 1);
}

int hmpo_laplacian_blend_f32(const float* const* inputs, int n, const float* mask, int k, int w, int h, int levels,
                             int rule, float* out) {
  if (n < 2 || n > 8 || levels < 1)
    return HMPO_EINVAL;
  return laplacian_blend_f32(inputs, n, mask, k, w, h, effective_levels(w, h, levels), rule, HMPO_FILTER_REFBOX, 1,
                             out);
}

int hmpo_laplacian_blend_ch_f32(const float* const* inputs, int n, const float* mask, int k, int w, int h,
                                int levels, int rule, int channels, float* out) {
  if (channels != 3 && channels != 4)
    return HMPO_EINVAL;
  g_ch = channels;
  const int rc = hmpo_laplacian_blend_f32(inputs, n, mask, k, w, h, levels, rule, out);
  g_ch = 4;
  return rc;
}
