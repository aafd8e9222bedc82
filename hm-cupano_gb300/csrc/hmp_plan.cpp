// hmp_plan.cpp -- construct-time planning of a stitch. See hmp_plan.h.
#include "hmp_plan.h"

#include <algorithm>
#include <cstring>

namespace hmp {
namespace {

int fail(std::string& message, int code, const std::string& text) {
  message = text;
  return code;
}

inline uint32_t pack_entry(uint16_t sx, uint16_t sy) { return uint32_t(sx) | (uint32_t(sy) << 16); }

// Seam value at canvas (x, y) after convertMaskMat's replicate padding to the canvas
// (src/pano/canvasManager.cpp:63-85).
inline uint8_t seam_at(const hmp_config& c, int x, int y) {
  const int sx = std::min(x, c.seam_width - 1), sy = std::min(y, c.seam_height - 1);
  return c.seam[size_t(sy) * c.seam_width + sx];
}

// Table entry of image i at canvas (x, y), or kNoEntry outside its table.
inline uint32_t table_at(const hmp_config& c, int i, int x, int y) {
  const hmp_remap& r = c.remaps[i];
  const int rx = x - r.xpos, ry = y - r.ypos;
  if (rx < 0 || ry < 0 || rx >= r.width || ry >= r.height) return kNoEntry;
  const size_t k = size_t(ry) * r.width + rx;
  return pack_entry(r.map_x[k], r.map_y[k]);
}

inline bool in_table(const hmp_config& c, int i, int x, int y) {
  const hmp_remap& r = c.remaps[i];
  return x >= r.xpos && y >= r.ypos && x < r.xpos + r.width && y < r.ypos + r.height;
}

Rect intersect(const Rect& a, const Rect& b) {
  const int x0 = std::max(a.x, b.x), y0 = std::max(a.y, b.y);
  const int x1 = std::min(a.x + a.w, b.x + b.w), y1 = std::min(a.y + a.h, b.y + b.h);
  if (x1 <= x0 || y1 <= y0) return Rect{};
  return Rect{x0, y0, x1 - x0, y1 - y0};
}

// Bounding box of label changes (right and down neighbours), src/pano/cudaPanoN.inl:38-75.
bool seam_boundary_bbox(const hmp_config& c, int W, int H, Rect& out) {
  if (W <= 1 || H <= 1) return false;
  int min_x = W, min_y = H, max_x = -1, max_y = -1;
  for (int y = 0; y < H; ++y) {
    for (int x = 0; x < W; ++x) {
      const uint8_t v = seam_at(c, x, y);
      if (x + 1 < W && v != seam_at(c, x + 1, y)) {
        min_x = std::min(min_x, x);
        max_x = std::max(max_x, x + 1);
        min_y = std::min(min_y, y);
        max_y = std::max(max_y, y);
      }
      if (y + 1 < H && v != seam_at(c, x, y + 1)) {
        min_x = std::min(min_x, x);
        max_x = std::max(max_x, x);
        min_y = std::min(min_y, y);
        max_y = std::max(max_y, y + 1);
      }
    }
  }
  if (max_x < 0 || max_y < 0) return false;
  out = Rect{min_x, min_y, max_x - min_x + 1, max_y - min_y + 1};
  return true;
}

// src/pano/cudaPanoN.inl:77-90.
Rect expand_and_clamp(const Rect& r, int pad, int W, int H) {
  if (r.empty()) return Rect{};
  const int x0 = std::max(0, r.x - pad), y0 = std::max(0, r.y - pad);
  const int x1 = std::min(W, r.x + r.w + pad), y1 = std::min(H, r.y + r.h + pad);
  return Rect{x0, y0, std::max(0, x1 - x0), std::max(0, y1 - y0)};
}

// src/pano/cudaPanoN.inl:92-105.
Rect align_and_clamp(const Rect& r, int align, int W, int H) {
  if (r.empty()) return Rect{};
  if (align <= 1) return r;
  const int x0 = std::max(0, (r.x / align) * align), y0 = std::max(0, (r.y / align) * align);
  const int x1 = std::min(W, ((r.x + r.w + align - 1) / align) * align);
  const int y1 = std::min(H, ((r.y + r.h + align - 1) / align) * align);
  return Rect{x0, y0, std::max(0, x1 - x0), std::max(0, y1 - y0)};
}

int validate(const hmp_config& c, std::string& m) {
  if (c.kind != HMP_KIND_PANO2 && c.kind != HMP_KIND_PANO3 && c.kind != HMP_KIND_PANON)
    return fail(m, HMP_ERR_INVALID_VALUE, "unknown stitcher kind");
  if (c.kind == HMP_KIND_PANO2 && c.n_images != 2)
    return fail(m, HMP_ERR_INVALID_VALUE, "two-image stitcher needs exactly 2 remaps");
  if (c.kind == HMP_KIND_PANO3 && c.n_images != 3)
    return fail(m, HMP_ERR_INVALID_VALUE, "three-image stitcher needs exactly 3 remaps");
  if (c.n_images < 2 || c.n_images > kMaxImages)
    return fail(m, HMP_ERR_INVALID_VALUE, "Unsupported N for blend (supported 2..8)");
  if (c.num_levels < 0 || c.num_levels > 30) return fail(m, HMP_ERR_INVALID_VALUE, "num_levels out of range");
  // With canvases below 2^20 pixels per side, 2^16 frames keep every byte count below 2^60.
  if (c.batch_size < 1 || c.batch_size > 65536)
    return fail(m, HMP_ERR_INVALID_VALUE, "batch_size must be in 1..65536");
  if (c.channels != 4 && c.channels != 3) return fail(m, HMP_ERR_NOT_SUPPORTED, "only 3- and 4-channel pixels are supported");
  if (c.pixel_format != HMP_PIXEL_U8 && c.pixel_format != HMP_PIXEL_F32)
    return fail(m, HMP_ERR_INVALID_VALUE, "unknown pixel format");
  if ((c.channels != 4 || c.pixel_format != HMP_PIXEL_U8) &&
      (c.storage != HMP_STORAGE_F32 || c.filter != HMP_FILTER_REFBOX))
    return fail(m, HMP_ERR_NOT_SUPPORTED, "FP16 storage and the Binomial5 filter are RGBA8-only");
  if (c.storage != HMP_STORAGE_F32 && c.storage != HMP_STORAGE_F16)
    return fail(m, HMP_ERR_INVALID_VALUE, "unknown pyramid storage");
  if (c.filter != HMP_FILTER_REFBOX && c.filter != HMP_FILTER_BINOMIAL5)
    return fail(m, HMP_ERR_INVALID_VALUE, "unknown pyramid filter");
  // ControlMasks::is_valid (src/pano/controlMasks.h:30-66): missing tables or seam.
  if (!c.remaps || !c.seam || c.seam_width <= 0 || c.seam_height <= 0)
    return fail(m, HMP_ERR_FILE_NOT_FOUND, "Stitching masks were not able to be loaded");
  for (int i = 0; i < c.n_images; ++i) {
    const hmp_remap& r = c.remaps[i];
    if (!r.map_x || !r.map_y || r.width <= 0 || r.height <= 0)
      return fail(m, HMP_ERR_FILE_NOT_FOUND, "Stitching masks were not able to be loaded");
    if (r.xpos < 0 || r.ypos < 0)
      return fail(m, HMP_ERR_INVALID_VALUE, "canvas positions must be normalised (>= 0)");
    // Keeps position + size (the canvas extent) and every pixel count far from int overflow.
    if (int64_t(r.xpos) + r.width > (int64_t(1) << 20) || int64_t(r.ypos) + r.height > (int64_t(1) << 20))
      return fail(m, HMP_ERR_NOT_SUPPORTED, "canvas larger than 2^20 pixels per side");
  }
  return HMP_OK;
}

// Crops a full-domain plane (dw x dh) to the bounding box of mapped pixels and drops the owner
// array when all mapped pixels share one owner equal to `implied_owner` (the owner the kernels
// assume for a plane without an owner array).
GatherPlane crop_plane(std::vector<uint8_t>& owner, std::vector<uint32_t>& map, int dw, int dh,
                       int implied_owner) {
  GatherPlane p;
  int x0 = dw, y0 = dh, x1 = -1, y1 = -1;
  int first_owner = -1;
  bool uniform = true;
  for (int y = 0; y < dh; ++y)
    for (int x = 0; x < dw; ++x) {
      const size_t k = size_t(y) * dw + x;
      if (owner[k] == kNoOwner) map[k] = kNoEntry;
      if (map[k] == kNoEntry) continue;
      x0 = std::min(x0, x);
      x1 = std::max(x1, x);
      y0 = std::min(y0, y);
      y1 = std::max(y1, y);
      if (first_owner < 0)
        first_owner = owner[k];
      else if (owner[k] != first_owner)
        uniform = false;
    }
  if (x1 < 0) return p;  // nothing mapped
  if (first_owner != implied_owner) uniform = false;
  p.rect = Rect{x0, y0, x1 - x0 + 1, y1 - y0 + 1};
  p.default_owner = first_owner;
  p.map.resize(size_t(p.rect.w) * p.rect.h);
  if (!uniform) p.owner.resize(p.map.size());
  for (int y = 0; y < p.rect.h; ++y) {
    std::memcpy(&p.map[size_t(y) * p.rect.w], &map[size_t(y0 + y) * dw + x0], size_t(p.rect.w) * 4);
    if (!uniform) std::memcpy(&p.owner[size_t(y) * p.rect.w], &owner[size_t(y0 + y) * dw + x0], p.rect.w);
  }
  return p;
}

// Canvas plane selected by the seam labels (hard seam; also the baseline of the minimised
// N-image soft seam): src/cuda/cudaRemap.cu:203-294, src/cuda/cudaFusedKernels3.cu:124-217.
void seam_owner_plane(const hmp_config& c, Plan& p) {
  const int W = p.canvas_w, H = p.canvas_h, n = p.n;
  GatherPlane& g = p.canvas;
  g.rect = Rect{0, 0, W, H};
  g.owner.assign(size_t(W) * H, kNoOwner);
  g.map.assign(size_t(W) * H, kNoEntry);
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      const int label = seam_at(c, x, y);
      int o = -1;
      if (c.kind == HMP_KIND_PANO2)
        o = label == 1 ? 0 : (label == 0 ? 1 : -1);  // seam inverted at load (cudaPano.inl:262-359)
      else if (label < n)
        o = label;
      if (o < 0) continue;
      const uint32_t e = table_at(c, o, x, y);
      if (e == kNoEntry && !in_table(c, o, x, y)) continue;
      g.owner[size_t(y) * W + x] = uint8_t(o);
      g.map[size_t(y) * W + x] = e;
    }
}

// Two-image soft seam, canvas outside the blend strip: image 2's table overwrites image 1's
// (cudaPano.inl:210-302; both remaps write every table pixel).
void last_writer_plane(const hmp_config& c, Plan& p) {
  const int W = p.canvas_w, H = p.canvas_h;
  GatherPlane& g = p.canvas;
  g.rect = Rect{0, 0, W, H};
  g.owner.assign(size_t(W) * H, kNoOwner);
  g.map.assign(size_t(W) * H, kNoEntry);
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      for (int o : {1, 0}) {
        if (!in_table(c, o, x, y)) continue;
        g.owner[size_t(y) * W + x] = uint8_t(o);
        g.map[size_t(y) * W + x] = table_at(c, o, x, y);
        break;
      }
    }
}

}  // namespace

int effective_levels(int w, int h, int requested) {
  const int levels = std::max(1, requested);
  int cw = w, ch = h, count = 1;
  for (int l = 1; l < levels; ++l) {
    if (cw < 2 || ch < 2) break;
    cw = (cw + 1) / 2;
    ch = (ch + 1) / 2;
    ++count;
  }
  return count;
}

int plan_geometry(const hmp_config& c, Plan& p, std::string& m) {
  int rc = validate(c, m);
  if (rc != HMP_OK) return rc;
  p = Plan{};
  p.kind = c.kind;
  p.n = c.n_images;
  p.batch = c.batch_size;
  p.levels_requested = c.num_levels;
  p.storage = c.storage;
  p.filter = c.filter;
  p.channels = c.channels;
  p.pixel_float = c.pixel_format == HMP_PIXEL_F32;
  // Canvas = max(position + table size) (src/pano/controlMasks.cpp:265-271).
  for (int i = 0; i < p.n; ++i) {
    p.canvas_w = std::max(p.canvas_w, c.remaps[i].xpos + c.remaps[i].width);
    p.canvas_h = std::max(p.canvas_h, c.remaps[i].ypos + c.remaps[i].height);
  }
  const int W = p.canvas_w, H = p.canvas_h, L = c.num_levels;
  if (c.seam_width > W || c.seam_height > H)
    return fail(m, HMP_ERR_INVALID_VALUE, "seam mask is larger than the canvas");
  p.blend = Rect{0, 0, W, H};
  p.write = p.blend;
  p.rule = kRuleNway;
  p.mask_k = p.n;
  p.slot_opaque = true;
  if (c.kind == HMP_KIND_PANO2) {
    p.rule = kRuleTwo;
    p.mask_k = 1;
    // updateMinimizeBlend (canvasManager.cpp:16-61): the tables must overlap.
    const int x1 = c.remaps[0].xpos, x2 = c.remaps[1].xpos, w1 = c.remaps[0].width;
    if (w1 - x2 <= 0) return fail(m, HMP_ERR_INVALID_VALUE, "Images do not overlap; invalid two-image configuration");
    if (L > 0 && c.minimize_blend) {
      const int x_start = x2 - kOverlapPad, x_end = w1 + kOverlapPad;
      // convertMaskMat asserts (canvasManager.cpp:88-92) and the strip copy's source origin.
      if (x_start < 0 || x_end > W || x2 - kOverlapPad - x1 < 0)
        return fail(m, HMP_ERR_INVALID_VALUE, "blend strip (overlap +/- 128 px) does not fit the canvas");
      p.minimized = true;
      p.blend = Rect{x_start, 0, x_end - x_start, H};
      p.write = p.blend;
      p.strip_shift = x1;
    }
  } else if (c.kind == HMP_KIND_PANO3) {
    p.rule = kRuleThree;
    p.mask_k = 3;
    p.slot_opaque = !c.fused;  // the fused remap leaves invalid pixels at 0 (cudaFusedKernels3.cu:25-119)
  } else if (L > 0 && c.minimize_blend) {
    Rect bbox;
    if (seam_boundary_bbox(c, W, H, bbox)) {
      const int margin = 1 << std::min(L, 30);
      const int align = L <= 1 ? 1 : 1 << std::min(L - 1, 30);
      p.write = expand_and_clamp(bbox, kOverlapPad, W, H);
      p.blend = align_and_clamp(expand_and_clamp(p.write, margin, W, H), align, W, H);
      p.minimized = !p.write.empty() && !p.blend.empty();
      if (!p.minimized) {
        p.blend = Rect{0, 0, W, H};
        p.write = p.blend;
      }
    }
  }
  if (L == 0) {
    p.levels = 0;
    p.write = Rect{};
    p.blend = Rect{};
  } else {
    p.levels = effective_levels(p.blend.w, p.blend.h, L);
    p.lw.assign(p.levels, 0);
    p.lh.assign(p.levels, 0);
    p.lw[0] = p.blend.w;
    p.lh[0] = p.blend.h;
    for (int l = 1; l < p.levels; ++l) {
      p.lw[l] = (p.lw[l - 1] + 1) / 2;
      p.lh[l] = (p.lh[l - 1] + 1) / 2;
    }
  }
  return HMP_OK;
}

int build_plan(const hmp_config& c, Plan& p, std::string& m) {
  int rc = plan_geometry(c, p, m);
  if (rc != HMP_OK) return rc;
  if (p.levels > kMaxLevels)
    return fail(m, HMP_ERR_NOT_SUPPORTED, "more than 7 effective pyramid levels are not supported");
  const int W = p.canvas_w, H = p.canvas_h, n = p.n;

  // ---- canvas plane (everything the pyramid does not write) ----
  if (p.levels == 0) {
    seam_owner_plane(c, p);
    p.canvas_plane_used = true;
    p.canvas_opaque = false;
    return HMP_OK;
  }
  if (p.kind == HMP_KIND_PANO2 && p.minimized) {
    last_writer_plane(c, p);
    p.canvas_plane_used = true;
    p.canvas_opaque = true;
  } else if (p.kind == HMP_KIND_PANON && p.minimized) {
    seam_owner_plane(c, p);
    p.canvas_plane_used = true;
    p.canvas_opaque = false;
  } else if (p.rule != kRuleTwo && p.n >= 3 && p.levels >= 2 && p.filter == HMP_FILTER_REFBOX && !p.generic()) {
    // Three images, or N without a minimised blend region: the pyramid covers the whole canvas,
    // and the seam-selected plane serves the copy blocks, where the pyramid's result is the
    // label's pixel (hmp_copyplan.h).
    seam_owner_plane(c, p);
    p.canvas_plane_used = true;
    p.canvas_opaque = false;
  }

  // ---- blend slots: level-0 pyramid input of each image over the blend region ----
  const Rect& B = p.blend;
  const int bw = B.w, bh = B.h;
  p.slots.resize(n);
  std::vector<uint8_t> owner;
  std::vector<uint32_t> map;
  for (int k = 0; k < n; ++k) {
    owner.assign(size_t(bw) * bh, kNoOwner);
    map.assign(size_t(bw) * bh, kNoEntry);
    if (p.kind == HMP_KIND_PANO2 && p.minimized) {
      // full1/full2 are copied out of the canvas after remap 1 / remap 2 (cudaPano.inl:225-318):
      // full1[y][x1 + i] = canvas1[y][x2 - pad - x1 + i], full2[y][x1 + pad + i] = canvas2[y][x2 + i]
      // for i < overlap + pad, where canvas1 holds image 1's table and canvas2 image 2's over it.
      const int x1 = c.remaps[0].xpos, x2 = c.remaps[1].xpos;
      const int rw = (c.remaps[0].width - x2) + kOverlapPad;
      for (int v = 0; v < bh; ++v)
        for (int i = 0; i < rw; ++i) {
          const int src_c = k == 0 ? (x2 - kOverlapPad - x1) + i : x2 + i;
          const int dst_u = k == 0 ? x1 + i : x1 + kOverlapPad + i;
          if (src_c < 0 || src_c >= W || v >= H || dst_u < 0 || dst_u >= bw) continue;
          const size_t d = size_t(v) * bw + dst_u;
          const int order[2] = {1, 0};
          for (int j = (k == 0 ? 1 : 0); j < 2; ++j) {
            const int o = order[j];
            if (!in_table(c, o, src_c, v)) continue;
            owner[d] = uint8_t(o);
            map[d] = table_at(c, o, src_c, v);
            break;
          }
        }
    } else {
      // Image k's table over the blend region (remap into a zeroed buffer, or the ROI remap of
      // the minimised N-image path: cudaRemap.cu:60-198, cudaPanoN.inl:590-615).
      const hmp_remap& r = c.remaps[k];
      const Rect tr{r.xpos, r.ypos, r.width, r.height};
      const Rect in = intersect(tr, B);
      for (int y = in.y; y < in.y + in.h; ++y)
        for (int x = in.x; x < in.x + in.w; ++x) {
          const size_t d = size_t(y - B.y) * bw + (x - B.x);
          owner[d] = uint8_t(k);
          map[d] = table_at(c, k, x, y);
        }
    }
    p.slots[k] = crop_plane(owner, map, bw, bh, k);
    if (p.slots[k].rect.empty()) p.slots[k].default_owner = k;
  }

  // ---- mask pyramid (constant per configuration) ----
  p.mask0.resize(size_t(bw) * bh);
  for (int v = 0; v < bh; ++v)
    for (int u = 0; u < bw; ++u) p.mask0[size_t(v) * bw + u] = seam_at(c, B.x + u, B.y + v);
  const int K = p.mask_k;
  std::vector<float> cur(size_t(bw) * bh * K);
  for (size_t i = 0; i < size_t(bw) * bh; ++i) {
    const uint8_t v = p.mask0[i];
    if (K == 1)
      cur[i] = float(v);
    else
      for (int ch = 0; ch < K; ++ch) cur[i * K + ch] = v == ch ? 1.0f : 0.0f;
  }
  p.mask_levels.assign(p.levels, {});
  for (int l = 1; l < p.levels; ++l) {
    const int iw = p.lw[l - 1], ih = p.lh[l - 1], ow = p.lw[l], oh = p.lh[l];
    std::vector<float> nxt(size_t(ow) * oh * K);
    float sums[kMaxImages];
    // 2x2 mean over in-bounds pixels, dy outer / dx inner (src/cuda/cudaBlend.cu:268-296,
    // src/cuda/cudaBlendN.cu:19-48).
    for (int y = 0; y < oh; ++y)
      for (int x = 0; x < ow; ++x) {
        for (int ch = 0; ch < K; ++ch) sums[ch] = 0.0f;
        int cnt = 0;
        for (int dy = 0; dy < 2; ++dy)
          for (int dx = 0; dx < 2; ++dx) {
            const int ix = 2 * x + dx, iy = 2 * y + dy;
            if (ix >= iw || iy >= ih) continue;
            for (int ch = 0; ch < K; ++ch) sums[ch] += cur[(size_t(iy) * iw + ix) * K + ch];
            ++cnt;
          }
        for (int ch = 0; ch < K; ++ch) nxt[(size_t(y) * ow + x) * K + ch] = sums[ch] / float(cnt);
      }
    p.mask_levels[l] = nxt;
    cur.swap(nxt);
  }
  // The N-way kernels pick from the class alone unless the weights are fractional.
  p.mask_hot.assign(p.levels, {});
  for (int l = 1; p.rule == kRuleNway && l < p.levels; ++l) {
    const std::vector<float>& wts = p.mask_levels[l];
    std::vector<uint8_t>& h = p.mask_hot[l];
    h.resize(size_t(p.lw[l]) * p.lh[l]);
    for (size_t i = 0; i < h.size(); ++i) {
      int hot = kHotNone;
      for (int k = 0; k < K && hot != kHotFrac; ++k) {
        const float w = wts[i * K + k];
        if (w == 1.0f)
          hot = hot == kHotNone ? k : kHotFrac;
        else if (w != 0.0f)
          hot = kHotFrac;
      }
      h[i] = uint8_t(hot);
    }
  }
  return HMP_OK;
}

}  // namespace hmp
