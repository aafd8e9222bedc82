// hmp_plan.h -- construct-time planning of a stitch (host only, no device code).
//
// The reference re-derives, every frame, which source pixel lands on which canvas pixel: it
// remaps each image onto the canvas, copies blend strips out of the canvas into float buffers,
// and pastes the blended strip back (src/pano/cudaPano.inl:167-418, cudaPanoN.inl:489-685).
// All of that is fixed per configuration, so the planner resolves it once into "gather planes":
// for every destination pixel, the owning image (uint8, 0xFF = none) and the packed table entry
// (sx | sy << 16). A frame then costs one gather per destination pixel and nothing else.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "hmpano.h"

namespace hmp {

constexpr int kOverlapPad = 128;       // CanvasManager overlap_pad (src/pano/canvasManager.h:65)
constexpr uint8_t kNoOwner = 0xFF;     // plane owner: nothing maps here
constexpr uint32_t kNoEntry = 0xFFFFFFFFu;  // packed (65535, 65535): unmapped
constexpr int kMaxImages = 8;
constexpr int kMaxLevels = 7;          // levels one fused pyramid pass supports

enum BlendRule : int { kRuleNway = 1, kRuleTwo = 2, kRuleThree = 3 };

// Mask class of an N-way pixel at level l >= 1 (values shared with the kernels): 0..n-1 = the
// image whose weight is 1 while the others are 0; kHotNone = every weight 0; kHotFrac = any other
// weights (the blend then reads the K mask values).
enum MaskHot : uint8_t { kHotNone = 0xFE, kHotFrac = 0xFF };

struct Rect {
  int x = 0, y = 0, w = 0, h = 0;
  bool empty() const { return w <= 0 || h <= 0; }
  bool contains(int px, int py) const { return px >= x && py >= y && px < x + w && py < y + h; }
};

// One gather plane over `rect` (coordinates of the plane's domain: canvas or blend region).
struct GatherPlane {
  Rect rect;                   // bounding box of mapped pixels (empty: nothing mapped)
  int default_owner = 0;       // owner when `owner` is empty
  std::vector<uint8_t> owner;  // rect.w * rect.h, row-major, or empty (single owner)
  std::vector<uint32_t> map;   // rect.w * rect.h, packed sx | sy << 16
};

struct Plan {
  int kind = 0;
  int n = 0;
  int batch = 1;
  int levels_requested = 0;
  int levels = 0;  // effective (compute_num_levels); 0 = hard seam
  int canvas_w = 0, canvas_h = 0;
  int storage = HMP_STORAGE_F32;
  int filter = HMP_FILTER_REFBOX;
  int rule = kRuleTwo;
  int mask_k = 1;        // mask channels of the pyramid blend
  int channels = 4;      // 4 (RGBA) or 3 (RGB)
  bool pixel_float = false;  // float samples (HMP_PIXEL_F32) instead of uint8
  // Everything but RGBA8 runs the level-by-level kernels (hmp_generic.cu).
  bool generic() const { return channels != 4 || pixel_float; }
  int pixel_bytes() const { return channels * (pixel_float ? 4 : 1); }
  bool minimized = false;
  bool slot_opaque = true;    // soft-seam rule: out-of-range, non-sentinel entries give alpha 255
  bool canvas_opaque = false; // same rule for the canvas plane
  Rect blend;  // pyramid domain, canvas coordinates
  Rect write;  // pyramid write-back region, canvas coordinates (inside blend)
  bool canvas_plane_used = false;
  GatherPlane canvas;               // canvas coordinates; pixels in `write` are skipped (all of
                                    // them, or those of pyramid blocks in copy-block mode)
  std::vector<GatherPlane> slots;   // n, blend coordinates
  std::vector<uint8_t> mask0;       // blend.w * blend.h: two-image weight value or label
  std::vector<std::vector<float>> mask_levels;  // levels >= 1: lw*lh*mask_k floats
  std::vector<std::vector<uint8_t>> mask_hot;   // N-way rule, levels >= 1: lw*lh MaskHot classes
  std::vector<int> lw, lh;          // level dims
  // Two images, minimised: the blend strip's content is the canvas shifted by image 1's table
  // column (the reference copies full1 / full2 out of the canvas at that offset).
  int strip_shift = 0;
  std::vector<int> src_w, src_h;    // expected source sizes (0 = unknown)
};

// Validates `cfg` and fills `plan`. Returns a cudaError_t value and a message on failure.
int build_plan(const hmp_config& cfg, Plan& plan, std::string& message);

// Geometry only (cheap): canvas size, blend/write rects, effective levels.
int plan_geometry(const hmp_config& cfg, Plan& plan, std::string& message);

// Effective pyramid depth for a w x h domain (cupano/ops.py compute_num_levels,
// src/cuda/cudaBlendN.cu:680-688): stop once a side of the previous level is below 2.
int effective_levels(int w, int h, int requested);

}  // namespace hmp
