// hmp_copyplan.h -- construct-time planning of copy blocks (host only).
//
// Three- and N-image blend regions cover most of the canvas, yet almost all of their pixels are
// far from every seam: the mask is one-hot on one image at every level of the pixel's
// reconstruction, and that image is valid throughout. There the reference's pyramid returns that
// image's pixel exactly. With the 2x2 box filter and bilinear upsample every value involved is a
// short dyadic fraction when all the image's pixels in the reconstruction's support have alpha != 0:
//   G^l holds multiples of 2^-2l below 256, a bilinear tap of weight 1, 1/2 or 1/4 adds two
//   bits, so the downsample sums, the upsample sums, Lap = G^l - up(G^(l+1)) and
//   R^l = up(R^(l+1)) + Lap all fit FP32's 24 bits (at most 8 integer + 14 fractional bits for
//   seven levels) and are exact. Then R^(L-1) = G^(L-1) and, by induction,
//   R^l = up(G^(l+1)) + (G^l - up(G^(l+1))) = G^l at every level, so the packed result is the
//   source pixel itself (truncation of an exact integer), alpha included.
// (With FP16 level storage the same pixels equal the FP64 result, which is exact there too.)
// A pixel whose support holds no valid pixel of any image reconstructs to (0, 0, 0, 0).
//
// The support of a level-0 pixel: level l reads level l+1 at floor(q/2) and floor(q/2)+1 (clamped),
// so the levels it depends on span the level-(L-1) pixels [x >> (L-1), hi] with
// hi = min((hi_prev >> 1) + 1, w_l - 1) chained from x, and their level-0 footprint, which holds
// every lower level's. Blocks of 64 x 16 write-rect pixels (pyr_fine's) are classified over the
// union of their pixels' supports:
//   copy-k  : every label there is k < n and image k's table holds a non-sentinel entry at every
//             pixel (the canvas gather then writes image k's pixel, which is also the hard seam's);
//   empty   : no image has a non-sentinel entry anywhere there (the gather writes 0);
//   pyramid : anything else (pyr_fine writes it).
// Per frame two conditions are checked, and either failure falls back to the full pyramid:
//   * the table entries the copy blocks read must lie inside the frames (need_w / need_h, checked
//     by the host per call: an out-of-range entry would read as a fill);
//   * every source pixel in a copy block's support must have alpha != 0 (checked on the device:
//     by the gather over the blend region, for the pixels it copies and those outside the write
//     rect, and by pyr_fine for the pyramid-block pixels inside a support, the only others a
//     support holds; any alpha 0 gates on the fallback launches, which recompute the write rect).
// The pyramid then runs only where it is needed: pyr_fine over the pyramid blocks, pyr_coarse over
// the level-1 tiles those read (R^1), pyr_down over the level-0 tiles whose levels either reads.
#pragma once

#include <cstdint>
#include <vector>

#include "hmp_plan.h"

namespace hmp {

constexpr uint8_t kBlockCopy = 0, kBlockPyramid = 1, kBlockEmpty = 2;

struct CopyPlan {
  bool usable = false;
  int fx0 = 0, fy0 = 0, nfx = 0, nfy = 0;   // pyr_fine block grid, blend coordinates
  std::vector<uint8_t> pyramid_block;       // [nfy][nfx]: 1 = written by the pyramid
  std::vector<uint8_t> block_class;         // [nfy][nfx]: kBlockCopy, kBlockPyramid or kBlockEmpty
  std::vector<uint32_t> fine_list;          // tx | ty << 16 of the pyramid blocks
  std::vector<uint32_t> coarse_list;        // absolute level-1 tiles of edge tile_coarse
  std::vector<uint32_t> down_list;          // level-0 tiles of edge tile_down; bit 31: pyr_fine reads
                                            // the tile's kept level-0 pixels
  // [gy][gx], one byte per 2^(L-1) block of the blend region: 1 + the slot a copy block copies
  // inside its support (one label there, and that slot has a source pixel at every pixel), else 0.
  std::vector<uint8_t> support_mark;
  int support_pitch = 0, support_shift = 0;
  uint32_t need_w[kMaxImages] = {}, need_h[kMaxImages] = {};  // frame size the copy blocks' entries need
  int copy_blocks = 0, empty_blocks = 0, pyramid_blocks = 0;
  long long pyramid_pixels = 0;  // write-rect pixels of the pyramid blocks
  long long dense_down = 0, dense_coarse = 0;  // tiles of the dense grids, for reports
};

// Plans copy blocks for `p` (its slot planes and level-0 labels must still be held on the host).
// Leaves out.usable false where they do not apply: two images without the minimised strip (or with
// image 1's table off column 0, which shifts the strip's content against the canvas), N-image
// stitchers of two images, fewer than two levels, the Binomial5 filter (its 5-tap sums are not
// short dyadic fractions), and non-RGBA8 pixels.
void plan_copy_blocks(const Plan& p, int tile_down, int tile_coarse, CopyPlan& out);

}  // namespace hmp
