// hmp_copyplan.cpp -- construct-time planning of copy blocks. See hmp_copyplan.h.
#include "hmp_copyplan.h"

#include <algorithm>

namespace hmp {

void plan_copy_blocks(const Plan& p, int td, int t1, CopyPlan& cp) {
  cp = CopyPlan{};
  const int L = p.levels, n = p.n;
  if (L < 2 || p.filter != HMP_FILTER_REFBOX || p.generic() || !p.canvas_plane_used) return;
  const bool two = p.rule == kRuleTwo;
  // Two images: the minimised strip only, whose content lines up with the canvas (image 1's table
  // at column 0); three or more: any blend region.
  if (two ? (!p.minimized || p.strip_shift != 0) : n < 3) return;
  const int bw = p.lw[0], bh = p.lh[0];
  if (bw <= 0 || bh <= 0 || int(p.mask0.size()) != bw * bh || int(p.slots.size()) != n) return;
  // Level-(L-1) pixel q covers level-0 block q of edge G; per block: the label if uniform, and per
  // image whether every pixel / any pixel has a non-sentinel entry, with the largest coordinates.
  const int G = 1 << (L - 1);
  const int gx = (bw + G - 1) / G, gy = (bh + G - 1) / G;
  constexpr uint8_t kUnset = 0xFE, kMixed = 0xFF;
  std::vector<uint8_t> lab(size_t(gx) * gy, kUnset);
  for (int y = 0; y < bh; ++y) {
    const uint8_t* row = &p.mask0[size_t(y) * bw];
    uint8_t* lb = &lab[size_t(y / G) * gx];
    for (int x = 0; x < bw; ++x) {
      uint8_t& b = lb[x / G];
      if (b == kUnset)
        b = row[x];
      else if (b != row[x])
        b = kMixed;
    }
  }
  // Per slot: whether every / any pixel of a block has a non-sentinel entry; per image: the largest
  // coordinates its entries there hold (a two-image strip's second slot mixes images 1 and 2).
  const size_t nb = size_t(gx) * gy;
  std::vector<uint8_t> all_valid(size_t(n) * nb, 1), any_valid(size_t(n) * nb, 0);
  std::vector<uint16_t> max_sx(size_t(n) * nb, 0), max_sy(size_t(n) * nb, 0);
  std::vector<uint8_t> img2_any(two ? nb : 0, 0);  // two images: any entry of image 2 in the block
  for (int k = 0; k < n; ++k) {
    const GatherPlane& s = p.slots[k];
    uint8_t* av = &all_valid[size_t(k) * nb];
    uint8_t* an = &any_valid[size_t(k) * nb];
    // Blocks not wholly inside the plane's rect hold pixels without an entry.
    for (int by = 0; by < gy; ++by)
      for (int bx = 0; bx < gx; ++bx) {
        const int x0 = bx * G, y0 = by * G, x1 = std::min(x0 + G, bw), y1 = std::min(y0 + G, bh);
        if (s.rect.empty() || x0 < s.rect.x || y0 < s.rect.y || x1 > s.rect.x + s.rect.w || y1 > s.rect.y + s.rect.h)
          av[size_t(by) * gx + bx] = 0;
      }
    if (s.rect.empty()) continue;
    for (int ry = 0; ry < s.rect.h; ++ry) {
      const int y = s.rect.y + ry;
      for (int rx = 0; rx < s.rect.w; ++rx) {
        const int x = s.rect.x + rx;
        const size_t i = size_t(ry) * s.rect.w + rx;
        const uint32_t e = s.map[i];
        const int o = s.owner.empty() ? s.default_owner : s.owner[i];
        const size_t b = size_t(y / G) * gx + x / G;
        if (two && o == 1) img2_any[b] = 1;
        // Three or more images: each slot holds its own image only.
        if (o >= n || (!two && o != k) || (e & 0xFFFFu) == 0xFFFFu) {
          av[b] = 0;
          continue;
        }
        an[b] = 1;
        uint16_t& mx = max_sx[size_t(o) * nb + b];
        uint16_t& my = max_sy[size_t(o) * nb + b];
        mx = std::max<uint16_t>(mx, uint16_t(e & 0xFFFFu));
        my = std::max<uint16_t>(my, uint16_t(e >> 16));
      }
    }
  }

  // pyr_fine's blocks over the write rect (blend coordinates), and each block's support.
  const int wx0 = p.write.x - p.blend.x, wy0 = p.write.y - p.blend.y;
  const int wx1 = wx0 + p.write.w, wy1 = wy0 + p.write.h;
  cp.fx0 = wx0 & ~1;
  cp.fy0 = wy0 & ~1;
  cp.nfx = (wx1 - cp.fx0 + 63) / 64;
  cp.nfy = (wy1 - cp.fy0 + 15) / 16;
  const auto hi_chain = [&](int h, const std::vector<int>& dims) {
    for (int l = 1; l < L; ++l) h = std::min((h >> 1) + 1, dims[l] - 1);
    return h;
  };
  cp.pyramid_block.assign(size_t(cp.nfx) * cp.nfy, 0);
  cp.block_class.assign(size_t(cp.nfx) * cp.nfy, kBlockPyramid);
  std::vector<uint8_t> support_mark(nb, 0);  // blocks inside some copy block's support
  for (int j = 0; j < cp.nfy; ++j)
    for (int i = 0; i < cp.nfx; ++i) {
      const int x0 = std::max(cp.fx0 + 64 * i, wx0), x1 = std::min(cp.fx0 + 64 * i + 64, wx1);
      const int y0 = std::max(cp.fy0 + 16 * j, wy0), y1 = std::min(cp.fy0 + 16 * j + 16, wy1);
      const int sx0 = x0 >> (L - 1), sx1 = hi_chain(x1 - 1, p.lw);
      const int sy0 = y0 >> (L - 1), sy1 = hi_chain(y1 - 1, p.lh);
      // The slot whose pixel the block copies: the label's image; with two images the seam value
      // 1 selects slot 0 (image 1) and 0 slot 1 (image 2, or image 1 where image 2 has no table).
      const int label = lab[size_t(sy0) * gx + sx0];
      const int k = two ? (label == 1 ? 0 : (label == 0 ? 1 : n)) : label;
      bool copy = k < n, empty = true;
      for (int by = sy0; by <= sy1; ++by)
        for (int bx = sx0; bx <= sx1; ++bx) {
          const size_t b = size_t(by) * gx + bx;
          if (copy && (lab[b] != label || !all_valid[size_t(k) * nb + b])) copy = false;
          // Two images, slot 0: the blend keeps slot 1's alpha where slot 1 has any, and the canvas
          // plane there holds image 2, so image 2's table must be absent from the support.
          if (copy && two && k == 0 && img2_any[b]) copy = false;
          for (int q = 0; q < n && empty; ++q)
            if (any_valid[size_t(q) * nb + b]) empty = false;
        }
      uint8_t& cls = cp.block_class[size_t(j) * cp.nfx + i];
      if (copy) {
        ++cp.copy_blocks;
        cls = kBlockCopy;
        for (int by = sy0; by <= sy1; ++by)
          for (int bx = sx0; bx <= sx1; ++bx) {
            const size_t b = size_t(by) * gx + bx;
            support_mark[b] = uint8_t(1 + k);
            for (int o = 0; o < n; ++o) {  // every image the slot's entries select (one, or two)
              if (!two && o != k) continue;
              cp.need_w[o] = std::max<uint32_t>(cp.need_w[o], uint32_t(max_sx[size_t(o) * nb + b]) + 1u);
              cp.need_h[o] = std::max<uint32_t>(cp.need_h[o], uint32_t(max_sy[size_t(o) * nb + b]) + 1u);
            }
          }
      } else if (empty) {
        ++cp.empty_blocks;
        cls = kBlockEmpty;
      } else {
        ++cp.pyramid_blocks;
        cp.pyramid_pixels += (long long)(x1 - x0) * (y1 - y0);
        cp.pyramid_block[size_t(j) * cp.nfx + i] = 1;
        cp.fine_list.push_back(uint32_t(i) | (uint32_t(j) << 16));
      }
    }

  // Level-1 tiles whose R^1 the pyramid blocks read (pyr_fine's 33 x 9 level-1 tile from
  // (bx0 / 2, by0 / 2), coordinates clamped to the level), and level-0 tiles whose G^l levels (or
  // kept level-0 pixels) pyr_fine and pyr_coarse read.
  const int lw1 = p.lw[1], lh1 = p.lh[1];
  const int ncx = (lw1 + t1 - 1) / t1, ncy = (lh1 + t1 - 1) / t1;
  const int ndx = (bw + td - 1) / td, ndy = (bh + td - 1) / td;
  cp.dense_coarse = (long long)ncx * ncy;
  cp.dense_down = (long long)ndx * ndy;
  std::vector<uint8_t> cmark(size_t(ncx) * ncy, 0), dmark(size_t(ndx) * ndy, 0);
  const auto mark_down = [&](int lx0, int ly0, int lx1, int ly1) {  // level-0 pixels, inclusive
    lx0 = std::max(lx0, 0);
    ly0 = std::max(ly0, 0);
    lx1 = std::min(lx1, bw - 1);
    ly1 = std::min(ly1, bh - 1);
    for (int ty = ly0 / td; ty <= ly1 / td; ++ty)
      for (int tx = lx0 / td; tx <= lx1 / td; ++tx) dmark[size_t(ty) * ndx + tx] = 1;
  };
  for (uint32_t f : cp.fine_list) {
    const int bx0 = cp.fx0 + 64 * int(f & 0xFFFFu), by0 = cp.fy0 + 16 * int(f >> 16);
    const int tx0 = bx0 >> 1, ty0 = by0 >> 1;
    const int tx1 = std::min(tx0 + 32, lw1 - 1), ty1 = std::min(ty0 + 8, lh1 - 1);
    for (int ty = ty0 / t1; ty <= ty1 / t1; ++ty)
      for (int tx = tx0 / t1; tx <= tx1 / t1; ++tx) cmark[size_t(ty) * ncx + tx] = 1;
    mark_down(2 * tx0, 2 * ty0, 2 * tx1 + 1, 2 * ty1 + 1);  // G^1 taps; the block's own pixels lie inside
  }
  for (int ty = 0; ty < ncy; ++ty)
    for (int tx = 0; tx < ncx; ++tx) {
      if (!cmark[size_t(ty) * ncx + tx]) continue;
      cp.coarse_list.push_back(uint32_t(tx) | (uint32_t(ty) << 16));
      // pyr_coarse's regions: the tile at level 1, then per level the tile's footprint plus the
      // upsample halo (the kernel's own recursion), as level-0 pixels.
      int ax = tx * t1, ay = ty * t1, bx = std::min(ax + t1, lw1), by = std::min(ay + t1, lh1);
      int f0x = ax << 1, f0y = ay << 1, f1x = bx << 1, f1y = by << 1;
      for (int l = 2; l < L; ++l) {
        ax >>= 1;
        ay >>= 1;
        bx = std::min(((bx - 1) >> 1) + 2, p.lw[l]);
        by = std::min(((by - 1) >> 1) + 2, p.lh[l]);
        f0x = std::min(f0x, ax << l);
        f0y = std::min(f0y, ay << l);
        f1x = std::max(f1x, bx << l);
        f1y = std::max(f1y, by << l);
      }
      mark_down(f0x, f0y, f1x - 1, f1y - 1);
    }
  // Down tiles that meet a pyramid block's pixels: pyr_fine reads their kept level-0 pixels.
  std::vector<uint8_t> keep0(size_t(ndx) * ndy, 0);
  for (uint32_t f : cp.fine_list) {
    const int i = int(f & 0xFFFFu), j = int(f >> 16);
    const int x0 = std::max(cp.fx0 + 64 * i, wx0), x1 = std::min(cp.fx0 + 64 * i + 64, wx1) - 1;
    const int y0 = std::max(cp.fy0 + 16 * j, wy0), y1 = std::min(cp.fy0 + 16 * j + 16, wy1) - 1;
    for (int ty = y0 / td; ty <= y1 / td; ++ty)
      for (int tx = x0 / td; tx <= x1 / td; ++tx) keep0[size_t(ty) * ndx + tx] = 1;
  }
  for (int ty = 0; ty < ndy; ++ty)
    for (int tx = 0; tx < ndx; ++tx) {
      if (!dmark[size_t(ty) * ndx + tx]) continue;
      cp.down_list.push_back(uint32_t(tx) | (uint32_t(ty) << 16) | (keep0[size_t(ty) * ndx + tx] ? 0x80000000u : 0u));
    }
  cp.support_mark = std::move(support_mark);
  cp.support_pitch = gx;
  cp.support_shift = L - 1;
  cp.usable = cp.copy_blocks + cp.empty_blocks > 0 && ndx < 0x8000 && ndy < 0x8000 && ncx < 0x8000 &&
              ncy < 0x8000 && cp.nfx < 0x8000 && cp.nfy < 0x8000;
}

}  // namespace hmp
