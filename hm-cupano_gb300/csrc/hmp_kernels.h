// hmp_kernels.h -- launch interface of the stitching kernels (host-visible).
#pragma once

#include <cuda_runtime.h>

#include "hmp_device.cuh"

namespace hmp {

// Canvas gather: every canvas pixel outside `skip` takes its gather-plane pixel.
struct GatherArgs {
  SrcSet S;
  PlaneDev P;  // canvas plane (entries resolved to offsets), rect = whole canvas
  CanvasDev C;
  int batch;
  int skip_x0, skip_y0, skip_x1, skip_y1;  // pixels written by the pyramid (end exclusive)
  int n_owners;  // images the plane can select (owners are < n_owners)
  // Per 256-pixel row segment [y][x / 256] (written with the resolved plane): kSegMixed if its
  // entries have several owners; else their one owner (0 if only fills), plus kSegFills if any
  // entry is a fill. A one-owner segment's entries are stored without the owner bits.
  const uint8_t* seg_owner;
  int seg_pitch;
  // Copy-block mode: every source pixel the gather reads inside [chk_x0, chk_x1) x [chk_y0, chk_y1)
  // (the blend region) must have alpha != 0 for the copy blocks to equal the pyramid; one with
  // alpha 0 sets *alpha_flag (nullptr: no check).
  int* alpha_flag;
  int chk_x0, chk_y0, chk_x1, chk_y1;
};
constexpr int kSegPixels = 256;
constexpr unsigned kSegFills = 8u, kSegMixed = 0xFFu;

// Shared by the Gaussian-pyramid (down) and blend/reconstruct (up) kernels.
struct PyrArgs {
  SrcSet S;
  PlaneDev slot[kDevMaxImages];
  int n;
  int levels;  // effective L >= 1
  int lw[kDevMaxLevels + 1];
  int lh[kDevMaxLevels + 1];
  void* G[kDevMaxImages][kDevMaxLevels];  // level l >= 1 of slot k: [batch][lh][lw] storage pixels
  const uint8_t* mask0;                   // level-0 weight value (two-image) or label, blend coords
  int mask0_pitch;
  const float* maskL[kDevMaxLevels];      // level l >= 1: [lh][lw][K]
  const uint8_t* hotL[kDevMaxLevels];     // N-way rule, level l >= 1: [lh][lw] mask class
  int K;
  int opaque;
  int tile;  // tile edge (level 0 for pyr_down, level 1 for pyr_coarse)
  float4* R1;  // level-1 reconstruction [batch][lh1][lw1] (levels >= 2)
  float4* Rl[kDevMaxLevels];  // Binomial5 filter: reconstruction R^l, l = 1..L-1, [batch][lh][lw]
  // Level-0 pixels of each slot over its plane rect, [batch][P.h][P.w] RGBA8, written by pyr_down
  // and read by pyr_fine (when use_p0; levels >= 2 with the box filter).
  uint32_t* P0[kDevMaxImages];
  int use_p0;
  int slots_cap;  // N-way pyr_down: shared memory holds this many slots (the most any tile has)
  // pyr_down's dynamic shared memory is at least this many bytes (0: what it needs). Reserving
  // more caps how many of its CTAs share an SM, which shapes how it packs beside the gather.
  int down_smem_floor;
  int coarse_cap; // N-way pyr_coarse: likewise, per coarse tile
  int fine_cap;   // N-way pyr_fine: likewise, per 64 x 16 level-0 block (with its upsample halo)
  int pdl;        // launch pyr_coarse / pyr_fine as programmatic dependents of the kernel before them
  // Work list of the launch (copy-block mode): entry blockIdx.x is the CTA's tile, tx | ty << 16;
  // in pyr_down's list bit 31 marks the tiles whose kept level-0 pixels pyr_fine reads.
  // nullptr: the dense grid.
  const uint32_t* tiles;
  int list_frames;  // listed launches: grid.x = entries x list_frames, frame = blockIdx.x % list_frames
  // Copy-block mode, pyr_fine: a level-0 pixel whose block of 2^sm_shift pixels is marked in
  // support_mark ([.][sm_pitch], blend coordinates) lies in a copy block's reconstruction support;
  // alpha 0 of its label image's pixel there sets *alpha_flag.
  int* alpha_flag;
  const uint8_t* support_mark;
  int sm_pitch, sm_shift;
  // Fallback launches: every CTA returns at once unless gate[0] != 0 (a copy block's source pixels
  // held alpha 0, so the whole write rect is recomputed); then the launch's CTAs walk the dense
  // grid of fb_nx x fb_ny tiles of fb_batch frames with a grid stride, and the last CTA of the
  // last fallback launch (pyr_fine's) to finish clears gate[0] (gate[1] counts them), so the flag
  // is 0 again when the next call's kernels start. nullptr: no gate.
  int* gate;
  int fb_nx, fb_ny, fb_batch;
  CanvasDev C;
  int wx0, wy0, wx1, wy1;  // write rect, blend coordinates, end exclusive
  int cx_off, cy_off;      // canvas = blend + offset
  int tx0, ty0;            // first up-tile index
};

// Pyramid dump (two-image box filter): the levels the fused kernels keep on chip, materialised
// as float4 [batch][lh][lw] buffers by plain kernels that use the same device functions.
cudaError_t launch_dump_level0(const PyrArgs& a, int k, float4* out, int batch, cudaStream_t stream);
cudaError_t launch_dump_widen(const void* level, int storage, long long n, float4* out, cudaStream_t stream);
cudaError_t launch_dump_lap(const float4* hi, int hw, int hh, const float4* lo, int lw, int lh, float4* lap, int batch,
                            cudaStream_t stream);
cudaError_t launch_dump_blend2(const float4* l0, const float4* l1, const float* m, const uint8_t* m0, int m0_pitch, int w,
                               int h, float4* out, int batch, cudaStream_t stream);
cudaError_t launch_dump_recon(const float4* lo, int lw, int lh, const float4* bl, int w, int h, float4* out, int batch,
                              cudaStream_t stream);

// Level-by-level stitch of the uchar3 / float4 / float3 pipelines (hmp_generic.cu).
struct GenArgs {
  SrcSet S;  // frames; ptr is the first pixel of any sample type
  PlaneDev slot[kDevMaxImages];
  int n;
  int levels;
  int lw[kDevMaxLevels + 1];
  int lh[kDevMaxLevels + 1];
  float4* G[kDevMaxImages][kDevMaxLevels];  // level l of slot k (level 0 included), [batch][lh][lw]
  const uint8_t* mask0;
  int mask0_pitch;
  const float* maskL[kDevMaxLevels];
  int K;
  int opaque;
  CanvasDev C;             // ptr is the first pixel of any sample type
  int wx0, wy0, wx1, wy1;  // write rect, blend coordinates, end exclusive
  int cx_off, cy_off;      // canvas = blend + offset
};
// r[0], r[1]: reconstruction buffers of level-1 size (levels alternate between them).
cudaError_t launch_generic_pyramid(const GenArgs& a, int channels, bool is_float, int rule, int batch,
                                   float4* const* r, cudaStream_t stream);
// The canvas outside g's skip rect from the raw (packed) canvas plane g.P.
cudaError_t launch_generic_canvas(const GatherArgs& g, int channels, bool is_float, bool opaque, cudaStream_t stream);
int generic_launches(int levels, bool canvas);

// One-time attribute setup (dynamic shared memory limits). Call before capture.
cudaError_t kernels_init();
// Copy-block fallback (hmp_fallback.cu): one single-thread launch after the frame's other kernels;
// when the alpha flag (a.gate[0]) is set it clears it and tail-launches the dense pyramid chain
// over the given dense grids. fallback_init sets the shared-memory limits of its kernels.
cudaError_t fallback_init();
cudaError_t launch_fallback_gate(const PyrArgs& a, int rule, int storage, int tile_down, int tile_coarse, dim3 down,
                                 dim3 coarse, dim3 fine, size_t coarse_smem, cudaStream_t stream);

// Resolves a plane's packed entries (raw.map) into offsets for the frames S (res: raw's layout).
// opaque: the soft-seam rule for entries outside their source.
// Also writes seg_owner (see GatherArgs) for the plane's 256-pixel row segments.
// Copy-block mode: canvas pixels inside `wr` whose 64 x 16 block (grid origin x0, y0, nx x ny
// blocks, one byte each at map[by * pitch + bx]) is marked resolve to kOffSkip. map nullptr: none.
struct SkipMap {
  const uint8_t* map;
  int pitch, x0, y0, nx, ny;
  int wr_x0, wr_y0, wr_x1, wr_y1;  // canvas coordinates, end exclusive
};
cudaError_t launch_resolve_plane(const PlaneDev& raw, uint32_t* res, uint8_t* seg_owner, int seg_pitch, const SrcSet& S,
                                 int n, bool opaque, const SkipMap& skip, cudaStream_t stream);

// copy_blocks: the plane holds copy-block skips (kOffSkip) or the call checks source alpha.
cudaError_t launch_canvas_gather(const GatherArgs& a, bool copy_blocks, cudaStream_t stream);

// Gaussian levels 1..L-1 of every slot; grid = tiles over the blend region x batch.
cudaError_t launch_pyr_down(const PyrArgs& a, int storage, dim3 grid, cudaStream_t stream);

// R^1 over the level-1 tiles the write rect needs; grid = level-1 tiles x batch (levels >= 2).
cudaError_t launch_pyr_coarse(const PyrArgs& a, int rule, int storage, dim3 grid, size_t smem, cudaStream_t stream);

// Level 0 of the write rect: blend + reconstruct + pack; grid = 64 x 16 pixel blocks x batch.
cudaError_t launch_pyr_fine(const PyrArgs& a, int rule, int storage, dim3 grid, cudaStream_t stream);

// Binomial5 filter: the whole pyramid (levels >= 2) as a level-by-level chain of launches.
cudaError_t launch_b5_pyramid(const PyrArgs& a, int rule, int storage, int batch, cudaStream_t stream);
int b5_launches(int levels);

size_t pyr_down_smem(int n, int tile);
// Dynamic shared memory per CTA that leaves room for at most `ctas_per_sm` CTAs on an SM of the
// current device (1 KB of it reserved per CTA); 0 for no cap.
size_t residency_smem(int ctas_per_sm);
// Shared memory of a pyr_coarse CTA (levels 2..L-1 of its tile with halos).
size_t pyr_coarse_smem(int n, int k, int tile1, int levels, int storage);

}  // namespace hmp
