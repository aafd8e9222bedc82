/*
 * hmp_oracle.h -- CPU restatement of hm-cupano's per-frame stitching path.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker for the CUDA path:
 * only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg may
 * load it. The product (libhmpano) never links, loads or calls it.
 *
 * It restates, step by step and with materialised buffers, what the
 * reference does per frame:
 *   - remap kernels            src/cuda/cudaRemap.cu:60-294
 *   - make-full / ROI copy     src/cuda/cudaMakeFull.cu:40-69, 173-258
 *   - uint8 pack (truncating)  src/cuda/cudaUtils.cuh:18-28, 118-127
 *   - 2-image pyramid blend    src/cuda/cudaBlend.cu:46-672, 847-1049
 *   - 3-image pyramid blend    src/cuda/cudaBlend3.cu:220-627, 881-1206
 *   - N-image pyramid blend    src/cuda/cudaBlendN.cu:19-447, 649-828
 *   - stitcher orchestration   src/pano/cudaPano.inl:167-418,
 *                              src/pano/cudaPanoN.inl:489-685,
 *                              src/pano/cudaPano3_optimized.inl:19-140
 *   - geometry                 src/pano/canvasManager.cpp:16-101,
 *                              src/pano/cudaPanoN.inl:20-105, 156-190
 * Operation order follows the reference (and its Python port cupano/ops.py)
 * so that the float build reproduces the reference's FP32 results bit for bit
 * where the reference is deterministic. The double build is the FP64 oracle.
 *
 * Parity pin: the float build is checked against golden vectors produced by
 * the reference's own Python implementation (tests/golden/make_golden.py).
 */
#ifndef HMP_ORACLE_H
#define HMP_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Stitcher kinds (which reference class is restated). */
#define HMPO_KIND_PANON 1 /* CudaStitchPanoN  (src/pano/cudaPanoN.h) */
#define HMPO_KIND_PANO2 2 /* CudaStitchPano   (src/pano/cudaPano.h)  */
#define HMPO_KIND_PANO3 3 /* CudaStitchPano3  (src/pano/cudaPano3.h) */

/* Filters. */
#define HMPO_FILTER_REFBOX 0    /* the reference's 2x2 box / bilinear pyramid */
#define HMPO_FILTER_BINOMIAL5 1 /* 5-tap [1,4,6,4,1]/16, reflect-101 (no reference code) */

/* Error codes (negative). */
#define HMPO_OK 0
#define HMPO_EINVAL -1
#define HMPO_ENOMEM -2
#define HMPO_EGEOM -3

typedef struct hmpo_config {
  int kind;           /* HMPO_KIND_* */
  int n_images;       /* 2 for PANO2, 3 for PANO3, 2..8 for PANON */
  int num_levels;     /* 0 = hard seam */
  int batch;          /* frames per call */
  int minimize_blend; /* PANO2 / PANON */
  int fused3;         /* PANO3: 1 = fused remap (default in the reference), 0 = legacy */
  int filter;         /* HMPO_FILTER_* (Binomial5 is only meaningful for the f64 build) */
  const uint16_t* const* map_x; /* per image, row-major map_h x map_w */
  const uint16_t* const* map_y;
  const int* map_w;
  const int* map_h;
  const int* pos_x; /* normalised canvas positions */
  const int* pos_y;
  const uint8_t* seam; /* PANO2: inverted seam (1 = image 1); PANO3/PANON: labels */
  int seam_w;
  int seam_h;
  int channels; /* pixel channels of frames and canvas: 4 (RGBA; 0 means 4) or 3 (RGB, box filter only) */
} hmpo_config;

/* Canvas size = max(pos + map size) (src/pano/controlMasks.cpp:265-271). */
int hmpo_canvas_size(const hmpo_config* cfg, int* width, int* height);

/* Geometry of the soft-seam path: blend region and write ROI in canvas
 * coordinates, and the effective level count. out[0..3] = blend x,y,w,h;
 * out[4..7] = write x,y,w,h; out[8] = effective levels. */
int hmpo_blend_geometry(const hmpo_config* cfg, int* out9);

/* Full stitch. inputs[i]: RGBA8, batch frames contiguous, in_w[i] x in_h[i].
 * canvas: RGBA8, batch frames contiguous, canvas_size(). */
int hmpo_stitch_f32(const hmpo_config* cfg, const uint8_t* const* inputs, const int* in_w, const int* in_h,
                    uint8_t* canvas);
int hmpo_stitch_f64(const hmpo_config* cfg, const uint8_t* const* inputs, const int* in_w, const int* in_h,
                    uint8_t* canvas);
/* Same, but returns the pre-pack blend result of the write ROI (float RGBA)
 * for error analysis in fractional LSBs (soft-seam only). */
int hmpo_stitch_f64_unpacked(const hmpo_config* cfg, const uint8_t* const* inputs, const int* in_w,
                             const int* in_h, double* roi_out);

/* Single pyramid operations (float build), for pinning against the
 * reference's op-level known-answer tests. Images are RGBA float, batch 1. */
void hmpo_downsample_rgba_f32(const float* in, int iw, int ih, float* out);
void hmpo_laplacian_rgba_f32(const float* high, int hw, int hh, const float* low, float* lap);
void hmpo_reconstruct_rgba_f32(const float* low, const float* lap, int hw, int hh, float* out);
void hmpo_downsample_mask_f32(const float* in, int iw, int ih, int k, float* out);
/* Level-wise N-way blend with a K=n mask (cudaBlendN.cu:199-288). */
void hmpo_blend_nway_f32(const float* const* laps, int n, const float* mask, int w, int h, float* out);
/* Two-image blend of one level (src/cuda/cudaBlend.cu:520-576), mask = weight of image 1. */
void hmpo_blend_two_f32(const float* l1, const float* l2, const float* mask, int w, int h, float* out);
/* Full Laplacian blend of n full buffers (rule: 2 = two-image, 3 = three-image, 1 = N-way). */
int hmpo_laplacian_blend_f32(const float* const* inputs, int n, const float* mask, int k, int w, int h, int levels,
                             int rule, float* out);
/* The same with the arithmetic of 3 (RGB, no alpha) or 4 (RGBA) channels; buffers hold 4 floats
 * per pixel either way (the fourth is ignored for 3). */
int hmpo_laplacian_blend_ch_f32(const float* const* inputs, int n, const float* mask, int k, int w, int h,
                                int levels, int rule, int channels, float* out);

/* Threads used by the OpenMP loops (0 = library default). */
void hmpo_set_threads(int n);
int hmpo_get_threads(void);

/* Frame stabiliser (src/cuda/cudaStabilize.cu; hmp_stabilize_oracle.c). Grayscale float frames,
 * w x h contiguous. gx, gy, resp: w*h scratch / output (the Harris response, 0 on the border).
 * hmpo_stab_corners returns the number of corners and writes the first `cap` as (x, y) pairs. */
void hmpo_stab_harris(const float* img, int w, int h, float k, float* gx, float* gy, float* resp);
int hmpo_stab_corners(const float* resp, int w, int h, float threshold, int* xy, int cap);
void hmpo_stab_flow(const float* prev, const float* next, const int* xy, int n, int w, int h, int window,
                    float* flow);
void hmpo_stab_mean(const float* flow, int n, float* dx, float* dy);
void hmpo_stab_warp(const float* in, int w, int h, float dx, float dy, float* out);

#ifdef __cplusplus
}
#endif

#endif
