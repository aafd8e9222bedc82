/*
 * hmpano.h -- C ABI of the GB300-native stitching path (libhmpano.so).
 *
 * This is the boundary a host program binds to (ctypes, cgo, JNI, N-API or plain C/C++). It
 * replaces the per-frame stitcher objects of hm-cupano:
 *
 *   hmp_stitcher_create   <- hm::pano::cuda::CudaStitchPano<T,T>::CudaStitchPano(batch, levels,
 *                            masks, quiet, minimize_blend)          src/pano/cudaPano.h:71-77
 *                            CudaStitchPano3(batch, levels, masks)   src/pano/cudaPano3.h:70-75
 *                            CudaStitchPanoN(batch, levels, masks, minimize_blend)
 *                                                                    src/pano/cudaPanoN.h:83-88
 *   hmp_stitcher_process  <- CudaStitchPano::process(in1, in2, stream, canvas)
 *                                                                    src/pano/cudaPano.h:95-99
 *                            CudaStitchPano3::process(in0, in1, in2, stream, canvas, fused)
 *                                                                    src/pano/cudaPano3.h:99-107
 *                            CudaStitchPanoN::process(inputs, stream, canvas)
 *                                                                    src/pano/cudaPanoN.h:97-101
 *   hmp_stitcher_status   <- CudaStitchPano*::status()               src/pano/cudaPano.h:91-93
 *   hmp_stitcher_canvas_* <- canvas_width() / canvas_height()        src/pano/cudaPano.h:79-85
 *   hmp_stitcher_dump_pyramid <- CudaStitchPano::dump_soft_blend_pyramid(directory, stream)
 *                                                                    src/pano/cudaPano.h:101
 *   hmp_stitcher_destroy  <- ~CudaStitchPano*()
 *   hmp_control_dir_load  <- ControlMasks::load / ControlMasks3::load / ControlMasksN::load
 *                            src/pano/controlMasks.cpp:133-326, controlMasks3.cpp:186-300,
 *                            controlMasksN.cpp:22-193
 *   hmp_stabilizer_*      <- the frame stabiliser src/cuda/cudaStabilize.cu: harrisCornerDetection
 *                            (:157-204), computeOpticalFlow (:210-238), stabilizeFrame (:243-267)
 *   hmp_batch_*, hmp_server_*, hmp_blend2_noalloc: no counterpart (the reference stitches one
 *                            configuration per process, one call at a time, and every blend it
 *                            offers allocates its own device buffers)
 *
 * Error convention (src/cuda/cudaStatus.h:12-75): every call returns an hmp_status whose code is
 * a cudaError_t value (0 = success) with a message. Construction errors are also kept as the
 * stitcher's sticky status; process() first returns the sticky status, then the per-call error,
 * and a per-call error becomes sticky (src/pano/cudaPano.inl:460-472).
 *
 * Data: images are RGBA8 (uchar4) unless hmp_config.channels / pixel_format select uchar3, float4
 * or float3; device memory, frame b of a batch at data + b*pitch*height.
 * Remap tables, positions and the seam are host data consumed at create time (the ControlMasks
 * of the reference, already loaded: the two-image seam is in its inverted form, 1 = image 1;
 * the three/N-image seam holds labels 0..n-1). Positions are normalised (minimum 0).
 *
 * All device memory a stitcher needs is allocated by hmp_stitcher_create; process() allocates
 * nothing, so it can be captured in a CUDA graph. One process() may be in flight per stitcher.
 */
#ifndef HMPANO_H
#define HMPANO_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define HMP_API __attribute__((visibility("default")))
#else
#define HMP_API
#endif

/* Stitcher kinds. */
#define HMP_KIND_PANON 1 /* CudaStitchPanoN: 2..8 images, N-way blend */
#define HMP_KIND_PANO2 2 /* CudaStitchPano: 2 images, two-image blend */
#define HMP_KIND_PANO3 3 /* CudaStitchPano3: 3 images, three-way blend */

/* Pyramid storage precision for levels >= 1 (arithmetic is always FP32). */
#define HMP_STORAGE_F32 0
#define HMP_STORAGE_F16 1

/* Pyramid filter. */
#define HMP_FILTER_REFBOX 0    /* the reference's 2x2 box downsample / bilinear upsample */
#define HMP_FILTER_BINOMIAL5 1 /* 5-tap [1,4,6,4,1]/16, reflect-101 (no reference counterpart) */

/* Status codes are cudaError_t values; these are the ones the library produces itself. */
#define HMP_OK 0
#define HMP_ERR_INVALID_VALUE 1        /* cudaErrorInvalidValue */
#define HMP_ERR_MEMORY_ALLOCATION 2    /* cudaErrorMemoryAllocation */
#define HMP_ERR_INVALID_DEVICE_POINTER 17 /* cudaErrorInvalidDevicePointer */
#define HMP_ERR_FILE_NOT_FOUND 301     /* cudaErrorFileNotFound: masks not loaded (cudaPano.inl:28-31) */
#define HMP_ERR_NOT_SUPPORTED 801      /* cudaErrorNotSupported */
#define HMP_ERR_TIMEOUT 909            /* cudaErrorTimeout: a bounded wait gave up */
#define HMP_ERR_UNKNOWN 999            /* cudaErrorUnknown: a file or directory could not be written */

typedef struct hmp_status {
  int code;          /* cudaError_t value, 0 = success */
  char message[252]; /* NUL-terminated */
} hmp_status;

typedef struct hmp_remap {
  const uint16_t* map_x; /* host, row-major height x width, CV_16U; 65535 = unmapped */
  const uint16_t* map_y;
  int width;
  int height;
  int xpos; /* canvas position of the table's top-left corner */
  int ypos;
} hmp_remap;

typedef struct hmp_config {
  int kind;           /* HMP_KIND_* */
  int n_images;       /* 2 (PANO2), 3 (PANO3), 2..8 (PANON) */
  int num_levels;     /* 0 = hard seam; pyramid levels otherwise */
  int batch_size;     /* frames per process() call, 1..65536 */
  int channels;       /* 4 (RGBA) or 3 (RGB) */
  int minimize_blend; /* PANO2 / PANON: blend only the seam region (reference default: 1) */
  int fused;          /* PANO3: 1 = fused remap (reference default), 0 = legacy remap+copy */
  int storage;        /* HMP_STORAGE_* */
  int filter;         /* HMP_FILTER_* */
  const hmp_remap* remaps; /* n_images entries */
  const uint8_t* seam;     /* host, seam_height x seam_width */
  int seam_width;
  int seam_height;
  int pixel_format;   /* HMP_PIXEL_U8 (default) or HMP_PIXEL_F32: the frames' and canvas's sample type */
} hmp_config;

/* Pixel sample types (the reference's CudaStitchPano<T_pipeline, T_compute> pipelines): uchar4 /
 * uchar3 (HMP_PIXEL_U8, canvas packed by truncation) and float4 / float3 (HMP_PIXEL_F32, canvas
 * stores the reconstruction as is). uchar4 runs the fused per-frame kernels; the other three run
 * level-by-level kernels with the same arithmetic (3-channel pixels have no alpha: plain means,
 * plain bilinear upsampling, blends without alpha tests). */
#define HMP_PIXEL_U8 0
#define HMP_PIXEL_F32 1

typedef struct hmp_image {
  void* data; /* device pointer to pixels of the stitcher's type (RGBA8 unless configured otherwise) */
  int width;
  int height;
  size_t pitch; /* bytes per row (>= pixel size * width); frame stride = pitch*height */
} hmp_image;

typedef struct hmp_stitcher hmp_stitcher;

/* Geometry and cost model of a stitcher (for reports and tests). Rectangles are x, y, w, h in
 * canvas pixels. */
typedef struct hmp_stitcher_info {
  int canvas_width;
  int canvas_height;
  int batch_size;
  int n_images;
  int levels;        /* effective pyramid levels (0 = hard seam) */
  int blend_rect[4]; /* pyramid domain */
  int write_rect[4]; /* region the pyramid writes back to the canvas */
  int tile_down;     /* level-0 tile edge of the Gaussian-pyramid kernel */
  int tile_coarse;   /* level-1 tile edge of the coarse reconstruction kernel */
  int launches_per_process; /* kernels one process() launches */
  double m0_bytes;   /* compulsory bytes per frame (maps, seam, sources, canvas) */
  double device_bytes; /* device memory held by the stitcher */
  /* Copy blocks (three- and N-image box pyramids; see hmp_stitcher_set_copy_blocks): 1 if they
   * are planned and switched on; the write rect's 64 x 16 blocks the canvas gather copies (one
   * image's pixels) or zeroes, and those the pyramid computes; the pyramid kernels' work-list
   * lengths (down tiles, coarse tiles, fine blocks). */
  int copy_mode;
  int copy_blocks;
  int empty_blocks;
  int pyramid_blocks;
  int pyramid_tiles[3];
  double gather_pixels; /* canvas pixels the canvas gather writes per frame */
} hmp_stitcher_info;

/* ---- Control directory (host only; no GPU needed) ----
 * Replaces ControlMasks::load / ControlMasks3::load / ControlMasksN::load
 * (src/pano/controlMasks.cpp:133-326, src/pano/controlMasks3.cpp:186-300,
 * src/pano/controlMasksN.cpp:22-193): reads mapping_000i_x.tif / mapping_000i_y.tif (16-bit
 * coordinate tables; uncompressed, LZW, Deflate or PackBits, strips or tiles), the XPosition /
 * YPosition x resolution tags of mapping_000i.tif (normalised so that the smallest is 0) and
 * seam_file.png (8-bit palette indices, else grayscale). The seam is processed as the reference
 * does for `kind`: two images -> smallest value 1 (weight of image 1), largest 0; three images ->
 * an 8-bit paletted seam with labels exactly 0, 1, 2; N images -> exactly n_images distinct values
 * remapped to 0..n_images-1. Errors: HMP_ERR_FILE_NOT_FOUND for a missing file,
 * HMP_ERR_NOT_SUPPORTED for an unsupported encoding, HMP_ERR_INVALID_VALUE otherwise. */
typedef struct hmp_control_dir {
  int kind;                  /* HMP_KIND_* the seam was processed for */
  int n;                     /* images */
  int map_width[8], map_height[8];
  const uint16_t* map_x[8];  /* [map_height][map_width] source column, 65535 = unmapped */
  const uint16_t* map_y[8];  /* source row */
  float xpos[8], ypos[8];    /* canvas position of each table */
  int seam_width, seam_height;
  const uint8_t* seam;       /* [seam_height][seam_width] */
  void* internal;            /* owner of the arrays */
} hmp_control_dir;

/* n_images is used for HMP_KIND_PANON (2 and 3 are implied by the other kinds). */
HMP_API hmp_status hmp_control_dir_load(const char* directory, int kind, int n_images, hmp_control_dir** out);
HMP_API void hmp_control_dir_free(hmp_control_dir* dir);

/* The loader's decoders on their own: a seam PNG (palette indices if 8-bit paletted, else
 * grayscale) and a single-channel 16-bit TIFF. With out == NULL only the size is returned;
 * otherwise out must hold width * height samples (`capacity`). */
HMP_API hmp_status hmp_read_seam_png(const char* path, int* width, int* height, int* paletted, uint8_t* out,
                                     size_t capacity);
HMP_API hmp_status hmp_read_tiff_u16(const char* path, int* width, int* height, uint16_t* out, size_t capacity);

/* Library version string. */
HMP_API const char* hmp_version(void);

/* Construct a stitcher: validates the configuration, plans the per-pixel gather tables and
 * allocates every device buffer. On failure *out is still set (unless NULL) to a stitcher
 * object carrying the sticky error status, like the reference's constructors; pass it to
 * hmp_stitcher_destroy. */
HMP_API hmp_status hmp_stitcher_create(const hmp_config* cfg, hmp_stitcher** out);

/* Alpha-aware Laplacian of one pyramid level, as the stitchers form it: out = high minus the
 * bilinear upsample of low over its taps with alpha != 0 (renormalised), in colour, and high's
 * alpha (cupano/ops.py compute_laplacian; src/cuda/cudaBlend.cu:356-456). Float RGBA levels on the
 * device, [batch][h][w][4], 16-byte aligned; low is the next level (at most high's size). */
HMP_API hmp_status hmp_laplacian_rgba(const float* high, int high_w, int high_h, const float* low, int low_w,
                                      int low_h, float* out, int batch, void* stream);

/* For tests of the construction-error path (no counterpart in the reference, whose construct
 * errors come from cudaMalloc itself, src/pano/cudaPano.inl:28-31): the k-th device allocation a
 * stitcher makes from now on (any stitcher of the process, counting from 1) fails with
 * HMP_ERR_MEMORY_ALLOCATION without allocating; 0 switches it off. hmp_debug_allocation_count()
 * returns how many device allocations stitchers have made so far (injected failures included). */
HMP_API void hmp_debug_fail_allocation(long long k);
HMP_API long long hmp_debug_allocation_count(void);

HMP_API void hmp_stitcher_destroy(hmp_stitcher* st);

/* Sticky status (construction error or the first failed process()). */
HMP_API hmp_status hmp_stitcher_status(const hmp_stitcher* st);

HMP_API int hmp_stitcher_canvas_width(const hmp_stitcher* st);
HMP_API int hmp_stitcher_canvas_height(const hmp_stitcher* st);
HMP_API int hmp_stitcher_batch_size(const hmp_stitcher* st);
HMP_API hmp_status hmp_stitcher_get_info(const hmp_stitcher* st, hmp_stitcher_info* info);

/* Stitch one batch: inputs[0..n_inputs) -> canvas, enqueued on `stream` (a cudaStream_t; NULL =
 * legacy default stream). Every canvas pixel is written, so the canvas needs no clearing. */
HMP_API hmp_status hmp_stitcher_process(hmp_stitcher* st, const hmp_image* inputs, int n_inputs,
                                        const hmp_image* canvas, void* stream);

/* Replaces CudaStitchPano::dump_soft_blend_pyramid(directory, stream) (src/pano/cudaPano.h:101,
 * src/pano/cudaPano.inl:420-458): synchronises `stream`, then writes the soft-blend pyramid of the
 * last process() under `directory`: metadata.txt (num_levels, batch_size, channels, level_<l>=WxH)
 * and float32 TIFF files gauss1, gauss2, lap1, lap2, blend, reconstruct
 * `<label>/level_<l>_batch_<b>.tiff` (RGBA) and `mask/level_<l>.tiff` (weight of image 1). The
 * per-frame kernels keep these levels on chip, so the dump recomputes them from the last call's
 * frames, which must still hold their contents. Two-image stitchers with the reference box filter;
 * HMP_ERR_INVALID_VALUE when num_levels is 0 or no frame was processed yet, HMP_ERR_UNKNOWN when a
 * file cannot be written. A debugging call: it allocates and synchronises. */
HMP_API hmp_status hmp_stitcher_dump_pyramid(hmp_stitcher* st, const char* directory, void* stream);

/* Tile edges of the pyramid kernels (a tuning knob, results are identical for every choice):
 * tile_down 32 or 64 level-0 pixels (a multiple of 2^(levels-1)), tile_coarse 32 level-1
 * pixels. Takes effect from the next process(); no counterpart in the reference. */
HMP_API hmp_status hmp_stitcher_set_tiles(hmp_stitcher* st, int tile_down, int tile_coarse);

/* Per-kernel device time of process() calls made while timing is enabled, measured with CUDA
 * events recorded on the stream each kernel is launched on (the pyramid kernels run on the
 * stitcher's auxiliary stream). Index 0 = canvas_gather, 1 = pyr_down, 2 = pyr_coarse,
 * 3 = pyr_fine; with the Binomial5 filter index 1 holds its whole pyramid chain. */
typedef struct hmp_kernel_timing {
  double total_ms[4];
  long long launches[4];
} hmp_kernel_timing;

/* Caps the Gaussian-pyramid kernel at ctas_per_sm CTAs per SM (0 = no cap) by reserving shared
 * memory for it. Tuning only (every setting gives the same bits): with the pyramid running beside
 * the canvas gather, how its few CTAs spread over the SMs changes the frame time. The default is 4
 * for two-image stitchers with 64-pixel down tiles, else 0; hmp_stitcher_set_tiles restores it.
 * No counterpart in the reference. */
HMP_API hmp_status hmp_stitcher_set_down_residency(hmp_stitcher* st, int ctas_per_sm);

/* Copy blocks: on (1, the default), off (0), or on for frames the caller promises are opaque (2).
 * No counterpart in the reference.
 * Three-image and N-image blend regions cover most of the canvas, but wherever the seam mask is
 * one image's at every level of a pixel's reconstruction and that image is valid there, the
 * pyramid's result is that image's pixel exactly (the box filter and bilinear upsample keep every
 * value a short dyadic fraction, so FP32 rounds nothing). The stitcher plans such 64 x 16 blocks
 * of the write rect at construction; per call the canvas gather copies them and the pyramid runs
 * over the remaining blocks and the tiles their reconstruction reads. Two conditions are checked
 * per call, and the full pyramid runs when either fails: the frames must contain every table
 * entry the copy blocks read (host check), and every source pixel behind a copy block must have
 * alpha != 0 (device check; a failure runs the whole write rect through the pyramid, launched
 * from one single-thread kernel that otherwise returns at once, or under stream capture from three
 * gated launches). Results are identical either way; off forces the full pyramid every call.
 * Applies to RGBA8 stitchers with the box filter and two or more levels: 3..8 images, and two
 * images whose minimised blend strip lines up with the canvas. Mode 2 drops the device check and
 * its fallback (one launch fewer per call): for frames whose source pixels all have alpha != 0
 * (camera and video frames, alpha 255); a source pixel with alpha 0 behind a copy block then gives
 * that block the source pixel where the reference's pyramid would blend it out. */
HMP_API hmp_status hmp_stitcher_set_copy_blocks(hmp_stitcher* st, int enable);

/* Enable (1) or disable (0) per-kernel event timing; enabling clears the accumulated times.
 * Mode 2 also serialises the kernels on the caller stream (no concurrent pyramid stream), so that
 * each kernel's time is its time alone. At most 4096 process() calls are recorded between two
 * hmp_stitcher_get_timing() calls. */
HMP_API hmp_status hmp_stitcher_set_timing(hmp_stitcher* st, int enable);

/* Accumulated kernel times since timing was enabled or last read; waits for the recorded
 * events, then resets the accumulators. No counterpart in the reference (its benchmark times
 * whole frames with a host clock, tests/testCudaBlend.cpp:224-241). */
HMP_API hmp_status hmp_stitcher_get_timing(hmp_stitcher* st, hmp_kernel_timing* out);

/* Size of the static device array hmp_blend2_noalloc works in: 48 MiB, about 2.3 million pixels
 * per frame at batch 1 (e.g. 1920 x 1080). */
#define HMP_NOALLOC_SCRATCH_BYTES (48u * 1024u * 1024u)

/* Two-image Laplacian pyramid blend that allocates no device memory. No counterpart in the
 * reference.
 *
 * For callers that cannot call cudaMalloc, and so cannot create a stitcher: a plugin inside a
 * host application that owns all device memory through its own pool (a raw cudaMalloc escapes
 * the host's budget and accounting), or code on a real-time frame path, where cudaMalloc and
 * cudaFree may synchronise the device and stall every stream. The caller passes the inputs and
 * the output; every intermediate lives in one file-scope device array of
 * HMP_NOALLOC_SCRATCH_BYTES, which every GPU that loads the library holds until the process exits.
 * The call allocates nothing (no cudaMalloc, cudaFree or allocating library routine).
 *
 * image1, image2: already-remapped RGBA8 frames of the same size (device, batch_size frames each
 * at data + b*pitch*height); seam: device, height rows of seam_pitch bytes, 1 = image 1, 0 =
 * image 2 (the two-image seam in its inverted form). Seam bytes must be exactly 0 or 1: the seam
 * is device data, so it is not checked, and any other value (a 0/255 mask, say) gives an
 * undefined blend, as it does in a stitcher. out: same size as the images. The result
 * equals hmp_stitcher_process of a two-image stitcher whose tables are the identity, with both
 * images at (0, 0) and minimize_blend = 0. Work is enqueued on `stream`.
 *
 * batch_size is 1..65536. Sizes whose scratch exceeds HMP_NOALLOC_SCRATCH_BYTES are rejected with
 * HMP_ERR_INVALID_VALUE and a message giving the bytes needed. The first call on a device does the
 * set-up (it looks up the array's device address and sets kernel attributes), so make it before
 * any stream capture.
 * Every call shares the one array, which keeps the last call's contents; calls whose work
 * overlaps on the GPU (other streams, other host threads) race on it and must be serialised. */
HMP_API hmp_status hmp_blend2_noalloc(const hmp_image* image1, const hmp_image* image2, const uint8_t* seam,
                                      size_t seam_pitch, int num_levels, int batch_size, const hmp_image* out,
                                      void* stream);

/* ---- Stitch server: continuous batching of requests for many pano configurations. ----
 * No counterpart in the reference (it stitches one configuration per process). Configurations are
 * registered once (host tables copied); requests (configuration, device inputs, device canvas)
 * are submitted from any thread and run as soon as one of `slots` streams and a resident stitcher
 * of their configuration are free, so requests that arrive while others run overlap on the GPU.
 * Stitchers stay resident (tables, seam, pyramid scratch) within `hbm_budget_bytes`; idle ones are
 * evicted least-recently-used when a new one does not fit. Inputs and canvas must stay valid until
 * the request finishes (hmp_server_wait / hmp_server_drain). */
typedef struct hmp_server hmp_server;

typedef struct hmp_server_options {
  size_t hbm_budget_bytes;      /* device bytes resident stitchers may hold together */
  int slots;                    /* streams (1..64): each runs one request and queues the next */
  int max_instances_per_config; /* resident stitchers per configuration (one request each at a time) */
} hmp_server_options;

typedef struct hmp_server_stats {
  long long submitted, completed, failed;
  long long instances_created, instances_evicted;
  int max_in_flight;
  double p50_ms, p99_ms, mean_ms, max_ms; /* latency: observed completion - submission (host clock) */
  double span_ms;                         /* first submission to last completion */
  double canvas_mpix;                     /* canvas megapixels completed (frames x canvas) */
  double resident_bytes, resident_bytes_peak;
} hmp_server_stats;

HMP_API hmp_status hmp_server_create(const hmp_server_options* options, hmp_server** out);
/* Finishes every submitted request, then releases the server's streams and stitchers. */
HMP_API void hmp_server_destroy(hmp_server* server);
/* Register a configuration (as for hmp_stitcher_create) while no request is outstanding. */
HMP_API hmp_status hmp_server_add_config(hmp_server* server, const hmp_config* cfg, int* config_id);
HMP_API hmp_status hmp_server_submit(hmp_server* server, int config_id, const hmp_image* inputs, int n_inputs,
                                     const hmp_image* canvas, long long* request_id);
/* The request's own status once it finished, or HMP_ERR_TIMEOUT after timeout_ms. */
HMP_API hmp_status hmp_server_wait(hmp_server* server, long long request_id, int timeout_ms);
/* Wait until no request is outstanding (HMP_ERR_TIMEOUT after timeout_ms). */
HMP_API hmp_status hmp_server_drain(hmp_server* server, int timeout_ms);
HMP_API hmp_status hmp_server_get_stats(hmp_server* server, hmp_server_stats* stats);
HMP_API void hmp_server_reset_stats(hmp_server* server);

/* Geometry of a configuration computed on the host only (no device work): blend rect, write
 * rect and effective levels, out9 = {bx, by, bw, bh, wx, wy, ww, wh, levels}; also the canvas
 * size. Mirrors CanvasManager::updateMinimizeBlend / convertMaskMat (src/pano/canvasManager.cpp:
 * 16-101) and the N-image ROI logic (src/pano/cudaPanoN.inl:156-190). */
/* ---- Batched job (config 4's native form) ----
 * Many process() calls of several stitchers captured once into a CUDA graph and replayed with one
 * launch; no counterpart in the reference (its batched use runs process() per frame). Calls added
 * under one stream index run in order; different indices run concurrently, so a stitcher's calls
 * must all use one index (HMP_ERR_INVALID_VALUE otherwise). The first capture
 * (hmp_batch_capture, or the first hmp_batch_launch) runs the job once eagerly, then captures it;
 * replays use the device buffers given at add time. Stitchers must outlive the batch, and a
 * stitcher called directly between replays must be given frames of the sizes and pitches it was
 * captured with (a call with other frames re-resolves its canvas table, which the graph reads). */
typedef struct hmp_batch hmp_batch;
HMP_API hmp_status hmp_batch_create(hmp_batch** out);
HMP_API void hmp_batch_destroy(hmp_batch* batch);
HMP_API hmp_status hmp_batch_add(hmp_batch* batch, hmp_stitcher* st, const hmp_image* inputs, int n_inputs,
                                 const hmp_image* canvas, int stream_index);
HMP_API hmp_status hmp_batch_capture(hmp_batch* batch, void* stream);
HMP_API hmp_status hmp_batch_launch(hmp_batch* batch, void* stream);

HMP_API hmp_status hmp_plan_geometry(const hmp_config* cfg, int* canvas_w, int* canvas_h, int* out9);

/* The copy-block classes a stitcher of `cfg` plans (see hmp_stitcher_set_copy_blocks), host only,
 * for inspection and tests; no counterpart in the reference. grid receives the canvas position of
 * block (0, 0) and the block counts across and down (blocks are 64 x 16 pixels of the write rect;
 * all zero when the configuration has no copy blocks). With classes non-NULL it receives one byte
 * per block, row-major: 0 = copy (the label image's pixel), 1 = pyramid, 2 = empty (0, 0, 0, 0). */
HMP_API hmp_status hmp_plan_copy_blocks(const hmp_config* cfg, int* grid, uint8_t* classes, size_t capacity);

/* Frame stabiliser (src/cuda/cudaStabilize.cu): Harris corners of the previous frame, their
 * Lucas-Kanade flow into the next frame, the mean flow as the global motion, and the next frame
 * translated by its rounding. Frames are grayscale float, width x height contiguous, on the device.
 * The reference copies the response map, the features and the flow through the host between
 * steps and allocates per call; a stabiliser allocates at create (max_features corners, 0 = as
 * many as the frame has interior pixels) and every step stays on the device, asynchronous on
 * `stream`, so a whole run can be captured in a CUDA graph. Corners are listed in raster order;
 * beyond max_features they are counted but not tracked. Reference defaults: k 0.04,
 * threshold 1e6, window 15 (cudaStabilize.cu:294-300). */
typedef struct hmp_stabilizer hmp_stabilizer;
typedef struct hmp_stabilize_info {
  int corners;          /* corners found in the previous frame */
  int kept;             /* of them, tracked (min(corners, max_features)) */
  float dx, dy;         /* mean flow, next relative to previous (0, 0 without corners) */
  int shift_x, shift_y; /* the translation applied: dx, dy rounded to whole pixels */
} hmp_stabilize_info;
HMP_API hmp_status hmp_stabilizer_create(int width, int height, int max_features, hmp_stabilizer** out);
HMP_API void hmp_stabilizer_destroy(hmp_stabilizer* st);
/* harrisCornerDetection(d_img, width, height, k, threshold, corners) cudaStabilize.cu:157 */
HMP_API hmp_status hmp_stabilizer_corners(hmp_stabilizer* st, const float* img, float k, float threshold,
                                          void* stream);
/* computeOpticalFlow(d_prev, d_next, features, flow, ..., window_size) cudaStabilize.cu:210, over
 * the stabiliser's current features, then the mean flow (stabilizeFrame's first half, :244-252). */
HMP_API hmp_status hmp_stabilizer_flow(hmp_stabilizer* st, const float* prev, const float* next, int window_size,
                                       void* stream);
/* The warp of stabilizeFrame (:254-266, warpFrameKernel :137-150) by the current motion; out may be frame (in place, as the
 * reference does it). */
HMP_API hmp_status hmp_stabilizer_warp(hmp_stabilizer* st, const float* frame, float* out, void* stream);
/* corners(prev) + flow(prev, next) + warp(next -> out): the reference's main() (:274-314). */
HMP_API hmp_status hmp_stabilizer_run(hmp_stabilizer* st, const float* prev, const float* next, float* out, float k,
                                      float threshold, int window_size, void* stream);
/* Waits for `stream`, then reads the motion and the first min(kept, capacity) features: xy as
 * (x, y) int pairs, flow as (dx, dy) float pairs (both may be NULL when capacity is 0). */
HMP_API hmp_status hmp_stabilizer_get_features(hmp_stabilizer* st, int* xy, float* flow, int capacity,
                                               hmp_stabilize_info* info, void* stream);
/* Waits for `stream`, then copies the last Harris response map (width * height floats, 0 on the
 * border) to host memory `out` of `capacity` floats (the map harrisCornerDetection reads back,
 * cudaStabilize.cu:176-177). */
HMP_API hmp_status hmp_stabilizer_get_response(hmp_stabilizer* st, float* out, size_t capacity, void* stream);
/* Replaces the features with n host (x, y) pairs (the reference's computeOpticalFlow takes any
 * feature list); n <= max_features, each point on the frame (HMP_ERR_INVALID_VALUE otherwise).
 * Waits for the upload before returning. */
HMP_API hmp_status hmp_stabilizer_set_features(hmp_stabilizer* st, const int* xy, int n, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* HMPANO_H */
