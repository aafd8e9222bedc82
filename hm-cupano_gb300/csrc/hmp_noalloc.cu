// hmp_noalloc.cu -- two-image pyramid blend that allocates no device memory
// (hmp_blend2_noalloc in include/hmpano.h).
//
// For callers that cannot call cudaMalloc: a plugin inside a host application that owns all device
// memory through its own pool (a raw cudaMalloc escapes the host's budget and accounting), or code
// on a real-time frame path, where cudaMalloc and cudaFree may synchronise the device and stall
// every stream. Such callers cannot construct a stitcher (hmp_stitcher_create allocates its tables
// and pyramid), so this entry point takes two already-remapped images, the seam and the output,
// and keeps every intermediate (pixel table, seam pyramid, Gaussian levels, level-1
// reconstruction) in one file-scope device array of HMP_NOALLOC_SCRATCH_BYTES.
//
// The blend itself is the stitcher's two-image pyramid (pyr_down, pyr_coarse, pyr_fine with the
// two-image rule) over the whole image, so its output equals a two-image stitcher's whose tables
// are the identity and whose images both sit at (0, 0) with minimize_blend off.
//
// The array is shared by every call on a device and keeps the last call's contents. Each call
// rewrites all of the scratch it reads before reading it (the kernels' tiles cover every level
// pixel), so nothing has to start at zero; calls whose work overlaps on the GPU race on it.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdio>
#include <mutex>

#include "hmp_kernels.h"
#include "hmp_plan.h"
#include "hmpano.h"

namespace {

// The scratch. Every GPU that loads the library holds it until the process exits. In host code
// this name is a stand-in for the symbol, not a device address: the address comes from
// cudaGetSymbolAddress (blend_scratch_for_current_device).
static __device__ __align__(256) unsigned char g_blend2_scratch[HMP_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
unsigned char* g_scratch_ptr[kMaxDevices] = {};

hmp_status status_of(int code, const char* msg) {
  hmp_status s;
  s.code = code;
  std::snprintf(s.message, sizeof(s.message), "%s", msg);
  return s;
}

hmp_status cuda_failure(cudaError_t e, const char* what) {
  hmp_status s;
  s.code = int(e);
  std::snprintf(s.message, sizeof(s.message), "%s: %s", what, cudaGetErrorString(e));
  return s;
}

// Set-up, once per device with that device current: the scratch's device address and the
// kernels' shared-memory limits. Runs inside the first hmp_blend2_noalloc call on a device.
cudaError_t blend_scratch_for_current_device(int dev, unsigned char** out) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_ptr[dev]) {
    unsigned char* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(reinterpret_cast<void**>(&ptr), g_blend2_scratch);
    if (e != cudaSuccess) return e;
    e = hmp::kernels_init();
    if (e != cudaSuccess) return e;
    g_scratch_ptr[dev] = ptr;
  }
  *out = g_scratch_ptr[dev];
  return cudaSuccess;
}

// Identity pixel table of a w x h image: entry (x, y) = x | y << 16.
__global__ void identity_table_kernel(uint32_t* map, int pitch, int w, int h) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x < w && y < h) map[(long long)y * pitch + x] = uint32_t(x) | (uint32_t(y) << 16);
}

// One seam-pyramid level: mean of the in-bounds pixels of each 2x2 block of the level above,
// summed dy-outer / dx-inner in FP32 and divided by the count (the stitcher's host planner does
// the same; src/cuda/cudaBlend.cu:268-296).
template <typename Tin>
__global__ void seam_level_kernel(const Tin* src, long long src_pitch, int iw, int ih, float* dst, int ow, int oh) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= ow || y >= oh) return;
  float s = 0.0f;
  int cnt = 0;
  for (int dy = 0; dy < 2; ++dy)
    for (int dx = 0; dx < 2; ++dx) {
      const int ix = 2 * x + dx, iy = 2 * y + dy;
      if (ix >= iw || iy >= ih) continue;
      s += float(src[iy * src_pitch + ix]);
      ++cnt;
    }
  dst[(long long)y * ow + x] = s / float(cnt);
}

inline size_t align256(size_t v) { return (v + 255) / 256 * 256; }

bool valid_image(const hmp_image* im) {
  return im && im->data && im->width > 0 && im->height > 0 && im->pitch >= size_t(im->width) * 4 &&
         im->pitch % 4 == 0 && reinterpret_cast<uintptr_t>(im->data) % 4 == 0;
}

}  // namespace

extern "C" HMP_API hmp_status hmp_blend2_noalloc(const hmp_image* image1, const hmp_image* image2,
                                                 const uint8_t* seam, size_t seam_pitch, int num_levels,
                                                 int batch_size, const hmp_image* out, void* stream) {
  if (!valid_image(image1) || !valid_image(image2) || !valid_image(out))
    return status_of(HMP_ERR_INVALID_VALUE, "images must be non-null RGBA8 with 4-byte aligned data and pitch");
  const int w = out->width, h = out->height;
  if (image1->width != w || image1->height != h || image2->width != w || image2->height != h)
    return status_of(HMP_ERR_INVALID_VALUE, "both images and the output must have the same size");
  if (w >= 65535 || h >= 65535)
    return status_of(HMP_ERR_INVALID_VALUE, "images must be smaller than 65535 pixels per side");
  if (!seam || seam_pitch < size_t(w) || seam_pitch > size_t(INT_MAX))
    return status_of(HMP_ERR_INVALID_VALUE, "seam must be a device pointer with pitch >= width");
  if (num_levels < 1 || num_levels > 30) return status_of(HMP_ERR_INVALID_VALUE, "num_levels must be in 1..30");
  // Bounds every scratch size below (batch x level pixels x 16 bytes) far from overflow.
  if (batch_size < 1 || batch_size > 65536) return status_of(HMP_ERR_INVALID_VALUE, "batch_size must be in 1..65536");
  const int L = hmp::effective_levels(w, h, num_levels);
  if (L > hmp::kMaxLevels)
    return status_of(HMP_ERR_NOT_SUPPORTED, "more than 7 effective pyramid levels are not supported");

  // Scratch layout (each part 256-byte aligned): pixel table, seam levels 1..L-1, Gaussian levels
  // 1..L-1 of both images, level-1 reconstruction.
  int lw[hmp::kMaxLevels], lh[hmp::kMaxLevels];
  lw[0] = w;
  lh[0] = h;
  for (int l = 1; l < L; ++l) lw[l] = (lw[l - 1] + 1) / 2, lh[l] = (lh[l - 1] + 1) / 2;
  const int map_pitch = (w + 7) / 8 * 8;
  const size_t B = size_t(batch_size);
  size_t off_mask[hmp::kMaxLevels] = {}, off_g[2][hmp::kMaxLevels] = {}, off_r1 = 0;
  size_t need = align256(size_t(map_pitch) * 4 * h);
  for (int l = 1; l < L; ++l) {
    off_mask[l] = need;
    need += align256(size_t(lw[l]) * lh[l] * sizeof(float));
  }
  for (int k = 0; k < 2; ++k)
    for (int l = 1; l < L; ++l) {
      off_g[k][l] = need;
      need += align256(B * lw[l] * lh[l] * sizeof(float4));
    }
  if (L > 1) {
    off_r1 = need;
    need += align256(B * lw[1] * lh[1] * sizeof(float4));
  }
  if (need > size_t(HMP_NOALLOC_SCRATCH_BYTES)) {
    char msg[200];
    std::snprintf(msg, sizeof(msg),
                  "blend needs %zu bytes of scratch, more than the library's static maximum of %zu bytes "
                  "(HMP_NOALLOC_SCRATCH_BYTES)",
                  need, size_t(HMP_NOALLOC_SCRATCH_BYTES));
    return status_of(HMP_ERR_INVALID_VALUE, msg);
  }

  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_failure(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return status_of(HMP_ERR_NOT_SUPPORTED, "device ordinal above 63");
  unsigned char* scratch = nullptr;
  e = blend_scratch_for_current_device(dev, &scratch);
  if (e != cudaSuccess) return cuda_failure(e, "static scratch set-up");

  const cudaStream_t s = static_cast<cudaStream_t>(stream);
  uint32_t* map = reinterpret_cast<uint32_t*>(scratch);
  identity_table_kernel<<<dim3((w + 255) / 256, h), 256, 0, s>>>(map, map_pitch, w, h);
  for (int l = 1; l < L; ++l) {
    float* dst = reinterpret_cast<float*>(scratch + off_mask[l]);
    const dim3 grid((lw[l] + 255) / 256, lh[l]);
    if (l == 1)
      seam_level_kernel<uint8_t><<<grid, 256, 0, s>>>(seam, (long long)seam_pitch, w, h, dst, lw[1], lh[1]);
    else
      seam_level_kernel<float><<<grid, 256, 0, s>>>(reinterpret_cast<const float*>(scratch + off_mask[l - 1]),
                                                    lw[l - 1], lw[l - 1], lh[l - 1], dst, lw[l], lh[l]);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_failure(e, "table/seam launch");

  hmp::PyrArgs a{};
  const hmp_image* ims[2] = {image1, image2};
  for (int k = 0; k < 2; ++k) {
    a.S.ptr[k] = static_cast<const uchar4*>(ims[k]->data);
    a.S.pitch[k] = (long long)ims[k]->pitch;
    a.S.bstride[k] = (long long)ims[k]->pitch * h;
    a.S.w[k] = w;
    a.S.h[k] = h;
    hmp::PlaneDev& P = a.slot[k];
    P.owner = nullptr;
    P.map = map;
    P.map_pitch = map_pitch;
    P.x0 = P.y0 = 0;
    P.w = w;
    P.h = h;
    P.default_owner = k;
  }
  a.n = 2;
  a.levels = L;
  for (int l = 0; l < L; ++l) {
    a.lw[l] = lw[l];
    a.lh[l] = lh[l];
    if (l > 0) {
      a.maskL[l] = reinterpret_cast<const float*>(scratch + off_mask[l]);
      for (int k = 0; k < 2; ++k) a.G[k][l] = scratch + off_g[k][l];
    }
  }
  a.mask0 = seam;
  a.mask0_pitch = int(seam_pitch);
  a.K = 1;
  a.opaque = 1;
  a.C.ptr = static_cast<uchar4*>(out->data);
  a.C.pitch = (long long)out->pitch;
  a.C.bstride = (long long)out->pitch * h;
  a.C.w = w;
  a.C.h = h;
  a.wx0 = a.wy0 = 0;
  a.wx1 = w;
  a.wy1 = h;
  a.cx_off = a.cy_off = 0;
  if (L > 1) {
    // Same tiles as a two-image stitcher of this depth.
    const int align = 1 << (L - 1);
    const int tile_down = std::max(64, align), tile_coarse = std::max(32, align / 2);
    const size_t coarse_smem = hmp::pyr_coarse_smem(2, 1, tile_coarse, L, HMP_STORAGE_F32);
    if (hmp::pyr_down_smem(2, tile_down) > 227 * 1024 || coarse_smem > 227 * 1024)
      return status_of(HMP_ERR_NOT_SUPPORTED, "pyramid tile does not fit in shared memory");
    a.tile = tile_down;
    e = hmp::launch_pyr_down(a, HMP_STORAGE_F32,
                             dim3((w + tile_down - 1) / tile_down, (h + tile_down - 1) / tile_down, batch_size), s);
    if (e != cudaSuccess) return cuda_failure(e, "pyr_down launch");
    a.R1 = reinterpret_cast<float4*>(scratch + off_r1);
    const int x1hi = std::min(((w - 1) >> 1) + 2, lw[1]), y1hi = std::min(((h - 1) >> 1) + 2, lh[1]);
    a.tile = tile_coarse;
    a.tx0 = a.ty0 = 0;
    e = hmp::launch_pyr_coarse(a, hmp::kRuleTwo, HMP_STORAGE_F32,
                               dim3((x1hi + tile_coarse - 1) / tile_coarse, (y1hi + tile_coarse - 1) / tile_coarse,
                                    batch_size),
                               coarse_smem, s);
    if (e != cudaSuccess) return cuda_failure(e, "pyr_coarse launch");
  }
  e = hmp::launch_pyr_fine(a, hmp::kRuleTwo, HMP_STORAGE_F32, dim3((w + 63) / 64, (h + 15) / 16, batch_size), s);
  if (e != cudaSuccess) return cuda_failure(e, "pyr_fine launch");
  return status_of(HMP_OK, "");
}
