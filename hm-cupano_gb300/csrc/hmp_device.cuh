// hmp_device.cuh -- device-side parameter blocks and helpers shared by the stitching kernels.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace hmp {

constexpr int kDevMaxImages = 8;
constexpr int kDevMaxLevels = 7;

// The frames of one process() call (RGBA8, pitched, batch-strided).
struct SrcSet {
  const uchar4* ptr[kDevMaxImages];
  long long pitch[kDevMaxImages];   // bytes per row
  long long bstride[kDevMaxImages]; // bytes per frame
  int w[kDevMaxImages];
  int h[kDevMaxImages];
};

// A gather plane on the device (see hmp_plan.h): owner (u8, optional) and packed table entries.
struct PlaneDev {
  const uint8_t* owner;  // nullptr: every pixel belongs to default_owner
  const uint32_t* map;
  int owner_pitch;  // bytes
  int map_pitch;    // entries
  int x0, y0, w, h; // rect in domain coordinates
  int default_owner;
};

struct CanvasDev {
  uchar4* ptr;
  long long pitch;   // bytes
  long long bstride; // bytes
  int w, h;
};

// 8-byte half-precision RGBA for FP16 pyramid storage.
struct __align__(8) half4 {
  __half x, y, z, w;
};

__device__ __forceinline__ float4 to_f4(const uchar4 v) {
  return make_float4(float(v.x), float(v.y), float(v.z), float(v.w));
}

__device__ __forceinline__ float4 load_level(const float4* p) { return *p; }
__device__ __forceinline__ float4 load_level(const half4* p) {
  const uint2 raw = *reinterpret_cast<const uint2*>(p);
  const __half2 a = *reinterpret_cast<const __half2*>(&raw.x);
  const __half2 b = *reinterpret_cast<const __half2*>(&raw.y);
  const float2 fa = __half22float2(a), fb = __half22float2(b);
  return make_float4(fa.x, fa.y, fb.x, fb.y);
}
__device__ __forceinline__ void store_level(float4* p, const float4 v) { *p = v; }
__device__ __forceinline__ void store_level(half4* p, const float4 v) {
  const __half2 a = __floats2half2_rn(v.x, v.y);
  const __half2 b = __floats2half2_rn(v.z, v.w);
  uint2 raw;
  raw.x = *reinterpret_cast<const uint32_t*>(&a);
  raw.y = *reinterpret_cast<const uint32_t*>(&b);
  *reinterpret_cast<uint2*>(p) = raw;
}

// Owner and packed table entry of one plane pixel (domain coordinates); owner 0xFF and entry
// 0xFFFFFFFF outside the plane.
__device__ __forceinline__ void plane_lookup(const PlaneDev& P, int x, int y, int& owner, uint32_t& entry) {
  const int rx = x - P.x0, ry = y - P.y0;
  owner = 0xFF;
  entry = 0xFFFFFFFFu;
  if ((unsigned)rx >= (unsigned)P.w || (unsigned)ry >= (unsigned)P.h) return;
  owner = P.owner ? int(__ldg(P.owner + (long long)ry * P.owner_pitch + rx)) : P.default_owner;
  entry = __ldg(P.map + (long long)ry * P.map_pitch + rx);
}

// Source pixel for (owner, entry): the source pixel when the entry lies inside the source;
// otherwise zero, with alpha 255 under the soft-seam ("opaque") rule when the x entry is not the
// 65535 sentinel (src/cuda/cudaRemap.cu:60-123).
__device__ __forceinline__ uchar4 fetch_src(const SrcSet& S, int o, uint32_t e, int b, bool opaque) {
  uchar4 out = make_uchar4(0, 0, 0, 0);
  if (o >= kDevMaxImages) return out;
  const int sx = int(e & 0xFFFFu), sy = int(e >> 16);
  if (sx < S.w[o] && sy < S.h[o]) {
    const char* base = reinterpret_cast<const char*>(S.ptr[o]) + b * S.bstride[o] + sy * S.pitch[o];
    return __ldg(reinterpret_cast<const uchar4*>(base) + sx);
  }
  if (opaque && sx != 0xFFFF) out.w = 255;
  return out;
}

// Source pixel of (owner, entry) with the owner resolved by a static select, so that the frame
// table in the kernel parameters is only ever indexed by constants.
template <int NMAX>
__device__ __forceinline__ uchar4 fetch_sel(const SrcSet& S, int o, uint32_t e, int b, bool opaque) {
  const int sx = int(e & 0xFFFFu), sy = int(e >> 16);
  uchar4 out = make_uchar4(0, 0, 0, 0);
#pragma unroll
  for (int q = 0; q < NMAX; ++q) {
    if (o == q) {
      if (sx < S.w[q] && sy < S.h[q]) {
        const char* base = reinterpret_cast<const char*>(S.ptr[q]) + b * S.bstride[q] + sy * S.pitch[q];
        out = __ldg(reinterpret_cast<const uchar4*>(base) + sx);
      } else if (opaque && sx != 0xFFFF) {
        out.w = 255;
      }
    }
  }
  return out;
}

// Level-0 value of one plane pixel (domain coordinates), the reference's remap rule
// (src/cuda/cudaRemap.cu:60-123): an entry inside the source gives the source pixel; otherwise
// zero, with alpha 255 under the soft-seam ("opaque") rule when the x entry is not the 65535
// sentinel. Pixels outside the plane, or with no owner, are zero.
__device__ __forceinline__ uchar4 plane_pixel(const SrcSet& S, const PlaneDev& P, int x, int y, int b,
                                              bool opaque) {
  const int rx = x - P.x0, ry = y - P.y0;
  uchar4 out = make_uchar4(0, 0, 0, 0);
  if ((unsigned)rx >= (unsigned)P.w || (unsigned)ry >= (unsigned)P.h) return out;
  const int o = P.owner ? int(P.owner[(long long)ry * P.owner_pitch + rx]) : P.default_owner;
  if (o >= kDevMaxImages) return out;
  const uint32_t e = P.map[(long long)ry * P.map_pitch + rx];
  const int sx = int(e & 0xFFFFu), sy = int(e >> 16);
  if (sx < S.w[o] && sy < S.h[o]) {
    const char* base = reinterpret_cast<const char*>(S.ptr[o]) + b * S.bstride[o] + sy * S.pitch[o];
    return __ldg(reinterpret_cast<const uchar4*>(base) + sx);
  }
  if (opaque && sx != 0xFFFF) out.w = 255;
  return out;
}

// Canvas-plane entries resolved for the frames being stitched (resolve_plane_kernel): the owner
// and a pixel offset within the owner's frame, owner << 29 | (sy * pitch / 4 + sx), or one of two
// fills -- the reference's remap rule (src/cuda/cudaRemap.cu:60-123): an entry outside the source
// reads zero, with alpha 255 under the soft-seam ("opaque") rule unless its x is the 65535
// sentinel.
constexpr uint32_t kOffZero = 0xFFFFFFFFu;    // (0, 0, 0, 0)
constexpr uint32_t kOffOpaque = 0xFFFFFFFEu;  // (0, 0, 0, 255)
// A canvas pixel the pyramid writes in copy-block mode (the gather leaves it alone). Frames hold
// at most kOffMask - 2 pixels (process() rejects larger ones), so offsets stay below kOffMask - 2
// and no resolved entry, owner 7 included, reaches this code.
constexpr uint32_t kOffSkip = 0xFFFFFFFDu;
constexpr int kOwnerShift = 29;
constexpr uint32_t kOffMask = (1u << kOwnerShift) - 1u;  // frames hold fewer than kOffMask - 1 pixels

__device__ __forceinline__ uint32_t fill_of(uint32_t off) { return off == kOffOpaque ? 0xFF000000u : 0u; }

// Truncating float -> uint8 pack (src/cuda/cudaUtils.cuh:18-28): v <= 0 -> 0, v >= 255 -> 255,
// otherwise truncation toward zero.
__device__ __forceinline__ unsigned char pack_u8(float v) {
  if (v <= 0.0f) return 0;
  if (v >= 255.0f) return 255;
  return (unsigned char)__float2uint_rz(v);
}

__device__ __forceinline__ uchar4 pack_rgba(const float4 v) {
  return make_uchar4(pack_u8(v.x), pack_u8(v.y), pack_u8(v.z), pack_u8(v.w));
}

}  // namespace hmp
