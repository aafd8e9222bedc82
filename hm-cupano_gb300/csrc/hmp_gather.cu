// hmp_gather.cu -- canvas gather kernel (hard seam, and the canvas outside the blend region).
//
// Replaces, per frame, the reference's canvas memset plus one remap launch per image
// (src/pano/cudaPano.inl:186-359 with src/cuda/cudaRemap.cu:203-294; the three-image fused hard
// seam src/cuda/cudaFusedKernels3.cu:124-217; the N-image fused hard seam cudaRemap.cu:251-294).
// One pass over the canvas: each warp owns a 256-pixel row segment, copies its owner bytes and
// packed table entries into shared memory, copies the source pixels they select (cp.async, for
// every frame of the batch) and stores them in full lines. Pixels with no owner get zero, so no memset is needed.
// HBM-bound: 1 + 4 + 4 + 4 = 13 bytes per canvas pixel.
#include <algorithm>

#include "hmp_kernels.h"

namespace hmp {
namespace {

// Table lookups of one 8-pixel row group: one 64-bit owner load (or none) and two 128-bit table
// loads when the group is complete, per-pixel loads at the right edge. Tables are read once per
// frame, so they bypass L1 and are marked evict-first in L2.
struct GroupMeta {
  uint32_t ent[8];
  uint32_t own[2];  // owner bytes of pixels 0-3 and 4-7
};

__device__ __forceinline__ void load_meta(const GatherArgs& a, int x8, int y, int nv, GroupMeta& m) {
  const uint8_t* orow = a.P.owner ? a.P.owner + (long long)y * a.P.owner_pitch : nullptr;
  const uint32_t* mrow = a.P.map + (long long)y * a.P.map_pitch;
  if (nv == 8) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const uint4 m4 = __ldcs(reinterpret_cast<const uint4*>(mrow + x8 + 4 * h));
      m.ent[4 * h + 0] = m4.x;
      m.ent[4 * h + 1] = m4.y;
      m.ent[4 * h + 2] = m4.z;
      m.ent[4 * h + 3] = m4.w;
    }
    if (orow) {
      const uint2 o8 = __ldcs(reinterpret_cast<const uint2*>(orow + x8));
      m.own[0] = o8.x;
      m.own[1] = o8.y;
    } else {
      m.own[0] = m.own[1] = 0x01010101u * uint32_t(a.P.default_owner);
    }
  } else {
    m.own[0] = m.own[1] = 0xFFFFFFFFu;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      if (j < nv) {
        m.ent[j] = __ldcs(mrow + x8 + j);
        const uint32_t o = orow ? uint32_t(__ldcs(orow + x8 + j)) : uint32_t(a.P.default_owner);
        const int sh = 8 * (j & 3);
        m.own[j >> 2] = (m.own[j >> 2] & ~(0xFFu << sh)) | (o << sh);
      } else {
        m.ent[j] = 0xFFFFFFFFu;
      }
    }
  }
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_addr(dst)), "l"(src));
}
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(smem_addr(dst)), "l"(src));
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(smem_addr(dst)), "l"(src));
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Each warp owns a 256-pixel segment of one canvas row; lane l handles pixels l, l+32, ...,
// l+224, so every warp instruction below touches 32 consecutive pixels: table entries and owner
// bytes are coalesced 128-byte copies, the source gathers of neighbouring canvas pixels land in
// the same few source lines, and the canvas stores are full 128-byte lines. All loads are
// cp.async copies into shared memory laid out [pixel group][lane] (conflict-free), so they need
// no destination registers and stay in flight together: table entries and owners first, then
// one 4-byte copy per source pixel and frame. Each lane reads back only what it copied itself
// (the owner bytes of a lane's pixels come from other lanes' 4-byte copies, hence a warp sync).
__global__ void __launch_bounds__(256) canvas_gather_kernel(const __grid_constant__ GatherArgs a) {
  constexpr int PX = 8;
  __shared__ __align__(16) uint32_t s_ent[8][PX][32];
  __shared__ __align__(16) uint8_t s_own[8][PX * 32];
  __shared__ __align__(16) uchar4 s_px[8][PX][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int x0 = blockIdx.x * (32 * PX);
  const int y = blockIdx.y * 8 + w;
  const int W = a.C.w, H = a.C.h;
  if (y >= H) return;
  const bool row_skip = y >= a.skip_y0 && y < a.skip_y1;
  if (row_skip && x0 >= a.skip_x0 && x0 + 32 * PX <= a.skip_x1) return;
  const uint8_t* orow = a.P.owner ? a.P.owner + (long long)y * a.P.owner_pitch : nullptr;
  const uint32_t* mrow = a.P.map + (long long)y * a.P.map_pitch;
  uint32_t (*ent)[32] = s_ent[w];
  uint8_t* own = s_own[w];
  uchar4 (*px)[32] = s_px[w];
#pragma unroll
  for (int j = 0; j < PX; ++j) {
    const int x = x0 + 32 * j + lane;
    if (x < W)
      cp_async4(&ent[j][lane], mrow + x);
    else
      ent[j][lane] = 0xFFFFFFFFu;
  }
  if (orow) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int xb = x0 + 128 * h + 4 * lane;
      if (xb < W) cp_async4(own + 128 * h + 4 * lane, orow + xb);
    }
  }
  cp_async_commit();
  cp_async_wait<0>();
  __syncwarp();
  const bool opaque = a.opaque != 0;
  for (int b = 0; b < a.batch; ++b) {
#pragma unroll
    for (int j = 0; j < PX; ++j) {
      const int x = x0 + 32 * j + lane;
      const int o = orow ? (x < W ? int(own[32 * j + lane]) : 0xFF) : a.P.default_owner;
      const uint32_t e = ent[j][lane];
      const int sx = int(e & 0xFFFFu), sy = int(e >> 16);
      if (o < kDevMaxImages && sx < a.S.w[o] && sy < a.S.h[o]) {
        const char* base = reinterpret_cast<const char*>(a.S.ptr[o]) + b * a.S.bstride[o] + sy * a.S.pitch[o];
        cp_async4(&px[j][lane], reinterpret_cast<const uchar4*>(base) + sx);
      } else {
        px[j][lane] = make_uchar4(0, 0, 0, (opaque && o < kDevMaxImages && sx != 0xFFFF) ? 255 : 0);
      }
    }
    cp_async_commit();
    cp_async_wait<0>();
    uint32_t* crow = reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(a.C.ptr) + b * a.C.bstride + y * a.C.pitch);
#pragma unroll
    for (int j = 0; j < PX; ++j) {
      const int x = x0 + 32 * j + lane;
      if (x < W && !(row_skip && x >= a.skip_x0 && x < a.skip_x1))
        __stcs(crow + x, *reinterpret_cast<const uint32_t*>(&px[j][lane]));
    }
  }
}

}  // namespace

cudaError_t launch_canvas_gather(const GatherArgs& a, cudaStream_t stream) {
  const dim3 grid((a.C.w + 255) / 256, (a.C.h + 7) / 8);
  canvas_gather_kernel<<<grid, 256, 0, stream>>>(a);
  return cudaGetLastError();
}

}  // namespace hmp
