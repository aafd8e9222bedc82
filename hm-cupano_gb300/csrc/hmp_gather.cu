// hmp_gather.cu -- canvas gather kernel (hard seam, and the canvas outside the blend region).
//
// Replaces, per frame, the reference's canvas memset plus one remap launch per image
// (src/pano/cudaPano.inl:186-359 with src/cuda/cudaRemap.cu:203-294; the three-image fused hard
// seam src/cuda/cudaFusedKernels3.cu:124-217; the N-image fused hard seam cudaRemap.cu:251-294).
// One pass over the canvas: each warp owns a 256-pixel row segment, loads its table entries, reads
// the source pixels they select (for every frame of the batch) and stores them in full lines.
// Pixels with no owner get zero, so no memset is needed. Table entries are resolved
// (resolve_plane_kernel below) to the owner and the pixel offset in its frame, and the resolve pass
// also records each segment's owner when it has only one and whether it holds fills, so a pixel of
// a fill-free one-owner segment costs a multiply-add besides its load and store.
// HBM-bound: 4 (entry) + 4 (source) + 4 (canvas) = 12 bytes per canvas pixel.
#include <algorithm>

#include "hmp_kernels.h"

namespace hmp {
namespace {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(smem_addr(dst)), "l"(src));
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Source pixel of a canvas pixel with resolved entry e in the frame at base (the entry's owner):
// a 4-byte copy into *dst, or its fill.
__device__ __forceinline__ void gather_one(uint32_t* dst, const uchar4* base, uint32_t e) {
  if (e < kOffOpaque)
    cp_async4(dst, base + e);
  else
    *dst = fill_of(e);
}

// Each warp owns a 256-pixel segment of one canvas row; lane l handles the pixel pairs
// (2l, 2l+1) + 64j, j = 0..3, so every warp instruction below touches 64 consecutive pixels:
// table entries are 8-byte loads (256 bytes per instruction), the source reads of neighbouring
// canvas pixels land in the same few source lines, and the canvas stores are 8-byte streaming
// stores of full lines. The segment's code from the resolve pass picks the path:
//   - one owner, no fills, whole segment stored (most of a canvas): the eight source pixels are
//     loaded into registers, all in flight together, and stored in pairs;
//   - otherwise they are cp.async copies into shared memory laid out [pixel step][lane]
//     (conflict-free; each lane reads back only what it copied), with fills written directly and
//     the owner taken per pixel from the entry (owner << 29 | offset) where a seam crosses the
//     segment.
// Measured: loading the entries into registers instead of staging them in shared memory, and the
// register path, each took about 4 % off the two-image 8500x3300 frame (fewer shared-memory
// instructions in the queue that the pyramid kernels running beside the gather also use).
// kCopy: the plane holds copy-block skips and the call may check source alpha (three or more
// images); without it the kernel is compiled free of that code.
template <bool kCopy>
__global__ void __launch_bounds__(256, 6) canvas_gather_kernel(const __grid_constant__ GatherArgs a) {
  constexpr int PJ = 4;  // 64-pixel steps per segment
  static_assert(64 * PJ == kSegPixels, "a warp's segment is the resolve pass's segment");
  __shared__ __align__(16) uint2 s_px[8][PJ][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int x0 = blockIdx.x * (64 * PJ);
  const int y = blockIdx.y * 8 + w;
  const int W = a.C.w, H = a.C.h;
  if (y >= H) return;
  const bool row_skip = y >= a.skip_y0 && y < a.skip_y1;
  if (row_skip && x0 >= a.skip_x0 && x0 + 64 * PJ <= a.skip_x1) return;
  const uint32_t* mrow = a.P.map + (long long)y * a.P.map_pitch;
  uint2* px = &s_px[w][0][0];
  uint2 er[PJ];
#pragma unroll
  for (int j = 0; j < PJ; ++j) {
    const int x = x0 + 64 * j + 2 * lane;
    if (x + 1 < W)
      er[j] = __ldg(reinterpret_cast<const uint2*>(mrow + x));  // map rows: 8-entry aligned pitch, x even
    else
      er[j] = make_uint2(x < W ? __ldg(mrow + x) : kOffZero, kOffZero);
  }
  // The segment's owner, from the resolve pass: one for all its entries (or only fills), or mixed.
  const unsigned so = __ldg(a.seg_owner + (long long)y * a.seg_pitch + blockIdx.x);
  const bool uniform = so != kSegMixed;
  const int uo = int(so & (kSegFills - 1));
  // Copy-block mode: pixels the pyramid writes carry kOffSkip (only in mixed segments).
  bool skips = false;
  if (kCopy && so == kSegMixed) {
#pragma unroll
    for (int j = 0; j < PJ; ++j) skips = skips || er[j].x == kOffSkip || er[j].y == kOffSkip;
    skips = __any_sync(0xFFFFFFFFu, skips);
  }
  // Segments wholly inside the canvas and outside the skipped rect store without checks.
  const bool plain = x0 + 64 * PJ <= W && !(row_skip && x0 < a.skip_x1 && x0 + 64 * PJ > a.skip_x0) && !skips;
  // Copy-block mode: source pixels read inside the blend region must have alpha != 0.
  const bool chk = kCopy && a.alpha_flag != nullptr && y >= a.chk_y0 && y < a.chk_y1 && x0 < a.chk_x1 && x0 + 64 * PJ > a.chk_x0;
  bool bad = false;
  for (int b = 0; b < a.batch; ++b) {
    uint32_t* pxw = reinterpret_cast<uint32_t*>(px);
    uint32_t* crow = reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(a.C.ptr) + b * a.C.bstride + y * a.C.pitch);
    if (so < kSegFills && plain && (reinterpret_cast<uintptr_t>(crow) & 7) == 0) {
      // One owner, no fills, whole segment stored: every load in flight from registers.
      const uint32_t* base =
          reinterpret_cast<const uint32_t*>(reinterpret_cast<const char*>(a.S.ptr[uo]) + b * a.S.bstride[uo]);
      uint32_t v[2 * PJ];
#pragma unroll
      for (int j = 0; j < PJ; ++j) {
        v[2 * j] = __ldg(base + er[j].x);
        v[2 * j + 1] = __ldg(base + er[j].y);
      }
#pragma unroll
      for (int j = 0; j < PJ; ++j)
        __stcs(reinterpret_cast<uint2*>(crow + x0 + 64 * j + 2 * lane), make_uint2(v[2 * j], v[2 * j + 1]));
      if (chk) {
#pragma unroll
        for (int i = 0; i < 2 * PJ; ++i) {
          const int x = x0 + 64 * (i >> 1) + 2 * lane + (i & 1);
          bad = bad || ((v[i] >> 24) == 0u && x >= a.chk_x0 && x < a.chk_x1);
        }
      }
      continue;
    }
    if (uniform) {
      // One owner: the entries are plain offsets into its frame (or fills, if the segment has any).
      const uchar4* base =
          reinterpret_cast<const uchar4*>(reinterpret_cast<const char*>(a.S.ptr[uo]) + b * a.S.bstride[uo]);
      if (so & kSegFills) {
#pragma unroll
        for (int j = 0; j < PJ; ++j) {
          const uint2 e = er[j];
          gather_one(pxw + 2 * (32 * j + lane), base, e.x);
          gather_one(pxw + 2 * (32 * j + lane) + 1, base, e.y);
        }
      } else {
#pragma unroll
        for (int j = 0; j < PJ; ++j) {
          const uint2 e = er[j];
          cp_async4(pxw + 2 * (32 * j + lane), base + e.x);
          cp_async4(pxw + 2 * (32 * j + lane) + 1, base + e.y);
        }
      }
    } else {
#pragma unroll
      for (int j = 0; j < PJ; ++j) {
        const uint2 e2 = er[j];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const uint32_t e = h ? e2.y : e2.x;
          uint32_t* d = pxw + 2 * (32 * j + lane) + h;
          if (e < kOffSkip) {
            const int o = int(e >> kOwnerShift);
            cp_async4(d, reinterpret_cast<const uchar4*>(reinterpret_cast<const char*>(a.S.ptr[o]) + b * a.S.bstride[o]) +
                             (e & kOffMask));
          } else {
            *d = fill_of(e);
          }
        }
      }
    }
    cp_async_commit();
    cp_async_wait<0>();
    if (chk) {
      // Source reads only: offsets and owner-tagged entries lie below every fill and skip code.
#pragma unroll
      for (int j = 0; j < PJ; ++j) {
        const uint2 v = px[32 * j + lane];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int x = x0 + 64 * j + 2 * lane + h;
          const uint32_t e = h ? er[j].y : er[j].x;
          bad = bad || (e < kOffSkip && ((h ? v.y : v.x) >> 24) == 0u && x >= a.chk_x0 && x < a.chk_x1);
        }
      }
    }
    if (plain && (reinterpret_cast<uintptr_t>(crow) & 7) == 0) {
#pragma unroll
      for (int j = 0; j < PJ; ++j)
        __stcs(reinterpret_cast<uint2*>(crow + x0 + 64 * j + 2 * lane), px[32 * j + lane]);
    } else {
#pragma unroll
      for (int j = 0; j < PJ; ++j) {
        const uint2 v = px[32 * j + lane];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int x = x0 + 64 * j + 2 * lane + h;
          const uint32_t e = h ? er[j].y : er[j].x;
          if (x < W && !(row_skip && x >= a.skip_x0 && x < a.skip_x1) && (!kCopy || e != kOffSkip))
            __stcs(crow + x, h ? v.y : v.x);
        }
      }
    }
  }
  if constexpr (kCopy) {
    if (chk && __any_sync(0xFFFFFFFFu, bad) && lane == 0) atomicOr(a.alpha_flag, 1);
  }
}

// Resolves one plane's packed entries (raw.map) for the frames' geometry (res, same layout):
// owner o < n and (sx, sy) inside image o give o << 29 | (sy * pitch / 4 + sx); anything else
// kOffZero, or kOffOpaque under the soft-seam rule when the owner is valid and sx is not the
// 65535 sentinel. (Frames hold fewer than kOffMask - 1 pixels, so no offset meets a fill code.)
__global__ void __launch_bounds__(kSegPixels) resolve_plane_kernel(const __grid_constant__ PlaneDev raw, uint32_t* res,
                                                                   uint8_t* seg_owner, int seg_pitch,
                                                                   const __grid_constant__ SrcSet S, int n, int opaque,
                                                                   const __grid_constant__ SkipMap skip) {
  // One CTA per 256-pixel row segment, the gather's unit.
  const int x = blockIdx.x * kSegPixels + threadIdx.x, y = blockIdx.y;
  uint32_t r = kOffZero;  // pixels past the plane's width read as fills
  const bool in = x < raw.w;
  if (in) {
    const int o = raw.owner ? int(raw.owner[(long long)y * raw.owner_pitch + x]) : raw.default_owner;
    const uint32_t e = raw.map[(long long)y * raw.map_pitch + x];
    const int sx = int(e & 0xFFFFu), sy = int(e >> 16);
    if (o < n) {
      if (sx < S.w[o] && sy < S.h[o])
        r = (uint32_t(o) << kOwnerShift) | (uint32_t(sy) * uint32_t(S.pitch[o] / 4) + uint32_t(sx));
      else if (opaque && sx != 0xFFFF)
        r = kOffOpaque;
    }
    // Copy-block mode: a pixel of a block the pyramid writes.
    if (skip.map && x >= skip.wr_x0 && x < skip.wr_x1 && y >= skip.wr_y0 && y < skip.wr_y1) {
      const int bx = (x - skip.x0) >> 6, by = (y - skip.y0) >> 4;
      if (bx >= 0 && by >= 0 && bx < skip.nx && by < skip.ny && skip.map[(long long)by * skip.pitch + bx]) r = kOffSkip;
    }
  }
  // The segment's range of owners and whether it holds fills.
  // A segment holding a skip is mixed: its entries keep their owners and the gather stores pixel
  // by pixel.
  __shared__ unsigned s_lo[kSegPixels / 32], s_hi[kSegPixels / 32], s_fill[kSegPixels / 32];
  __shared__ unsigned s_code;
  unsigned lo = r < kOffSkip ? r >> kOwnerShift : 8u, hi = r < kOffSkip ? r >> kOwnerShift : 0u;
  if (r == kOffSkip) lo = 1u, hi = 2u;
  lo = __reduce_min_sync(0xFFFFFFFFu, lo);
  hi = __reduce_max_sync(0xFFFFFFFFu, hi);
  const unsigned fill = __reduce_or_sync(0xFFFFFFFFu, r >= kOffSkip ? 1u : 0u);
  if ((threadIdx.x & 31) == 0) {
    s_lo[threadIdx.x >> 5] = lo;
    s_hi[threadIdx.x >> 5] = hi;
    s_fill[threadIdx.x >> 5] = fill;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned f = fill;
    for (int w = 1; w < kSegPixels / 32; ++w) {
      lo = min(lo, s_lo[w]);
      hi = max(hi, s_hi[w]);
      f |= s_fill[w];
    }
    s_code = lo >= hi ? ((lo < 8u ? lo : 0u) | (f ? kSegFills : 0u)) : kSegMixed;
    if (seg_owner) seg_owner[(long long)y * seg_pitch + blockIdx.x] = uint8_t(s_code);
  }
  __syncthreads();
  // Entries of a one-owner segment are stored without their owner (the segment has it).
  if (in) res[(long long)y * raw.map_pitch + x] = (s_code != kSegMixed && r < kOffSkip) ? (r & kOffMask) : r;
}

}  // namespace

cudaError_t launch_resolve_plane(const PlaneDev& raw, uint32_t* res, uint8_t* seg_owner, int seg_pitch, const SrcSet& S,
                                 int n, bool opaque, const SkipMap& skip, cudaStream_t stream) {
  if (raw.w <= 0 || raw.h <= 0) return cudaSuccess;
  resolve_plane_kernel<<<dim3((raw.w + kSegPixels - 1) / kSegPixels, raw.h), kSegPixels, 0, stream>>>(
      raw, res, seg_owner, seg_pitch, S, n, opaque ? 1 : 0, skip);
  return cudaGetLastError();
}

cudaError_t launch_canvas_gather(const GatherArgs& a, bool copy_blocks, cudaStream_t stream) {
  const dim3 grid((a.C.w + 255) / 256, (a.C.h + 7) / 8);
  if (copy_blocks)
    canvas_gather_kernel<true><<<grid, 256, 0, stream>>>(a);
  else
    canvas_gather_kernel<false><<<grid, 256, 0, stream>>>(a);
  return cudaGetLastError();
}

}  // namespace hmp
