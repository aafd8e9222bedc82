// hmp_gather.cu -- canvas gather kernel (hard seam, and the canvas outside the blend region).
//
// Replaces, per frame, the reference's canvas memset plus one remap launch per image
// (src/pano/cudaPano.inl:186-359 with src/cuda/cudaRemap.cu:203-294; the three-image fused hard
// seam src/cuda/cudaFusedKernels3.cu:124-217; the N-image fused hard seam cudaRemap.cu:251-294).
// One pass over the canvas: each thread owns 4 consecutive pixels of a row, loads their 4 owner
// bytes (32-bit load) and 4 packed table entries (128-bit load), gathers the source pixels
// (read-only path) for every frame of the batch and stores 16 bytes. Pixels with no owner get
// zero, so no memset is needed. HBM-bound: 1 + 4 + 4 + 4 = 13 bytes per canvas pixel.
#include "hmp_kernels.h"

namespace hmp {
namespace {

__device__ __forceinline__ uchar4 fetch(const SrcSet& S, int o, uint32_t e, int b, bool opaque) {
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

template <bool kVec>
__global__ void __launch_bounds__(256) canvas_gather_kernel(const __grid_constant__ GatherArgs a) {
  const int x4 = (blockIdx.x * blockDim.x + threadIdx.x) * 4;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int W = a.C.w;
  if (y >= a.C.h || x4 >= W) return;
  const bool row_skip = y >= a.skip_y0 && y < a.skip_y1;
  if (row_skip && x4 >= a.skip_x0 && x4 + 4 <= a.skip_x1) return;
  const int nv = min(4, W - x4);
  const bool partial = nv < 4 || (row_skip && x4 + 4 > a.skip_x0 && x4 < a.skip_x1);

  int own[4];
  uint32_t ent[4];
  const uint8_t* orow = a.P.owner ? a.P.owner + (long long)y * a.P.owner_pitch : nullptr;
  const uint32_t* mrow = a.P.map + (long long)y * a.P.map_pitch;
  if (kVec && nv == 4) {
    const uint4 m4 = __ldg(reinterpret_cast<const uint4*>(mrow + x4));
    ent[0] = m4.x;
    ent[1] = m4.y;
    ent[2] = m4.z;
    ent[3] = m4.w;
    if (orow) {
      const uchar4 o4 = __ldg(reinterpret_cast<const uchar4*>(orow + x4));
      own[0] = o4.x;
      own[1] = o4.y;
      own[2] = o4.z;
      own[3] = o4.w;
    } else {
      own[0] = own[1] = own[2] = own[3] = a.P.default_owner;
    }
  } else {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if (j < nv) {
        ent[j] = __ldg(mrow + x4 + j);
        own[j] = orow ? int(__ldg(orow + x4 + j)) : a.P.default_owner;
      } else {
        ent[j] = 0xFFFFFFFFu;
        own[j] = 0xFF;
      }
    }
  }
  const bool opaque = a.opaque != 0;
  for (int b = 0; b < a.batch; ++b) {
    uchar4 px[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) px[j] = fetch(a.S, own[j], ent[j], b, opaque);
    uchar4* crow = reinterpret_cast<uchar4*>(reinterpret_cast<char*>(a.C.ptr) + b * a.C.bstride + y * a.C.pitch);
    if (kVec && !partial) {
      uint4 v;
      v.x = *reinterpret_cast<const uint32_t*>(&px[0]);
      v.y = *reinterpret_cast<const uint32_t*>(&px[1]);
      v.z = *reinterpret_cast<const uint32_t*>(&px[2]);
      v.w = *reinterpret_cast<const uint32_t*>(&px[3]);
      *reinterpret_cast<uint4*>(crow + x4) = v;
    } else {
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int x = x4 + j;
        if (j < nv && !(row_skip && x >= a.skip_x0 && x < a.skip_x1)) crow[x] = px[j];
      }
    }
  }
}

}  // namespace

cudaError_t launch_canvas_gather(const GatherArgs& a, bool vec, cudaStream_t stream) {
  const dim3 block(64, 4);
  const int groups = (a.C.w + 3) / 4;
  const dim3 grid((groups + block.x - 1) / block.x, (a.C.h + block.y - 1) / block.y);
  if (vec)
    canvas_gather_kernel<true><<<grid, block, 0, stream>>>(a);
  else
    canvas_gather_kernel<false><<<grid, block, 0, stream>>>(a);
  return cudaGetLastError();
}

}  // namespace hmp
