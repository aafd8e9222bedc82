// hmp_generic.cu -- the stitch for the reference's other pixel pipelines: uchar3, float4 and float3
// (CudaStitchPano*<uchar3, float3>, <float4, float4>, <float3, float3>; src/pano/cudaPano3_test.cpp,
// tests/testCudaBlend.cpp). RGBA8 runs the fused kernels of hmp_gather.cu / hmp_pyramid.cu; these
// pipelines are used by the reference's tests and tools rather than its video path, so they run
// plain level-by-level kernels over float4 level buffers in HBM, with the reference's arithmetic:
//   level 0   per image, the remap over the blend region (cudaRemap.cu:60-123): the source pixel if
//             the table entry is inside the frame, else 0 (4 channels: alpha 255 under the soft-seam
//             rule for an entry that is not the 65535 sentinel)
//   down      4 channels: the alpha-aware 2x2 mean (DownAcc); 3 channels: the plain mean of the
//             in-bounds pixels (cudaBlend.cu:46-144)
//   up        4 channels: the alpha-aware bilinear upsample (up_alpha); 3 channels: the separable
//             bilinear one in the Laplacian (cudaBlend.cu:389-455) and the sequential four-tap sum
//             in the reconstruction (up_taps; cudaBlend.cu:581-672, cudaBlendN.cu:372-447)
//   blend     4 channels: blend_level / blend_level0 (the reference rules, alpha tests included);
//             3 channels: two images m*a + (1-m)*b (cudaBlend.cu:520-576), three m1*v1 + m2*v2 +
//             m3*v3 (cudaBlend3.cu:376-531), N the mask normalised by its sum (cudaBlendN.cu:199-288)
//   reconstruct  up(R^(l+1)) + blend^l; level 0 written into the canvas's write rect, packed by
//             truncation for uint8 pipelines, as is for float ones (cudaMakeFull.cu:241-258)
// and the canvas outside the write rect (or all of it for the hard seam) copied from the canvas
// plane's entries. Compiled with -fmad=false, like the fused kernels.
#include <cuda_runtime.h>

#include "hmp_blend.cuh"
#include "hmp_kernels.h"

namespace hmp {
namespace {

// Pixel of C channels, uint8 or float samples (F), at byte address p.
template <int C, bool F>
struct Px {
  static constexpr int kBytes = C * (F ? 4 : 1);
  __device__ __forceinline__ static float4 load(const char* p) {
    if constexpr (F) {
      const float* f = reinterpret_cast<const float*>(p);
      return make_float4(f[0], f[1], f[2], C == 4 ? f[3] : 0.f);
    } else {
      const unsigned char* u = reinterpret_cast<const unsigned char*>(p);
      return make_float4(float(u[0]), float(u[1]), float(u[2]), C == 4 ? float(u[3]) : 0.f);
    }
  }
  __device__ __forceinline__ static void store(char* p, const float4 v) {
    if constexpr (F) {
      float* f = reinterpret_cast<float*>(p);
      f[0] = v.x;
      f[1] = v.y;
      f[2] = v.z;
      if (C == 4) f[3] = v.w;
    } else {
      unsigned char* u = reinterpret_cast<unsigned char*>(p);
      u[0] = pack_u8(v.x);
      u[1] = pack_u8(v.y);
      u[2] = pack_u8(v.z);
      if (C == 4) u[3] = pack_u8(v.w);
    }
  }
};

// Source pixel for (owner o, packed entry e) in frame b, or the remap's fill.
template <int C, bool F>
__device__ __forceinline__ float4 fetch(const SrcSet& S, int n, int o, uint32_t e, int b, bool opaque) {
  float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
  if (o >= n) return v;
  const int sx = int(e & 0xFFFFu), sy = int(e >> 16);
  if (sx < S.w[o] && sy < S.h[o]) {
    const char* base = reinterpret_cast<const char*>(S.ptr[o]) + b * S.bstride[o] + (long long)sy * S.pitch[o];
    return Px<C, F>::load(base + (long long)sx * Px<C, F>::kBytes);
  }
  if (C == 4 && opaque && sx != 0xFFFF) v.w = 255.f;
  return v;
}

// Plain (3-channel) separable bilinear upsample of level `lo` (lw x lh) at high-res (x, y).
__device__ __forceinline__ float3 up_plain(const float4* lo, int lw, int lh, int x, int y) {
  const int gxi = x >> 1, gyi = y >> 1;
  const float dx = (x & 1) ? 0.5f : 0.f, dy = (y & 1) ? 0.5f : 0.f;
  const int gxi1 = min(gxi + 1, lw - 1), gyi1 = min(gyi + 1, lh - 1);
  const float4 v00 = lo[(long long)gyi * lw + gxi], v10 = lo[(long long)gyi * lw + gxi1];
  const float4 v01 = lo[(long long)gyi1 * lw + gxi], v11 = lo[(long long)gyi1 * lw + gxi1];
  const float ex = 1.f - dx, ey = 1.f - dy;
  const float a0 = v00.x * ex + v10.x * dx, a1 = v01.x * ex + v11.x * dx;
  const float b0 = v00.y * ex + v10.y * dx, b1 = v01.y * ex + v11.y * dx;
  const float c0 = v00.z * ex + v10.z * dx, c1 = v01.z * ex + v11.z * dx;
  return make_float3(a0 * ey + a1 * dy, b0 * ey + b1 * dy, c0 * ey + c1 * dy);
}

template <int C>
__device__ __forceinline__ float3 up_level(const float4* lo, int lw, int lh, int x, int y) {
  if constexpr (C == 4)
    return up_alpha(lo, lw, 0, 0, lw, lh, x, y);
  else
    return up_plain(lo, lw, lh, x, y);
}

// The reconstruction's upsample of 3-channel pixels: the sequential four-tap sum
// (((0 + v00 w00) + v10 w10) + v01 w01) + v11 w11 of the reference's reconstructions
// (src/cuda/cudaBlend.cu:581-672 and src/cuda/cudaBlendN.cu:372-447, whose weight sum is exactly 1
// here; cupano/ops.py:514-565). It rounds differently from the Laplacian's separable form at pixels
// with odd x and odd y once a level holds blended (non-dyadic) values.
__device__ __forceinline__ float3 up_taps(const float4* lo, int lw, int lh, int x, int y) {
  const int gxi = x >> 1, gyi = y >> 1;
  const float dx = (x & 1) ? 0.5f : 0.f, dy = (y & 1) ? 0.5f : 0.f;
  const int gxi1 = min(gxi + 1, lw - 1), gyi1 = min(gyi + 1, lh - 1);
  const float4 v00 = lo[(long long)gyi * lw + gxi], v10 = lo[(long long)gyi * lw + gxi1];
  const float4 v01 = lo[(long long)gyi1 * lw + gxi], v11 = lo[(long long)gyi1 * lw + gxi1];
  const float ex = 1.f - dx, ey = 1.f - dy;
  const float w00 = ex * ey, w10 = dx * ey, w01 = ex * dy, w11 = dx * dy;
  return make_float3((((0.f + v00.x * w00) + v10.x * w10) + v01.x * w01) + v11.x * w11,
                     (((0.f + v00.y * w00) + v10.y * w10) + v01.y * w01) + v11.y * w11,
                     (((0.f + v00.z * w00) + v10.z * w10) + v01.z * w01) + v11.z * w11);
}

// The reconstruction's upsample: alpha-aware for 4 channels, the four-tap sum for 3.
template <int C>
__device__ __forceinline__ float3 up_recon(const float4* lo, int lw, int lh, int x, int y) {
  if constexpr (C == 4)
    return up_alpha(lo, lw, 0, 0, lw, lh, x, y);
  else
    return up_taps(lo, lw, lh, x, y);
}

// 3-channel blends (no alpha): weights m[0..n) of the level's pixel.
template <int RULE, int NMAX>
__device__ __forceinline__ float4 blend_rgb(int n, const float4* L, const float* m) {
  float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
  if constexpr (RULE == kRuleTwo) {
    const float m0 = m[0], mm1 = 1.f - m0;
    r = make_float4(m0 * L[0].x + mm1 * L[1].x, m0 * L[0].y + mm1 * L[1].y, m0 * L[0].z + mm1 * L[1].z, 0.f);
  } else if constexpr (RULE == kRuleThree) {
    r = make_float4((m[0] * L[0].x + m[1] * L[1].x) + m[2] * L[2].x, (m[0] * L[0].y + m[1] * L[1].y) + m[2] * L[2].y,
                    (m[0] * L[0].z + m[1] * L[1].z) + m[2] * L[2].z, 0.f);
  } else {
    float w[NMAX], sum = 0.f;
#pragma unroll
    for (int k = 0; k < NMAX; ++k) {
      w[k] = k < n ? m[k] : 0.f;
      if (k < n) sum += w[k];
    }
    if (sum > 0.f) {
#pragma unroll
      for (int k = 0; k < NMAX; ++k)
        if (k < n) w[k] /= sum;
    }
#pragma unroll
    for (int k = 0; k < NMAX; ++k) {
      if (k < n) {
        r.x += w[k] * L[k].x;
        r.y += w[k] * L[k].y;
        r.z += w[k] * L[k].z;
      }
    }
  }
  return r;
}

template <int C, bool F>
__global__ void gen_level0_kernel(const __grid_constant__ GenArgs a) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  const int k = int(blockIdx.z) % a.n, b = int(blockIdx.z) / a.n;
  const int lw0 = a.lw[0], lh0 = a.lh[0];
  if (x >= lw0) return;
  const PlaneDev& P = a.slot[k];
  const int rx = x - P.x0, ry = y - P.y0;
  uint32_t e = 0xFFFFFFFFu;
  int o = P.owner != nullptr ? 0xFF : k;
  if ((unsigned)rx < (unsigned)P.w && (unsigned)ry < (unsigned)P.h) {
    e = P.map[(long long)ry * P.map_pitch + rx];
    if (P.owner != nullptr) o = int(P.owner[(long long)ry * P.owner_pitch + rx]);
  }
  a.G[k][0][((long long)b * lh0 + y) * lw0 + x] = fetch<C, F>(a.S, a.n, o, e, b, a.opaque != 0);
}

template <int C>
__global__ void gen_down_kernel(const __grid_constant__ GenArgs a, int l) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  const int k = int(blockIdx.z) % a.n, b = int(blockIdx.z) / a.n;
  const int iw = a.lw[l - 1], ih = a.lh[l - 1], ow = a.lw[l], oh = a.lh[l];
  if (x >= ow) return;
  const float4* in = a.G[k][l - 1] + (long long)b * iw * ih;
  float4 r;
  if constexpr (C == 4) {
    DownAcc acc;
    for (int dy = 0; dy < 2; ++dy)
      for (int dx = 0; dx < 2; ++dx) {
        const int ix = 2 * x + dx, iy = 2 * y + dy;
        if (ix < iw && iy < ih) acc.add(in[(long long)iy * iw + ix]);
      }
    r = acc.result();
  } else {
    float s0 = 0.f, s1 = 0.f, s2 = 0.f;
    int cnt = 0;
    for (int dy = 0; dy < 2; ++dy)
      for (int dx = 0; dx < 2; ++dx) {
        const int ix = 2 * x + dx, iy = 2 * y + dy;
        if (ix < iw && iy < ih) {
          const float4 p = in[(long long)iy * iw + ix];
          s0 += p.x;
          s1 += p.y;
          s2 += p.z;
          ++cnt;
        }
      }
    const float c = float(cnt);  // 1, 2 or 4 (3 taps never occur without alpha holes)
    r = make_float4(s0 / c, s1 / c, s2 / c, 0.f);
  }
  a.G[k][l][((long long)b * oh + y) * ow + x] = r;
}

// Level l: the Laplacians of every image, their blend and the reconstruction (into `rout`, or into
// the canvas's write rect at level 0).
template <int C, bool F, int RULE, int NMAX>
__global__ void gen_up_kernel(const __grid_constant__ GenArgs a, int l, const float4* rnext, float4* rout) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, b = blockIdx.z;
  const int w = a.lw[l], h = a.lh[l];
  if (x >= w) return;
  const bool last = l == a.levels - 1;
  const int nw = a.lw[l + 1], nh = a.lh[l + 1];
  const int n = RULE == kRuleNway ? a.n : NMAX;
  float4 lap[NMAX];
#pragma unroll
  for (int k = 0; k < NMAX; ++k) {
    lap[k] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (k < n) {
      float4 g = a.G[k][l][((long long)b * h + y) * w + x];
      if (!last) {
        const float3 up = up_level<C>(a.G[k][l + 1] + (long long)b * nw * nh, nw, nh, x, y);
        g.x = g.x - up.x;
        g.y = g.y - up.y;
        g.z = g.z - up.z;
      }
      lap[k] = g;
    }
  }
  float4 r;
  if constexpr (C == 4) {
    r = l == 0 ? blend_level0<RULE, NMAX>(n, lap, int(a.mask0[(long long)y * a.mask0_pitch + x]))
               : blend_level<RULE, NMAX>(n, lap, a.maskL[l] + ((long long)y * w + x) * a.K);
  } else {
    float m[NMAX];
    if (l == 0) {
      const int v = int(a.mask0[(long long)y * a.mask0_pitch + x]);
#pragma unroll
      for (int k = 0; k < NMAX; ++k) m[k] = RULE == kRuleTwo ? (k == 0 ? float(v) : 0.f) : (k == v ? 1.f : 0.f);
    } else {
      const float* ml = a.maskL[l] + ((long long)y * w + x) * a.K;
#pragma unroll
      for (int k = 0; k < NMAX; ++k) m[k] = k < a.K ? ml[k] : 0.f;
    }
    r = blend_rgb<RULE, NMAX>(n, lap, m);
  }
  if (!last) {
    const float3 up = up_recon<C>(rnext + (long long)b * nw * nh, nw, nh, x, y);
    r.x = up.x + r.x;
    r.y = up.y + r.y;
    r.z = up.z + r.z;
  }
  if (l > 0) {
    rout[((long long)b * h + y) * w + x] = r;
    return;
  }
  if (x < a.wx0 || x >= a.wx1 || y < a.wy0 || y >= a.wy1) return;
  char* row = reinterpret_cast<char*>(a.C.ptr) + b * a.C.bstride + (long long)(y + a.cy_off) * a.C.pitch;
  Px<C, F>::store(row + (long long)(x + a.cx_off) * Px<C, F>::kBytes, r);
}

// Canvas pixels outside the skipped rect from the canvas plane's packed entries.
template <int C, bool F>
__global__ void gen_canvas_kernel(const __grid_constant__ GatherArgs g, int opaque) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, b = blockIdx.z;
  if (x >= g.C.w) return;
  if (x >= g.skip_x0 && x < g.skip_x1 && y >= g.skip_y0 && y < g.skip_y1) return;
  const PlaneDev& P = g.P;
  const int o = P.owner ? int(P.owner[(long long)y * P.owner_pitch + x]) : P.default_owner;
  const uint32_t e = P.map[(long long)y * P.map_pitch + x];
  const float4 v = fetch<C, F>(g.S, g.n_owners, o, e, b, opaque != 0);
  char* row = reinterpret_cast<char*>(g.C.ptr) + b * g.C.bstride + (long long)y * g.C.pitch;
  Px<C, F>::store(row + (long long)x * Px<C, F>::kBytes, v);
}

dim3 grid_of(int w, int h, int z) { return dim3((w + 255) / 256, h, z); }

template <int C, bool F>
cudaError_t run_pyramid(const GenArgs& a, int rule, int batch, float4* const* r, cudaStream_t s) {
  const int L = a.levels;
  gen_level0_kernel<C, F><<<grid_of(a.lw[0], a.lh[0], batch * a.n), 256, 0, s>>>(a);
  for (int l = 1; l < L; ++l) gen_down_kernel<C><<<grid_of(a.lw[l], a.lh[l], batch * a.n), 256, 0, s>>>(a, l);
  for (int l = L - 1; l >= 0; --l) {
    const float4* rnext = l + 1 < L ? r[(l + 1) & 1] : nullptr;
    float4* rout = l > 0 ? r[l & 1] : nullptr;
    const dim3 grid = grid_of(a.lw[l], a.lh[l], batch);
    if (rule == kRuleTwo)
      gen_up_kernel<C, F, kRuleTwo, 2><<<grid, 256, 0, s>>>(a, l, rnext, rout);
    else if (rule == kRuleThree)
      gen_up_kernel<C, F, kRuleThree, 3><<<grid, 256, 0, s>>>(a, l, rnext, rout);
    else
      gen_up_kernel<C, F, kRuleNway, kDevMaxImages><<<grid, 256, 0, s>>>(a, l, rnext, rout);
  }
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_generic_pyramid(const GenArgs& a, int channels, bool is_float, int rule, int batch,
                                   float4* const* r, cudaStream_t stream) {
  if (channels == 4) return is_float ? run_pyramid<4, true>(a, rule, batch, r, stream)
                                     : run_pyramid<4, false>(a, rule, batch, r, stream);
  return is_float ? run_pyramid<3, true>(a, rule, batch, r, stream) : run_pyramid<3, false>(a, rule, batch, r, stream);
}

cudaError_t launch_generic_canvas(const GatherArgs& g, int channels, bool is_float, bool opaque, cudaStream_t stream) {
  const dim3 grid = grid_of(g.C.w, g.C.h, g.batch);
  if (channels == 4 && is_float)
    gen_canvas_kernel<4, true><<<grid, 256, 0, stream>>>(g, opaque ? 1 : 0);
  else if (channels == 4)
    gen_canvas_kernel<4, false><<<grid, 256, 0, stream>>>(g, opaque ? 1 : 0);
  else if (is_float)
    gen_canvas_kernel<3, true><<<grid, 256, 0, stream>>>(g, opaque ? 1 : 0);
  else
    gen_canvas_kernel<3, false><<<grid, 256, 0, stream>>>(g, opaque ? 1 : 0);
  return cudaGetLastError();
}

int generic_launches(int levels, bool canvas) { return (canvas ? 1 : 0) + (levels > 0 ? 2 * levels : 0); }

}  // namespace hmp
