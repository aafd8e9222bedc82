// hmp_pyramid.cu -- fused Laplacian-pyramid blend of the reference's soft seam.
//
// The reference runs ~6L launches per frame: a downsample and a mask downsample per level, a
// Laplacian per image and level, a blend per level, a reconstruct per level, plus device copies
// (src/cuda/cudaBlend.cu:847-1049, cudaBlend3.cu:881-1206, cudaBlendN.cu:649-828). Here the whole
// pyramid is two launches:
//
//  * pyr_down: the 2x2 box downsample has no halo, so a CTA that owns an aligned T x T level-0
//    tile (T a multiple of 2^(L-1)) builds every Gaussian level of that tile in shared memory,
//    gathering level 0 straight from the sources through the slot planes (remap + level-0
//    downsample fused). Levels >= 1 go to HBM (FP32 or FP16 storage).
//  * pyr_up: a CTA that owns a level-0 tile of the write region walks from the coarsest level
//    down. At level l it needs its tile plus a 1-2 pixel halo (the bilinear upsample reads
//    floor(x/2) and floor(x/2)+1), so it loads G_k^l of every image for that region, forms the
//    Laplacians G_k^l - up(G_k^{l+1}), blends them with the mask pyramid, adds up(R^{l+1}) and
//    keeps R^l in shared memory. At level 0 it packs straight into the canvas. Laplacians,
//    blended levels and reconstructions never touch HBM.
//
// Arithmetic follows the reference order exactly (this file is compiled with -fmad=false so no
// product is fused into a sum): downsample sums in (0,0),(1,0),(0,1),(1,1) order divided by the
// count; alpha-aware bilinear taps in 00,10,01,11 order over taps with alpha != 0; blends as in
// cudaBlend.cu:520-576, cudaBlend3.cu:376-531, cudaBlendN.cu:199-288.
#include "hmp_kernels.h"

namespace hmp {
namespace {

constexpr int kRuleNway = 1, kRuleTwo = 2, kRuleThree = 3;

// Alpha-aware 2x2 mean of four level-l pixels (src/cuda/cudaBlend.cu:46-144).
struct DownAcc {
  float s0 = 0.f, s1 = 0.f, s2 = 0.f, amax = 0.f;
  int cnt = 0;
  __device__ __forceinline__ void add(const float4 p) {
    if (p.w > amax) amax = p.w;
    if (p.w != 0.f) {
      s0 += p.x;
      s1 += p.y;
      s2 += p.z;
      ++cnt;
    }
  }
  __device__ __forceinline__ float4 result() const {
    if (cnt == 0) return make_float4(0.f, 0.f, 0.f, amax);
    const float c = float(cnt);
    return make_float4(s0 / c, s1 / c, s2 / c, amax);
  }
};

template <typename Store>
__global__ void __launch_bounds__(256) pyr_down_kernel(const __grid_constant__ PyrArgs a) {
  extern __shared__ float4 sm[];
  const int TD = a.tile, T1 = TD >> 1;
  float4* bufA = sm;
  float4* bufB = sm + T1 * T1;
  const int b = blockIdx.z;
  const int X0 = blockIdx.x * TD, Y0 = blockIdx.y * TD;
  const bool opaque = a.opaque != 0;
  const int L = a.levels;
  for (int k = 0; k < a.n; ++k) {
    const PlaneDev& P = a.slot[k];
    // A tile that misses the slot's rect only produces zeros, which the buffers already hold.
    if (X0 >= P.x0 + P.w || Y0 >= P.y0 + P.h || X0 + TD <= P.x0 || Y0 + TD <= P.y0) continue;
    // Level 1 straight from the sources.
    {
      Store* G1 = static_cast<Store*>(a.G[k][1]) + (long long)b * a.lw[1] * a.lh[1];
      for (int i = threadIdx.x; i < T1 * T1; i += blockDim.x) {
        const int tx = i % T1, ty = i / T1;
        const int gx = (X0 >> 1) + tx, gy = (Y0 >> 1) + ty;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (gx < a.lw[1] && gy < a.lh[1]) {
          DownAcc acc;
#pragma unroll
          for (int dy = 0; dy < 2; ++dy)
#pragma unroll
            for (int dx = 0; dx < 2; ++dx) {
              const int ix = 2 * gx + dx, iy = 2 * gy + dy;
              if (ix < a.lw[0] && iy < a.lh[0]) acc.add(to_f4(plane_pixel(a.S, P, ix, iy, b, opaque)));
            }
          v = acc.result();
          store_level(G1 + (long long)gy * a.lw[1] + gx, v);
        }
        bufA[i] = v;
      }
    }
    __syncthreads();
    float4* src = bufA;
    float4* dst = bufB;
    int T = T1;
    for (int l = 2; l < L; ++l) {
      const int Tn = T >> 1;
      Store* Gl = static_cast<Store*>(a.G[k][l]) + (long long)b * a.lw[l] * a.lh[l];
      for (int i = threadIdx.x; i < Tn * Tn; i += blockDim.x) {
        const int tx = i % Tn, ty = i / Tn;
        const int gx = (X0 >> l) + tx, gy = (Y0 >> l) + ty;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (gx < a.lw[l] && gy < a.lh[l]) {
          DownAcc acc;
#pragma unroll
          for (int dy = 0; dy < 2; ++dy)
#pragma unroll
            for (int dx = 0; dx < 2; ++dx) {
              if (2 * gx + dx < a.lw[l - 1] && 2 * gy + dy < a.lh[l - 1])
                acc.add(src[(2 * ty + dy) * T + 2 * tx + dx]);
            }
          v = acc.result();
          store_level(Gl + (long long)gy * a.lw[l] + gx, v);
        }
        dst[i] = v;
      }
      __syncthreads();
      float4* t = src;
      src = dst;
      dst = t;
      T = Tn;
    }
  }
}

// Alpha-aware bilinear upsample of a shared-memory region (origin ax, ay; row width rw) of a
// level of size lw x lh, sampled for high-res pixel (x, y): top-left aligned, gx = x/2, taps
// floor and floor+1 clamped to the level, only taps with alpha != 0, renormalised
// (src/cuda/cudaBlend.cu:389-455, 581-672).
__device__ __forceinline__ float3 up_alpha(const float4* buf, int rw, int ax, int ay, int lw, int lh, int x, int y) {
  const int gxi = x >> 1, gyi = y >> 1;
  const int gxi1 = min(gxi + 1, lw - 1), gyi1 = min(gyi + 1, lh - 1);
  const float dx = (x & 1) ? 0.5f : 0.f, dy = (y & 1) ? 0.5f : 0.f;
  const float w00 = (1.f - dx) * (1.f - dy), w10 = dx * (1.f - dy), w01 = (1.f - dx) * dy, w11 = dx * dy;
  const float4 p00 = buf[(gyi - ay) * rw + (gxi - ax)];
  const float4 p10 = buf[(gyi - ay) * rw + (gxi1 - ax)];
  const float4 p01 = buf[(gyi1 - ay) * rw + (gxi - ax)];
  const float4 p11 = buf[(gyi1 - ay) * rw + (gxi1 - ax)];
  float sw = 0.f, s0 = 0.f, s1 = 0.f, s2 = 0.f;
  if (p00.w != 0.f) {
    sw += w00;
    s0 += p00.x * w00;
    s1 += p00.y * w00;
    s2 += p00.z * w00;
  }
  if (p10.w != 0.f) {
    sw += w10;
    s0 += p10.x * w10;
    s1 += p10.y * w10;
    s2 += p10.z * w10;
  }
  if (p01.w != 0.f) {
    sw += w01;
    s0 += p01.x * w01;
    s1 += p01.y * w01;
    s2 += p01.z * w01;
  }
  if (p11.w != 0.f) {
    sw += w11;
    s0 += p11.x * w11;
    s1 += p11.y * w11;
    s2 += p11.z * w11;
  }
  if (sw > 0.f) return make_float3(s0 / sw, s1 / sw, s2 / sw);
  return make_float3(0.f, 0.f, 0.f);
}

// Two-image rule (src/cuda/cudaBlend.cu:520-576).
__device__ __forceinline__ float4 blend_two(const float4 a, const float4 b, const float m) {
  if (a.w == 0.f) return b;
  if (b.w == 0.f) return a;
  const float mm1 = 1.f - m;
  return make_float4(m * a.x + mm1 * b.x, m * a.y + mm1 * b.y, m * a.z + mm1 * b.z, b.w);
}

// Three-image rule (src/cuda/cudaBlend3.cu:376-531).
__device__ __forceinline__ float4 blend_three(const float4* L, float m0, float m1, float m2) {
  if (L[0].w == 0.f) m0 = 0.f;
  if (L[1].w == 0.f) m1 = 0.f;
  if (L[2].w == 0.f) m2 = 0.f;
  const float sum = (m0 + m1) + m2;
  if (!(sum > 0.f)) {
    int src = -1;
    float amax = 0.f;
#pragma unroll
    for (int k = 0; k < 3; ++k)
      if (L[k].w > amax) {
        amax = L[k].w;
        src = k;
      }
    return src < 0 ? make_float4(0.f, 0.f, 0.f, 0.f) : L[src];
  }
  m0 /= sum;
  m1 /= sum;
  m2 /= sum;
  float aout = 0.f;
  if (m0 > 0.f && L[0].w > aout) aout = L[0].w;
  if (m1 > 0.f && L[1].w > aout) aout = L[1].w;
  if (m2 > 0.f && L[2].w > aout) aout = L[2].w;
  return make_float4((m0 * L[0].x + m1 * L[1].x) + m2 * L[2].x, (m0 * L[0].y + m1 * L[1].y) + m2 * L[2].y,
                     (m0 * L[0].z + m1 * L[1].z) + m2 * L[2].z, aout);
}

// N-way rule (src/cuda/cudaBlendN.cu:199-288).
template <int NMAX>
__device__ __forceinline__ float4 blend_nway(const float4* L, int n, float* w) {
  float sumw = 0.f;
#pragma unroll
  for (int k = 0; k < NMAX; ++k)
    if (k < n) sumw += w[k];
  if (sumw > 0.f) {
#pragma unroll
    for (int k = 0; k < NMAX; ++k)
      if (k < n) w[k] /= sumw;
  }
  float sumw2 = 0.f, amax = 0.f;
  int aidx = -1;
#pragma unroll
  for (int k = 0; k < NMAX; ++k) {
    if (k < n) {
      const float al = L[k].w;
      if (al > amax) {
        amax = al;
        aidx = k;
      }
      if (al == 0.f) w[k] = 0.f;
      sumw2 += w[k];
    }
  }
  if (!(sumw2 > 0.f)) {
    float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int k = 0; k < NMAX; ++k)
      if (k == aidx && amax != 0.f) r = L[k];
    return r;
  }
#pragma unroll
  for (int k = 0; k < NMAX; ++k)
    if (k < n) w[k] /= sumw2;
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
  for (int k = 0; k < NMAX; ++k) {
    if (k < n) {
      acc.x += w[k] * L[k].x;
      acc.y += w[k] * L[k].y;
      acc.z += w[k] * L[k].z;
      if (w[k] != 0.f && L[k].w > acc.w) acc.w = L[k].w;
    }
  }
  return acc;
}

template <int RULE, int NMAX>
__device__ __forceinline__ float4 blend_pixel(const PyrArgs& a, const float4* lap, int l, int px, int py) {
  if (RULE == kRuleTwo) {
    float m;
    if (l == 0)
      m = float(a.mask0[(long long)py * a.mask0_pitch + px]);
    else
      m = a.maskL[l][(long long)py * a.lw[l] + px];
    return blend_two(lap[0], lap[1], m);
  } else if (RULE == kRuleThree) {
    float m[3];
    if (l == 0) {
      const int label = a.mask0[(long long)py * a.mask0_pitch + px];
#pragma unroll
      for (int k = 0; k < 3; ++k) m[k] = label == k ? 1.f : 0.f;
    } else {
      const float* mp = a.maskL[l] + ((long long)py * a.lw[l] + px) * 3;
#pragma unroll
      for (int k = 0; k < 3; ++k) m[k] = mp[k];
    }
    return blend_three(lap, m[0], m[1], m[2]);
  } else {
    float w[NMAX];
    if (l == 0) {
      const int label = a.mask0[(long long)py * a.mask0_pitch + px];
#pragma unroll
      for (int k = 0; k < NMAX; ++k) w[k] = label == k ? 1.f : 0.f;
    } else {
      const float* mp = a.maskL[l] + ((long long)py * a.lw[l] + px) * a.K;
#pragma unroll
      for (int k = 0; k < NMAX; ++k) w[k] = k < a.n ? mp[k] : 0.f;
    }
    return blend_nway<NMAX>(lap, a.n, w);
  }
}

template <int RULE, int NMAX, typename Store>
__global__ void __launch_bounds__(256) pyr_up_kernel(const __grid_constant__ PyrArgs a) {
  extern __shared__ float4 sm[];
  const int n = a.n;
  // Shared memory: G for odd levels [n][rm_odd], G for even levels [n][rm_even], then R for odd
  // and even levels. Level 0 is never stored.
  float4* g_odd = sm;
  float4* g_even = g_odd + n * a.rm_odd;
  float4* r_odd = g_even + n * a.rm_even;
  float4* r_even = r_odd + a.rm_odd;
  const int TU = a.tile;
  const int b = blockIdx.z;
  const int X0 = (a.tx0 + blockIdx.x) * TU, Y0 = (a.ty0 + blockIdx.y) * TU;
  const int L = a.levels, c = L - 1;
  int ax[kDevMaxLevels], ay[kDevMaxLevels], bx[kDevMaxLevels], by[kDevMaxLevels];
  ax[0] = X0;
  ay[0] = Y0;
  bx[0] = min(X0 + TU, a.lw[0]);
  by[0] = min(Y0 + TU, a.lh[0]);
#pragma unroll
  for (int l = 1; l < kDevMaxLevels; ++l) {
    if (l < L) {
      ax[l] = ax[l - 1] >> 1;
      ay[l] = ay[l - 1] >> 1;
      bx[l] = min(((bx[l - 1] - 1) >> 1) + 2, a.lw[l]);
      by[l] = min(((by[l - 1] - 1) >> 1) + 2, a.lh[l]);
    }
  }
  const bool opaque = a.opaque != 0;
  for (int l = c; l >= 0; --l) {
    const int rw = bx[l] - ax[l], rh = by[l] - ay[l];
    float4* gcur = (l & 1) ? g_odd : g_even;
    float4* gprev = (l & 1) ? g_even : g_odd;
    const int rm_cur = (l & 1) ? a.rm_odd : a.rm_even;
    const int rm_prev = (l & 1) ? a.rm_even : a.rm_odd;
    float4* rcur = (l & 1) ? r_odd : r_even;
    const float4* rprev = (l & 1) ? r_even : r_odd;
    if (l >= 1) {
      const int npx = rw * rh;
      for (int i = threadIdx.x; i < n * npx; i += blockDim.x) {
        const int k = i / npx, j = i - k * npx;
        const int py = ay[l] + j / rw, px = ax[l] + j % rw;
        const Store* Gl = static_cast<const Store*>(a.G[k][l]) + (long long)b * a.lw[l] * a.lh[l];
        gcur[k * rm_cur + j] = load_level(Gl + (long long)py * a.lw[l] + px);
      }
      __syncthreads();
    }
    const int rw1 = l < c ? bx[l + 1] - ax[l + 1] : 0;
    for (int i = threadIdx.x; i < rw * rh; i += blockDim.x) {
      const int py = ay[l] + i / rw, px = ax[l] + i % rw;
      if (l == 0 && (px < a.wx0 || px >= a.wx1 || py < a.wy0 || py >= a.wy1)) continue;
      float4 lap[NMAX];
#pragma unroll
      for (int k = 0; k < NMAX; ++k) {
        if (k < n) {
          float4 g = l == 0 ? to_f4(plane_pixel(a.S, a.slot[k], px, py, b, opaque)) : gcur[k * rm_cur + i];
          if (l < c) {
            const float3 up = up_alpha(gprev + k * rm_prev, rw1, ax[l + 1], ay[l + 1], a.lw[l + 1], a.lh[l + 1], px, py);
            g.x = g.x - up.x;
            g.y = g.y - up.y;
            g.z = g.z - up.z;
          }
          lap[k] = g;
        } else {
          lap[k] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
      }
      float4 r = blend_pixel<RULE, NMAX>(a, lap, l, px, py);
      if (l < c) {
        const float3 up = up_alpha(rprev, rw1, ax[l + 1], ay[l + 1], a.lw[l + 1], a.lh[l + 1], px, py);
        r.x = up.x + r.x;
        r.y = up.y + r.y;
        r.z = up.z + r.z;
      }
      if (l > 0) {
        rcur[i] = r;
      } else {
        uchar4* crow = reinterpret_cast<uchar4*>(reinterpret_cast<char*>(a.C.ptr) + b * a.C.bstride +
                                                 (long long)(py + a.cy_off) * a.C.pitch);
        crow[px + a.cx_off] = pack_rgba(r);
      }
    }
    __syncthreads();
  }
}

template <int RULE, int NMAX, typename Store>
void set_up_attr() {
  cudaFuncSetAttribute(pyr_up_kernel<RULE, NMAX, Store>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
}

}  // namespace

size_t pyr_down_smem(int tile) {
  const int t1 = tile / 2, t2 = tile / 4;
  return size_t(t1 * t1 + t2 * t2) * sizeof(float4);
}

size_t pyr_up_smem(int n, int rm_odd, int rm_even) {
  return size_t((n + 1) * (rm_odd + rm_even)) * sizeof(float4);
}

cudaError_t kernels_init() {
  cudaFuncSetAttribute(pyr_down_kernel<float4>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
  cudaFuncSetAttribute(pyr_down_kernel<half4>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
  set_up_attr<kRuleTwo, 2, float4>();
  set_up_attr<kRuleTwo, 2, half4>();
  set_up_attr<kRuleThree, 3, float4>();
  set_up_attr<kRuleThree, 3, half4>();
  set_up_attr<kRuleNway, 8, float4>();
  set_up_attr<kRuleNway, 8, half4>();
  return cudaGetLastError();
}

cudaError_t launch_pyr_down(const PyrArgs& a, int storage, dim3 grid, cudaStream_t stream) {
  const size_t smem = pyr_down_smem(a.tile);
  if (storage == 1)
    pyr_down_kernel<half4><<<grid, 256, smem, stream>>>(a);
  else
    pyr_down_kernel<float4><<<grid, 256, smem, stream>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_pyr_up(const PyrArgs& a, int rule, int storage, dim3 grid, size_t smem, cudaStream_t stream) {
  const bool h = storage == 1;
  if (rule == kRuleTwo) {
    if (h)
      pyr_up_kernel<kRuleTwo, 2, half4><<<grid, 256, smem, stream>>>(a);
    else
      pyr_up_kernel<kRuleTwo, 2, float4><<<grid, 256, smem, stream>>>(a);
  } else if (rule == kRuleThree) {
    if (h)
      pyr_up_kernel<kRuleThree, 3, half4><<<grid, 256, smem, stream>>>(a);
    else
      pyr_up_kernel<kRuleThree, 3, float4><<<grid, 256, smem, stream>>>(a);
  } else {
    if (h)
      pyr_up_kernel<kRuleNway, 8, half4><<<grid, 256, smem, stream>>>(a);
    else
      pyr_up_kernel<kRuleNway, 8, float4><<<grid, 256, smem, stream>>>(a);
  }
  return cudaGetLastError();
}

}  // namespace hmp
