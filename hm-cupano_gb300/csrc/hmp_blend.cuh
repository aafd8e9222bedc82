// hmp_blend.cuh -- device helpers shared by the pyramid kernels (box and Binomial5 filters):
// slot-plane lookups, the reference's blend rules, and the one-hot "pick" that lets the up-pass
// compute a single Laplacian where the blend weights are one-hot.
#pragma once

#include "hmp_kernels.h"

namespace hmp {

constexpr int kRuleNway = 1, kRuleTwo = 2, kRuleThree = 3;

// Table lookup of slot k at (x, y); the owner is k unless the slot has an owner plane.
__device__ __forceinline__ void slot_lookup(const PlaneDev& P, int k, int x, int y, int& owner, uint32_t& entry) {
  const int rx = x - P.x0, ry = y - P.y0;
  owner = 0xFF;
  entry = 0xFFFFFFFFu;
  if ((unsigned)rx >= (unsigned)P.w || (unsigned)ry >= (unsigned)P.h) return;
  owner = P.owner ? int(__ldg(P.owner + (long long)ry * P.owner_pitch + rx)) : k;
  entry = __ldg(P.map + (long long)ry * P.map_pitch + rx);
}

// Source pixel of slot k for a looked-up (owner, entry). A slot without an owner plane only ever
// reads image k (outside its plane the entry is the sentinel, which reads as zero), so it skips
// the owner select.
template <int NMAX>
__device__ __forceinline__ uchar4 slot_fetch(const PyrArgs& a, int k, int own, uint32_t e, int b, bool opaque) {
  if (a.slot[k].owner != nullptr) return fetch_sel<NMAX>(a.S, own, e, b, opaque);
  const int sx = int(e & 0xFFFFu), sy = int(e >> 16);
  uchar4 out = make_uchar4(0, 0, 0, 0);
  if (sx < a.S.w[k] && sy < a.S.h[k]) {
    const char* base = reinterpret_cast<const char*>(a.S.ptr[k]) + b * a.S.bstride[k];
    out = __ldg(reinterpret_cast<const uchar4*>(base + (long long)sy * int(a.S.pitch[k])) + sx);
  } else if (opaque && sx != 0xFFFF) {
    out.w = 255;
  }
  return out;
}

// Blends whose weights are one-hot need a single Laplacian. With weight 1 on image s and 0 on
// the others, every rule below returns Lap_s's colour up to the sign of a zero (1*x + 0*y = x
// unless x is a zero) and an alpha known from the alphas alone; a zero's sign never changes a
// later non-zero sum, product or alpha test, and the uint8 pack maps both zeros to 0. So the
// up-pass computes the Laplacian of the picked image only:
//   pick >= 0 : the result is Lap_pick's colour with the alpha of blend_alpha();
//   kPickNone : the result is (0, 0, 0, 0);
//   kPickAll  : fractional weights, the full blend of every Laplacian.
constexpr int kPickNone = -1, kPickAll = -2;

// First image of strictly largest non-zero alpha (the rules' fallback when no weighted image has
// alpha), or kPickNone.
template <int NMAX>
__device__ __forceinline__ int pick_max_alpha(int n, const float* al) {
  float amax = 0.f;
  int idx = kPickNone;
#pragma unroll
  for (int k = 0; k < NMAX; ++k)
    if (k < n && al[k] > amax) {
      amax = al[k];
      idx = k;
    }
  return idx;
}

// Level 0: the seam value v is the two-image weight of image 1, or the label (one-hot weights).
template <int RULE, int NMAX>
__device__ __forceinline__ int blend_pick0(int n, const float* al, int v) {
  if (RULE == kRuleTwo) {
    if (al[0] == 0.f) return 1;  // blend_two returns b
    if (al[1] == 0.f) return 0;  // blend_two returns a
    if (v == 1) return 0;
    if (v == 0) return 1;
    return kPickAll;
  }
  float alv = 0.f;
#pragma unroll
  for (int k = 0; k < NMAX; ++k)
    if (k == v) alv = al[k];
  if (v < n && alv != 0.f) return v;
  return pick_max_alpha<NMAX>(n, al);
}

// Levels >= 1: mask values m[0..K).
template <int RULE, int NMAX>
__device__ __forceinline__ int blend_pick(int n, const float* al, const float* m) {
  if (RULE == kRuleTwo) {
    if (al[0] == 0.f) return 1;
    if (al[1] == 0.f) return 0;
    if (m[0] == 1.f) return 0;
    if (m[0] == 0.f) return 1;
    return kPickAll;
  }
  int hot = kPickNone;
  bool onehot = true;
#pragma unroll
  for (int k = 0; k < NMAX; ++k) {
    if (k >= n) break;
    if (m[k] == 1.f) {
      if (hot != kPickNone) onehot = false;
      hot = k;
    } else if (m[k] != 0.f) {
      onehot = false;
    }
  }
  if (!onehot) return kPickAll;
  float alh = 0.f;
#pragma unroll
  for (int k = 0; k < NMAX; ++k)
    if (k == hot) alh = al[k];
  if (hot != kPickNone && alh != 0.f) return hot;
  return pick_max_alpha<NMAX>(n, al);
}

// Alpha of a picked blend: the two-image rule keeps b's alpha unless b has none; the others
// keep the picked image's.
template <int RULE, int NMAX>
__device__ __forceinline__ float blend_alpha(const float* al, int pick) {
  if (RULE == kRuleTwo) return al[1] == 0.f ? al[0] : al[1];
  float r = 0.f;
#pragma unroll
  for (int k = 0; k < NMAX; ++k)
    if (k == pick) r = al[k];
  return r;
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
    float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
    float amax = 0.f;
#pragma unroll
    for (int k = 0; k < 3; ++k)
      if (L[k].w > amax) {
        amax = L[k].w;
        r = L[k];
      }
    return r;
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

// Blend of one pixel at level l >= 1 with mask values m[0..K).
template <int RULE, int NMAX>
__device__ __forceinline__ float4 blend_level(int n, const float4* lap, const float* m) {
  if constexpr (RULE == kRuleTwo) {
    return blend_two(lap[0], lap[1], m[0]);
  } else if constexpr (RULE == kRuleThree) {
    return blend_three(lap, m[0], m[1], m[2]);
  } else {
    float w[NMAX];
#pragma unroll
    for (int k = 0; k < NMAX; ++k) w[k] = k < n ? m[k] : 0.f;
    return blend_nway<NMAX>(lap, n, w);
  }
}

// ---- Level arithmetic shared by the pyramid kernels ----

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
  // s / count. Division by 1, 2 or 4 equals the (correctly rounded) product with 1, 0.5 or 0.25,
  // so only a count of 3 needs a division.
  __device__ __forceinline__ float4 result() const {
    if (cnt == 4) return make_float4(s0 * 0.25f, s1 * 0.25f, s2 * 0.25f, amax);
    if (cnt == 0) return make_float4(0.f, 0.f, 0.f, amax);
    if (cnt == 2) return make_float4(s0 * 0.5f, s1 * 0.5f, s2 * 0.5f, amax);
    if (cnt == 1) return make_float4(s0, s1, s2, amax);
    return make_float4(s0 / 3.f, s1 / 3.f, s2 / 3.f, amax);
  }
};

// Alpha-aware bilinear upsample of a shared-memory region (origin ax, ay; row stride cw) of a
// level of size lw x lh, sampled for high-res pixel (x, y): top-left aligned, gx = x/2, taps
// floor and floor+1 clamped to the level, only taps with alpha != 0, renormalised
// (src/cuda/cudaBlend.cu:389-455, 581-672). Callers order pixels so that the parity of (x, y) is
// the same across a warp, which keeps the branches below uniform.
//
// Same bits as the reference, with less work. The weights are products of {1, 0.5}, so a tap of
// weight 0 adds an exact zero and is skipped (the remaining taps keep their order; skipping can
// only turn a -0 sum into +0, and the uint8 pack maps both to 0). Every other product v*w is
// exact. The weight sum is 1, 0.5, 0.25 or 0.75; dividing by the first three is an exact scaling
// by 1, 2 or 4, so only a 0.75 sum (three of four taps valid) needs a division.
template <typename T>
__device__ __forceinline__ float3 up_alpha(const T* buf, int cw, int ax, int ay, int lw, int lh, int x, int y) {
  const int gxi = x >> 1, gyi = y >> 1;
  const T* r0 = buf + (gyi - ay) * cw - ax;
  const float4 p00 = load_level(r0 + gxi);
  const bool ox = (x & 1) != 0, oy = (y & 1) != 0;
  if (!ox && !oy) {
    if (p00.w != 0.f) return make_float3(p00.x, p00.y, p00.z);
    return make_float3(0.f, 0.f, 0.f);
  }
  if (ox != oy) {
    // Two taps of weight 0.5: (00, 10) for odd x, (00, 01) for odd y.
    const float4 p1 = ox ? load_level(r0 + min(gxi + 1, lw - 1)) : load_level(buf + (min(gyi + 1, lh - 1) - ay) * cw + (gxi - ax));
    const bool v0 = p00.w != 0.f, v1 = p1.w != 0.f;
    if (v0 && v1)  // (p00*0.5 + p1*0.5) / 1
      return make_float3(p00.x * 0.5f + p1.x * 0.5f, p00.y * 0.5f + p1.y * 0.5f, p00.z * 0.5f + p1.z * 0.5f);
    // (p*0.5) / 0.5: dividing by 0.5 is an exact doubling (kept explicit for subnormal p)
    if (v0) return make_float3((p00.x * 0.5f) * 2.f, (p00.y * 0.5f) * 2.f, (p00.z * 0.5f) * 2.f);
    if (v1) return make_float3((p1.x * 0.5f) * 2.f, (p1.y * 0.5f) * 2.f, (p1.z * 0.5f) * 2.f);
    return make_float3(0.f, 0.f, 0.f);
  }
  // Four taps of weight 0.25.
  const int gxi1 = min(gxi + 1, lw - 1), gyi1 = min(gyi + 1, lh - 1);
  const T* r1 = buf + (gyi1 - ay) * cw - ax;
  const float4 q[4] = {p00, load_level(r0 + gxi1), load_level(r1 + gxi), load_level(r1 + gxi1)};
  float sw = 0.f, s0 = 0.f, s1 = 0.f, s2 = 0.f;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    if (q[i].w != 0.f) {
      sw += 0.25f;
      s0 += q[i].x * 0.25f;
      s1 += q[i].y * 0.25f;
      s2 += q[i].z * 0.25f;
    }
  }
  if (sw == 1.f) return make_float3(s0, s1, s2);
  if (sw == 0.5f) return make_float3(s0 * 2.f, s1 * 2.f, s2 * 2.f);
  if (sw == 0.25f) return make_float3(s0 * 4.f, s1 * 4.f, s2 * 4.f);
  if (sw > 0.f) return make_float3(s0 / sw, s1 / sw, s2 / sw);
  return make_float3(0.f, 0.f, 0.f);
}

// Mask class of an N-way pixel at level l >= 1, from the planner (same values as its MaskHot):
// 0..n-1 = the one-hot image, kHotNone = all weights 0, kHotFrac = fractional weights.
constexpr int kHotNone = 0xFE, kHotFrac = 0xFF;

// One N-way blended Laplacian pixel at level l >= 1, visiting only a tile's compact slot list
// (slot order; slots off the list read as zero there, so they change no pick, sum or alpha):
//   pix(c)    : G^l pixel of list entry c;
//   lap(c, g) : g minus entry c's upsampled G^(l+1) in colour (g itself at the coarsest level);
//   hot       : the pixel's mask class; mk: its mask values, read only for kHotFrac.
// The result equals blend_pick + blend_alpha, or blend_level for fractional weights (up to the
// sign of a zero), restated over the list: the one-hot image when it has alpha, else the first
// image of strictly largest alpha; for fractional weights blend_nway's normalised sums.
template <class Pix, class Lap>
__device__ __forceinline__ float4 nway_lap_blend(int n, int na, uint32_t list, uint32_t cmap, int hot,
                                                 const float* mk, Pix pix, Lap lap) {
  if (hot < 16) {
    const uint32_t c = (cmap >> (4 * hot)) & 15u;
    if (c < 15u) {
      const float4 g = pix(int(c));
      if (g.w != 0.f) return lap(int(c), g);
    }
  }
  float amax = 0.f;
  int mc = -1;
  float4 mg = make_float4(0.f, 0.f, 0.f, 0.f);
  if (hot != kHotFrac) {
    for (int c = 0; c < na; ++c) {
      const float4 g = pix(c);
      if (g.w > amax) {
        amax = g.w;
        mc = c;
        mg = g;
      }
    }
    return mc >= 0 ? lap(mc, mg) : make_float4(0.f, 0.f, 0.f, 0.f);
  }
  float sumw = 0.f;
  for (int k = 0; k < n; ++k) sumw += __ldg(mk + k);
  float sumw2 = 0.f;
  for (int c = 0; c < na; ++c) {
    float w = __ldg(mk + ((list >> (4 * c)) & 15u));
    if (sumw > 0.f) w /= sumw;
    const float4 g = pix(c);
    if (g.w > amax) {
      amax = g.w;
      mc = c;
      mg = g;
    }
    if (g.w == 0.f) w = 0.f;
    sumw2 += w;
  }
  if (!(sumw2 > 0.f)) return mc >= 0 ? lap(mc, mg) : make_float4(0.f, 0.f, 0.f, 0.f);
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int c = 0; c < na; ++c) {
    float w = __ldg(mk + ((list >> (4 * c)) & 15u));
    if (sumw > 0.f) w /= sumw;
    const float4 g = pix(c);
    if (g.w == 0.f) w = 0.f;
    w /= sumw2;
    const float4 L = lap(c, g);
    acc.x += w * L.x;
    acc.y += w * L.y;
    acc.z += w * L.z;
    if (w != 0.f && L.w > acc.w) acc.w = L.w;
  }
  return acc;
}

// Blend of one level-0 pixel from its seam value (two-image weight) or label (one-hot).
template <int RULE, int NMAX>
__device__ __forceinline__ float4 blend_level0(int n, const float4* lap, int v) {
  if constexpr (RULE == kRuleTwo) {
    return blend_two(lap[0], lap[1], float(v));
  } else if constexpr (RULE == kRuleThree) {
    return blend_three(lap, v == 0 ? 1.f : 0.f, v == 1 ? 1.f : 0.f, v == 2 ? 1.f : 0.f);
  } else {
    float w[NMAX];
#pragma unroll
    for (int k = 0; k < NMAX; ++k) w[k] = v == k ? 1.f : 0.f;
    return blend_nway<NMAX>(lap, n, w);
  }
}

// Read-only loads of a level buffer in HBM (through the non-coherent cache).
__device__ __forceinline__ float4 ldg_level(const float4* p) { return __ldg(p); }
__device__ __forceinline__ float4 ldg_level(const half4* p) {
  const uint2 raw = __ldg(reinterpret_cast<const uint2*>(p));
  const __half2 a = *reinterpret_cast<const __half2*>(&raw.x);
  const __half2 b = *reinterpret_cast<const __half2*>(&raw.y);
  const float2 fa = __half22float2(a), fb = __half22float2(b);
  return make_float4(fa.x, fa.y, fb.x, fb.y);
}

}  // namespace hmp
