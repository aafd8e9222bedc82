// hmp_binomial.cu -- the Binomial5 pyramid: 5-tap [1,4,6,4,1]/16 separable filter with reflect-101
// borders in place of the reference's 2x2 box / bilinear pair (no reference implementation; parity
// is checked against the oracle: its FP64 build for accuracy, its FP32 build bit for bit).
//
//   down:  G^{l+1}(x, y) = sum over taps (2x+i, 2y+j), i, j in -2..2 with alpha != 0, of
//          w_i w_j / 256 * G^l, divided by the sum of those weights (0 if none); alpha is the
//          max over the in-bounds 2x2 block (2x..2x+1, 2y..2y+1), as in the box pyramid.
//   up:    Burt-Adelson expand: per axis, even x reads x/2-1, x/2, x/2+1 with weights 1, 6, 1,
//          odd x reads (x-1)/2, (x+1)/2 with weights 4, 4; weight w_x w_y / 64; alpha-aware
//          (alpha-0 taps dropped, renormalised).
//   blend, reconstruct, pack: as in the box pyramid (the reference's rules).
//
// The 5-tap filter has a halo, so the box pyramid's tile-local level walk does not apply; the
// pyramid is built level by level through HBM (L2-resident at these sizes):
//   b5_down0   level 0 (gathered through the slot planes) -> G^1, 16x16 output tiles; the 35x35
//              source tile of every image is staged in shared memory as stored (uint8), all its
//              table lookups in flight together, then all its pixel fetches; exact integer sums,
//              separably (row pass, column pass)
//   b5_down    G^l -> G^{l+1}
//   b5_up      R^l = up(R^{l+1}) + blend(G^l - up(G^{l+1}))         (l = L-1 .. 1; no up at L-1)
//   b5_fine    level 0 of the write rect: blend(G^0 - up(G^1)) + up(R^1), packed into the canvas
// b5_fine gives each thread a 2x2 quad (64x16 pixels a block), so that every pixel's tap parity,
// and with it its expand weights, is known at compile time; b5_up takes one pixel a thread (32x8
// blocks). The coarser-level pixels a block's expands read (34x10 or 19x7, reflected at the
// borders) of every image and of R are staged in shared memory first. Where every tap of a filter
// has alpha, its weights sum to exactly 1 and the normalising divisions are skipped. Every launch after the first is a programmatic dependent of the one before
// (griddepcontrol.wait before any global access), so a launch's CTAs are resident as its
// predecessor drains.
// Arithmetic order follows the oracle term by term (this file is compiled with -fmad=false).
#include "hmp_blend.cuh"

namespace hmp {
namespace {

constexpr int kB5Tile = 16;                    // output tile edge of the down kernels
constexpr int kB5Src = 2 * kB5Tile + 3;        // source tile edge: 2x-2 .. 2x+2 of 16 outputs
constexpr int kB5SrcArea = kB5Src * kB5Src;
constexpr int kB5Per = (kB5SrcArea + 255) / 256;  // source elements per thread
// b5_fine: a thread takes a 2x2 quad at even coordinates, a 32x8-thread block 64x16 pixels, whose
// expands read the 34x10 coarser-level pixels from (X0/2 - 1, Y0/2 - 1).
constexpr int kQW = 34, kQH = 10, kQArea = kQW * kQH;
constexpr int kUpW = 19, kUpArea = kUpW * 7;   // b5_up: coarser-level pixels of a 32x8 block
constexpr int kRowSums = kB5Src * kB5Tile;     // b5_down0: row sums of a tile (35 rows x 16 columns)

__device__ __forceinline__ void b5_dep_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }

// Reflect-101 of coordinate m into [0, n). A tap an output reads is at most 2 outside, which
// these steps settle (the second only for n == 2); staged tiles also hold elements past the
// level's far edge that no output reads, and those are clamped into the level so that every load
// stays inside the buffer.
__device__ __forceinline__ int reflect101(int m, int n) {
  if (n == 1) return 0;
  if (m < 0) m = -m;
  if (m >= n) m = 2 * n - 2 - m;
  if (m < 0) m = -m;
  return min(max(m, 0), n - 1);
}

// Down-filter output (ox, oy) of a source tile `t` whose element (p, q) is source pixel
// (reflect(2*X0 - 2 + p), reflect(2*Y0 - 2 + q)); (tx, ty) = output position in the tile.
__device__ __forceinline__ float4 tile_f4(const float4 v) { return v; }
__device__ __forceinline__ float4 tile_f4(const uchar4 v) { return to_f4(v); }

template <typename T>
__device__ __forceinline__ float4 down5(const T* t, int tx, int ty, int ox, int oy, int iw, int ih) {
  const float k5[5] = {1.f, 4.f, 6.f, 4.f, 1.f};
  float sw = 0.f, s0 = 0.f, s1 = 0.f, s2 = 0.f;
#pragma unroll
  for (int j = 0; j < 5; ++j)
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      const float4 p = tile_f4(t[(2 * ty + j) * kB5Src + 2 * tx + i]);
      if (p.w == 0.f) continue;
      const float wgt = (k5[i] * k5[j]) / 256.f;
      sw += wgt;
      s0 += wgt * p.x;
      s1 += wgt * p.y;
      s2 += wgt * p.z;
    }
  float amax = 0.f;
#pragma unroll
  for (int dy = 0; dy < 2; ++dy)
#pragma unroll
    for (int dx = 0; dx < 2; ++dx) {
      if (2 * ox + dx < iw && 2 * oy + dy < ih) {
        const float a = tile_f4(t[(2 * ty + 2 + dy) * kB5Src + 2 * tx + 2 + dx]).w;
        if (a > amax) amax = a;
      }
    }
  if (sw == 1.f) return make_float4(s0, s1, s2, amax);  // every tap in: x / 1 is x
  if (sw > 0.f) return make_float4(s0 / sw, s1 / sw, s2 / sw, amax);
  return make_float4(0.f, 0.f, 0.f, amax);
}

// Stages coarser-level pixels for a block's expands: element (u, v) of `t` (pitch `pitch`, `area`
// elements) = level buffer `low` (lw x lh) at (reflect(U0 + u), reflect(V0 + v)).
template <typename T>
__device__ __forceinline__ void stage_tile(float4* t, const T* low, int lw, int lh, int U0, int V0, int pitch,
                                           int area) {
  for (int i = threadIdx.y * 32 + threadIdx.x; i < area; i += 256) {
    const int sx = reflect101(U0 + i % pitch, lw), sy = reflect101(V0 + i / pitch, lh);
    t[i] = ldg_level(low + (long long)sy * lw + sx);
  }
}

// Burt-Adelson expand of the pixel of parity (PX, PY) whose coarser-level pixel (x >> 1, y >> 1)
// is element (cu, cv) of a staged tile: the taps, weights and order of up5 with the parity known
// at compile time (even: -1, 0, +1 with weights 1, 6, 1; odd: 0, +1 with weights 4, 4).
__device__ constexpr float up_w(int par, int i) { return par ? 4.f : (i == 1 ? 6.f : 1.f); }

template <int PX, int PY>
__device__ __forceinline__ float3 up5q(const float4* t, int cu, int cv) {
  constexpr int NX = PX ? 2 : 3, NY = PY ? 2 : 3;
  const int c0 = PX ? cu : cu - 1, r0 = PY ? cv : cv - 1;
  float sw = 0.f, s0 = 0.f, s1 = 0.f, s2 = 0.f;
#pragma unroll
  for (int j = 0; j < NY; ++j)
#pragma unroll
    for (int i = 0; i < NX; ++i) {
      const float4 p = t[(r0 + j) * kQW + c0 + i];
      if (p.w == 0.f) continue;
      constexpr float kInv = 1.f / 64.f;
      const float wgt = (up_w(PX, i) * up_w(PY, j)) * kInv;  // exact: (w_x w_y) / 64
      sw += wgt;
      s0 += wgt * p.x;
      s1 += wgt * p.y;
      s2 += wgt * p.z;
    }
  if (sw == 1.f) return make_float3(s0, s1, s2);  // every tap in: x / 1 is x
  if (sw > 0.f) return make_float3(s0 / sw, s1 / sw, s2 / sw);
  return make_float3(0.f, 0.f, 0.f);
}

template <int NMAX, typename Store>
__device__ __forceinline__ const Store* g_of(const PyrArgs& a, int k, int l, int b) {
  const void* p = a.G[0][l];
#pragma unroll
  for (int j = 1; j < NMAX; ++j)
    if (j == k) p = a.G[j][l];
  return static_cast<const Store*>(p) + (long long)b * a.lw[l] * a.lh[l];
}

// Level 0 -> G^1 for every slot: the source tiles are gathered through the slot planes at
// reflected level-0 coordinates, every image's together (the table lookups of all of them in
// flight, then all the pixel fetches), and kept as stored (uint8).
// Level-0 values are integers 0..255 and the weights k_i k_j / 256 are dyadic, so every partial
// sum of down5 is a multiple of 1/256 below 256 and exact in FP32 whatever the order: the sums are
// formed here in integers, separably (5-tap row sums of the tile, then 5-tap column sums), with
// (R, G) and (B, weight) packed as two 16-bit halves of one word (no half exceeds 255 * 256).
// sum / weight is then the same IEEE quotient as down5's (sum/256) / (weight/256).
template <int NMAX, typename Store>
__global__ void __launch_bounds__(256) b5_down0_kernel(const __grid_constant__ PyrArgs a) {
  __shared__ uchar4 t[NMAX][kB5SrcArea];
  __shared__ uint2 rs[kRowSums];  // row sums of one image, column-major: (c, r) at c * 35 + r
  constexpr int kGroup = NMAX <= 3 ? NMAX : 2;  // images whose loads are in flight together
  b5_dep_wait();
  const int n = a.n, b = blockIdx.z, tid = threadIdx.x;
  const int X0 = blockIdx.x * kB5Tile, Y0 = blockIdx.y * kB5Tile;
  const int iw = a.lw[0], ih = a.lh[0], ow = a.lw[1], oh = a.lh[1];
  const int tx = tid % kB5Tile, ty = tid / kB5Tile, ox = X0 + tx, oy = Y0 + ty;
  int sx[kB5Per], sy[kB5Per];
#pragma unroll
  for (int u = 0; u < kB5Per; ++u) {
    const int i = min(tid + 256 * u, kB5SrcArea - 1);
    sx[u] = reflect101(2 * X0 - 2 + i % kB5Src, iw);
    sy[u] = reflect101(2 * Y0 - 2 + i / kB5Src, ih);
  }
#pragma unroll
  for (int k0 = 0; k0 < NMAX; k0 += kGroup) {
    if (k0 >= n) break;
    int own[kGroup][kB5Per];
    uint32_t ent[kGroup][kB5Per];
#pragma unroll
    for (int g = 0; g < kGroup; ++g)
#pragma unroll
      for (int u = 0; u < kB5Per; ++u) {
        own[g][u] = 0xFF;
        ent[g][u] = 0xFFFFFFFFu;
        if (k0 + g < n && tid + 256 * u < kB5SrcArea) slot_lookup(a.slot[k0 + g], k0 + g, sx[u], sy[u], own[g][u], ent[g][u]);
      }
#pragma unroll
    for (int g = 0; g < kGroup; ++g)
#pragma unroll
      for (int u = 0; u < kB5Per; ++u)
        if (k0 + g < n && tid + 256 * u < kB5SrcArea)
          t[k0 + g][tid + 256 * u] = slot_fetch<NMAX>(a, k0 + g, own[g][u], ent[g][u], b, a.opaque != 0);
  }
  constexpr uint32_t k5[5] = {1u, 4u, 6u, 4u, 1u};
#pragma unroll
  for (int k = 0; k < NMAX; ++k) {
    if (k >= n) break;
    __syncthreads();  // the tiles are in (k == 0); the previous image's column pass is done
    const uint32_t* tk = reinterpret_cast<const uint32_t*>(t[k]);
    for (int e = tid; e < kRowSums; e += 256) {
      const int c = e / kB5Src, r = e - c * kB5Src;
      uint32_t lo = 0u, hi = 0u;
#pragma unroll
      for (int i = 0; i < 5; ++i) {
        const uint32_t w = tk[r * kB5Src + 2 * c + i];
        const uint32_t m = (w >> 24) != 0u ? 0xFFFFFFFFu : 0u;  // alpha 0: the tap is dropped
        lo += k5[i] * (__byte_perm(w, 0u, 0x4140) & m);         // R | G << 16
        hi += k5[i] * (__byte_perm(w, 1u, 0x5452) & m);         // B | 1 << 16
      }
      rs[e] = make_uint2(lo, hi);
    }
    __syncthreads();
    if (ox < ow && oy < oh) {
      uint32_t lo = 0u, hi = 0u;
#pragma unroll
      for (int j = 0; j < 5; ++j) {
        const uint2 v = rs[tx * kB5Src + 2 * ty + j];
        lo += k5[j] * v.x;
        hi += k5[j] * v.y;
      }
      const uint32_t wsum = hi >> 16;
      float amax = 0.f;
#pragma unroll
      for (int dy = 0; dy < 2; ++dy)
#pragma unroll
        for (int dx = 0; dx < 2; ++dx)
          if (2 * ox + dx < iw && 2 * oy + dy < ih) {
            const float al = float(t[k][(2 * ty + 2 + dy) * kB5Src + 2 * tx + 2 + dx].w);
            if (al > amax) amax = al;
          }
      float4 v = make_float4(0.f, 0.f, 0.f, amax);
      if (wsum == 256u) {  // every tap in: a division by 256 is the exact product by 2^-8
        v.x = float(lo & 0xFFFFu) * 0.00390625f;
        v.y = float(lo >> 16) * 0.00390625f;
        v.z = float(hi & 0xFFFFu) * 0.00390625f;
      } else if (wsum > 0u) {
        const float sw = float(wsum);
        v.x = float(lo & 0xFFFFu) / sw;
        v.y = float(lo >> 16) / sw;
        v.z = float(hi & 0xFFFFu) / sw;
      }
      Store* G1 = static_cast<Store*>(a.G[k][1]) + (long long)b * ow * oh;
      store_level(G1 + (long long)oy * ow + ox, v);
    }
  }
}

// G^l -> G^{l+1} (l >= 1) for every slot; with two slots both source tiles are loaded together
// (one memory round trip), with more one slot at a time (the tiles would not fit).
template <int NMAX, typename Store>
__global__ void __launch_bounds__(256) b5_down_kernel(const __grid_constant__ PyrArgs a, int l) {
  constexpr int kGroup = NMAX == 2 ? 2 : 1;
  __shared__ float4 t[kGroup][kB5SrcArea];
  b5_dep_wait();
  const int n = a.n, b = blockIdx.z, tid = threadIdx.x;
  const int X0 = blockIdx.x * kB5Tile, Y0 = blockIdx.y * kB5Tile;
  const int iw = a.lw[l], ih = a.lh[l], ow = a.lw[l + 1], oh = a.lh[l + 1];
  const int tx = tid % kB5Tile, ty = tid / kB5Tile, ox = X0 + tx, oy = Y0 + ty;
  int so[kB5Per];  // reflected source offset of each of the thread's tile elements
#pragma unroll
  for (int u = 0; u < kB5Per; ++u) {
    const int i = min(tid + 256 * u, kB5SrcArea - 1);
    so[u] = reflect101(2 * Y0 - 2 + i / kB5Src, ih) * iw + reflect101(2 * X0 - 2 + i % kB5Src, iw);
  }
  for (int k0 = 0; k0 < n; k0 += kGroup) {
    if (k0 > 0) __syncthreads();  // the previous group's outputs are done with the tiles
#pragma unroll
    for (int g = 0; g < kGroup; ++g) {
      if (k0 + g >= n) break;
      const Store* src = static_cast<const Store*>(a.G[k0 + g][l]) + (long long)b * iw * ih;
#pragma unroll
      for (int u = 0; u < kB5Per; ++u)
        if (tid + 256 * u < kB5SrcArea) t[g][tid + 256 * u] = ldg_level(src + so[u]);
    }
    __syncthreads();
    if (ox < ow && oy < oh) {
#pragma unroll
      for (int g = 0; g < kGroup; ++g) {
        if (k0 + g >= n) break;
        Store* dst = static_cast<Store*>(a.G[k0 + g][l + 1]) + (long long)b * ow * oh;
        store_level(dst + (long long)oy * ow + ox, down5(t[g], tx, ty, ox, oy, iw, ih));
      }
    }
  }
}

// Expand at pixel (x, y) of parity known only at run time (b5_up), from a staged tile of pitch
// kUpW whose element (u, v) is the coarser-level pixel (reflect(U0 + u), reflect(V0 + v)); the
// taps, weights and order of up5q.
__device__ __forceinline__ float3 up5r(const float4* t, int U0, int V0, int x, int y) {
  const int px = x & 1, py = y & 1;
  const int c0 = (x >> 1) - U0 - (px ? 0 : 1), r0 = (y >> 1) - V0 - (py ? 0 : 1);
  const int nx = px ? 2 : 3, ny = py ? 2 : 3;
  float sw = 0.f, s0 = 0.f, s1 = 0.f, s2 = 0.f;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    if (j >= ny) break;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      if (i >= nx) break;
      const float4 p = t[(r0 + j) * kUpW + c0 + i];
      if (p.w == 0.f) continue;
      const float wgt = (up_w(px, i) * up_w(py, j)) / 64.f;
      sw += wgt;
      s0 += wgt * p.x;
      s1 += wgt * p.y;
      s2 += wgt * p.z;
    }
  }
  if (sw == 1.f) return make_float3(s0, s1, s2);
  if (sw > 0.f) return make_float3(s0 / sw, s1 / sw, s2 / sw);
  return make_float3(0.f, 0.f, 0.f);
}

// R^l, l >= 1, one pixel a thread over 32x8 blocks (the coarse levels have few pixels: more,
// smaller blocks keep more of their loads in flight). The pixel's own loads are issued before the
// staging loads.
template <int RULE, int NMAX, typename Store>
__global__ void __launch_bounds__(256) b5_up_kernel(const __grid_constant__ PyrArgs a, int l) {
  __shared__ float4 tg[NMAX][kUpArea];  // G^{l+1} of every image
  __shared__ float4 tr[kUpArea];        // R^{l+1}
  b5_dep_wait();
  const int n = RULE == kRuleNway ? a.n : NMAX;
  const int K = RULE == kRuleTwo ? 1 : (RULE == kRuleThree ? 3 : a.K);
  const int b = blockIdx.z;
  const int X0 = blockIdx.x * 32, Y0 = blockIdx.y * 8;
  const int x = X0 + threadIdx.x, y = Y0 + threadIdx.y;
  const int lw = a.lw[l], lh = a.lh[l];
  const bool has_next = l + 1 < a.levels;
  const bool inside = x < lw && y < lh;
  const long long o = inside ? (long long)y * lw + x : 0;
  float4 g[NMAX];
  float al[NMAX], m[NMAX];
#pragma unroll
  for (int k = 0; k < NMAX; ++k) {
    g[k] = k < n && inside ? ldg_level(g_of<NMAX, Store>(a, k, l, b) + o) : make_float4(0.f, 0.f, 0.f, 0.f);
    m[k] = k < K && inside ? __ldg(a.maskL[l] + o * K + k) : 0.f;
  }
  const int U0 = (X0 >> 1) - 1, V0 = (Y0 >> 1) - 1;
  if (has_next) {
    const int lwn = a.lw[l + 1], lhn = a.lh[l + 1];
#pragma unroll
    for (int k = 0; k < NMAX; ++k)
      if (k < n) stage_tile(tg[k], g_of<NMAX, Store>(a, k, l + 1, b), lwn, lhn, U0, V0, kUpW, kUpArea);
    stage_tile(tr, a.Rl[l + 1] + (long long)b * lwn * lhn, lwn, lhn, U0, V0, kUpW, kUpArea);
    __syncthreads();
  }
  if (!inside) return;
#pragma unroll
  for (int k = 0; k < NMAX; ++k) al[k] = g[k].w;
  const int pk = blend_pick<RULE, NMAX>(n, al, m);
  float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
  if (pk >= 0) {
    float4 v = g[0];
#pragma unroll
    for (int k = 1; k < NMAX; ++k)
      if (k == pk) v = g[k];
    if (has_next) {
      const float3 up = up5r(tg[pk], U0, V0, x, y);
      v.x = v.x - up.x;
      v.y = v.y - up.y;
      v.z = v.z - up.z;
    }
    r = make_float4(v.x, v.y, v.z, blend_alpha<RULE, NMAX>(al, pk));
  } else if (pk == kPickAll) {
#pragma unroll
    for (int k = 0; k < NMAX; ++k) {
      if (k < n && has_next) {
        const float3 up = up5r(tg[k], U0, V0, x, y);
        g[k].x = g[k].x - up.x;
        g[k].y = g[k].y - up.y;
        g[k].z = g[k].z - up.z;
      }
    }
    r = blend_level<RULE, NMAX>(n, g, m);
  }
  if (has_next) {
    const float3 up = up5r(tr, U0, V0, x, y);
    r.x = up.x + r.x;
    r.y = up.y + r.y;
    r.z = up.z + r.z;
  }
  a.Rl[l][(long long)b * lw * lh + o] = r;
}

// One level-0 pixel of parity (PX, PY): Laplacians against up(G^1), blend with the level-0 seam
// value, add up(R^1), truncating pack into the canvas.
template <int RULE, int NMAX, int PX, int PY>
__device__ __forceinline__ void fine_pixel(const PyrArgs& a, int n, int b, int x, int y, int mv, const uchar4* src,
                                           const float4 (*tg)[kQArea], const float4* tr, int cu, int cv) {
  float al[NMAX];
#pragma unroll
  for (int k = 0; k < NMAX; ++k) al[k] = float(src[k].w);
  const int pk = blend_pick0<RULE, NMAX>(n, al, mv);
  float4 res = make_float4(0.f, 0.f, 0.f, 0.f);
  if (pk >= 0) {
    uchar4 s0 = src[0];
#pragma unroll
    for (int k = 1; k < NMAX; ++k)
      if (k == pk) s0 = src[k];
    const float4 v = to_f4(s0);
    const float3 up = up5q<PX, PY>(tg[pk], cu, cv);
    res = make_float4(v.x - up.x, v.y - up.y, v.z - up.z, blend_alpha<RULE, NMAX>(al, pk));
  } else if (pk == kPickAll) {
    float4 lap[NMAX];
#pragma unroll
    for (int k = 0; k < NMAX; ++k) {
      float4 v = to_f4(src[k]);
      if (k < n) {
        const float3 up = up5q<PX, PY>(tg[k], cu, cv);
        v.x = v.x - up.x;
        v.y = v.y - up.y;
        v.z = v.z - up.z;
      }
      lap[k] = v;
    }
    res = blend_level0<RULE, NMAX>(n, lap, mv);
  }
  const float3 up = up5q<PX, PY>(tr, cu, cv);
  res.x = up.x + res.x;
  res.y = up.y + res.y;
  res.z = up.z + res.z;
  uchar4* crow = reinterpret_cast<uchar4*>(reinterpret_cast<char*>(a.C.ptr) + b * a.C.bstride +
                                           (long long)(y + a.cy_off) * a.C.pitch);
  crow[x + a.cx_off] = pack_rgba(res);
}

// Level 0 of the write rect over 64x16-pixel blocks of 2x2 quads at even coordinates. A thread's
// table lookups are issued before the staging loads and its pixel fetches right after them, so a
// block waits for two memory round trips before it computes.
template <int RULE, int NMAX, typename Store>
__global__ void __launch_bounds__(256) b5_fine_kernel(const __grid_constant__ PyrArgs a) {
  __shared__ float4 tg[NMAX][kQArea];  // G^1 of every image
  __shared__ float4 tr[kQArea];        // R^1
  b5_dep_wait();
  const int n = RULE == kRuleNway ? a.n : NMAX;
  const int b = blockIdx.z;
  const int X0 = (a.wx0 & ~1) + blockIdx.x * 64, Y0 = (a.wy0 & ~1) + blockIdx.y * 16;
  const int qx = X0 + 2 * threadIdx.x, qy = Y0 + 2 * threadIdx.y;
  const int lw1 = a.lw[1], lh1 = a.lh[1];
  int mv[4], own[4][NMAX];
  uint32_t ent[4][NMAX];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int x = qx + (q & 1), y = qy + (q >> 1);
    const bool inside = x >= a.wx0 && x < a.wx1 && y >= a.wy0 && y < a.wy1;
    mv[q] = inside ? int(__ldg(a.mask0 + (long long)y * a.mask0_pitch + x)) : 0;
#pragma unroll
    for (int k = 0; k < NMAX; ++k) {
      own[q][k] = 0xFF;
      ent[q][k] = 0xFFFFFFFFu;
      if (k < n && inside) slot_lookup(a.slot[k], k, x, y, own[q][k], ent[q][k]);
    }
  }
  const int U0 = (X0 >> 1) - 1, V0 = (Y0 >> 1) - 1;
#pragma unroll
  for (int k = 0; k < NMAX; ++k)
    if (k < n) stage_tile(tg[k], g_of<NMAX, Store>(a, k, 1, b), lw1, lh1, U0, V0, kQW, kQArea);
  stage_tile(tr, a.Rl[1] + (long long)b * lw1 * lh1, lw1, lh1, U0, V0, kQW, kQArea);
  uchar4 src[4][NMAX];
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int k = 0; k < NMAX; ++k) src[q][k] = slot_fetch<NMAX>(a, k, own[q][k], ent[q][k], b, a.opaque != 0);
  __syncthreads();
  const int cu = threadIdx.x + 1, cv = threadIdx.y + 1;
#define HMP_B5_FINE(Q)                                                                              \
  {                                                                                                 \
    const int x = qx + ((Q) & 1), y = qy + ((Q) >> 1);                                              \
    if (x >= a.wx0 && x < a.wx1 && y >= a.wy0 && y < a.wy1)                                        \
      fine_pixel<RULE, NMAX, ((Q) & 1), ((Q) >> 1)>(a, n, b, x, y, mv[Q], src[Q], tg, tr, cu, cv);      \
  }
  HMP_B5_FINE(0)
  HMP_B5_FINE(1)
  HMP_B5_FINE(2)
  HMP_B5_FINE(3)
#undef HMP_B5_FINE
}

// Launches `k` on `s`; with `pdl` as a programmatic dependent of the kernel before it.
template <typename Kern, typename... Args>
void b5_launch(Kern k, dim3 grid, dim3 block, bool pdl, cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl ? 1 : 0;
  cudaLaunchKernelEx(&cfg, k, args...);
}

template <int RULE, int NMAX, typename Store>
cudaError_t b5_chain(const PyrArgs& a, int batch, cudaStream_t s) {
  const int L = a.levels;
  for (int l = 0; l + 1 < L; ++l) {
    const dim3 grid((a.lw[l + 1] + kB5Tile - 1) / kB5Tile, (a.lh[l + 1] + kB5Tile - 1) / kB5Tile, batch);
    if (l == 0)
      b5_launch(b5_down0_kernel<NMAX, Store>, grid, dim3(256), false, s, a);
    else
      b5_launch(b5_down_kernel<NMAX, Store>, grid, dim3(256), true, s, a, l);
  }
  const dim3 blk(32, 8);
  for (int l = L - 1; l >= 1; --l)
    b5_launch(b5_up_kernel<RULE, NMAX, Store>, dim3((a.lw[l] + 31) / 32, (a.lh[l] + 7) / 8, batch), blk, true, s, a, l);
  const int fx0 = a.wx0 & ~1, fy0 = a.wy0 & ~1;
  b5_launch(b5_fine_kernel<RULE, NMAX, Store>, dim3((a.wx1 - fx0 + 63) / 64, (a.wy1 - fy0 + 15) / 16, batch), blk,
            true, s, a);
  return cudaGetLastError();
}

template <typename Store>
cudaError_t b5_dispatch(const PyrArgs& a, int rule, int batch, cudaStream_t s) {
  if (rule == kRuleTwo) return b5_chain<kRuleTwo, 2, Store>(a, batch, s);
  if (rule == kRuleThree) return b5_chain<kRuleThree, 3, Store>(a, batch, s);
  return b5_chain<kRuleNway, 8, Store>(a, batch, s);
}

}  // namespace

cudaError_t launch_b5_pyramid(const PyrArgs& a, int rule, int storage, int batch, cudaStream_t stream) {
  if (a.levels < 2) return cudaErrorInvalidValue;
  return storage == 1 ? b5_dispatch<half4>(a, rule, batch, stream) : b5_dispatch<float4>(a, rule, batch, stream);
}

int b5_launches(int levels) { return levels < 2 ? 0 : 2 * levels - 1; }

}  // namespace hmp
