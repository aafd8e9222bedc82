// hmp_pyramid_kernels.cuh -- the box-filter pyramid kernels (pyr_down, pyr_coarse, pyr_fine and
// their N-way forms) and their device helpers, in an unnamed namespace: hmp_pyramid.cu launches
// them, and hmp_fallback.cu holds its own copies of the dense forms for the copy-block fallback.
//
// The reference runs ~6L launches per frame: a downsample and a mask downsample per level, a
// Laplacian per image and level, a blend per level, a reconstruct per level, plus device copies
// (src/cuda/cudaBlend.cu:847-1049, cudaBlend3.cu:881-1206, cudaBlendN.cu:649-828). Here the whole
// pyramid is three launches:
//
//  * pyr_down: the 2x2 box downsample has no halo, so a CTA that owns an aligned T x T level-0
//    tile (T a multiple of 2^(L-1)) builds every Gaussian level of that tile in shared memory,
//    gathering level 0 straight from the sources through the slot planes (remap + level-0
//    downsample fused). Levels >= 1 go to HBM (FP32 or FP16 storage).
//  * pyr_coarse: a CTA that owns a tile of level-1 pixels loads, all at once, every coarser level
//    it needs (its tile plus a 1-2 pixel halo per level: the bilinear upsample reads floor(x/2)
//    and floor(x/2)+1) into shared memory and walks from the coarsest level down: Laplacians
//    G_k^l - up(G_k^{l+1}), the seam-weighted blend, R^l = up(R^{l+1}) + blend. It writes R^1.
//  * pyr_fine: level 0 (three quarters of the pixels) as a streaming kernel: gather the level-0
//    pixels through the slot planes, Laplacians against up(G_k^1), blend, add up(R^1), pack
//    into the canvas. Laplacians and blended levels never touch HBM.
//
// Tile edges are template parameters and level loops are unrolled, so shared-memory strides and
// per-level geometry are compile-time constants or registers (no local memory, no integer
// division by runtime values).
//
// Arithmetic follows the reference order exactly (this file is compiled with -fmad=false so no
// product is fused into a sum): downsample sums in (0,0),(1,0),(0,1),(1,1) order divided by the
// count; alpha-aware bilinear taps in 00,10,01,11 order over taps with alpha != 0; blends as in
// cudaBlend.cu:520-576, cudaBlend3.cu:376-531, cudaBlendN.cu:199-288.
#pragma once

#include <algorithm>
#include "hmp_blend.cuh"

namespace hmp {
namespace {

constexpr int kL = kDevMaxLevels;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
template <int BYTES>
__device__ __forceinline__ void cp_async(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(smem_u32(dst)), "l"(src), "n"(BYTES));
}
__device__ __forceinline__ void cp_async_commit_wait_all() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}


// Source pixel address of slot k for table entry e (owner o when the slot has an owner plane),
// or nullptr with the pixel to store instead: zero, or alpha 255 under the soft-seam ("opaque")
// rule for an out-of-range entry that is not the 65535 sentinel (src/cuda/cudaRemap.cu:60-123).
template <int NMAX>
__device__ __forceinline__ const uchar4* slot_src(const PyrArgs& a, int k, int o, uint32_t e, int b, bool opaque,
                                                  uint32_t& fill) {
  const int sx = int(e & 0xFFFFu), sy = int(e >> 16);
  fill = 0u;
  if (a.slot[k].owner == nullptr) o = k;
  const uchar4* p = nullptr;
  bool known = false;
#pragma unroll
  for (int q = 0; q < NMAX; ++q) {
    if (o == q) {
      known = true;
      if (sx < a.S.w[q] && sy < a.S.h[q])
        p = reinterpret_cast<const uchar4*>(reinterpret_cast<const char*>(a.S.ptr[q]) + b * a.S.bstride[q] +
                                            (long long)sy * int(a.S.pitch[q])) + sx;
    }
  }
  if (!p && known && opaque && sx != 0xFFFF) fill = 0xFF000000u;
  return p;
}

__device__ __forceinline__ float4 u32_to_f4(uint32_t v) {
  return make_float4(float(v & 0xFFu), float((v >> 8) & 0xFFu), float((v >> 16) & 0xFFu), float(v >> 24));
}

// Level-l buffer of slot k, frame b (k selected at run time among the NMAX slots).
template <int NMAX, typename Store>
__device__ __forceinline__ Store* level_of(const PyrArgs& a, int k, int l, int b) {
  void* p = a.G[0][l];
#pragma unroll
  for (int j = 1; j < NMAX; ++j)
    if (j == k) p = a.G[j][l];
  return static_cast<Store*>(p) + (long long)b * a.lw[l] * a.lh[l];
}

// Gaussian levels 1..L-1 of every slot for one TD x TD level-0 tile (TD a multiple of 2^(L-1),
// so no level needs a neighbouring tile). Level 0 is gathered like the canvas: each warp owns
// tile rows, copies their table entries into shared memory (cp.async, 32 consecutive entries
// per instruction), then replaces every entry by its source pixel (one 4-byte cp.async each, all
// in flight together). One pass then reduces each 4x4 pixel block to its four level-1 pixels
// (kept in registers and stored to HBM) and their level-2 pixel; deeper levels reduce the
// previous level in shared memory (levels 3, 5 reuse the level-0 buffer). Every level >= 1 goes
// to HBM. A slot whose plane misses the tile produces zeros, which its level buffers already
// hold, so it is skipped entirely.
// Programmatic dependent launch: pyr_coarse and pyr_fine are launched with programmatic stream
// serialization, so their CTAs can be scheduled as the kernel before them on the stream drains
// (its CTAs trigger implicitly at exit; an explicit early trigger measured slower beside the
// canvas gather, the waiting CTAs holding SM resources). griddepcontrol.wait returns once that
// kernel has completed and its writes are visible (at once after a normal launch).
__device__ __forceinline__ void grid_dep_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }

// The gated fallback launches (copy-block mode) let their dependents start at once: a fallback CTA
// whose gate is clear only reads it and returns, so the next fallback launch need not wait for the
// previous one to drain before its own CTAs are placed (they wait for its results, if any, with
// grid_dep_wait). Only the walking instantiations do this.
__device__ __forceinline__ void grid_dep_launch() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }

// The last fallback launch (pyr_fine's), when its gate was set: every CTA counts itself out once it
// is done walking, and the last one clears the gate and the count, so that the flag is 0 when the
// next call's kernels start. Nothing waits: a CTA counts and returns.
__device__ __forceinline__ void walk_done(const PyrArgs& a) {
  if (threadIdx.x != 0) return;
  volatile int* g = a.gate;
  if (g[0] == 0) return;
  __threadfence();
  if (atomicAdd(a.gate + 1, 1) == int(gridDim.x * gridDim.y * gridDim.z) - 1) {
    g[1] = 0;
    g[0] = 0;
    __threadfence();
  }
}

// pyr_down in copy-block mode: bit 31 of a listed tile says whether pyr_fine reads the tile's kept
// level-0 pixels (the tile meets a pyramid block); other listed tiles feed only coarser levels.
// Dense and walking launches keep every tile's.
template <bool kLists, bool kWalk>
__device__ __forceinline__ bool keeps_level0(const PyrArgs& a) {
  if constexpr (kLists && !kWalk) {
    if (a.tiles != nullptr) return (__ldg(a.tiles + blockIdx.x / a.list_frames) >> 31) != 0u;
  }
  return true;
}

// Work item w (0, 1, ...) of this CTA: its tile (tx, ty) and frame b. Without kWalk, one item:
// blockIdx.x / y of the dense grid, or entry blockIdx.x of the launch's work list (copy-block mode:
// tx | ty << 16), frame blockIdx.z. kWalk (the gated fallback of copy-block mode): false at once
// unless *gate is set (so that the launch costs little when nothing falls back), then a grid-stride
// walk of the launch's few CTAs over every dense tile of every frame. The gate is written before the
// launch's stream reaches it, so every thread of every CTA reads the same value and leaves
// together. Copy blocks apply to three or more images, and to two through separate instantiations
// (kLists): the dense two-image kernels stay free of this code, since extra code in them measured
// slower beside the canvas gather.
template <bool kLists, bool kWalk>
__device__ __forceinline__ bool cta_tile(const PyrArgs& a, int w, int& tx, int& ty, int& b) {
  b = int(blockIdx.z);
  tx = int(blockIdx.x);
  ty = int(blockIdx.y);
  if constexpr (kWalk) {
    if (*a.gate == 0) return false;
    const long long per = (long long)a.fb_nx * a.fb_ny;
    const long long i = (long long)blockIdx.x + (long long)w * gridDim.x;
    if (i >= per * a.fb_batch) return false;
    b = int(i / per);
    const int r = int(i - b * per);
    ty = r / a.fb_nx;
    tx = r - ty * a.fb_nx;
    return true;
  } else {
    if constexpr (kLists) {
      if (a.tiles != nullptr) {
        // Listed launches put the frame fastest: the CTAs of one tile for every frame of the call
        // run together and share its table entries in L2.
        const int i = int(blockIdx.x) / a.list_frames;
        b = int(blockIdx.x) - i * a.list_frames;
        const uint32_t t = __ldg(a.tiles + i);
        tx = int(t & 0xFFFFu);
        ty = int((t >> 16) & 0x7FFFu);
      }
    }
    return true;
  }
}

// Copy-block mode, at a pyramid-block pixel (blend coordinates x, y) with the label image's level-0
// value v: inside a copy block's reconstruction support (support_mark, one byte per 2^(L-1) block)
// that image's table entry is a source pixel, so alpha 0 there is the source's own, which breaks
// the exactness the copy blocks rely on.
__device__ __forceinline__ bool support_alpha_zero(const PyrArgs& a, int x, int y, uint32_t v) {
  return (v >> 24) == 0u && __ldg(a.support_mark + (long long)(y >> a.sm_shift) * a.sm_pitch + (x >> a.sm_shift)) != 0;
}

// kListed: work lists and the fallback gate (copy-block mode); always on for three or more images,
// a separate instantiation for two, whose dense kernels stay free of that code.
template <int NMAX, typename Store, int TD, bool kListed = false, bool kWalk = false>
__global__ void __launch_bounds__(256) pyr_down_kernel(const __grid_constant__ PyrArgs a) {
  extern __shared__ float4 sm[];
  // One tile, or (kWalk: the gated fallback) a grid-stride walk over the dense tiles.
  if constexpr (kWalk) grid_dep_launch();
  for (int w = 0;; ++w) {
    int tx, ty, b;
    if (!cta_tile<(NMAX >= 3 || kListed), kWalk>(a, w, tx, ty, b)) return;
    if (kWalk && w) __syncthreads();  // the previous tile is done with shared memory
    // Only the three- and N-image kernels keep level 0 for pyr_fine; the two-image kernel is
    // compiled without that code (it measured faster that way, running beside the canvas gather).
    constexpr bool kKeepLevel0 = NMAX >= 3;
    constexpr int T1 = TD / 2, T2 = TD / 4, A2 = T2 * T2;
    const int n = a.n;
    uint32_t* pix = reinterpret_cast<uint32_t*>(sm);  // level 0: [n][TD][TD] pixels
    float4* bufA = sm;                                // levels 3, 5: [n][T1*T1], over level 0
    float4* bufB = sm + n * T1 * T1;                  // levels 2, 4, 6: [n][T2*T2]
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int X0 = tx * TD, Y0 = ty * TD;
    const bool opaque = a.opaque != 0;
    const int L = a.levels;
    const int lw0 = a.lw[0], lh0 = a.lh[0], lw1 = a.lw[1], lh1 = a.lh[1];
    bool active[NMAX];
    uint32_t amask = 0;
  #pragma unroll
    for (int k = 0; k < NMAX; ++k) {
      const PlaneDev& P = a.slot[k];
      active[k] = k < n && !(X0 >= P.x0 + P.w || Y0 >= P.y0 + P.h || X0 + TD <= P.x0 || Y0 + TD <= P.y0);
      if (active[k]) amask |= 1u << k;
    }
    // Level 0, step 1: table entries (the sentinel outside the level or the plane).
  #pragma unroll
    for (int k = 0; k < NMAX; ++k) {
      if (!active[k]) continue;
      const PlaneDev& P = a.slot[k];
      uint32_t* pk = pix + k * TD * TD;
      for (int r = warp; r < TD; r += 8) {
        const int y = Y0 + r, ry = y - P.y0;
  #pragma unroll
        for (int j = 0; j < TD / 32; ++j) {
          const int x = X0 + 32 * j + lane, rx = x - P.x0;
          uint32_t* d = pk + r * TD + 32 * j + lane;
          if (x < lw0 && y < lh0 && (unsigned)rx < (unsigned)P.w && (unsigned)ry < (unsigned)P.h)
            cp_async<4>(d, P.map + (long long)ry * P.map_pitch + rx);
          else
            *d = 0xFFFFFFFFu;
        }
      }
    }
    cp_async_commit_wait_all();
    // Step 2: each thread replaces the entries it copied by their source pixels.
  #pragma unroll
    for (int k = 0; k < NMAX; ++k) {
      if (!active[k]) continue;
      const PlaneDev& P = a.slot[k];
      uint32_t* pk = pix + k * TD * TD;
      for (int r = warp; r < TD; r += 8) {
        const int y = Y0 + r, ry = y - P.y0;
  #pragma unroll
        for (int j = 0; j < TD / 32; ++j) {
          const int x = X0 + 32 * j + lane, rx = x - P.x0;
          uint32_t* d = pk + r * TD + 32 * j + lane;
          const uint32_t e = *d;
          int o = k;
          if (P.owner != nullptr)
            o = (x < lw0 && y < lh0 && (unsigned)rx < (unsigned)P.w && (unsigned)ry < (unsigned)P.h)
                    ? int(__ldg(P.owner + (long long)ry * P.owner_pitch + rx))
                    : 0xFF;
          uint32_t fill;
          const uchar4* sp = slot_src<NMAX>(a, k, o, e, b, opaque, fill);
          if (sp)
            cp_async<4>(d, sp);
          else
            *d = fill;
        }
      }
    }
    cp_async_commit_wait_all();
    __syncthreads();
    // Level 0 for pyr_fine: each slot's gathered pixels inside its plane rect, so that the level-0
    // pass reads them back directly instead of repeating the table lookups and gathers.
    if constexpr (kKeepLevel0) {
  #pragma unroll
      for (int k = 0; k < NMAX; ++k) {
        if (!active[k] || !a.use_p0 || !keeps_level0<(NMAX >= 3 || kListed), kWalk>(a)) continue;
        const PlaneDev& P = a.slot[k];
        uint32_t* dst = a.P0[k] + (long long)b * P.w * P.h;
        const uint32_t* pk = pix + k * TD * TD;
        for (int r = warp; r < TD; r += 8) {
          const int ry = Y0 + r - P.y0;
          if ((unsigned)ry >= (unsigned)P.h) continue;
  #pragma unroll
          for (int j = 0; j < TD / 32; ++j) {
            const int x = X0 + 32 * j + lane, rx = x - P.x0;
            if ((unsigned)rx < (unsigned)P.w) dst[(long long)ry * P.w + rx] = pk[r * TD + 32 * j + lane];
          }
        }
      }
    }
    // Levels 1 and 2: one item = one level-2 pixel of one slot = its four level-1 pixels, each the
    // alpha-aware mean of a 2x2 level-0 block (two 8-byte shared loads), summed in (0,0), (1,0),
    // (0,1), (1,1) order at both levels.
    const bool has2 = L > 2;
    const int lw2 = a.lw[has2 ? 2 : 1], lh2 = a.lh[has2 ? 2 : 1];
    for (int it = tid; it < n * A2; it += 256) {
      const int k = it / A2, j = it - k * A2;
      if (!((amask >> k) & 1u)) continue;
      const int tx2 = j % T2, ty2 = j / T2;
      const int gx2 = (X0 >> 2) + tx2, gy2 = (Y0 >> 2) + ty2;
      const uint32_t* pk = pix + k * TD * TD;
      Store* G1 = level_of<NMAX, Store>(a, k, 1, b);
      DownAcc acc2;
  #pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int tx = 2 * tx2 + (q & 1), ty = 2 * ty2 + (q >> 1);
        const int gx = (X0 >> 1) + tx, gy = (Y0 >> 1) + ty;
        if (gx < lw1 && gy < lh1) {
          const uint2 r0 = *reinterpret_cast<const uint2*>(pk + (2 * ty) * TD + 2 * tx);
          const uint2 r1 = *reinterpret_cast<const uint2*>(pk + (2 * ty + 1) * TD + 2 * tx);
          const bool xin = 2 * gx + 1 < lw0, yin = 2 * gy + 1 < lh0;
          DownAcc acc;
          acc.add(u32_to_f4(r0.x));
          if (xin) acc.add(u32_to_f4(r0.y));
          if (yin) acc.add(u32_to_f4(r1.x));
          if (xin && yin) acc.add(u32_to_f4(r1.y));
          const float4 v = acc.result();
          store_level(G1 + (long long)gy * lw1 + gx, v);
          acc2.add(v);
        }
      }
      if (has2) {
        float4 v2 = make_float4(0.f, 0.f, 0.f, 0.f);
        if (gx2 < lw2 && gy2 < lh2) {
          v2 = acc2.result();
          store_level(level_of<NMAX, Store>(a, k, 2, b) + (long long)gy2 * lw2 + gx2, v2);
        }
        bufB[k * A2 + j] = v2;
      }
    }
    __syncthreads();
  #pragma unroll
    for (int l = 3; l < kL; ++l) {
      if (l >= L) break;
      const int Tp = TD >> (l - 1), Tn = TD >> l;
      const int area = Tn * Tn;
      const float4* src = (l & 1) ? bufB : bufA;
      float4* dst = (l & 1) ? bufA : bufB;
      const int sstride = (l & 1) ? T2 * T2 : T1 * T1;
      const int dstride = (l & 1) ? T1 * T1 : T2 * T2;
      const int lwl = a.lw[l], lhl = a.lh[l], lwp = a.lw[l - 1], lhp = a.lh[l - 1];
  #pragma unroll
      for (int k = 0; k < NMAX; ++k) {
        if (!active[k]) continue;
        for (int j = threadIdx.x; j < area; j += blockDim.x) {
          const int tx = j % Tn, ty = j / Tn;
          const int gx = (X0 >> l) + tx, gy = (Y0 >> l) + ty;
          float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
          if (gx < lwl && gy < lhl) {
            DownAcc acc;
            const float4* sk = src + k * sstride;
  #pragma unroll
            for (int q = 0; q < 4; ++q) {
              const int dx = q & 1, dy = q >> 1;
              if (2 * gx + dx < lwp && 2 * gy + dy < lhp) acc.add(sk[(2 * ty + dy) * Tp + 2 * tx + dx]);
            }
            v = acc.result();
            Store* Gl = static_cast<Store*>(a.G[k][l]) + (long long)b * lwl * lhl;
            store_level(Gl + (long long)gy * lwl + gx, v);
          }
          dst[k * dstride + j] = v;
        }
      }
      __syncthreads();
    }
    if constexpr (!kWalk) return;
  }
}

// Source pixel address of slot k (k and the owner known only at run time), as slot_src.
__device__ __forceinline__ const uchar4* slot_src_dyn(const PyrArgs& a, int k, int o, uint32_t e, int b, bool opaque,
                                                      uint32_t& fill) {
  const int sx = int(e & 0xFFFFu), sy = int(e >> 16);
  fill = 0u;
  if (a.slot[k].owner == nullptr) o = k;
  if (o >= kDevMaxImages) return nullptr;
  if (sx < a.S.w[o] && sy < a.S.h[o])
    return reinterpret_cast<const uchar4*>(reinterpret_cast<const char*>(a.S.ptr[o]) + b * a.S.bstride[o] +
                                           (long long)sy * int(a.S.pitch[o])) + sx;
  if (opaque && sx != 0xFFFF) fill = 0xFF000000u;
  return nullptr;
}

// pyr_down for the N-way rule (up to eight slots). A tile of the N-image blend region overlaps
// only one to three slots' planes, so instead of loops unrolled over all eight slots (whose code
// and per-slot checks dominated: instruction-cache stalls) the tile's active slots form a run-time
// list, and shared memory holds `a.slots_cap` slots (the most any tile has, from the planner).
// Same steps and arithmetic as pyr_down_kernel; level 0 is kept for pyr_fine.
template <typename Store, int TD, bool kWalk = false>
__global__ void __launch_bounds__(256) pyr_down_n_kernel(const __grid_constant__ PyrArgs a) {
  extern __shared__ float4 sm[];
  // One tile, or (kWalk: the gated fallback) a grid-stride walk over the dense tiles.
  if constexpr (kWalk) grid_dep_launch();
  for (int w = 0;; ++w) {
    int tx, ty, b;
    if (!cta_tile<true, kWalk>(a, w, tx, ty, b)) return;
    if (kWalk && w) __syncthreads();  // the previous tile is done with shared memory
    constexpr int T1 = TD / 2, T2 = TD / 4, A2 = T2 * T2;
    const int n = a.n, cap = a.slots_cap;
    uint32_t* pix = reinterpret_cast<uint32_t*>(sm);  // level 0: [cap][TD][TD]
    float4* bufA = sm;                                // levels 3, 5: [cap][T1*T1], over level 0
    float4* bufB = sm + cap * T1 * T1;                // levels 2, 4, 6: [cap][T2*T2]
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int X0 = tx * TD, Y0 = ty * TD;
    const bool opaque = a.opaque != 0;
    const int L = a.levels;
    const int lw0 = a.lw[0], lh0 = a.lh[0], lw1 = a.lw[1], lh1 = a.lh[1];
    uint32_t list = 0;  // active slots, four bits each
    int na = 0;
    for (int k = 0; k < n; ++k) {
      const PlaneDev& P = a.slot[k];
      if (!(X0 >= P.x0 + P.w || Y0 >= P.y0 + P.h || X0 + TD <= P.x0 || Y0 + TD <= P.y0) && na < cap)
        list |= uint32_t(k) << (4 * na++);
    }
  #pragma unroll 1
    for (int c = 0; c < na; ++c) {
      const PlaneDev& P = a.slot[(list >> (4 * c)) & 15u];
      uint32_t* pk = pix + c * TD * TD;
      for (int r = warp; r < TD; r += 8) {
        const int y = Y0 + r, ry = y - P.y0;
  #pragma unroll
        for (int j = 0; j < TD / 32; ++j) {
          const int x = X0 + 32 * j + lane, rx = x - P.x0;
          uint32_t* d = pk + r * TD + 32 * j + lane;
          if (x < lw0 && y < lh0 && (unsigned)rx < (unsigned)P.w && (unsigned)ry < (unsigned)P.h)
            cp_async<4>(d, P.map + (long long)ry * P.map_pitch + rx);
          else
            *d = 0xFFFFFFFFu;
        }
      }
    }
    cp_async_commit_wait_all();
  #pragma unroll 1
    for (int c = 0; c < na; ++c) {
      const int k = (list >> (4 * c)) & 15u;
      const PlaneDev& P = a.slot[k];
      uint32_t* pk = pix + c * TD * TD;
      for (int r = warp; r < TD; r += 8) {
        const int y = Y0 + r, ry = y - P.y0;
  #pragma unroll
        for (int j = 0; j < TD / 32; ++j) {
          const int x = X0 + 32 * j + lane, rx = x - P.x0;
          uint32_t* d = pk + r * TD + 32 * j + lane;
          const uint32_t e = *d;
          int o = k;
          if (P.owner != nullptr)
            o = (x < lw0 && y < lh0 && (unsigned)rx < (unsigned)P.w && (unsigned)ry < (unsigned)P.h)
                    ? int(__ldg(P.owner + (long long)ry * P.owner_pitch + rx))
                    : 0xFF;
          uint32_t fill;
          const uchar4* sp = slot_src_dyn(a, k, o, e, b, opaque, fill);
          if (sp)
            cp_async<4>(d, sp);
          else
            *d = fill;
        }
      }
    }
    cp_async_commit_wait_all();
    __syncthreads();
    if (a.use_p0 && keeps_level0<true, kWalk>(a)) {
  #pragma unroll 1
      for (int c = 0; c < na; ++c) {
        const int k = (list >> (4 * c)) & 15u;
        const PlaneDev& P = a.slot[k];
        uint32_t* dst = a.P0[k] + (long long)b * P.w * P.h;
        const uint32_t* pk = pix + c * TD * TD;
        for (int r = warp; r < TD; r += 8) {
          const int ry = Y0 + r - P.y0;
          if ((unsigned)ry >= (unsigned)P.h) continue;
  #pragma unroll
          for (int j = 0; j < TD / 32; ++j) {
            const int x = X0 + 32 * j + lane, rx = x - P.x0;
            if ((unsigned)rx < (unsigned)P.w) dst[(long long)ry * P.w + rx] = pk[r * TD + 32 * j + lane];
          }
        }
      }
    }
    const bool has2 = L > 2;
    const int lw2 = a.lw[has2 ? 2 : 1], lh2 = a.lh[has2 ? 2 : 1];
  #pragma unroll 1
    for (int it = tid; it < na * A2; it += 256) {
      const int c = it / A2, j = it - c * A2;
      const int k = (list >> (4 * c)) & 15u;
      const int tx2 = j % T2, ty2 = j / T2;
      const int gx2 = (X0 >> 2) + tx2, gy2 = (Y0 >> 2) + ty2;
      const uint32_t* pk = pix + c * TD * TD;
      Store* G1 = static_cast<Store*>(a.G[k][1]) + (long long)b * lw1 * lh1;
      DownAcc acc2;
  #pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int tx = 2 * tx2 + (q & 1), ty = 2 * ty2 + (q >> 1);
        const int gx = (X0 >> 1) + tx, gy = (Y0 >> 1) + ty;
        if (gx < lw1 && gy < lh1) {
          const uint2 r0 = *reinterpret_cast<const uint2*>(pk + (2 * ty) * TD + 2 * tx);
          const uint2 r1 = *reinterpret_cast<const uint2*>(pk + (2 * ty + 1) * TD + 2 * tx);
          const bool xin = 2 * gx + 1 < lw0, yin = 2 * gy + 1 < lh0;
          DownAcc acc;
          acc.add(u32_to_f4(r0.x));
          if (xin) acc.add(u32_to_f4(r0.y));
          if (yin) acc.add(u32_to_f4(r1.x));
          if (xin && yin) acc.add(u32_to_f4(r1.y));
          const float4 v = acc.result();
          store_level(G1 + (long long)gy * lw1 + gx, v);
          acc2.add(v);
        }
      }
      if (has2) {
        float4 v2 = make_float4(0.f, 0.f, 0.f, 0.f);
        if (gx2 < lw2 && gy2 < lh2) {
          v2 = acc2.result();
          store_level(static_cast<Store*>(a.G[k][2]) + (long long)b * lw2 * lh2 + (long long)gy2 * lw2 + gx2, v2);
        }
        bufB[c * A2 + j] = v2;
      }
    }
    __syncthreads();
  #pragma unroll
    for (int l = 3; l < kL; ++l) {
      if (l >= L) break;
      const int Tp = TD >> (l - 1), Tn = TD >> l;
      const int area = Tn * Tn;
      const float4* src = (l & 1) ? bufB : bufA;
      float4* dst = (l & 1) ? bufA : bufB;
      const int sstride = (l & 1) ? T2 * T2 : T1 * T1;
      const int dstride = (l & 1) ? T1 * T1 : T2 * T2;
      const int lwl = a.lw[l], lhl = a.lh[l], lwp = a.lw[l - 1], lhp = a.lh[l - 1];
  #pragma unroll 1
      for (int it = tid; it < na * area; it += 256) {
        const int c = it / area, j = it - c * area;
        const int k = (list >> (4 * c)) & 15u;
        const int tx = j % Tn, ty = j / Tn;
        const int gx = (X0 >> l) + tx, gy = (Y0 >> l) + ty;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (gx < lwl && gy < lhl) {
          DownAcc acc;
          const float4* sk = src + c * sstride;
  #pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int dx = q & 1, dy = q >> 1;
            if (2 * gx + dx < lwp && 2 * gy + dy < lhp) acc.add(sk[(2 * ty + dy) * Tp + 2 * tx + dx]);
          }
          v = acc.result();
          Store* Gl = static_cast<Store*>(a.G[k][l]) + (long long)b * lwl * lhl;
          store_level(Gl + (long long)gy * lwl + gx, v);
        }
        dst[c * dstride + j] = v;
      }
      __syncthreads();
    }
    if constexpr (!kWalk) return;
  }
}


// Shared-memory row stride and capacity (pixels) of level l >= 1 for an up-tile of edge TU: the
// tile's footprint at that level plus the upsample halo.
__host__ __device__ constexpr int up_cw(int tile, int l) { return (tile >> l) + 2; }
__host__ __device__ constexpr int up_cap(int tile, int l) { return up_cw(tile, l) * up_cw(tile, l); }

// pyr_coarse: R^1 (the reconstruction at level 1) for one T1 x T1 tile of level-1 pixels.
// Shared memory holds, per level l >= 2, the tile's footprint plus the upsample halo (G of every
// slot, the mask values, R once computed), all copied in with cp.async up front (one wait on
// memory). The CTA then blends and reconstructs from the coarsest level down; level 1 reads G^1
// and the level-1 mask from HBM and writes R^1 to HBM for pyr_fine. Pixels are processed
// parity-class-major so that the upsample branches stay uniform across a warp.
struct CoarseLayout {
  int g[kL], r[kL], m[kL];  // byte offsets of G (n x cap, storage type), R (cap float4), mask (cap x K)
  int total;
};

__host__ __device__ constexpr int align16(int v) { return (v + 15) & ~15; }

__host__ __device__ inline CoarseLayout coarse_layout(int n, int K, int T1, int L, int store_bytes) {
  CoarseLayout o{};
  int t = 0;
  for (int l = 1; l < kL; ++l) {
    const int cap = (l > 1 && l < L) ? up_cap(T1, l - 1) : 0;
    o.g[l] = t;
    t += align16(n * cap * store_bytes);
    o.r[l] = t;
    t += l > 1 ? cap * 16 : 0;
    o.m[l] = t;
    t += align16(cap * K * 4);
  }
  o.total = t;
  return o;
}

template <int RULE, int NMAX, typename Store, int T1, bool kListed = false, bool kWalk = false>
__global__ void __launch_bounds__(256) pyr_coarse_kernel(const __grid_constant__ PyrArgs a) {
  extern __shared__ float4 sm[];
  // One tile, or (kWalk: the gated fallback) a grid-stride walk over the dense tiles.
  if constexpr (kWalk) grid_dep_launch();
  for (int w = 0;; ++w) {
    int tx, ty, b;
    if (!cta_tile<(RULE != kRuleTwo || kListed), kWalk>(a, w, tx, ty, b)) return;
    if (kWalk && w) __syncthreads();  // the previous tile is done with shared memory
    char* smb = reinterpret_cast<char*>(sm);
    constexpr bool kLists = RULE != kRuleTwo || kListed;
    if (!kLists || a.tiles == nullptr) tx += a.tx0, ty += a.ty0;
    grid_dep_wait();  // G^l of pyr_down
    const int n = RULE == kRuleNway ? a.n : NMAX;
    const int K = RULE == kRuleTwo ? 1 : (RULE == kRuleThree ? 3 : a.K);
    const int X1 = tx * T1, Y1 = ty * T1;
    const int L = a.levels, c = L - 1;
    const int tid = threadIdx.x;
    const CoarseLayout lo = coarse_layout(n, K, T1, L, int(sizeof(Store)));
    // Regions: level 1 is the tile itself; level l >= 2 adds the halo read by level l-1's upsample.
    int rax[kL], ray[kL], rbx[kL], rby[kL];
    {
      int ax = X1, ay = Y1, bx = min(X1 + T1, a.lw[1]), by = min(Y1 + T1, a.lh[1]);
  #pragma unroll
      for (int l = 1; l < kL; ++l) {
        if (l > 1 && l < L) {
          ax >>= 1;
          ay >>= 1;
          bx = min(((bx - 1) >> 1) + 2, a.lw[l]);
          by = min(((by - 1) >> 1) + 2, a.lh[l]);
        }
        rax[l] = ax;
        ray[l] = ay;
        rbx[l] = bx;
        rby[l] = by;
      }
    }
    // Slots whose plane misses the level-0 footprint of every region read here have all-zero levels
    // (alpha 0) in it: the blend never picks them, so their loads are skipped and they read as 0.
    uint32_t amask = 0;
    {
      int fx0 = rax[1] << 1, fy0 = ray[1] << 1, fx1 = rbx[1] << 1, fy1 = rby[1] << 1;
  #pragma unroll
      for (int l = 2; l < kL; ++l) {
        if (l >= L) break;
        fx0 = min(fx0, rax[l] << l);
        fy0 = min(fy0, ray[l] << l);
        fx1 = max(fx1, rbx[l] << l);
        fy1 = max(fy1, rby[l] << l);
      }
  #pragma unroll
      for (int k = 0; k < NMAX; ++k) {
        const PlaneDev& P = a.slot[k];
        if (k < n && fx0 < P.x0 + P.w && P.x0 < fx1 && fy0 < P.y0 + P.h && P.y0 < fy1) amask |= 1u << k;
      }
    }
  #pragma unroll
    for (int l = 2; l < kL; ++l) {
      if (l >= L) break;
      const int CW = up_cw(T1, l - 1), CAP = CW * CW;
      const int lax = rax[l], lay = ray[l], rw = rbx[l] - lax, rh = rby[l] - lay;
      const int lw = a.lw[l], lh = a.lh[l];
  #pragma unroll
      for (int k = 0; k < NMAX; ++k) {
        if (k >= n) break;
        if (!((amask >> k) & 1u)) continue;
        const Store* Gl = static_cast<const Store*>(a.G[k][l]) + (long long)b * lw * lh;
        Store* gl = reinterpret_cast<Store*>(smb + lo.g[l]) + k * CAP;
        for (int i = tid; i < CAP; i += 256) {
          const int x = i % CW, y = i / CW;
          if (x < rw && y < rh) cp_async<int(sizeof(Store))>(gl + i, Gl + (long long)(lay + y) * lw + (lax + x));
        }
      }
      const float* ml = a.maskL[l];
      float* mb = reinterpret_cast<float*>(smb + lo.m[l]);
      for (int p = tid; p < CAP; p += 256) {
        const int x = p % CW, y = p / CW;
        if (x < rw && y < rh) {
          const float* src = ml + ((long long)(lay + y) * lw + (lax + x)) * K;
          for (int q = 0; q < K; ++q) cp_async<4>(mb + p * K + q, src + q);
        }
      }
    }
    cp_async_commit_wait_all();
    __syncthreads();
  #pragma unroll
    for (int l = kL - 1; l >= 2; --l) {
      if (l > c) continue;
      const int CW = up_cw(T1, l - 1), CAP = CW * CW;
      const int QW = (CW + 1) / 2, QC = QW * QW;
      const int lax = rax[l], lay = ray[l], rw = rbx[l] - lax, rh = rby[l] - lay;
      const Store* gcur = reinterpret_cast<const Store*>(smb + lo.g[l]);
      float4* rcur = reinterpret_cast<float4*>(smb + lo.r[l]);
      const float* mb = reinterpret_cast<const float*>(smb + lo.m[l]);
      const bool has_next = l < c;
      const int nl = l + 1 < kL ? l + 1 : l;
      const int CWN = up_cw(T1, nl - 1), CAPN = CWN * CWN;
      const int nax = rax[nl], nay = ray[nl];
      const int lwn = a.lw[nl], lhn = a.lh[nl];
      const Store* gnext = reinterpret_cast<const Store*>(smb + lo.g[nl]);
      const float4* rnext = reinterpret_cast<const float4*>(smb + lo.r[nl]);
      for (int t = tid; t < 4 * QC; t += 256) {
        const int cls = t / QC, j = t - cls * QC;
        const int x = 2 * (j % QW) + (cls & 1), y = 2 * (j / QW) + (cls >> 1);
        if (x >= rw || y >= rh) continue;
        const int i = y * CW + x;
        const int px = lax + x, py = lay + y;
        float al[NMAX];
  #pragma unroll
        for (int k = 0; k < NMAX; ++k) al[k] = ((amask >> k) & 1u) ? load_level(gcur + k * CAP + i).w : 0.f;
        const int pk = blend_pick<RULE, NMAX>(n, al, mb + i * K);
        float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
        if (pk >= 0) {
          // The two-image rule can pick an inactive slot (image 2 where neither has alpha); its
          // levels are all zero here, so its Laplacian is zero.
          const bool act = (amask >> pk) & 1u;
          float4 g = act ? load_level(gcur + pk * CAP + i) : make_float4(0.f, 0.f, 0.f, 0.f);
          if (has_next && act) {
            const float3 up = up_alpha(gnext + pk * CAPN, CWN, nax, nay, lwn, lhn, px, py);
            g.x = g.x - up.x;
            g.y = g.y - up.y;
            g.z = g.z - up.z;
          }
          r = make_float4(g.x, g.y, g.z, blend_alpha<RULE, NMAX>(al, pk));
        } else if (pk == kPickAll) {
          float4 lap[NMAX];
  #pragma unroll
          for (int k = 0; k < NMAX; ++k) {
            if ((amask >> k) & 1u) {
              float4 g = load_level(gcur + k * CAP + i);
              if (has_next) {
                const float3 up = up_alpha(gnext + k * CAPN, CWN, nax, nay, lwn, lhn, px, py);
                g.x = g.x - up.x;
                g.y = g.y - up.y;
                g.z = g.z - up.z;
              }
              lap[k] = g;
            } else {
              lap[k] = make_float4(0.f, 0.f, 0.f, 0.f);
            }
          }
          r = blend_level<RULE, NMAX>(n, lap, mb + i * K);
        }
        if (has_next) {
          const float3 up = up_alpha(rnext, CWN, nax, nay, lwn, lhn, px, py);
          r.x = up.x + r.x;
          r.y = up.y + r.y;
          r.z = up.z + r.z;
        }
        rcur[i] = r;
      }
      __syncthreads();
    }
    // Level 1: the tile's own pixels, R^1 to HBM.
    constexpr int HALF = T1 / 2, CLS = HALF * HALF, PER = (T1 * T1 + 255) / 256;
    static_assert(CLS % 32 == 0, "tile");
    const int lw1 = a.lw[1], lh1 = a.lh[1];
    const bool has2 = c >= 2;
    const int CW2 = up_cw(T1, 1), CAP2 = CW2 * CW2;
    const int nax = rax[2], nay = ray[2];
    const int lw2 = a.lw[2 < kL ? 2 : 1], lh2 = a.lh[2 < kL ? 2 : 1];
    const Store* g2 = reinterpret_cast<const Store*>(smb + lo.g[2]);
    const float4* r2 = reinterpret_cast<const float4*>(smb + lo.r[2]);
    float4* R1 = a.R1 + (long long)b * lw1 * lh1;
  #pragma unroll 2
    for (int p = 0; p < PER; ++p) {
      const int i = p * 256 + tid;
      const int lx = 2 * ((i % CLS) % HALF) + ((i / CLS) & 1), ly = 2 * ((i % CLS) / HALF) + ((i / CLS) >> 1);
      const int px = X1 + lx, py = Y1 + ly;
      if (px >= lw1 || py >= lh1) continue;
      const long long o1 = (long long)py * lw1 + px;
      float m[NMAX];
      float4 g1[NMAX];
      float al[NMAX];
  #pragma unroll
      for (int q = 0; q < NMAX; ++q)
        m[q] = q < K ? __ldg(a.maskL[1] + o1 * K + q) : 0.f;
  #pragma unroll
      for (int k = 0; k < NMAX; ++k) {
        g1[k] = ((amask >> k) & 1u) ? ldg_level(static_cast<const Store*>(a.G[k][1]) + (long long)b * lw1 * lh1 + o1)
                                    : make_float4(0.f, 0.f, 0.f, 0.f);
        al[k] = g1[k].w;
      }
      const int pk = blend_pick<RULE, NMAX>(n, al, m);
      float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
      if (pk >= 0) {
        float4 g = g1[0];
  #pragma unroll
        for (int k = 1; k < NMAX; ++k)
          if (k == pk) g = g1[k];
        if (has2 && ((amask >> pk) & 1u)) {
          const float3 up = up_alpha(g2 + pk * CAP2, CW2, nax, nay, lw2, lh2, px, py);
          g.x = g.x - up.x;
          g.y = g.y - up.y;
          g.z = g.z - up.z;
        }
        r = make_float4(g.x, g.y, g.z, blend_alpha<RULE, NMAX>(al, pk));
      } else if (pk == kPickAll) {
  #pragma unroll
        for (int k = 0; k < NMAX; ++k) {
          if (((amask >> k) & 1u) && has2) {
            const float3 up = up_alpha(g2 + k * CAP2, CW2, nax, nay, lw2, lh2, px, py);
            g1[k].x = g1[k].x - up.x;
            g1[k].y = g1[k].y - up.y;
            g1[k].z = g1[k].z - up.z;
          }
        }
        r = blend_level<RULE, NMAX>(n, g1, m);
      }
      if (has2) {
        const float3 up = up_alpha(r2, CW2, nax, nay, lw2, lh2, px, py);
        r.x = up.x + r.x;
        r.y = up.y + r.y;
        r.z = up.z + r.z;
      }
      R1[o1] = r;
    }
    if constexpr (!kWalk) return;
  }
}

// pyr_coarse for the N-way rule: the tile's active slots (those whose plane meets the footprint
// of the regions read) form a run-time list, shared memory holds `a.coarse_cap` slots (the most
// any tile has, from the planner) and no mask values: each pixel reads its mask class (one byte)
// and, where the weights are one-hot, first the class image's pixel, which decides the pick when
// it has alpha (nway_lap_blend). Same results as pyr_coarse_kernel (inactive slots read as zero).
template <typename Store, int T1, bool kWalk = false>
__global__ void __launch_bounds__(256) pyr_coarse_n_kernel(const __grid_constant__ PyrArgs a) {
  extern __shared__ float4 sm[];
  // One tile, or (kWalk: the gated fallback) a grid-stride walk over the dense tiles.
  if constexpr (kWalk) grid_dep_launch();
  for (int w = 0;; ++w) {
    int tx, ty, b;
    if (!cta_tile<true, kWalk>(a, w, tx, ty, b)) return;
    if (kWalk && w) __syncthreads();  // the previous tile is done with shared memory
    char* smb = reinterpret_cast<char*>(sm);
    if (a.tiles == nullptr) tx += a.tx0, ty += a.ty0;
    grid_dep_wait();  // G^l of pyr_down
    const int n = a.n, K = a.K, cap = a.coarse_cap;
    const int X1 = tx * T1, Y1 = ty * T1;
    const int L = a.levels, c = L - 1;
    const int tid = threadIdx.x;
    const CoarseLayout lo = coarse_layout(cap, 0, T1, L, int(sizeof(Store)));
    int rax[kL], ray[kL], rbx[kL], rby[kL];
    {
      int ax = X1, ay = Y1, bx = min(X1 + T1, a.lw[1]), by = min(Y1 + T1, a.lh[1]);
  #pragma unroll
      for (int l = 1; l < kL; ++l) {
        if (l > 1 && l < L) {
          ax >>= 1;
          ay >>= 1;
          bx = min(((bx - 1) >> 1) + 2, a.lw[l]);
          by = min(((by - 1) >> 1) + 2, a.lh[l]);
        }
        rax[l] = ax;
        ray[l] = ay;
        rbx[l] = bx;
        rby[l] = by;
      }
    }
    uint32_t list = 0, cmap = 0xFFFFFFFFu;  // compact list (slot per nibble), slot -> compact index
    int na = 0;
    {
      int fx0 = rax[1] << 1, fy0 = ray[1] << 1, fx1 = rbx[1] << 1, fy1 = rby[1] << 1;
  #pragma unroll
      for (int l = 2; l < kL; ++l) {
        if (l >= L) break;
        fx0 = min(fx0, rax[l] << l);
        fy0 = min(fy0, ray[l] << l);
        fx1 = max(fx1, rbx[l] << l);
        fy1 = max(fy1, rby[l] << l);
      }
      for (int k = 0; k < n; ++k) {
        const PlaneDev& P = a.slot[k];
        if (fx0 < P.x0 + P.w && P.x0 < fx1 && fy0 < P.y0 + P.h && P.y0 < fy1 && na < cap) {
          list |= uint32_t(k) << (4 * na);
          cmap = (cmap & ~(0xFu << (4 * k))) | (uint32_t(na) << (4 * k));
          ++na;
        }
      }
    }
  #pragma unroll
    for (int l = 2; l < kL; ++l) {
      if (l >= L) break;
      const int CW = up_cw(T1, l - 1), CAP = CW * CW;
      const int lax = rax[l], lay = ray[l], rw = rbx[l] - lax, rh = rby[l] - lay;
      const int lw = a.lw[l], lh = a.lh[l];
  #pragma unroll 1
      for (int ci = 0; ci < na; ++ci) {
        const int k = (list >> (4 * ci)) & 15u;
        const Store* Gl = static_cast<const Store*>(a.G[k][l]) + (long long)b * lw * lh;
        Store* gl = reinterpret_cast<Store*>(smb + lo.g[l]) + ci * CAP;
        for (int i = tid; i < CAP; i += 256) {
          const int x = i % CW, y = i / CW;
          if (x < rw && y < rh) cp_async<int(sizeof(Store))>(gl + i, Gl + (long long)(lay + y) * lw + (lax + x));
        }
      }
    }
    cp_async_commit_wait_all();
    __syncthreads();
  #pragma unroll
    for (int l = kL - 1; l >= 2; --l) {
      if (l > c) continue;
      const int CW = up_cw(T1, l - 1), CAP = CW * CW;
      const int QW = (CW + 1) / 2, QC = QW * QW;
      const int lax = rax[l], lay = ray[l], rw = rbx[l] - lax, rh = rby[l] - lay;
      const int lw = a.lw[l];
      const Store* gcur = reinterpret_cast<const Store*>(smb + lo.g[l]);
      float4* rcur = reinterpret_cast<float4*>(smb + lo.r[l]);
      const uint8_t* hl = a.hotL[l];
      const float* ml = a.maskL[l];
      const bool has_next = l < c;
      const int nl = l + 1 < kL ? l + 1 : l;
      const int CWN = up_cw(T1, nl - 1), CAPN = CWN * CWN;
      const int nax = rax[nl], nay = ray[nl];
      const int lwn = a.lw[nl], lhn = a.lh[nl];
      const Store* gnext = reinterpret_cast<const Store*>(smb + lo.g[nl]);
      const float4* rnext = reinterpret_cast<const float4*>(smb + lo.r[nl]);
      for (int t = tid; t < 4 * QC; t += 256) {
        const int cls = t / QC, j = t - cls * QC;
        const int x = 2 * (j % QW) + (cls & 1), y = 2 * (j / QW) + (cls >> 1);
        if (x >= rw || y >= rh) continue;
        const int i = y * CW + x;
        const int px = lax + x, py = lay + y;
        const long long o = (long long)py * lw + px;
        const auto pix = [&](int ci) { return load_level(gcur + ci * CAP + i); };
        const auto lap = [&](int ci, float4 g) {
          if (has_next) {
            const float3 up = up_alpha(gnext + ci * CAPN, CWN, nax, nay, lwn, lhn, px, py);
            g.x = g.x - up.x;
            g.y = g.y - up.y;
            g.z = g.z - up.z;
          }
          return g;
        };
        float4 r = nway_lap_blend(n, na, list, cmap, int(__ldg(hl + o)), ml + o * K, pix, lap);
        if (has_next) {
          const float3 up = up_alpha(rnext, CWN, nax, nay, lwn, lhn, px, py);
          r.x = up.x + r.x;
          r.y = up.y + r.y;
          r.z = up.z + r.z;
        }
        rcur[i] = r;
      }
      __syncthreads();
    }
    constexpr int HALF = T1 / 2, CLS = HALF * HALF, PER = (T1 * T1 + 255) / 256;
    const int lw1 = a.lw[1], lh1 = a.lh[1];
    const bool has2 = c >= 2;
    const int CW2 = up_cw(T1, 1), CAP2 = CW2 * CW2;
    const int nax = rax[2], nay = ray[2];
    const int lw2 = a.lw[2 < kL ? 2 : 1], lh2 = a.lh[2 < kL ? 2 : 1];
    const Store* g2 = reinterpret_cast<const Store*>(smb + lo.g[2]);
    const float4* r2 = reinterpret_cast<const float4*>(smb + lo.r[2]);
    const long long boff = (long long)b * lw1 * lh1;
    float4* R1 = a.R1 + boff;
  #pragma unroll 1
    for (int p = 0; p < PER; ++p) {
      const int i = p * 256 + tid;
      const int lx = 2 * ((i % CLS) % HALF) + ((i / CLS) & 1), ly = 2 * ((i % CLS) / HALF) + ((i / CLS) >> 1);
      const int px = X1 + lx, py = Y1 + ly;
      if (px >= lw1 || py >= lh1) continue;
      const long long o1 = (long long)py * lw1 + px;
      const auto pix = [&](int ci) {
        return ldg_level(static_cast<const Store*>(a.G[(list >> (4 * ci)) & 15u][1]) + boff + o1);
      };
      const auto lap = [&](int ci, float4 g) {
        if (has2) {
          const float3 up = up_alpha(g2 + ci * CAP2, CW2, nax, nay, lw2, lh2, px, py);
          g.x = g.x - up.x;
          g.y = g.y - up.y;
          g.z = g.z - up.z;
        }
        return g;
      };
      float4 r = nway_lap_blend(n, na, list, cmap, int(__ldg(a.hotL[1] + o1)), a.maskL[1] + o1 * K, pix, lap);
      if (has2) {
        const float3 up = up_alpha(r2, CW2, nax, nay, lw2, lh2, px, py);
        r.x = up.x + r.x;
        r.y = up.y + r.y;
        r.z = up.z + r.z;
      }
      R1[o1] = r;
    }
    if constexpr (!kWalk) return;
  }
}

// Level-1 tile of a pyr_fine CTA: the 32 x 8 level-1 pixels under its 64 x 16 level-0 block
// plus the +1 column and row the bilinear upsample reads, with coordinates clamped to the level
// (so the tile holds the clamped taps and the upsample needs no bounds checks).
constexpr int kFineTW = 33, kFineTH = 9, kFineTA = kFineTW * kFineTH;


// up_alpha from a pyr_fine tile: tap (0,0) at t[i]; (1,0) at t[i+1], (0,1) at t[i+TW]. Same
// taps, order and exact shortcuts as up_alpha.
template <typename T>
__device__ __forceinline__ float3 up_tile(const T* t, int i, bool ox, bool oy) {
  const float4 p00 = load_level(t + i);
  if (!ox && !oy) {
    if (p00.w != 0.f) return make_float3(p00.x, p00.y, p00.z);
    return make_float3(0.f, 0.f, 0.f);
  }
  if (ox != oy) {
    const float4 p1 = load_level(t + i + (ox ? 1 : kFineTW));
    const bool v0 = p00.w != 0.f, v1 = p1.w != 0.f;
    if (v0 && v1)
      return make_float3(p00.x * 0.5f + p1.x * 0.5f, p00.y * 0.5f + p1.y * 0.5f, p00.z * 0.5f + p1.z * 0.5f);
    if (v0) return make_float3((p00.x * 0.5f) * 2.f, (p00.y * 0.5f) * 2.f, (p00.z * 0.5f) * 2.f);
    if (v1) return make_float3((p1.x * 0.5f) * 2.f, (p1.y * 0.5f) * 2.f, (p1.z * 0.5f) * 2.f);
    return make_float3(0.f, 0.f, 0.f);
  }
  const float4 q[4] = {p00, load_level(t + i + 1), load_level(t + i + kFineTW), load_level(t + i + kFineTW + 1)};
  float sw = 0.f, s0 = 0.f, s1 = 0.f, s2 = 0.f;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    if (q[j].w != 0.f) {
      sw += 0.25f;
      s0 += q[j].x * 0.25f;
      s1 += q[j].y * 0.25f;
      s2 += q[j].z * 0.25f;
    }
  }
  if (sw == 1.f) return make_float3(s0, s1, s2);
  if (sw == 0.5f) return make_float3(s0 * 2.f, s1 * 2.f, s2 * 2.f);
  if (sw == 0.25f) return make_float3(s0 * 4.f, s1 * 4.f, s2 * 4.f);
  if (sw > 0.f) return make_float3(s0 / sw, s1 / sw, s2 / sw);
  return make_float3(0.f, 0.f, 0.f);
}

// pyr_fine: level 0 of the write region. A CTA owns a 64 x 16 pixel block, each warp 64 x 2 of
// it, each lane the 2x2 quad (X, Y)..(X+1, Y+1). The CTA first copies its level-1 tiles (G^1 of
// every slot, R^1) into shared memory with cp.async, then issues all its table lookups and
// source gathers, and waits for the tiles only after that. Per pixel: Lap = G^0 - up(G^1) of the
// picked image (of every image where the weights are fractional), blend, add up(R^1), truncating
// pack into the canvas.
template <int RULE, int NMAX, typename Store, bool P0M, bool kListed = false, bool kWalk = false>
__global__ void __launch_bounds__(256) pyr_fine_kernel(const __grid_constant__ PyrArgs a) {
  extern __shared__ float4 fsm[];  // R^1 tile, then G^1 tiles of slots 0..n-1 (Store)
  // One tile, or (kWalk: the gated fallback) a grid-stride walk over the dense tiles.
  if constexpr (kWalk) grid_dep_launch();
  for (int w = 0;; ++w) {
    int tx, ty, b;
    if (!cta_tile<(RULE != kRuleTwo || kListed), kWalk>(a, w, tx, ty, b)) {
      if constexpr (kWalk) walk_done(a);
      return;
    }
    if (kWalk && w) __syncthreads();  // the previous tile is done with shared memory
    const int n = RULE == kRuleNway ? a.n : NMAX;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int bx0 = (a.wx0 & ~1) + tx * 64, by0 = (a.wy0 & ~1) + ty * 16;
    const int X = bx0 + 2 * lane, Y = by0 + 2 * warp;
    const bool opaque = a.opaque != 0;
    const bool has1 = a.levels > 1;
    const int lw0 = a.lw[0], lh0 = a.lh[0], lw1 = a.lw[1], lh1 = a.lh[1];
    float4* rs = fsm;
    Store* gs = reinterpret_cast<Store*>(fsm + kFineTA);
    // A slot whose plane misses the level-0 footprint of this block's G^1 taps (the block plus the
    // 2-pixel upsample halo) has zero pixels (alpha 0) and zero G^1 taps here, so the blend reads
    // nothing non-zero from it: its lookups and G^1 tiles are skipped. (The halo matters: the
    // two-image rule returns image 2's Laplacian, 0 - up(G^1), where neither image has alpha.)
    uint32_t amask = 0;
  #pragma unroll
    for (int k = 0; k < NMAX; ++k) {
      const PlaneDev& P = a.slot[k];
      if (k < n && bx0 < P.x0 + P.w && P.x0 < bx0 + 66 && by0 < P.y0 + P.h && P.y0 < by0 + 18) amask |= 1u << k;
    }
    if (P0M) grid_dep_wait();  // level 0 of pyr_down
    // Pixels of the quad are processed QB at a time: all four (every lookup and gather in flight
    // together) for up to three images; one at a time for the N-way kernel, whose eight images'
    // arrays would not fit in registers four times over.
    constexpr int QB = NMAX > 3 ? 1 : 4;
    const int ti = warp * kFineTW + lane;  // tap (0,0) of the quad in the tiles
  #pragma unroll
    for (int q0 = 0; q0 < 4; q0 += QB) {
      int own[QB][NMAX], mv[QB];
      uint32_t ent[QB][NMAX];
      bool live[QB];
  #pragma unroll
      for (int u = 0; u < QB; ++u) {
        const int q = q0 + u;
        const int x = X + (q & 1), y = Y + (q >> 1);
        live[u] = x < lw0 && y < lh0 && x >= a.wx0 && x < a.wx1 && y >= a.wy0 && y < a.wy1;
        mv[u] = live[u] ? int(__ldg(a.mask0 + (long long)y * a.mask0_pitch + x)) : 0;
  #pragma unroll
        for (int k = 0; k < NMAX; ++k) {
          own[u][k] = 0xFF;
          ent[u][k] = 0xFFFFFFFFu;
          if (P0M) {
            // Level-0 pixel kept by pyr_down (zero outside the slot's plane): in ent.
            const PlaneDev& P = a.slot[k];
            const int rx = x - P.x0, ry = y - P.y0;
            ent[u][k] = 0u;
            if (live[u] && ((amask >> k) & 1u) && (unsigned)rx < (unsigned)P.w && (unsigned)ry < (unsigned)P.h)
              ent[u][k] = __ldg(a.P0[k] + (long long)b * P.w * P.h + (long long)ry * P.w + rx);
          } else if (live[u] && ((amask >> k) & 1u)) {
            slot_lookup(a.slot[k], k, x, y, own[u][k], ent[u][k]);
          }
        }
      }
      // The tiles (R^1 of pyr_coarse, G^1 of pyr_down) are requested after the first lookups, which
      // read only the tables and the frames and so overlap the wait for pyr_coarse.
      if (q0 == 0 && has1) {
        if (!P0M) grid_dep_wait();
        const int tx0 = bx0 >> 1, ty0 = by0 >> 1;
        const long long fo = (long long)b * lw1 * lh1;
        for (int j = tid; j < kFineTA; j += 256) {
          const int y = min(ty0 + j / kFineTW, lh1 - 1), x = min(tx0 + j % kFineTW, lw1 - 1);
          const long long o = fo + (long long)y * lw1 + x;
          cp_async<16>(rs + j, a.R1 + o);
  #pragma unroll
          for (int k = 0; k < NMAX; ++k)
            if ((amask >> k) & 1u)
              cp_async<int(sizeof(Store))>(gs + k * kFineTA + j, static_cast<const Store*>(a.G[k][1]) + o);
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
      }
      uchar4 src[QB][NMAX];
  #pragma unroll
      for (int u = 0; u < QB; ++u)
  #pragma unroll
        for (int k = 0; k < NMAX; ++k) {
          if (P0M) {
            const uint32_t v = ent[u][k];
            src[u][k] = make_uchar4(v & 0xFF, (v >> 8) & 0xFF, (v >> 16) & 0xFF, v >> 24);
          } else {
            src[u][k] = ((amask >> k) & 1u) ? slot_fetch<NMAX>(a, k, own[u][k], ent[u][k], b, opaque)
                                            : make_uchar4(0, 0, 0, 0);
          }
        }
      if (q0 == 0 && has1) {
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        __syncthreads();
      }
      bool bad = false;  // copy-block mode: alpha 0 of the label image inside a copy block's support
  #pragma unroll
      for (int u = 0; u < QB; ++u) {
        const int q = q0 + u;
        if (!live[u]) continue;
        const bool ox = (q & 1) != 0, oy = (q >> 1) != 0;
        float al[NMAX];
  #pragma unroll
        for (int k = 0; k < NMAX; ++k) al[k] = float(src[u][k].w);

        const int pk = blend_pick0<RULE, NMAX>(n, al, mv[u]);
        if constexpr (P0M && RULE != kRuleTwo) {
          // The three- and N-way picks return the label's image exactly when it has alpha, so a
          // valid label picked otherwise had alpha 0.
          if (a.alpha_flag != nullptr && mv[u] < n && pk != mv[u])
            bad = bad || support_alpha_zero(a, X + (q & 1), Y + (q >> 1), 0u);
        } else if constexpr (RULE == kRuleTwo && kListed) {
          // Two images: the support's mark names the slot its copy block copies (1 + slot).
          if (a.alpha_flag != nullptr && (al[0] == 0.f || al[1] == 0.f)) {
            const int x = X + (q & 1), y = Y + (q >> 1);
            const int m = __ldg(a.support_mark + (long long)(y >> a.sm_shift) * a.sm_pitch + (x >> a.sm_shift));
            bad = bad || (m == 1 && al[0] == 0.f) || (m == 2 && al[1] == 0.f);
          }
        }
        float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
        if (pk >= 0) {
          uchar4 sp = src[u][0];
  #pragma unroll
          for (int k = 1; k < NMAX; ++k)
            if (k == pk) sp = src[u][k];
          float4 g = to_f4(sp);
          if (has1 && ((amask >> pk) & 1u)) {  // an inactive slot's G^1 taps are all zero here
            const float3 up = up_tile(gs + pk * kFineTA, ti, ox, oy);
            g.x = g.x - up.x;
            g.y = g.y - up.y;
            g.z = g.z - up.z;
          }
          r = make_float4(g.x, g.y, g.z, blend_alpha<RULE, NMAX>(al, pk));
        } else if (pk == kPickAll) {
          float4 lap[NMAX];
  #pragma unroll
          for (int k = 0; k < NMAX; ++k) {
            float4 g = to_f4(src[u][k]);
            if (has1 && ((amask >> k) & 1u)) {
              const float3 up = up_tile(gs + k * kFineTA, ti, ox, oy);
              g.x = g.x - up.x;
              g.y = g.y - up.y;
              g.z = g.z - up.z;
            }
            lap[k] = g;
          }
          r = blend_level0<RULE, NMAX>(n, lap, mv[u]);
        }
        if (has1) {
          const float3 up = up_tile(rs, ti, ox, oy);
          r.x = up.x + r.x;
          r.y = up.y + r.y;
          r.z = up.z + r.z;
        }
        const int px = X + (q & 1), py = Y + (q >> 1);
        uchar4* crow = reinterpret_cast<uchar4*>(reinterpret_cast<char*>(a.C.ptr) + b * a.C.bstride +
                                                 (long long)(py + a.cy_off) * a.C.pitch);
        crow[px + a.cx_off] = pack_rgba(r);
      }
      if constexpr ((P0M && RULE != kRuleTwo) || (RULE == kRuleTwo && kListed)) {
        if (a.alpha_flag != nullptr && __any_sync(0xFFFFFFFFu, bad) && lane == 0) atomicOr(a.alpha_flag, 1);
      }
    }
    if constexpr (!kWalk) return;
  }
}

// pyr_fine for the N-way rule with level 0 kept by pyr_down: the block's active slots (those
// whose plane meets its footprint with the upsample halo) form a run-time list, shared memory
// holds R^1 and `a.fine_cap` G^1 tiles. The label weights are one-hot, so the blend is the
// Laplacian of one image (blend_pick0): the label's image where it has alpha -- one load -- and
// otherwise the first image of strictly largest alpha, found by walking the list in slot order.
template <typename Store, bool kWalk = false>
__global__ void __launch_bounds__(256) pyr_fine_n_kernel(const __grid_constant__ PyrArgs a) {
  extern __shared__ float4 fsm[];
  // One tile, or (kWalk: the gated fallback) a grid-stride walk over the dense tiles.
  if constexpr (kWalk) grid_dep_launch();
  for (int w = 0;; ++w) {
    int tx, ty, b;
    if (!cta_tile<true, kWalk>(a, w, tx, ty, b)) {
      if constexpr (kWalk) walk_done(a);
      return;
    }
    if (kWalk && w) __syncthreads();  // the previous tile is done with shared memory
    grid_dep_wait();  // R^1 of pyr_coarse; G^1 and level 0 of pyr_down
    const int n = a.n, cap = a.fine_cap;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int bx0 = (a.wx0 & ~1) + tx * 64, by0 = (a.wy0 & ~1) + ty * 16;
    const int X = bx0 + 2 * lane, Y = by0 + 2 * warp;
    const int lw0 = a.lw[0], lh0 = a.lh[0], lw1 = a.lw[1], lh1 = a.lh[1];
    float4* rs = fsm;
    Store* gs = reinterpret_cast<Store*>(fsm + kFineTA);
    uint32_t list = 0, cmap = 0xFFFFFFFFu;  // compact list (slot per nibble), slot -> compact index
    int na = 0;
    for (int k = 0; k < n; ++k) {
      const PlaneDev& P = a.slot[k];
      if (bx0 < P.x0 + P.w && P.x0 < bx0 + 66 && by0 < P.y0 + P.h && P.y0 < by0 + 18 && na < cap) {
        list |= uint32_t(k) << (4 * na);
        cmap = (cmap & ~(0xFu << (4 * k))) | (uint32_t(na) << (4 * k));
        ++na;
      }
    }
    {
      const int tx0 = bx0 >> 1, ty0 = by0 >> 1;
      const long long fo = (long long)b * lw1 * lh1;
      for (int j = tid; j < kFineTA; j += 256) {
        const int y = min(ty0 + j / kFineTW, lh1 - 1), x = min(tx0 + j % kFineTW, lw1 - 1);
        const long long o = fo + (long long)y * lw1 + x;
        cp_async<16>(rs + j, a.R1 + o);
        for (int c = 0; c < na; ++c)
          cp_async<int(sizeof(Store))>(gs + c * kFineTA + j, static_cast<const Store*>(a.G[(list >> (4 * c)) & 15u][1]) + o);
      }
      asm volatile("cp.async.commit_group;\n" ::: "memory");
    }
    const int ti = warp * kFineTW + lane;
    bool live[4], done[4];
    int pc[4];
    uint32_t pp[4];
    {
      int v[4];
      uint32_t p[4];
  #pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int x = X + (q & 1), y = Y + (q >> 1);
        live[q] = x < lw0 && y < lh0 && x >= a.wx0 && x < a.wx1 && y >= a.wy0 && y < a.wy1;
        v[q] = live[q] ? int(__ldg(a.mask0 + (long long)y * a.mask0_pitch + x)) : 15;
        p[q] = 0u;
        if (v[q] < n) {  // an inactive label's plane misses the pixel: its alpha is 0
          const PlaneDev& P = a.slot[v[q]];
          const int rx = x - P.x0, ry = y - P.y0;
          if ((unsigned)rx < (unsigned)P.w && (unsigned)ry < (unsigned)P.h)
            p[q] = __ldg(a.P0[v[q]] + (long long)b * P.w * P.h + (long long)ry * P.w + rx);
        }
      }
      if (a.alpha_flag != nullptr) {  // copy-block mode, as in pyr_fine_kernel
        bool bad = false;
  #pragma unroll
        for (int q = 0; q < 4; ++q)
          bad = bad || (live[q] && v[q] < n && support_alpha_zero(a, X + (q & 1), Y + (q >> 1), p[q]));
        if (__any_sync(0xFFFFFFFFu, bad) && lane == 0) atomicOr(a.alpha_flag, 1);
      }
  #pragma unroll
      for (int q = 0; q < 4; ++q) {
        done[q] = !live[q] || (p[q] >> 24) != 0u;
        pc[q] = (p[q] >> 24) != 0u ? int((cmap >> (4 * v[q])) & 15u) : -1;
        pp[q] = p[q];
      }
    }
    if (!(done[0] && done[1] && done[2] && done[3])) {
      uint32_t amax[4] = {0u, 0u, 0u, 0u};
  #pragma unroll 1
      for (int c = 0; c < na; ++c) {
        const int k = (list >> (4 * c)) & 15u;
        const PlaneDev& P = a.slot[k];
        const uint32_t* p0 = a.P0[k] + (long long)b * P.w * P.h;
        uint32_t p[4];
  #pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int rx = X + (q & 1) - P.x0, ry = Y + (q >> 1) - P.y0;
          p[q] = 0u;
          if (!done[q] && (unsigned)rx < (unsigned)P.w && (unsigned)ry < (unsigned)P.h)
            p[q] = __ldg(p0 + (long long)ry * P.w + rx);
        }
  #pragma unroll
        for (int q = 0; q < 4; ++q)
          if ((p[q] >> 24) > amax[q]) {
            amax[q] = p[q] >> 24;
            pc[q] = c;
            pp[q] = p[q];
          }
      }
    }
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    __syncthreads();
  #pragma unroll
    for (int q = 0; q < 4; ++q) {
      if (!live[q]) continue;
      const int x = X + (q & 1), y = Y + (q >> 1);
      const bool ox = (q & 1) != 0, oy = (q >> 1) != 0;
      float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
      if (pc[q] >= 0) {
        const uint32_t g = pp[q];
        const float3 up = up_tile(gs + pc[q] * kFineTA, ti, ox, oy);
        r = make_float4(float(g & 0xFF) - up.x, float((g >> 8) & 0xFF) - up.y, float((g >> 16) & 0xFF) - up.z,
                        float(g >> 24));
      }
      const float3 up = up_tile(rs, ti, ox, oy);
      r.x = up.x + r.x;
      r.y = up.y + r.y;
      r.z = up.z + r.z;
      uchar4* crow = reinterpret_cast<uchar4*>(reinterpret_cast<char*>(a.C.ptr) + b * a.C.bstride +
                                               (long long)(y + a.cy_off) * a.C.pitch);
      crow[x + a.cx_off] = pack_rgba(r);
    }
    if constexpr (!kWalk) return;
  }
}

}  // namespace
}  // namespace hmp
