// hmp_stabilize.cu -- frame stabiliser (hmp_stabilizer_* in include/hmpano.h).
//
// The reference ships it as a demo beside the stitcher (src/cuda/cudaStabilize.cu): Harris corners
// of the previous frame, sparse Lucas-Kanade flow of each into the next frame, the mean flow as the
// global motion, and the next frame translated by it. There every step round-trips through the
// host (the response map is copied out for thresholding, the features copied in, the flow copied
// out and averaged on the CPU) with a synchronize after each kernel and allocations per call. Here
// a stabiliser allocates once and every step stays on the device, asynchronous on the caller's
// stream:
//   harris      Sobel gradients and the 3x3 Harris response of a 32 x 8 tile, the image tile (with
//               a 2-pixel halo) and its gradients staged in shared memory;
//   corners     threshold + 3x3 non-maximum suppression: a warp per row counts its corners with
//               ballots, one CTA scans the row counts, and a warp per row writes its corners at its
//               offset, so the list is in raster order as the reference's host loop builds it;
//   flow        Lucas-Kanade per feature, one thread each, the reference's sums in its order;
//   motion      one thread sums the flow in feature order (the reference's host sum) and rounds;
//   warp        translation by the rounded mean, zero fill.
// Operation order follows the reference (this file is compiled with -fmad=false); where the
// reference reads memory it never defines, the values are fixed as the oracle documents
// (oracle/hmp_stabilize_oracle.c): gradients and responses outside the interior are 0, flow taps
// in column 0 or row 0 are skipped, and no corners means no motion.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <new>

#include "hmpano.h"

namespace {

struct Motion {
  int corners;     // corners found (the list holds at most the stabiliser's capacity)
  float dx, dy;    // mean flow
  int sx, sy;      // its rounding, the translation applied
};

constexpr int kTX = 32, kTY = 8;

// A displacement rounded to whole pixels: the float-to-int conversion saturates and maps NaN to 0;
// the clamp at +-2^24 keeps the index sums in range (a shift that large leaves the frame either way).
__device__ __forceinline__ int shift_of(float v) {
  if (!(v == v)) return 0;
  return int(fminf(fmaxf(roundf(v), -16777216.0f), 16777216.0f));
}

__global__ void __launch_bounds__(256) harris_kernel(const float* __restrict__ img, int w, int h, float k,
                                                     float* __restrict__ resp) {
  __shared__ float t[kTY + 4][kTX + 4];      // image, origin (X0 - 2, Y0 - 2); 0 outside
  __shared__ float gx[kTY + 2][kTX + 2];     // gradients, origin (X0 - 1, Y0 - 1); 0 off the interior
  __shared__ float gy[kTY + 2][kTX + 2];
  const int X0 = blockIdx.x * kTX, Y0 = blockIdx.y * kTY;
  const int tid = threadIdx.y * kTX + threadIdx.x;
  for (int i = tid; i < (kTY + 4) * (kTX + 4); i += kTX * kTY) {
    const int tx = i % (kTX + 4), ty = i / (kTX + 4);
    const int x = X0 - 2 + tx, y = Y0 - 2 + ty;
    t[ty][tx] = (x >= 0 && x < w && y >= 0 && y < h) ? img[(long long)y * w + x] : 0.f;
  }
  __syncthreads();
  for (int i = tid; i < (kTY + 2) * (kTX + 2); i += kTX * kTY) {
    const int tx = i % (kTX + 2), ty = i / (kTX + 2);
    const int x = X0 - 1 + tx, y = Y0 - 1 + ty;
    float vx = 0.f, vy = 0.f;
    if (x > 0 && x < w - 1 && y > 0 && y < h - 1) {
      // t[ty + 1][tx + 1] is pixel (x, y)
      const float* r0 = &t[ty][tx + 1];
      const float* r1 = &t[ty + 1][tx + 1];
      const float* r2 = &t[ty + 2][tx + 1];
      vx = r0[1] + 2.0f * r1[1] + r2[1] - r0[-1] - 2.0f * r1[-1] - r2[-1];
      vy = r0[-1] + 2.0f * r0[0] + r0[1] - r2[-1] - 2.0f * r2[0] - r2[1];
    }
    gx[ty][tx] = vx;
    gy[ty][tx] = vy;
  }
  __syncthreads();
  const int x = X0 + threadIdx.x, y = Y0 + threadIdx.y;
  if (x >= w || y >= h) return;
  float r = 0.f;
  if (x > 0 && x < w - 1 && y > 0 && y < h - 1) {
    float sxx = 0.f, sxy = 0.f, syy = 0.f;
#pragma unroll
    for (int j = -1; j <= 1; ++j)
#pragma unroll
      for (int i = -1; i <= 1; ++i) {
        const float ix = gx[threadIdx.y + 1 + j][threadIdx.x + 1 + i];
        const float iy = gy[threadIdx.y + 1 + j][threadIdx.x + 1 + i];
        sxx += ix * ix;
        sxy += ix * iy;
        syy += iy * iy;
      }
    const float det = sxx * syy - sxy * sxy;
    const float tr = sxx + syy;
    r = det - k * tr * tr;
  }
  resp[(long long)y * w + x] = r;
}

// Threshold and 3x3 non-maximum suppression (a neighbour strictly above removes the pixel).
__device__ __forceinline__ bool is_corner(const float* resp, int w, int h, float thr, int x, int y) {
  if (x < 1 || x >= w - 1 || y < 1 || y >= h - 1) return false;
  const float r = __ldg(resp + (long long)y * w + x);
  if (!(r > thr)) return false;
  for (int j = -1; j <= 1; ++j)
    for (int i = -1; i <= 1; ++i)
      if (__ldg(resp + (long long)(y + j) * w + (x + i)) > r) return false;
  return true;
}

// Corners are counted and emitted by segments: kCornerSeg pixels of one row, a warp each. Rows
// split into segments give the count and emit passes many more warps than rows (a 3840-pixel row
// is 8 segments), and the segments' raster order keeps the corners in raster order.
constexpr int kCornerSeg = 512;
constexpr int kScanPerThread = 8;  // segment counts per thread in each pass of the scan

__host__ __device__ inline int corner_segments_per_row(int w) { return (w + kCornerSeg - 1) / kCornerSeg; }

// A warp per segment: its corner count.
__global__ void __launch_bounds__(256) corner_count_kernel(const float* resp, int w, int h, float thr, int segs,
                                                           int* seg_count) {
  const int lane = threadIdx.x & 31, g = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (g >= segs) return;
  const int spr = corner_segments_per_row(w), y = g / spr, xs = (g - y * spr) * kCornerSeg;
  const int xe = min(xs + kCornerSeg, w);
  int c = 0;
  for (int x0 = xs; x0 < xe; x0 += 32) c += __popc(__ballot_sync(0xFFFFFFFFu, is_corner(resp, w, h, thr, x0 + lane, y)));
  if (lane == 0) seg_count[g] = c;
}

// One CTA: segment offsets (exclusive scan of the counts, kScanPerThread consecutive counts per
// thread, 1024 threads a pass) and the total.
__global__ void __launch_bounds__(1024) corner_scan_kernel(const int* seg_count, int segs, int* seg_off, Motion* m) {
  __shared__ int warp_sum[32];
  __shared__ int carry;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < segs; base += 1024 * kScanPerThread) {
    const int i0 = base + threadIdx.x * kScanPerThread;
    int v[kScanPerThread];
    int t = 0;
#pragma unroll
    for (int e = 0; e < kScanPerThread; ++e) {
      v[e] = i0 + e < segs ? seg_count[i0 + e] : 0;
      t += v[e];
    }
    int s = t;  // inclusive scan of the threads' totals within the warp
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int u = __shfl_up_sync(0xFFFFFFFFu, s, d);
      if (lane >= d) s += u;
    }
    if (lane == 31) warp_sum[wid] = s;
    __syncthreads();
    if (wid == 0) {
      int ws = warp_sum[lane];
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const int u = __shfl_up_sync(0xFFFFFFFFu, ws, d);
        if (lane >= d) ws += u;
      }
      warp_sum[lane] = ws;  // inclusive over warps
    }
    __syncthreads();
    int before = carry + (wid > 0 ? warp_sum[wid - 1] : 0) + s - t;
#pragma unroll
    for (int e = 0; e < kScanPerThread; ++e) {
      if (i0 + e < segs) seg_off[i0 + e] = before;
      before += v[e];
    }
    __syncthreads();
    if (threadIdx.x == 1023) carry = before;  // this pass's total added
    __syncthreads();
  }
  if (threadIdx.x == 0) m->corners = carry;
}

// A warp per segment: its corners, in x order, at the segment's offset (those within the capacity).
__global__ void __launch_bounds__(256) corner_emit_kernel(const float* resp, int w, int h, float thr, int segs,
                                                          const int* seg_off, int2* xy, int cap) {
  const int lane = threadIdx.x & 31, g = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (g >= segs) return;
  const int spr = corner_segments_per_row(w), y = g / spr, xs = (g - y * spr) * kCornerSeg;
  const int xe = min(xs + kCornerSeg, w);
  int at = seg_off[g];
  for (int x0 = xs; x0 < xe; x0 += 32) {
    const bool c = is_corner(resp, w, h, thr, x0 + lane, y);
    const unsigned bits = __ballot_sync(0xFFFFFFFFu, c);
    const int pos = at + __popc(bits & ((1u << lane) - 1u));
    if (c && pos < cap) xy[pos] = make_int2(x0 + lane, y);
    at += __popc(bits);
  }
}

// Lucas-Kanade per feature: 10 iterations over a window_size window, the displacement rounded to
// whole pixels for sampling the next frame (the reference's scheme and sum order).
__global__ void __launch_bounds__(256) flow_kernel(const float* __restrict__ prev, const float* __restrict__ next,
                                                   const int2* xy, const Motion* m, int cap, int w, int h, int window,
                                                   float2* flow) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= min(m->corners, cap)) return;
  const int2 p = xy[f];
  const int half = window / 2;
  float dx = 0.f, dy = 0.f;
  for (int iter = 0; iter < 10; ++iter) {
    float sxx = 0.f, syy = 0.f, sxy = 0.f, stx = 0.f, sty = 0.f;
    const int rdx = shift_of(dx), rdy = shift_of(dy);
    for (int j = -half; j <= half; ++j)
      for (int i = -half; i <= half; ++i) {
        const int x = p.x + i, y = p.y + j, xn = x + rdx, yn = y + rdy;
        if (x < 1 || x >= w - 1 || y < 1 || y >= h - 1 || xn < 0 || xn >= w - 1 || yn < 0 || yn >= h - 1) continue;
        const long long o = (long long)y * w + x;
        const float ix = (__ldg(prev + o + 1) - __ldg(prev + o - 1)) * 0.5f;
        const float iy = (__ldg(prev + o + w) - __ldg(prev + o - w)) * 0.5f;
        const float it = __ldg(next + (long long)yn * w + xn) - __ldg(prev + o);
        sxx += ix * ix;
        syy += iy * iy;
        sxy += ix * iy;
        stx += ix * it;
        sty += iy * it;
      }
    const float det = sxx * syy - sxy * sxy;
    if (fabsf(det) < 1e-6f) break;
    const float ddx = (-syy * stx + sxy * sty) / det;
    const float ddy = (sxy * stx - sxx * sty) / det;
    dx += ddx;
    dy += ddy;
    if (sqrtf(ddx * ddx + ddy * ddy) < 0.01f) break;
  }
  flow[f] = make_float2(dx, dy);
}

// Lucas-Kanade per feature for the reference's default 15-pixel window, the same taps and sums in
// the same order as flow_kernel, loaded by rows: a row of the window is a few aligned 16-byte
// chunks (frames 16-byte aligned, checked on the host) instead of one 4-byte load per value, and
// the three rows of `prev` the gradients read slide down the window in registers. A warp's
// features sit at scattered places, so each load instruction touches about one cache line per
// lane; loading four values per instruction cuts those wavefronts about five-fold.
// v[c] = frame[L + c] for c < N (0 outside [0, total)).
template <int N>
__device__ __forceinline__ void load_row(const float* __restrict__ frame, long long total, long long L, float (&v)[N]) {
  constexpr int NC = (N + 6) / 4;  // chunks covering an offset of up to 3 plus N values
  const long long a0 = L & ~3LL;
  const int off = int(L - a0);
  float c4[NC * 4];
#pragma unroll
  for (int k = 0; k < NC; ++k) {
    const long long c = a0 + 4 * k;
    if (c >= 0 && c + 3 < total) {
      const float4 q = __ldg(reinterpret_cast<const float4*>(frame + c));
      c4[4 * k] = q.x, c4[4 * k + 1] = q.y, c4[4 * k + 2] = q.z, c4[4 * k + 3] = q.w;
    } else {
#pragma unroll
      for (int e = 0; e < 4; ++e) c4[4 * k + e] = (c + e >= 0 && c + e < total) ? __ldg(frame + c + e) : 0.f;
    }
  }
#pragma unroll
  for (int c = 0; c < N; ++c)
    v[c] = off == 0 ? c4[c] : off == 1 ? c4[c + 1] : off == 2 ? c4[c + 2] : c4[c + 3];
}

template <int W>
__global__ void __launch_bounds__(256) flow_rows_kernel(const float* __restrict__ prev, const float* __restrict__ next,
                                                        const int2* xy, const Motion* m, int cap, int w, int h,
                                                        float2* flow) {
  constexpr int HALF = W / 2;
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= min(m->corners, cap)) return;
  const int2 p = xy[f];
  const long long total = (long long)w * h;
  float dx = 0.f, dy = 0.f;
  for (int iter = 0; iter < 10; ++iter) {
    float sxx = 0.f, syy = 0.f, sxy = 0.f, stx = 0.f, sty = 0.f;
    const int rdx = shift_of(dx), rdy = shift_of(dy);
    // up, mid, dn: prev rows y-1, y, y+1 at columns p.x - HALF - 1 .. p.x + HALF + 1
    float up[W + 2], mid[W + 2], dn[W + 2];
    load_row(prev, total, (long long)(p.y - HALF - 1) * w + (p.x - HALF - 1), up);
    load_row(prev, total, (long long)(p.y - HALF) * w + (p.x - HALF - 1), mid);
    for (int j = -HALF; j <= HALF; ++j) {
      const int y = p.y + j, yn = y + rdy;
      load_row(prev, total, (long long)(y + 1) * w + (p.x - HALF - 1), dn);
      float nx[W];  // next row yn at columns p.x + rdx - HALF ..
      load_row(next, total, (long long)yn * w + (p.x + rdx - HALF), nx);
      const bool row_ok = y >= 1 && y < h - 1 && yn >= 0 && yn < h - 1;
#pragma unroll
      for (int i = 0; i < W; ++i) {
        const int x = p.x - HALF + i, xn = x + rdx;
        if (!row_ok || x < 1 || x >= w - 1 || xn < 0 || xn >= w - 1) continue;
        const float ix = (mid[i + 2] - mid[i]) * 0.5f;
        const float iy = (dn[i + 1] - up[i + 1]) * 0.5f;
        const float it = nx[i] - mid[i + 1];
        sxx += ix * ix;
        syy += iy * iy;
        sxy += ix * iy;
        stx += ix * it;
        sty += iy * it;
      }
#pragma unroll
      for (int c = 0; c < W + 2; ++c) {
        up[c] = mid[c];
        mid[c] = dn[c];
      }
    }
    const float det = sxx * syy - sxy * sxy;
    if (fabsf(det) < 1e-6f) break;
    const float ddx = (-syy * stx + sxy * sty) / det;
    const float ddy = (sxy * stx - sxx * sty) / det;
    dx += ddx;
    dy += ddy;
    if (sqrtf(ddx * ddx + ddy * ddy) < 0.01f) break;
  }
  flow[f] = make_float2(dx, dy);
}

// The global motion: the flow summed in feature order (as the reference's host loop), its mean and
// the rounded translation. The sum is one dependent chain of additions, so one thread makes it;
// the CTA's other threads stage the flow in shared memory ahead of it (double-buffered chunks,
// coalesced), so that the chain waits on shared-memory loads, not on global-memory latency.
constexpr int kMotionThreads = 1024, kMotionChunk = 2048;  // 2 x 16 KB of float2

__global__ void __launch_bounds__(kMotionThreads) motion_kernel(const float2* __restrict__ flow, int cap, Motion* m) {
  __shared__ float4 buf[2][kMotionChunk / 2];  // float2 pairs
  const int n = min(m->corners, cap);
  const int chunks = (n + kMotionChunk - 1) / kMotionChunk;
  const float4* f4 = reinterpret_cast<const float4*>(flow);  // flow is 16-byte aligned (cudaMalloc)
  const auto stage = [&](int c) {
    const int base = c * kMotionChunk;
    for (int i = threadIdx.x; i < kMotionChunk / 2; i += kMotionThreads) {
      const int e = base + 2 * i;  // feature index of the pair's first element
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (e + 1 < n) {
        v = __ldg(f4 + (e >> 1));
      } else if (e < n) {
        const float2 q = __ldg(flow + e);
        v.x = q.x, v.y = q.y;
      }
      buf[c & 1][i] = v;
    }
  };
  float sx = 0.f, sy = 0.f;
  if (chunks > 0) stage(0);
  __syncthreads();
  for (int c = 0; c < chunks; ++c) {
    if (c + 1 < chunks) stage(c + 1);
    if (threadIdx.x == 0) {
      const int cnt = min(kMotionChunk, n - c * kMotionChunk);
      const float4* b = buf[c & 1];
      int i = 0;
#pragma unroll 8
      for (; 2 * i + 1 < cnt; ++i) {
        const float4 v = b[i];
        sx += v.x;
        sy += v.y;
        sx += v.z;
        sy += v.w;
      }
      if (2 * i < cnt) {
        sx += b[i].x;
        sy += b[i].y;
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    m->dx = n > 0 ? sx / float(n) : 0.f;
    m->dy = n > 0 ? sy / float(n) : 0.f;
    m->sx = shift_of(m->dx);
    m->sy = shift_of(m->dy);
  }
}

__global__ void __launch_bounds__(256) warp_kernel(const float* __restrict__ in, float* __restrict__ out, int w, int h,
                                                   const Motion* m) {
  const int x = blockIdx.x * kTX + threadIdx.x, y = blockIdx.y * kTY + threadIdx.y;
  if (x >= w || y >= h) return;
  const int u = x - m->sx, v = y - m->sy;
  out[(long long)y * w + x] = (u >= 0 && u < w && v >= 0 && v < h) ? in[(long long)v * w + u] : 0.f;
}

__global__ void copy_kernel(const float* __restrict__ in, float* __restrict__ out, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = in[i];
}

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

}  // namespace

struct hmp_stabilizer {
  int w = 0, h = 0, cap = 0, device = -1;
  float* resp = nullptr;
  int segs = 0;  // corner segments (rows x corner_segments_per_row)
  int* seg_count = nullptr;
  int* seg_off = nullptr;
  int2* xy = nullptr;
  float2* flow = nullptr;
  Motion* motion = nullptr;
  float* temp = nullptr;  // an in-place warp's output before the copy back
  ~hmp_stabilizer() {
    for (void* p : {static_cast<void*>(resp), static_cast<void*>(seg_count), static_cast<void*>(seg_off),
                    static_cast<void*>(xy), static_cast<void*>(flow), static_cast<void*>(motion),
                    static_cast<void*>(temp)})
      if (p) cudaFree(p);
  }
  hmp_status check(const void* a, const void* b) const {
    int dev = -1;
    cudaGetDevice(&dev);
    if (dev != device) return status_of(HMP_ERR_INVALID_VALUE, "stabilizer used on another device");
    if (!a || !b) return status_of(HMP_ERR_INVALID_DEVICE_POINTER, "frame is null");
    return status_of(HMP_OK, "");
  }
};

extern "C" {

HMP_API hmp_status hmp_stabilizer_create(int width, int height, int max_features, hmp_stabilizer** out) {
  if (!out) return status_of(HMP_ERR_INVALID_VALUE, "out is null");
  *out = nullptr;
  if (width < 3 || height < 3 || width > (1 << 15) || height > (1 << 15))
    return status_of(HMP_ERR_INVALID_VALUE, "frames must be 3..32768 pixels per side");
  const long long interior = (long long)(width - 2) * (height - 2);
  if (max_features < 0) return status_of(HMP_ERR_INVALID_VALUE, "max_features must be >= 0 (0: every interior pixel)");
  hmp_stabilizer* st = new (std::nothrow) hmp_stabilizer();
  if (!st) return status_of(HMP_ERR_MEMORY_ALLOCATION, "out of host memory");
  st->w = width;
  st->h = height;
  st->cap = int(max_features == 0 ? interior : std::min<long long>(max_features, interior));
  st->segs = height * corner_segments_per_row(width);
  cudaError_t e = cudaGetDevice(&st->device);
  const size_t px = size_t(width) * height;
  if (e == cudaSuccess) e = cudaMalloc(&st->resp, px * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&st->seg_count, size_t(st->segs) * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&st->seg_off, size_t(st->segs) * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&st->xy, size_t(std::max(st->cap, 1)) * sizeof(int2));
  if (e == cudaSuccess) e = cudaMalloc(&st->flow, size_t(std::max(st->cap, 1)) * sizeof(float2));
  if (e == cudaSuccess) e = cudaMalloc(&st->motion, sizeof(Motion));
  if (e == cudaSuccess) e = cudaMalloc(&st->temp, px * sizeof(float));
  if (e == cudaSuccess) e = cudaMemset(st->motion, 0, sizeof(Motion));
  if (e != cudaSuccess) {
    delete st;
    return cuda_failure(e, "stabilizer allocation");
  }
  *out = st;
  return status_of(HMP_OK, "");
}

HMP_API void hmp_stabilizer_destroy(hmp_stabilizer* st) { delete st; }

HMP_API hmp_status hmp_stabilizer_corners(hmp_stabilizer* st, const float* img, float k, float threshold,
                                          void* stream) {
  if (!st) return status_of(HMP_ERR_INVALID_VALUE, "stabilizer is null");
  hmp_status s = st->check(img, img);
  if (s.code) return s;
  const cudaStream_t cs = static_cast<cudaStream_t>(stream);
  const dim3 tiles((st->w + kTX - 1) / kTX, (st->h + kTY - 1) / kTY);
  harris_kernel<<<tiles, dim3(kTX, kTY), 0, cs>>>(img, st->w, st->h, k, st->resp);
  const int seg_blocks = (st->segs + 7) / 8;
  corner_count_kernel<<<seg_blocks, 256, 0, cs>>>(st->resp, st->w, st->h, threshold, st->segs, st->seg_count);
  corner_scan_kernel<<<1, 1024, 0, cs>>>(st->seg_count, st->segs, st->seg_off, st->motion);
  corner_emit_kernel<<<seg_blocks, 256, 0, cs>>>(st->resp, st->w, st->h, threshold, st->segs, st->seg_off, st->xy,
                                                 st->cap);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? status_of(HMP_OK, "") : cuda_failure(e, "corner launch");
}

HMP_API hmp_status hmp_stabilizer_flow(hmp_stabilizer* st, const float* prev, const float* next, int window_size,
                                       void* stream) {
  if (!st) return status_of(HMP_ERR_INVALID_VALUE, "stabilizer is null");
  hmp_status s = st->check(prev, next);
  if (s.code) return s;
  if (window_size < 1 || window_size > 255) return status_of(HMP_ERR_INVALID_VALUE, "window_size must be in 1..255");
  const cudaStream_t cs = static_cast<cudaStream_t>(stream);
  const unsigned blocks = unsigned((std::max(st->cap, 1) + 255) / 256);
  const bool aligned = ((reinterpret_cast<uintptr_t>(prev) | reinterpret_cast<uintptr_t>(next)) & 15u) == 0;
  if (window_size == 15 && aligned)
    flow_rows_kernel<15><<<blocks, 256, 0, cs>>>(prev, next, st->xy, st->motion, st->cap, st->w, st->h, st->flow);
  else
    flow_kernel<<<blocks, 256, 0, cs>>>(prev, next, st->xy, st->motion, st->cap, st->w, st->h, window_size, st->flow);
  motion_kernel<<<1, kMotionThreads, 0, cs>>>(st->flow, st->cap, st->motion);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? status_of(HMP_OK, "") : cuda_failure(e, "flow launch");
}

HMP_API hmp_status hmp_stabilizer_warp(hmp_stabilizer* st, const float* frame, float* out, void* stream) {
  if (!st) return status_of(HMP_ERR_INVALID_VALUE, "stabilizer is null");
  hmp_status s = st->check(frame, out);
  if (s.code) return s;
  const cudaStream_t cs = static_cast<cudaStream_t>(stream);
  const dim3 tiles((st->w + kTX - 1) / kTX, (st->h + kTY - 1) / kTY);
  const long long px = (long long)st->w * st->h;
  if (out == frame) {
    warp_kernel<<<tiles, dim3(kTX, kTY), 0, cs>>>(frame, st->temp, st->w, st->h, st->motion);
    copy_kernel<<<unsigned((px + 255) / 256), 256, 0, cs>>>(st->temp, out, px);
  } else {
    warp_kernel<<<tiles, dim3(kTX, kTY), 0, cs>>>(frame, out, st->w, st->h, st->motion);
  }
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? status_of(HMP_OK, "") : cuda_failure(e, "warp launch");
}

HMP_API hmp_status hmp_stabilizer_run(hmp_stabilizer* st, const float* prev, const float* next, float* out, float k,
                                      float threshold, int window_size, void* stream) {
  hmp_status s = hmp_stabilizer_corners(st, prev, k, threshold, stream);
  if (s.code == HMP_OK) s = hmp_stabilizer_flow(st, prev, next, window_size, stream);
  if (s.code == HMP_OK) s = hmp_stabilizer_warp(st, next, out, stream);
  return s;
}

HMP_API hmp_status hmp_stabilizer_get_features(hmp_stabilizer* st, int* xy, float* flow, int capacity,
                                               hmp_stabilize_info* info, void* stream) {
  if (!st || !info || capacity < 0 || (capacity > 0 && (!xy || !flow)))
    return status_of(HMP_ERR_INVALID_VALUE, "invalid argument");
  const cudaStream_t cs = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaStreamSynchronize(cs);
  Motion m{};
  if (e == cudaSuccess) e = cudaMemcpy(&m, st->motion, sizeof(m), cudaMemcpyDeviceToHost);
  const int n = std::min({m.corners, st->cap, capacity});
  if (e == cudaSuccess && n > 0) e = cudaMemcpy(xy, st->xy, size_t(n) * sizeof(int2), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && n > 0) e = cudaMemcpy(flow, st->flow, size_t(n) * sizeof(float2), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_failure(e, "feature copy");
  info->corners = m.corners;
  info->kept = std::min(m.corners, st->cap);
  info->dx = m.dx;
  info->dy = m.dy;
  info->shift_x = m.sx;
  info->shift_y = m.sy;
  return status_of(HMP_OK, "");
}

HMP_API hmp_status hmp_stabilizer_get_response(hmp_stabilizer* st, float* out, size_t capacity, void* stream) {
  if (!st || !out) return status_of(HMP_ERR_INVALID_VALUE, "invalid argument");
  const size_t px = size_t(st->w) * st->h;
  if (capacity < px) return status_of(HMP_ERR_INVALID_VALUE, "capacity below width * height");
  const cudaStream_t cs = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaStreamSynchronize(cs);
  if (e == cudaSuccess) e = cudaMemcpy(out, st->resp, px * sizeof(float), cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? status_of(HMP_OK, "") : cuda_failure(e, "response copy");
}

HMP_API hmp_status hmp_stabilizer_set_features(hmp_stabilizer* st, const int* xy, int n, void* stream) {
  if (!st || n < 0 || (n > 0 && !xy)) return status_of(HMP_ERR_INVALID_VALUE, "invalid argument");
  if (n > st->cap) return status_of(HMP_ERR_INVALID_VALUE, "more features than the stabilizer holds");
  for (int i = 0; i < n; ++i)  // the window's index sums stay in range for points on the frame
    if (xy[2 * i] < 0 || xy[2 * i] >= st->w || xy[2 * i + 1] < 0 || xy[2 * i + 1] >= st->h)
      return status_of(HMP_ERR_INVALID_VALUE, "feature outside the frame");
  const cudaStream_t cs = static_cast<cudaStream_t>(stream);
  Motion m{};
  m.corners = n;
  cudaError_t e = cudaSuccess;
  if (n > 0) e = cudaMemcpyAsync(st->xy, xy, size_t(n) * sizeof(int2), cudaMemcpyHostToDevice, cs);
  if (e == cudaSuccess) e = cudaMemcpyAsync(st->motion, &m, sizeof(m), cudaMemcpyHostToDevice, cs);
  if (e == cudaSuccess) e = cudaStreamSynchronize(cs);  // the host arrays may go once this returns
  return e == cudaSuccess ? status_of(HMP_OK, "") : cuda_failure(e, "feature upload");
}

}  // extern "C"
