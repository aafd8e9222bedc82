// hmp_stitcher.cu -- stitcher object and the C ABI (include/hmpano.h).
//
// Construction plans the configuration on the host (hmp_plan.cpp), uploads the gather planes and
// the mask pyramid, and allocates the pyramid levels. The first process() -- and any call whose
// frames differ in size or pitch from the previous call's -- resolves the canvas plane's packed
// entries into pixel offsets for those frames (resolve_plane_kernel). process() then launches at
// most four kernels and allocates nothing:
//   aux stream (high priority) : pyr_down (Gaussian levels), pyr_coarse (reconstruction down to
//                                level 1), pyr_fine (level 0: blend + reconstruct + pack of the
//                                write rect), forked from and joined back to the caller stream
//   caller stream              : canvas_gather of everything outside the write rect
// The hard seam (levels == 0) is a single canvas_gather on the caller stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <climits>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <new>
#include <string>
#include <vector>

#include "hmp_copyplan.h"
#include "hmp_kernels.h"
#include "hmp_plan.h"
#include "hmpano.h"

namespace {

hmp_status make_status(int code, const std::string& msg) {
  hmp_status s;
  s.code = code;
  std::snprintf(s.message, sizeof(s.message), "%s", msg.c_str());
  return s;
}

hmp_status ok_status() { return make_status(HMP_OK, ""); }

hmp_status cuda_status(cudaError_t e, const char* what) {
  return make_status(int(e), std::string(what) + ": " + cudaGetErrorString(e));
}

inline int round_up(int v, int a) { return (v + a - 1) / a * a; }

// Allocation-failure injection for tests (hmp_debug_fail_allocation): the device allocation that
// brings this countdown from 1 to 0 fails without allocating. Also the count of allocations made.
std::atomic<long long> g_alloc_fail_countdown{0};
std::atomic<long long> g_alloc_count{0};

bool injected_allocation_failure() {
  long long v = g_alloc_fail_countdown.load();
  while (v > 0)
    if (g_alloc_fail_countdown.compare_exchange_weak(v, v - 1)) return v == 1;
  return false;
}

// Little-endian baseline TIFF of float32 samples, uncompressed, one strip: ch = 1 (grey) or 4
// (RGBA, unassociated alpha), rows top to bottom, `px` holding ch floats per pixel.
bool write_tiff_f32(const std::string& path, int w, int h, int ch, const float* px) {
  std::vector<uint8_t> b;
  const auto u16 = [&](uint32_t v) {
    b.push_back(uint8_t(v));
    b.push_back(uint8_t(v >> 8));
  };
  const auto u32 = [&](uint32_t v) {
    u16(v & 0xFFFFu);
    u16(v >> 16);
  };
  const uint32_t n_tags = ch == 4 ? 12 : 11;
  const uint32_t ifd = 8, arrays = ifd + 2 + 12 * n_tags + 4;
  const uint32_t bits_at = arrays, fmt_at = arrays + 2 * ch, data_at = fmt_at + 2 * ch;
  const uint64_t data_bytes = uint64_t(w) * h * ch * 4;
  if (data_at + data_bytes > 0xFFFFFFFFull) return false;
  b.push_back('I');
  b.push_back('I');
  u16(42);
  u32(ifd);
  u16(n_tags);
  const auto tag = [&](uint32_t id, uint32_t type, uint32_t count, uint32_t value) {
    u16(id);
    u16(type);
    u32(count);
    u32(value);  // a SHORT value sits in the low half, little-endian
  };
  constexpr uint32_t kShort = 3, kLong = 4;
  tag(256, kLong, 1, uint32_t(w));
  tag(257, kLong, 1, uint32_t(h));
  tag(258, kShort, ch, ch == 1 ? 32u : bits_at);     // BitsPerSample
  tag(259, kShort, 1, 1);                            // no compression
  tag(262, kShort, 1, ch == 4 ? 2u : 1u);           // RGB / BlackIsZero
  tag(273, kLong, 1, data_at);                       // StripOffsets
  tag(277, kShort, 1, uint32_t(ch));                 // SamplesPerPixel
  tag(278, kLong, 1, uint32_t(h));                   // RowsPerStrip
  tag(279, kLong, 1, uint32_t(data_bytes));          // StripByteCounts
  tag(284, kShort, 1, 1);                            // PlanarConfiguration: contiguous
  if (ch == 4) tag(338, kShort, 1, 2);               // ExtraSamples: unassociated alpha
  tag(339, kShort, ch, ch == 1 ? 3u : fmt_at);      // SampleFormat: IEEE float
  u32(0);                                            // no next IFD
  for (int i = 0; i < ch; ++i) u16(32);
  for (int i = 0; i < ch; ++i) u16(3);
  if (ch == 1) b.resize(data_at);  // the arrays are inline for one sample
  std::ofstream f(path, std::ios::binary);
  if (!f) return false;
  f.write(reinterpret_cast<const char*>(b.data()), std::streamsize(b.size()));
  f.write(reinterpret_cast<const char*>(px), std::streamsize(data_bytes));
  return bool(f);
}

}  // namespace

struct hmp_stitcher {
  hmp::Plan plan;  // geometry; the large host arrays are released after upload
  hmp_status status = ok_status();
  int device = -1;
  std::vector<void*> allocations;
  size_t device_bytes = 0;
  // Canvas plane as the gather reads it (entries resolved to offsets for the current frames'
  // geometry) and with the planned packed entries it is resolved from.
  hmp::PlaneDev canvas_plane{}, canvas_raw{};
  bool resolved = false;  // canvas_plane holds offsets for the geometry below
  uint8_t* seg_owner = nullptr;  // per 256-pixel canvas row segment, written with the resolve
  int seg_pitch = 0;
  int geo_w[hmp::kDevMaxImages]{}, geo_h[hmp::kDevMaxImages]{};
  long long geo_pitch[hmp::kDevMaxImages]{};
  hmp::PlaneDev slot_planes[hmp::kDevMaxImages]{};
  void* G[hmp::kDevMaxImages][hmp::kDevMaxLevels]{};
  const float* maskL[hmp::kDevMaxLevels]{};
  const uint8_t* hotL[hmp::kDevMaxLevels]{};
  const uint8_t* mask0 = nullptr;
  int mask0_pitch = 0;
  int tile_down = 0, tile_coarse = 0;
  int down_residency = 0;  // pyr_down CTAs per SM, capped through its shared memory (0: no cap)
  long long fallback_ctas = 608;  // CTAs of a gated fallback launch: four per SM
  int down_cap = 0;  // N-way pyr_down: slots held in shared memory (the most any tile overlaps)
  int coarse_cap = 0;  // N-way pyr_coarse: likewise per coarse tile
  int fine_cap = 0;    // N-way pyr_fine: likewise per 64 x 16 level-0 block and its upsample halo
  size_t coarse_smem = 0;
  float4* R1 = nullptr;
  bool b5 = false;  // Binomial5 filter with at least two levels
  float4* Rl[hmp::kDevMaxLevels]{};
  uint32_t* P0[hmp::kDevMaxImages]{};  // level-0 pixels per slot over its plane rect (box filter)
  bool use_p0 = false;
  // Copy blocks (three- and N-image box pyramids, hmp_copyplan.h): the pyramid runs over its work
  // lists only, the canvas gather copies the rest of the write rect, and gated fallback launches
  // recompute everything when a copy block's source pixels hold alpha 0.
  bool copy_plan = false;  // planned for this configuration
  bool copy_on = true;     // hmp_stitcher_set_copy_blocks
  bool copy_opaque = false;  // mode 2: frames promised opaque, no alpha checks and no fallback
  const uint32_t* fine_list = nullptr;
  const uint32_t* coarse_list = nullptr;
  const uint32_t* down_list[2] = {};  // tile_down 32, 64 (nullptr where that tile is not allowed)
  int n_fine = 0, n_coarse = 0, n_down[2] = {};
  int* alpha_flag = nullptr;
  const uint8_t* support_mark = nullptr;  // per 2^(L-1) block of the blend region (pyr_fine's check)
  int sm_pitch = 0, sm_shift = 0;
  hmp::SkipMap skip{};
  uint32_t need_w[hmp::kDevMaxImages]{}, need_h[hmp::kDevMaxImages]{};
  int copy_blocks = 0, empty_blocks = 0, pyramid_blocks = 0;
  long long pyramid_pixels = 0;
  cudaStream_t aux = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_gather = nullptr;
  double m0_bytes = 0;
  int launches = 0;
  hmp::SrcSet last_src{};  // frames of the last process(), for the pyramid dump
  bool have_last = false;
  bool generic = false;    // uchar3 / float4 / float3 pixels: the level-by-level kernels
  float4* G0[hmp::kDevMaxImages]{};  // generic: level 0 per slot
  float4* Rg[2]{};                   // generic: reconstruction buffers (level-1 size)
  // Optional per-kernel event timing (hmp_stitcher_set_timing).
  static constexpr int kTimingSlots = 4096;
  static constexpr int kTimed = 4;
  bool timing = false;
  bool serialize = false;  // timing mode 2: every kernel on the caller stream, one after another
  std::vector<cudaEvent_t> tev;  // [slot][kernel][begin/end], kernels: gather, down, coarse, fine
  std::vector<unsigned char> tused;
  int tnext = 0;
  double tms[4] = {0, 0, 0, 0};
  long long tcount[4] = {0, 0, 0, 0};

  ~hmp_stitcher() {
    for (cudaEvent_t e : tev) cudaEventDestroy(e);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    if (ev_gather) cudaEventDestroy(ev_gather);
    if (aux) cudaStreamDestroy(aux);
    for (void* p : allocations) cudaFree(p);
  }

  cudaError_t alloc(void** p, size_t bytes) {
    ++g_alloc_count;
    if (injected_allocation_failure()) {
      *p = nullptr;
      return cudaErrorMemoryAllocation;
    }
    cudaError_t e = cudaMalloc(p, bytes);
    if (e == cudaSuccess) {
      allocations.push_back(*p);
      device_bytes += bytes;
    }
    return e;
  }

  // Uploads one gather plane with 16-byte aligned rows.
  cudaError_t upload_plane(const hmp::GatherPlane& g, hmp::PlaneDev& d) {
    d = hmp::PlaneDev{};
    d.x0 = g.rect.x;
    d.y0 = g.rect.y;
    d.w = g.rect.w;
    d.h = g.rect.h;
    d.default_owner = g.default_owner;
    if (g.rect.empty()) {
      d.w = d.h = 0;
      return cudaSuccess;
    }
    const int mp = round_up(g.rect.w, 8);
    void* m = nullptr;
    cudaError_t e = alloc(&m, size_t(mp) * 4 * g.rect.h);
    if (e != cudaSuccess) return e;
    e = cudaMemcpy2D(m, size_t(mp) * 4, g.map.data(), size_t(g.rect.w) * 4, size_t(g.rect.w) * 4, g.rect.h,
                     cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return e;
    d.map = static_cast<const uint32_t*>(m);
    d.map_pitch = mp;
    if (!g.owner.empty()) {
      const int op = round_up(g.rect.w, 16);
      void* o = nullptr;
      e = alloc(&o, size_t(op) * g.rect.h);
      if (e != cudaSuccess) return e;
      e = cudaMemcpy2D(o, op, g.owner.data(), g.rect.w, g.rect.w, g.rect.h, cudaMemcpyHostToDevice);
      if (e != cudaSuccess) return e;
      d.owner = static_cast<const uint8_t*>(o);
      d.owner_pitch = op;
    }
    return cudaSuccess;
  }

  // The most slot planes the footprint of any coarse tile (level-1 edge t1, its regions of levels
  // 2..L-1 with their halos, in level-0 pixels) overlaps; the same footprint rule as the kernel.
  int coarse_cap_for(int t1) const {
    const hmp::Plan& p = plan;
    const int L = p.levels;
    int best = 1;
    for (int Y1 = 0; Y1 < p.lh[1]; Y1 += t1)
      for (int X1 = 0; X1 < p.lw[1]; X1 += t1) {
        int ax = X1, ay = Y1, bx = std::min(X1 + t1, p.lw[1]), by = std::min(Y1 + t1, p.lh[1]);
        int fx0 = ax << 1, fy0 = ay << 1, fx1 = bx << 1, fy1 = by << 1;
        for (int l = 2; l < L; ++l) {
          ax >>= 1;
          ay >>= 1;
          bx = std::min(((bx - 1) >> 1) + 2, p.lw[l]);
          by = std::min(((by - 1) >> 1) + 2, p.lh[l]);
          fx0 = std::min(fx0, ax << l);
          fy0 = std::min(fy0, ay << l);
          fx1 = std::max(fx1, bx << l);
          fy1 = std::max(fy1, by << l);
        }
        int c = 0;
        for (int k = 0; k < p.n; ++k) {
          const hmp::PlaneDev& P = slot_planes[k];
          if (fx0 < P.x0 + P.w && P.x0 < fx1 && fy0 < P.y0 + P.h && P.y0 < fy1) ++c;
        }
        best = std::max(best, c);
      }
    return best;
  }

  // The most slot planes the footprint of any pyr_fine block (64 x 16 level-0 pixels of the write
  // rect plus the 2-pixel upsample halo) overlaps; the same footprint rule as the kernel.
  int fine_cap_for() const {
    const hmp::Plan& p = plan;
    const int wx0 = p.write.x - p.blend.x, wy0 = p.write.y - p.blend.y;
    const int wx1 = wx0 + p.write.w, wy1 = wy0 + p.write.h;
    int best = 1;
    for (int by0 = wy0 & ~1; by0 < wy1; by0 += 16)
      for (int bx0 = wx0 & ~1; bx0 < wx1; bx0 += 64) {
        int c = 0;
        for (int k = 0; k < p.n; ++k) {
          const hmp::PlaneDev& P = slot_planes[k];
          if (bx0 < P.x0 + P.w && P.x0 < bx0 + 66 && by0 < P.y0 + P.h && P.y0 < by0 + 18) ++c;
        }
        best = std::max(best, c);
      }
    return best;
  }

  // Default cap on pyr_down's CTAs per SM, 64-pixel tiles. Two images: 4. Its 40 KB of shared
  // memory and ~48 registers would let five share an SM, and five measured slower beside the
  // canvas gather (8500x3300 at L=6: 0.103 -> 0.090 ms per frame with the cap; three would do as
  // well, two is slower); packed five to an SM the one-wave kernel bunches onto fewer SMs. Four
  // or more images (the N-way kernel): 4 as well (eight-image 9000x2400 at L=6: 0.2057 -> 0.1971
  // ms per frame FP32, 0.2015 -> 0.1955 FP16; 3 and 5 no better than none). Three images: no cap
  // (2 to 5 measured no better).
  int default_residency() const { return (plan.n == 2 || plan.n >= 4) && tile_down == 64 ? 4 : 0; }

  // pyr_coarse's shared memory: the N-way kernel holds `coarse_cap` slots and no mask values.
  size_t coarse_smem_for(int t1) const {
    const hmp::Plan& p = plan;
    if (coarse_cap > 0) return hmp::pyr_coarse_smem(coarse_cap, 0, t1, p.levels, p.storage);
    return hmp::pyr_coarse_smem(p.n, p.mask_k, t1, p.levels, p.storage);
  }

  // The most slot planes any td x td level-0 tile of the blend region overlaps.
  int down_cap_for(int td) const {
    const hmp::Plan& p = plan;
    int best = 1;
    for (int y0 = 0; y0 < p.lh[0]; y0 += td)
      for (int x0 = 0; x0 < p.lw[0]; x0 += td) {
        int c = 0;
        for (int k = 0; k < p.n; ++k) {
          const hmp::PlaneDev& P = slot_planes[k];
          if (!(x0 >= P.x0 + P.w || y0 >= P.y0 + P.h || x0 + td <= P.x0 || y0 + td <= P.y0)) ++c;
        }
        best = std::max(best, c);
      }
    return best;
  }

  hmp_status setup() {
    hmp::Plan& p = plan;
    generic = p.generic();
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) return cuda_status(e, "cudaGetDevice");
    e = hmp::kernels_init();
    if (e != cudaSuccess) return cuda_status(e, "kernel setup");
    if (p.canvas_plane_used) {
      e = upload_plane(p.canvas, canvas_plane);
      if (e != cudaSuccess) return cuda_status(e, "canvas plane upload");
      canvas_raw = canvas_plane;
      if (canvas_plane.w > 0 && !p.generic()) {
        void* r = nullptr;
        e = alloc(&r, size_t(canvas_plane.map_pitch) * 4 * canvas_plane.h);
        if (e != cudaSuccess) return cuda_status(e, "canvas plane allocation");
        canvas_plane.map = static_cast<const uint32_t*>(r);
        seg_pitch = round_up((canvas_plane.w + hmp::kSegPixels - 1) / hmp::kSegPixels, 16);
        void* so = nullptr;
        e = alloc(&so, size_t(seg_pitch) * canvas_plane.h);
        if (e != cudaSuccess) return cuda_status(e, "canvas segment allocation");
        seg_owner = static_cast<uint8_t*>(so);
      }
    }
    // The gather runs when the canvas plane has pixels outside the write rect to fill (copy-block
    // mode adds its own count below).
    launches = p.canvas_plane_used && (p.levels == 0 || p.write.w < p.canvas_w || p.write.h < p.canvas_h) ? 1 : 0;
    if (p.levels > 0) {
      const int n = p.n, B = p.batch, L = p.levels;
      for (int k = 0; k < n; ++k) {
        e = upload_plane(p.slots[k], slot_planes[k]);
        if (e != cudaSuccess) return cuda_status(e, "slot plane upload");
      }
      // Level-0 mask: weight value (two-image) or label per blend pixel.
      mask0_pitch = round_up(p.lw[0], 16);
      void* m0 = nullptr;
      e = alloc(&m0, size_t(mask0_pitch) * p.lh[0]);
      if (e != cudaSuccess) return cuda_status(e, "mask allocation");
      e = cudaMemcpy2D(m0, mask0_pitch, p.mask0.data(), p.lw[0], p.lw[0], p.lh[0], cudaMemcpyHostToDevice);
      if (e != cudaSuccess) return cuda_status(e, "mask upload");
      mask0 = static_cast<const uint8_t*>(m0);
      const size_t px_bytes = p.storage == HMP_STORAGE_F16 ? 8 : 16;
      for (int l = 1; l < L; ++l) {
        void* mk = nullptr;
        const size_t mb = p.mask_levels[l].size() * sizeof(float);
        e = alloc(&mk, mb);
        if (e != cudaSuccess) return cuda_status(e, "mask pyramid allocation");
        e = cudaMemcpy(mk, p.mask_levels[l].data(), mb, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cuda_status(e, "mask pyramid upload");
        maskL[l] = static_cast<const float*>(mk);
        if (l < int(p.mask_hot.size()) && !p.mask_hot[l].empty()) {
          void* hk = nullptr;
          e = alloc(&hk, p.mask_hot[l].size());
          if (e != cudaSuccess) return cuda_status(e, "mask class allocation");
          e = cudaMemcpy(hk, p.mask_hot[l].data(), p.mask_hot[l].size(), cudaMemcpyHostToDevice);
          if (e != cudaSuccess) return cuda_status(e, "mask class upload");
          hotL[l] = static_cast<const uint8_t*>(hk);
        }
        for (int k = 0; k < n; ++k) {
          const size_t gb = size_t(B) * p.lw[l] * p.lh[l] * px_bytes;
          e = alloc(&G[k][l], gb);
          if (e != cudaSuccess) return cuda_status(e, "pyramid allocation");
          // Tiles that miss a slot are never written; their levels must read as zero.
          e = cudaMemset(G[k][l], 0, gb);
          if (e != cudaSuccess) return cuda_status(e, "pyramid clear");
        }
      }
      if (generic) {
        for (int k = 0; k < n; ++k) {
          void* q = nullptr;
          e = alloc(&q, size_t(B) * p.lw[0] * p.lh[0] * sizeof(float4));
          if (e != cudaSuccess) return cuda_status(e, "pyramid allocation");
          G0[k] = static_cast<float4*>(q);
        }
        for (int i = 0; i < 2 && L > 1; ++i) {
          void* q = nullptr;
          e = alloc(&q, size_t(B) * p.lw[1] * p.lh[1] * sizeof(float4));
          if (e != cudaSuccess) return cuda_status(e, "reconstruction buffer");
          Rg[i] = static_cast<float4*>(q);
        }
      }
      // Tiles: level-0 edge a multiple of 2^(L-1); smaller up-tiles for many images keep the
      // per-CTA shared memory (n+1 images' worth of two levels) within the SM.
      const int align = 1 << (L - 1);
      // Down tiles: 64 level-0 pixels amortise the per-CTA level walk; with more than three images
      // the per-tile shared memory calls for 32. Coarse tiles: 32 level-1 pixels (a multiple of
      // 2^(L-2) for every supported L); smaller ones multiply the per-CTA halo and walk.
      tile_down = std::max(n <= 3 ? 64 : 32, align);
      if (n <= 3 && align <= 32) {
        // A small blend region gives few 64-pixel tiles: below two per SM, 32-pixel tiles (four
        // times as many CTAs) measured faster (two images 561x800 at L=6: 36.5 -> 32.3 us).
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
        const long long t64 = (long long)((p.lw[0] + 63) / 64) * ((p.lh[0] + 63) / 64);
        if (sms > 0 && t64 < 2LL * sms) tile_down = 32;
      }
      if (n > 3) {
        // The N-way pyr_down keeps only a tile's overlapping slots in shared memory; size it for
        // the most any tile overlaps and prefer 64-pixel tiles while two CTAs still fit an SM.
        const auto cap_for = [&](int td) { return down_cap_for(td); };
        const int c64 = cap_for(64);
        if (align <= 64 && hmp::pyr_down_smem(c64, 64) <= 113 * 1024) {
          tile_down = 64;
          down_cap = c64;
        } else {
          down_cap = cap_for(tile_down);
        }
      }
      tile_coarse = std::max(32, align / 2);
      down_residency = default_residency();
      {
        int sms = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) == cudaSuccess && sms > 0)
          fallback_ctas = 4LL * sms;
      }
      coarse_cap = (n > 3 && L > 2) ? coarse_cap_for(tile_coarse) : 0;
      coarse_smem = coarse_smem_for(tile_coarse);
      b5 = p.filter == HMP_FILTER_BINOMIAL5 && L > 1;
      if (L > 1 && !b5 && !generic) {
        void* r = nullptr;
        e = alloc(&r, size_t(B) * p.lw[1] * p.lh[1] * sizeof(float4));
        if (e != cudaSuccess) return cuda_status(e, "reconstruction buffer");
        R1 = static_cast<float4*>(r);
      }
      // With three or more images pyr_down keeps the level-0 pixels for pyr_fine (one load per slot
      // instead of a table lookup and a gather); with two it measured slower (the extra writes
      // lengthen pyr_down more than they shorten pyr_fine), so pyr_fine gathers again.
      use_p0 = L > 1 && !b5 && n >= 3 && !generic;
      fine_cap = (use_p0 && n > 3) ? fine_cap_for() : 0;
      for (int k = 0; use_p0 && k < n; ++k) {
        const hmp::PlaneDev& P = slot_planes[k];
        if (P.w <= 0 || P.h <= 0) continue;
        void* q = nullptr;
        e = alloc(&q, size_t(B) * P.w * P.h * sizeof(uint32_t));
        if (e != cudaSuccess) return cuda_status(e, "level-0 buffer");
        P0[k] = static_cast<uint32_t*>(q);
      }
      for (int l = 1; b5 && l < L; ++l) {
        void* r = nullptr;
        e = alloc(&r, size_t(B) * p.lw[l] * p.lh[l] * sizeof(float4));
        if (e != cudaSuccess) return cuda_status(e, "reconstruction buffer");
        Rl[l] = static_cast<float4*>(r);
      }
      if (hmp::pyr_down_smem(down_cap > 0 ? down_cap : n, tile_down) > 227 * 1024)
        return make_status(HMP_ERR_NOT_SUPPORTED, "pyramid tile does not fit in shared memory");
      if (coarse_smem > 227 * 1024)
        return make_status(HMP_ERR_NOT_SUPPORTED, "pyramid tile does not fit in shared memory");
      launches += b5 ? hmp::b5_launches(L) : (L > 1 ? 2 : 0) + 1;
    }
    if (generic) launches = hmp::generic_launches(p.levels, p.canvas_plane_used);
    if (p.levels > 1 && !b5 && !generic && p.canvas_plane_used) {
      const hmp_status cs = setup_copy_blocks();
      if (cs.code != HMP_OK) return cs;
    }
    if (p.canvas_plane_used && p.levels > 0 && !generic) {
      // The pyramid chain (latency-bound, few CTAs) runs on a high-priority stream so that its
      // CTAs are dispatched ahead of the bandwidth-bound canvas gather sharing the SMs.
      int least = 0, greatest = 0;
      cudaDeviceGetStreamPriorityRange(&least, &greatest);
      e = cudaStreamCreateWithPriority(&aux, cudaStreamNonBlocking, greatest);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev_gather, cudaEventDisableTiming);
      if (e != cudaSuccess) return cuda_status(e, "stream setup");
    }
    // The uploads and clears ran on the legacy default stream; wait for them only, so that a
    // stitcher created while others run (a server admitting a configuration) does not stall them.
    e = cudaStreamSynchronize(nullptr);
    if (e != cudaSuccess) return cuda_status(e, "upload");
    compute_m0();
    // Release the large host-side arrays; geometry stays.
    std::vector<uint8_t>().swap(p.canvas.owner);
    std::vector<uint32_t>().swap(p.canvas.map);
    for (auto& s : p.slots) {
      std::vector<uint8_t>().swap(s.owner);
      std::vector<uint32_t>().swap(s.map);
    }
    std::vector<uint8_t>().swap(p.mask0);
    for (auto& m : p.mask_levels) std::vector<float>().swap(m);
    for (auto& m : p.mask_hot) std::vector<uint8_t>().swap(m);
    return ok_status();
  }

  cudaError_t upload_list(const std::vector<uint32_t>& v, const uint32_t** out) {
    *out = nullptr;
    if (v.empty()) return cudaSuccess;
    void* d = nullptr;
    cudaError_t e = alloc(&d, v.size() * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemcpy(d, v.data(), v.size() * sizeof(uint32_t), cudaMemcpyHostToDevice);
    *out = static_cast<const uint32_t*>(d);
    return e;
  }

  // Copy blocks: plans them (for both pyramid down-tile edges the tile setter allows) and uploads
  // the work lists, the pyramid-block map the resolve pass marks and the alpha flag.
  hmp_status setup_copy_blocks() {
    const hmp::Plan& p = plan;
    const int align = 1 << (p.levels - 1);
    hmp::CopyPlan cps[2];
    for (int i = 0; i < 2; ++i) {
      const int td = i == 0 ? 32 : 64;
      if (td % align == 0) hmp::plan_copy_blocks(p, td, tile_coarse, cps[i]);
    }
    const hmp::CopyPlan& c = cps[1].usable ? cps[1] : cps[0];
    if (!c.usable) return ok_status();
    cudaError_t e = upload_list(c.fine_list, &fine_list);
    if (e == cudaSuccess) e = upload_list(c.coarse_list, &coarse_list);
    for (int i = 0; i < 2 && e == cudaSuccess; ++i) {
      if (!cps[i].usable) continue;
      e = upload_list(cps[i].down_list, &down_list[i]);
      n_down[i] = int(cps[i].down_list.size());
    }
    // The pyramid-block map, then the flag (4-byte aligned; allocations are 256-byte aligned).
    const size_t flag_off = (c.pyramid_block.size() + 3) / 4 * 4;
    void* m = nullptr;
    if (e == cudaSuccess) e = alloc(&m, flag_off + 2 * sizeof(int));
    if (e == cudaSuccess)
      e = cudaMemcpy(m, c.pyramid_block.data(), c.pyramid_block.size(), cudaMemcpyHostToDevice);
    // The flag and the fallback's CTA count start at 0; the fallback clears both whenever it ran.
    if (e == cudaSuccess) e = cudaMemset(static_cast<char*>(m) + flag_off, 0, 2 * sizeof(int));
    if (e != cudaSuccess) return cuda_status(e, "copy-block upload");
    n_fine = int(c.fine_list.size());
    n_coarse = int(c.coarse_list.size());
    alpha_flag = reinterpret_cast<int*>(static_cast<char*>(m) + flag_off);
    void* sm = nullptr;
    e = alloc(&sm, c.support_mark.size());
    if (e == cudaSuccess) e = cudaMemcpy(sm, c.support_mark.data(), c.support_mark.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_status(e, "copy-block support upload");
    support_mark = static_cast<const uint8_t*>(sm);
    sm_pitch = c.support_pitch;
    sm_shift = c.support_shift;
    skip.map = static_cast<const uint8_t*>(m);
    skip.pitch = c.nfx;
    skip.x0 = c.fx0 + p.blend.x;
    skip.y0 = c.fy0 + p.blend.y;
    skip.nx = c.nfx;
    skip.ny = c.nfy;
    skip.wr_x0 = p.write.x;
    skip.wr_y0 = p.write.y;
    skip.wr_x1 = p.write.x + p.write.w;
    skip.wr_y1 = p.write.y + p.write.h;
    for (int k = 0; k < p.n; ++k) {
      need_w[k] = c.need_w[k];
      need_h[k] = c.need_h[k];
    }
    copy_blocks = c.copy_blocks;
    empty_blocks = c.empty_blocks;
    pyramid_blocks = c.pyramid_blocks;
    pyramid_pixels = c.pyramid_pixels;
    copy_plan = true;
    return ok_status();
  }

  // Kernels one process() launches in copy-block mode: the flag reset, the listed pyramid kernels,
  // the gather and the three gated fallbacks.
  int copy_launches() const {
    return (n_down[tile_down == 64 ? 1 : 0] > 0) + (n_coarse > 0) + (n_fine > 0) + 1 + (copy_opaque ? 0 : 1);
  }

  // Compulsory bytes per process(): outside the write rect, 4 (table) + 1 (seam) + a source and
  // a canvas pixel per canvas pixel; inside it, 4 + a source pixel per mapped slot pixel, 1 (seam)
  // + a canvas pixel per pixel (4 bytes for RGBA8). Tables and seam are read once per call,
  // sources and canvas once per frame.
  void compute_m0() {
    const hmp::Plan& p = plan;
    const double B = p.batch;
    const double canvas_px = double(p.canvas_w) * p.canvas_h;
    const double a0 = p.levels > 0 ? double(p.write.w) * p.write.h : 0.0;
    const double px = p.pixel_bytes();
    double bytes = (canvas_px - a0) * (5.0 + 2.0 * px * B);
    if (p.levels > 0) {
      double mapped = 0;
      for (const auto& s : p.slots)
        for (uint32_t e : s.map) mapped += e != hmp::kNoEntry;
      bytes += mapped * (4.0 + px * B) + a0 * (1.0 + px * B);
    }
    m0_bytes = bytes;
  }

  // The soft-blend pyramid of the last process() (cudaPano.inl:420-458): every level of the two
  // Gaussian pyramids, the mask, both Laplacians, the blend and the reconstruction, as float32 TIFF
  // files `<label>/level_<l>_batch_<b>.tiff` (`mask/level_<l>.tiff`) plus metadata.txt. The fused
  // kernels keep these levels on chip, so they are recomputed here from the last frames (which must
  // still hold them) by plain kernels using the same device functions; not a per-frame call.
  hmp_status dump_pyramid(const char* directory, cudaStream_t s) {
    const hmp::Plan& p = plan;
    if (!directory) return make_status(HMP_ERR_INVALID_VALUE, "directory is null");
    if (p.levels == 0)
      return make_status(HMP_ERR_INVALID_VALUE, "Soft-blend pyramid is only available when num_levels > 0");
    if (p.rule != hmp::kRuleTwo || b5 || (generic && p.channels != 4))
      return make_status(HMP_ERR_NOT_SUPPORTED,
                         "the pyramid dump covers two-image stitchers of RGBA pixels with the box filter");
    if (!have_last) return make_status(HMP_ERR_INVALID_VALUE, "No Laplacian workspace is populated yet: call process() first");
    int dev = -1;
    cudaGetDevice(&dev);
    if (dev != device) return make_status(HMP_ERR_INVALID_VALUE, "dump called on another device");
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_status(e, "stream synchronize");
    namespace fs = std::filesystem;
    const fs::path root(directory);
    std::error_code ec;
    for (const char* sub : {"", "gauss1", "gauss2", "mask", "lap1", "lap2", "blend", "reconstruct"}) {
      fs::create_directories(root / sub, ec);
      if (ec) return make_status(HMP_ERR_UNKNOWN, "Unable to create directory " + (root / sub).string() + ": " + ec.message());
    }
    const int L = p.levels, B = p.batch;
    std::vector<void*> owned;
    struct Free {
      std::vector<void*>& v;
      ~Free() {
        for (void* q : v) cudaFree(q);
      }
    } free_all{owned};
    const auto level_bytes = [&](int l) { return size_t(B) * p.lw[l] * p.lh[l] * sizeof(float4); };
    std::vector<float4*> g[2], lap[2], bl(L), rc(L);
    for (int l = 0; l < L; ++l) {
      for (float4** slot : {&bl[l], &rc[l]}) {
        void* q = nullptr;
        if ((e = cudaMalloc(&q, level_bytes(l))) != cudaSuccess) return cuda_status(e, "dump allocation");
        owned.push_back(q);
        *slot = static_cast<float4*>(q);
      }
      for (int k = 0; k < 2; ++k)
        for (auto* v : {&g[k], &lap[k]}) {
          void* q = nullptr;
          if ((e = cudaMalloc(&q, level_bytes(l))) != cudaSuccess) return cuda_status(e, "dump allocation");
          owned.push_back(q);
          v->push_back(static_cast<float4*>(q));
        }
    }
    hmp::PyrArgs a = pyr_args(last_src, hmp::CanvasDev{});
    if (copy_plan && L > 1) {
      // Copy-block mode computes the Gaussian levels only where the pyramid runs: all of them here.
      const dim3 dgrid((p.lw[0] + tile_down - 1) / tile_down, (p.lh[0] + tile_down - 1) / tile_down, B);
      e = hmp::launch_pyr_down(a, p.storage, dgrid, s);
    }
    for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
      if (generic) {
        // float4 pixels: the level-by-level kernels keep every Gaussian level, level 0 included.
        e = cudaMemcpyAsync(g[k][0], G0[k], level_bytes(0), cudaMemcpyDeviceToDevice, s);
        for (int l = 1; l < L && e == cudaSuccess; ++l)
          e = cudaMemcpyAsync(g[k][l], G[k][l], level_bytes(l), cudaMemcpyDeviceToDevice, s);
      } else {
        e = hmp::launch_dump_level0(a, k, g[k][0], B, s);
        for (int l = 1; l < L && e == cudaSuccess; ++l)
          e = hmp::launch_dump_widen(G[k][l], p.storage, (long long)B * p.lw[l] * p.lh[l], g[k][l], s);
      }
      for (int l = 0; l + 1 < L && e == cudaSuccess; ++l)
        e = hmp::launch_dump_lap(g[k][l], p.lw[l], p.lh[l], g[k][l + 1], p.lw[l + 1], p.lh[l + 1], lap[k][l], B, s);
      if (e == cudaSuccess)  // the coarsest Laplacian is the Gaussian itself
        e = cudaMemcpyAsync(lap[k][L - 1], g[k][L - 1], level_bytes(L - 1), cudaMemcpyDeviceToDevice, s);
    }
    for (int l = 0; l < L && e == cudaSuccess; ++l)
      e = hmp::launch_dump_blend2(lap[0][l], lap[1][l], l ? maskL[l] : nullptr, mask0, mask0_pitch, p.lw[l], p.lh[l], bl[l],
                                  B, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(rc[L - 1], bl[L - 1], level_bytes(L - 1), cudaMemcpyDeviceToDevice, s);
    for (int l = L - 2; l >= 0 && e == cudaSuccess; --l)
      e = hmp::launch_dump_recon(rc[l + 1], p.lw[l + 1], p.lh[l + 1], bl[l], p.lw[l], p.lh[l], rc[l], B, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_status(e, "pyramid dump");
    {
      std::ofstream meta(root / "metadata.txt");
      meta << "num_levels=" << L << "\n" << "batch_size=" << B << "\n" << "channels=4\n";
      for (int l = 0; l < L; ++l) meta << "level_" << l << "=" << p.lw[l] << "x" << p.lh[l] << "\n";
      if (!meta) return make_status(HMP_ERR_UNKNOWN, "Unable to write " + (root / "metadata.txt").string());
    }
    std::vector<float> host;
    const auto write_level = [&](const float4* d, int l, const char* label) -> hmp_status {
      const size_t px = size_t(p.lw[l]) * p.lh[l];
      host.resize(px * 4 * B);
      const cudaError_t ce = cudaMemcpy(host.data(), d, level_bytes(l), cudaMemcpyDeviceToHost);
      if (ce != cudaSuccess) return cuda_status(ce, "pyramid dump copy");
      for (int b = 0; b < B; ++b) {
        const fs::path f = root / label / ("level_" + std::to_string(l) + "_batch_" + std::to_string(b) + ".tiff");
        if (!write_tiff_f32(f.string(), p.lw[l], p.lh[l], 4, host.data() + px * 4 * b))
          return make_status(HMP_ERR_UNKNOWN, "Unable to write " + f.string());
      }
      return ok_status();
    };
    for (int l = 0; l < L; ++l) {
      const std::pair<const float4*, const char*> items[] = {{g[0][l], "gauss1"}, {g[1][l], "gauss2"}, {lap[0][l], "lap1"},
                                                             {lap[1][l], "lap2"},  {bl[l], "blend"},     {rc[l], "reconstruct"}};
      for (const auto& it : items) {
        const hmp_status st = write_level(it.first, l, it.second);
        if (st.code != HMP_OK) return st;
      }
      // Mask level: the seam weights of image 1 at level 0, the mask pyramid above.
      const size_t px = size_t(p.lw[l]) * p.lh[l];
      std::vector<float> m(px);
      if (l == 0) {
        std::vector<uint8_t> m8(size_t(mask0_pitch) * p.lh[0]);
        e = cudaMemcpy(m8.data(), mask0, m8.size(), cudaMemcpyDeviceToHost);
        for (int y = 0; y < p.lh[0]; ++y)
          for (int x = 0; x < p.lw[0]; ++x) m[size_t(y) * p.lw[0] + x] = float(m8[size_t(y) * mask0_pitch + x]);
      } else {
        e = cudaMemcpy(m.data(), maskL[l], px * sizeof(float), cudaMemcpyDeviceToHost);
      }
      if (e != cudaSuccess) return cuda_status(e, "pyramid dump copy");
      const fs::path f = root / "mask" / ("level_" + std::to_string(l) + ".tiff");
      if (!write_tiff_f32(f.string(), p.lw[l], p.lh[l], 1, m.data()))
        return make_status(HMP_ERR_UNKNOWN, "Unable to write " + f.string());
    }
    return ok_status();
  }

  cudaError_t timing_enable(int mode) {
    const bool on = mode != 0;
    serialize = mode == 2;
    if (on && tev.empty()) {
      tev.resize(size_t(kTimingSlots) * kTimed * 2);
      for (auto& e : tev) {
        cudaError_t r = cudaEventCreate(&e);
        if (r != cudaSuccess) return r;
      }
      tused.assign(size_t(kTimingSlots) * kTimed, 0);
    }
    timing = on;
    tnext = 0;
    std::fill(tused.begin(), tused.end(), 0);
    for (int k = 0; k < kTimed; ++k) tms[k] = 0, tcount[k] = 0;
    return cudaSuccess;
  }

  cudaEvent_t tbegin(int kernel, cudaStream_t s) {
    if (!timing || tnext >= kTimingSlots) return nullptr;
    cudaEventRecord(tev[(size_t(tnext) * kTimed + kernel) * 2], s);
    return tev[(size_t(tnext) * kTimed + kernel) * 2];
  }
  void tend(int kernel, cudaStream_t s) {
    if (!timing || tnext >= kTimingSlots) return;
    cudaEventRecord(tev[(size_t(tnext) * kTimed + kernel) * 2 + 1], s);
    tused[size_t(tnext) * kTimed + kernel] = 1;
  }

  cudaError_t timing_collect(hmp_kernel_timing* out) {
    for (int slot = 0; slot < tnext; ++slot)
      for (int k = 0; k < kTimed; ++k) {
        if (!tused[size_t(slot) * kTimed + k]) continue;
        float ms = 0;
        cudaEvent_t e1 = tev[(size_t(slot) * kTimed + k) * 2 + 1];
        cudaError_t r = cudaEventSynchronize(e1);
        if (r == cudaSuccess) r = cudaEventElapsedTime(&ms, tev[(size_t(slot) * kTimed + k) * 2], e1);
        if (r != cudaSuccess) return r;
        tms[k] += ms;
        tcount[k] += 1;
      }
    for (int k = 0; k < kTimed; ++k) {
      out->total_ms[k] = tms[k];
      out->launches[k] = tcount[k];
      tms[k] = 0;
      tcount[k] = 0;
    }
    tnext = 0;
    std::fill(tused.begin(), tused.end(), 0);
    return cudaSuccess;
  }

  // Parameters of the pyramid kernels for frames S and canvas C (dense grids; no work lists).
  hmp::PyrArgs pyr_args(const hmp::SrcSet& S, const hmp::CanvasDev& C) const {
    const hmp::Plan& p = plan;
    hmp::PyrArgs a{};
    a.S = S;
    for (int k = 0; k < p.n; ++k) a.slot[k] = slot_planes[k];
    a.n = p.n;
    a.levels = p.levels;
    for (int l = 0; l < p.levels; ++l) {
      a.lw[l] = p.lw[l];
      a.lh[l] = p.lh[l];
      a.maskL[l] = maskL[l];
      a.hotL[l] = hotL[l];
      for (int k = 0; k < p.n; ++k) a.G[k][l] = G[k][l];
    }
    a.mask0 = mask0;
    a.mask0_pitch = mask0_pitch;
    a.K = p.mask_k;
    a.opaque = p.slot_opaque ? 1 : 0;
    a.C = C;
    a.wx0 = p.write.x - p.blend.x;
    a.wy0 = p.write.y - p.blend.y;
    a.wx1 = a.wx0 + p.write.w;
    a.wy1 = a.wy0 + p.write.h;
    a.cx_off = p.blend.x;
    a.cy_off = p.blend.y;
    a.use_p0 = use_p0 ? 1 : 0;
    a.fine_cap = fine_cap;
    a.pdl = p.levels > 1 && !b5 ? 1 : 0;  // pyr_coarse follows pyr_down, pyr_fine pyr_coarse
    for (int k = 0; k < p.n; ++k) a.P0[k] = P0[k];
    a.slots_cap = down_cap;
    a.coarse_cap = coarse_cap;
    a.tile = tile_down;
    a.down_smem_floor = int(hmp::residency_smem(down_residency));
    a.list_frames = 1;
    return a;
  }

  hmp::SrcSet sources(const hmp_image* inputs) const {
    hmp::SrcSet S{};
    for (int i = 0; i < plan.n; ++i) {
      S.ptr[i] = static_cast<const uchar4*>(inputs[i].data);
      S.pitch[i] = (long long)inputs[i].pitch;
      S.bstride[i] = (long long)inputs[i].pitch * inputs[i].height;
      S.w[i] = inputs[i].width;
      S.h[i] = inputs[i].height;
    }
    return S;
  }

  // uchar3 / float4 / float3 pixels: the canvas outside the write rect, then the pyramid level by
  // level, all on the caller's stream (hmp_generic.cu).
  hmp_status process_generic(const hmp::SrcSet& S, const hmp_image* canvas, cudaStream_t s) {
    const hmp::Plan& p = plan;
    hmp::CanvasDev C;
    C.ptr = static_cast<uchar4*>(canvas->data);
    C.pitch = (long long)canvas->pitch;
    C.bstride = (long long)canvas->pitch * canvas->height;
    C.w = canvas->width;
    C.h = canvas->height;
    cudaError_t e = cudaSuccess;
    if (p.canvas_plane_used) {
      hmp::GatherArgs g{};
      g.S = S;
      g.P = canvas_raw;
      g.C = C;
      g.batch = p.batch;
      g.n_owners = p.n;
      if (p.levels > 0) {
        g.skip_x0 = p.write.x;
        g.skip_y0 = p.write.y;
        g.skip_x1 = p.write.x + p.write.w;
        g.skip_y1 = p.write.y + p.write.h;
      }
      e = hmp::launch_generic_canvas(g, p.channels, p.pixel_float, p.canvas_opaque, s);
      if (e != cudaSuccess) return cuda_status(e, "canvas launch");
    }
    if (p.levels > 0) {
      hmp::GenArgs a{};
      a.S = S;
      for (int k = 0; k < p.n; ++k) a.slot[k] = slot_planes[k];
      a.n = p.n;
      a.levels = p.levels;
      for (int l = 0; l < p.levels; ++l) {
        a.lw[l] = p.lw[l];
        a.lh[l] = p.lh[l];
        a.maskL[l] = maskL[l];
        for (int k = 0; k < p.n; ++k) a.G[k][l] = l == 0 ? G0[k] : static_cast<float4*>(G[k][l]);
      }
      a.mask0 = mask0;
      a.mask0_pitch = mask0_pitch;
      a.K = p.mask_k;
      a.opaque = p.slot_opaque ? 1 : 0;
      a.C = C;
      a.wx0 = p.write.x - p.blend.x;
      a.wy0 = p.write.y - p.blend.y;
      a.wx1 = a.wx0 + p.write.w;
      a.wy1 = a.wy0 + p.write.h;
      a.cx_off = p.blend.x;
      a.cy_off = p.blend.y;
      e = hmp::launch_generic_pyramid(a, p.channels, p.pixel_float, p.rule, p.batch, Rg, s);
      if (e != cudaSuccess) return cuda_status(e, "pyramid launch");
    }
    return ok_status();
  }

  hmp_status process(const hmp_image* inputs, int n_inputs, const hmp_image* canvas, cudaStream_t s) {
    const hmp::Plan& p = plan;
    if (!inputs || n_inputs != p.n) return make_status(HMP_ERR_INVALID_VALUE, "inputs size != N");
    if (!canvas || !canvas->data) return make_status(HMP_ERR_INVALID_DEVICE_POINTER, "Canvas must be provided");
    const size_t pxb = size_t(p.pixel_bytes()), align = p.pixel_float ? 4 : (generic ? 1 : 4);
    if (canvas->width != p.canvas_w || canvas->height != p.canvas_h || canvas->pitch < size_t(canvas->width) * pxb ||
        canvas->pitch % align != 0)
      return make_status(HMP_ERR_INVALID_VALUE, "canvas size does not match the stitcher");
    // The kernels load and store whole 4-byte words of RGBA8 and float pixels.
    if (reinterpret_cast<uintptr_t>(canvas->data) % align != 0)
      return make_status(HMP_ERR_INVALID_VALUE, "canvas data must be aligned to 4 bytes");
    for (int i = 0; i < n_inputs; ++i) {
      const hmp_image& im = inputs[i];
      if (!im.data) return make_status(HMP_ERR_INVALID_DEVICE_POINTER, "input image is null");
      if (im.width <= 0 || im.height <= 0 || im.pitch < size_t(im.width) * pxb || im.pitch > size_t(INT_MAX) ||
          im.pitch % align != 0 || reinterpret_cast<uintptr_t>(im.data) % align != 0)
        return make_status(HMP_ERR_INVALID_VALUE, "input image has an invalid size, pitch or alignment");
      if (!generic && size_t(im.height) * (im.pitch / 4) >= size_t(hmp::kOffMask) - 1)
        return make_status(HMP_ERR_NOT_SUPPORTED, "input frames must hold fewer than 2^29 - 2 pixels");
      if (im.width >= 65535 || im.height >= 65535)
        return make_status(HMP_ERR_INVALID_VALUE, "input images must be smaller than 65535 pixels per side");
    }
    int dev = -1;
    cudaGetDevice(&dev);
    if (dev != device) return make_status(HMP_ERR_INVALID_VALUE, "process() called on another device");

    const hmp::SrcSet S = sources(inputs);
    last_src = S;
    have_last = true;
    if (generic) return process_generic(S, canvas, s);
    if (p.canvas_plane_used) {
      // The gather reads the canvas plane as offsets into these frames: resolve it for their
      // geometry on the first call and whenever a size or pitch changes.
      bool same = resolved;
      for (int i = 0; i < p.n; ++i)
        same = same && S.w[i] == geo_w[i] && S.h[i] == geo_h[i] && S.pitch[i] == geo_pitch[i];
      if (!same) {
        const cudaError_t re = hmp::launch_resolve_plane(canvas_raw, const_cast<uint32_t*>(canvas_plane.map), seg_owner,
                                                         seg_pitch, S, p.n, p.canvas_opaque,
                                                         copy_plan ? skip : hmp::SkipMap{}, s);
        if (re != cudaSuccess) return cuda_status(re, "canvas plane resolve launch");
        for (int i = 0; i < p.n; ++i) {
          geo_w[i] = S.w[i];
          geo_h[i] = S.h[i];
          geo_pitch[i] = S.pitch[i];
        }
        resolved = true;
      }
    }
    hmp::CanvasDev C;
    C.ptr = static_cast<uchar4*>(canvas->data);
    C.pitch = (long long)canvas->pitch;
    C.bstride = (long long)canvas->pitch * canvas->height;
    C.w = canvas->width;
    C.h = canvas->height;

    // Copy-block mode for this call: planned, switched on, and every table entry the copy blocks
    // read lies inside these frames (else it would read as a fill).
    const int di = tile_down == 64 ? 1 : 0;
    // Listed launches interleave the call's frames in grid.x, which must hold entries x frames.
    const long long longest = std::max<long long>({n_down[di], n_coarse, n_fine});
    bool copy = copy_plan && copy_on && (n_fine == 0 || down_list[di] != nullptr) &&
                longest * p.batch < (1LL << 31) - 1;
    for (int k = 0; copy && k < p.n; ++k) copy = uint32_t(S.w[k]) >= need_w[k] && uint32_t(S.h[k]) >= need_h[k];
    hmp::GatherArgs ga{};
    if (p.canvas_plane_used) {
      ga.S = S;
      ga.P = canvas_plane;
      ga.C = C;
      ga.batch = p.batch;
      ga.n_owners = p.n;
      ga.seg_owner = seg_owner;
      ga.seg_pitch = seg_pitch;
      if (copy) {
        // The gather writes the copy blocks too (the pyramid blocks' entries are skips) and checks
        // the alpha of every source pixel it reads over the blend region (unless the caller
        // promised opaque frames).
        ga.alpha_flag = copy_opaque ? nullptr : alpha_flag;
        ga.chk_x0 = p.blend.x;
        ga.chk_y0 = p.blend.y;
        ga.chk_x1 = p.blend.x + p.blend.w;
        ga.chk_y1 = p.blend.y + p.blend.h;
      } else if (p.levels > 0) {
        ga.skip_x0 = p.write.x;
        ga.skip_y0 = p.write.y;
        ga.skip_x1 = p.write.x + p.write.w;
        ga.skip_y1 = p.write.y + p.write.h;
      }
    }
    // Without copy blocks a write rect covering the canvas leaves the gather nothing to do.
    const bool gather = p.canvas_plane_used &&
                        (p.levels == 0 || copy || p.write.w < p.canvas_w || p.write.h < p.canvas_h);
    cudaError_t e;
    if (p.levels == 0) {
      tbegin(0, s);
      e = hmp::launch_canvas_gather(ga, copy_plan, s);
      tend(0, s);
      if (timing && tnext < kTimingSlots) ++tnext;
      if (e != cudaSuccess) return cuda_status(e, "canvas_gather launch");
      return ok_status();
    }
    // Fork: the pyramid goes to the high-priority stream `aux` when the canvas gather also
    // runs; the gather is launched on the caller stream after the pyramid kernels.
    const bool fork = gather && !serialize;
    cudaStream_t ps = s;
    if (fork) {
      e = cudaEventRecord(ev_fork, s);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(aux, ev_fork, 0);
      if (e != cudaSuccess) return cuda_status(e, "stream fork");
      ps = aux;
    }
    // A failed launch after the fork still joins the pyramid stream back, so that the caller's
    // stream waits for whatever was already queued there.
    const auto failed = [&](cudaError_t err, const char* what) {
      if (fork) {
        cudaEventRecord(ev_join, aux);
        cudaStreamWaitEvent(s, ev_join, 0);
      }
      return cuda_status(err, what);
    };
    hmp::PyrArgs a = pyr_args(S, C);
    if (b5) {
      // Binomial5: the level-by-level chain (its time is reported under pyr_down).
      for (int l = 1; l < p.levels; ++l) a.Rl[l] = Rl[l];
      tbegin(1, ps);
      e = hmp::launch_b5_pyramid(a, p.rule, p.storage, p.batch, ps);
      tend(1, ps);
      if (e != cudaSuccess) return failed(e, "Binomial5 pyramid launch");
    }
    // Dense grids: every down tile of the blend region, the level-1 tiles holding the level-1
    // pixels the fine pass reads (floor(x/2) and floor(x/2)+1 of the write rect), every 64 x 16
    // block of the write rect.
    a.R1 = R1;
    const dim3 dgrid((p.lw[0] + tile_down - 1) / tile_down, (p.lh[0] + tile_down - 1) / tile_down, p.batch);
    dim3 cgrid(1, 1, 1);
    if (p.levels > 1) {
      const int x1lo = a.wx0 >> 1, x1hi = std::min(((a.wx1 - 1) >> 1) + 2, p.lw[1]);
      const int y1lo = a.wy0 >> 1, y1hi = std::min(((a.wy1 - 1) >> 1) + 2, p.lh[1]);
      a.tx0 = x1lo / tile_coarse;
      a.ty0 = y1lo / tile_coarse;
      cgrid = dim3((x1hi + tile_coarse - 1) / tile_coarse - a.tx0, (y1hi + tile_coarse - 1) / tile_coarse - a.ty0,
                   p.batch);
    }
    const int fx0 = a.wx0 & ~1, fy0 = a.wy0 & ~1;
    const dim3 fgrid((a.wx1 - fx0 + 63) / 64, (a.wy1 - fy0 + 15) / 16, p.batch);
    // The pyramid chain: dense, or (copy-block mode) over the work lists, or as the gated fallback,
    // whose few CTAs walk the dense grids (every tile of every frame) only when the gate is set.
    const auto walk = [&](const dim3& dense) {
      const long long tiles = (long long)dense.x * dense.y * dense.z;
      return dim3(unsigned(std::min<long long>(tiles, fallback_ctas)), 1, 1);
    };
    const auto chain = [&](const hmp::PyrArgs& base, bool listed, cudaStream_t cs, bool timed) -> hmp_status {
      hmp::PyrArgs q = base;
      const bool gated = q.gate != nullptr;
      const auto grid_of = [&](const dim3& dense, int n_list) {
        if (listed) {
          q.list_frames = p.batch;
          return dim3(unsigned(n_list) * unsigned(p.batch), 1, 1);
        }
        if (gated) {
          q.fb_nx = int(dense.x);
          q.fb_ny = int(dense.y);
          q.fb_batch = int(dense.z);
          return walk(dense);
        }
        return dense;
      };
      if (p.levels > 1 && !b5 && (!listed || n_down[di] > 0)) {
        q.tile = tile_down;
        q.tiles = listed ? down_list[di] : nullptr;
        const dim3 g = grid_of(dgrid, n_down[di]);
        if (timed) tbegin(1, cs);
        e = hmp::launch_pyr_down(q, p.storage, g, cs);
        if (timed) tend(1, cs);
        if (e != cudaSuccess) return failed(e, "pyr_down launch");
      }
      if (p.levels > 1 && !b5 && (!listed || n_coarse > 0)) {
        q.tile = tile_coarse;
        q.tiles = listed ? coarse_list : nullptr;
        const dim3 g = grid_of(cgrid, n_coarse);
        if (timed) tbegin(2, cs);
        e = hmp::launch_pyr_coarse(q, p.rule, p.storage, g, coarse_smem, cs);
        if (timed) tend(2, cs);
        if (e != cudaSuccess) return failed(e, "pyr_coarse launch");
      }
      if (!b5 && (!listed || n_fine > 0)) {
        q.tiles = listed ? fine_list : nullptr;
        const dim3 g = grid_of(fgrid, n_fine);
        if (timed) tbegin(3, cs);
        e = hmp::launch_pyr_fine(q, p.rule, p.storage, g, cs);
        if (timed) tend(3, cs);
        if (e != cudaSuccess) return failed(e, "pyr_fine launch");
      }
      return ok_status();
    };
    if (copy) {  // pyr_fine checks the pyramid-block pixels inside copy blocks' supports
      a.alpha_flag = copy_opaque ? nullptr : alpha_flag;
      a.support_mark = support_mark;
      a.sm_pitch = sm_pitch;
      a.sm_shift = sm_shift;
    }
    hmp_status cst = chain(a, copy, ps, true);
    if (cst.code != HMP_OK) return cst;
    // Copy-block fallback, after the gather wrote the copy blocks: it recomputes the whole write
    // rect densely if a copy block's source pixels held alpha 0, and clears the flag. Outside a
    // stream capture it is one thread (hmp_fallback.cu) that returns at once unless the flag is
    // set, then tail-launches the dense chain; with the gather forked it runs on the pyramid
    // stream after pyr_fine and the gather, so the caller stream's join follows it directly.
    // In a CUDA graph the gate's device-side launches did not run (the graph replay test of copy
    // blocks on alpha-0 frames caught it), so a captured call keeps three gated launches whose
    // CTAs walk the dense tiles when the flag is set; the last one clears it.
    // With frames promised opaque (hmp_stitcher_set_copy_blocks mode 2) nothing is checked and no
    // fallback is launched.
    const bool checked = copy && !copy_opaque;
    cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
    if (checked) {
      e = cudaStreamIsCapturing(s, &capture);
      if (e != cudaSuccess) return failed(e, "stream capture query");
    }
    const bool gate = checked && capture == cudaStreamCaptureStatusNone;
    hmp::PyrArgs f = a;
    f.gate = alpha_flag;
    if (gather) {
      tbegin(0, s);
      e = hmp::launch_canvas_gather(ga, copy_plan, s);
      tend(0, s);
      if (e != cudaSuccess) return failed(e, "canvas_gather launch");
    }
    if (gate && fork) {
      e = cudaEventRecord(ev_gather, s);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(aux, ev_gather, 0);
      if (e == cudaSuccess)
        e = hmp::launch_fallback_gate(f, p.rule, p.storage, tile_down, tile_coarse, dgrid, cgrid, fgrid, coarse_smem,
                                      aux);
      if (e != cudaSuccess) return failed(e, "copy-block fallback launch");
    }
    if (fork) {
      e = cudaEventRecord(ev_join, aux);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(s, ev_join, 0);
      if (e != cudaSuccess) return cuda_status(e, "stream join");
    }
    if (gate && !fork) {
      e = hmp::launch_fallback_gate(f, p.rule, p.storage, tile_down, tile_coarse, dgrid, cgrid, fgrid, coarse_smem, s);
      if (e != cudaSuccess) return cuda_status(e, "copy-block fallback launch");
    } else if (checked && !gate) {
      f.alpha_flag = nullptr;
      cst = chain(f, false, s, false);
      if (cst.code != HMP_OK) return cst;
    }
    if (timing && tnext < kTimingSlots) ++tnext;
    return ok_status();
  }
};

extern "C" {

HMP_API const char* hmp_version(void) { return "hmpano-gb300 0.1 (sm_103a)"; }

HMP_API hmp_status hmp_stitcher_create(const hmp_config* cfg, hmp_stitcher** out) {
  if (out) *out = nullptr;
  if (!cfg) return make_status(HMP_ERR_INVALID_VALUE, "config is null");
  hmp_stitcher* st = new (std::nothrow) hmp_stitcher();
  if (!st) return make_status(HMP_ERR_MEMORY_ALLOCATION, "out of host memory");
  std::string msg;
  int rc = HMP_OK;
  try {
    rc = hmp::build_plan(*cfg, st->plan, msg);
  } catch (const std::bad_alloc&) {
    rc = HMP_ERR_MEMORY_ALLOCATION;
    msg = "out of host memory while planning";
  }
  if (rc != HMP_OK)
    st->status = make_status(rc, msg);
  else
    st->status = st->setup();
  if (st->status.code != HMP_OK) {
    // Release device memory now; keep the object for its sticky status.
    for (void* p : st->allocations) cudaFree(p);
    st->allocations.clear();
    st->device_bytes = 0;
  }
  if (out)
    *out = st;
  else if (st->status.code != HMP_OK) {
    hmp_status s = st->status;
    delete st;
    return s;
  }
  return st->status;
}

HMP_API void hmp_stitcher_destroy(hmp_stitcher* st) { delete st; }

HMP_API hmp_status hmp_laplacian_rgba(const float* high, int high_w, int high_h, const float* low, int low_w,
                                      int low_h, float* out, int batch, void* stream) {
  if (!high || !low || !out) return make_status(HMP_ERR_INVALID_VALUE, "null argument");
  if (high_w <= 0 || high_h <= 0 || low_w <= 0 || low_h <= 0 || batch <= 0 || high_w > (1 << 20) ||
      high_h > (1 << 20) || low_w > high_w || low_h > high_h || batch > 65536)
    return make_status(HMP_ERR_INVALID_VALUE, "invalid level sizes or batch");
  if (reinterpret_cast<uintptr_t>(high) % 16 || reinterpret_cast<uintptr_t>(low) % 16 ||
      reinterpret_cast<uintptr_t>(out) % 16)
    return make_status(HMP_ERR_INVALID_VALUE, "levels must be 16-byte aligned float RGBA");
  const cudaError_t e = hmp::launch_dump_lap(reinterpret_cast<const float4*>(high), high_w, high_h,
                                             reinterpret_cast<const float4*>(low), low_w, low_h,
                                             reinterpret_cast<float4*>(out), batch, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_status(e, "laplacian launch");
  return ok_status();
}

HMP_API void hmp_debug_fail_allocation(long long k) { g_alloc_fail_countdown.store(k > 0 ? k : 0); }

HMP_API long long hmp_debug_allocation_count(void) { return g_alloc_count.load(); }

HMP_API hmp_status hmp_stitcher_status(const hmp_stitcher* st) {
  if (!st) return make_status(HMP_ERR_INVALID_VALUE, "stitcher is null");
  return st->status;
}

HMP_API int hmp_stitcher_canvas_width(const hmp_stitcher* st) { return st ? st->plan.canvas_w : 0; }
HMP_API int hmp_stitcher_canvas_height(const hmp_stitcher* st) { return st ? st->plan.canvas_h : 0; }
HMP_API int hmp_stitcher_batch_size(const hmp_stitcher* st) { return st ? st->plan.batch : 0; }

HMP_API hmp_status hmp_stitcher_get_info(const hmp_stitcher* st, hmp_stitcher_info* info) {
  if (!st || !info) return make_status(HMP_ERR_INVALID_VALUE, "null argument");
  const hmp::Plan& p = st->plan;
  std::memset(info, 0, sizeof(*info));
  info->canvas_width = p.canvas_w;
  info->canvas_height = p.canvas_h;
  info->batch_size = p.batch;
  info->n_images = p.n;
  info->levels = p.levels;
  const int br[4] = {p.blend.x, p.blend.y, p.blend.w, p.blend.h};
  const int wr[4] = {p.write.x, p.write.y, p.write.w, p.write.h};
  std::memcpy(info->blend_rect, br, sizeof(br));
  std::memcpy(info->write_rect, wr, sizeof(wr));
  info->tile_down = st->tile_down;
  info->tile_coarse = st->tile_coarse;
  const bool copy = st->copy_plan && st->copy_on;
  info->launches_per_process = copy ? st->copy_launches() : st->launches;
  info->m0_bytes = st->m0_bytes;
  info->device_bytes = double(st->device_bytes);
  info->copy_mode = copy ? 1 : 0;
  info->copy_blocks = st->copy_blocks;
  info->empty_blocks = st->empty_blocks;
  info->pyramid_blocks = st->pyramid_blocks;
  info->pyramid_tiles[0] = st->n_down[st->tile_down == 64 ? 1 : 0];
  info->pyramid_tiles[1] = st->n_coarse;
  info->pyramid_tiles[2] = st->n_fine;
  const double canvas_px = double(p.canvas_w) * p.canvas_h;
  if (!p.canvas_plane_used)
    info->gather_pixels = 0;
  else if (p.levels == 0)
    info->gather_pixels = canvas_px;
  else if (copy)
    info->gather_pixels = canvas_px - double(st->pyramid_pixels);
  else
    info->gather_pixels = canvas_px - double(p.write.w) * p.write.h;
  return st->status;
}

HMP_API hmp_status hmp_stitcher_set_down_residency(hmp_stitcher* st, int ctas_per_sm) {
  if (!st) return make_status(HMP_ERR_INVALID_VALUE, "stitcher is null");
  if (st->status.code != HMP_OK) return st->status;
  if (ctas_per_sm < 0 || ctas_per_sm > 8) return make_status(HMP_ERR_INVALID_VALUE, "ctas_per_sm must be in 0..8");
  st->down_residency = ctas_per_sm;
  return ok_status();
}

HMP_API hmp_status hmp_stitcher_set_copy_blocks(hmp_stitcher* st, int enable) {
  if (!st) return make_status(HMP_ERR_INVALID_VALUE, "stitcher is null");
  if (st->status.code != HMP_OK) return st->status;
  if (enable < 0 || enable > 2) return make_status(HMP_ERR_INVALID_VALUE, "copy-block mode must be 0, 1 or 2");
  st->copy_on = enable != 0;
  st->copy_opaque = enable == 2;
  return ok_status();
}

HMP_API hmp_status hmp_stitcher_process(hmp_stitcher* st, const hmp_image* inputs, int n_inputs,
                                        const hmp_image* canvas, void* stream) {
  if (!st) return make_status(HMP_ERR_INVALID_VALUE, "stitcher is null");
  if (st->status.code != HMP_OK) return st->status;
  hmp_status s = st->process(inputs, n_inputs, canvas, static_cast<cudaStream_t>(stream));
  if (s.code != HMP_OK) st->status = s;
  return s;
}

HMP_API hmp_status hmp_stitcher_set_tiles(hmp_stitcher* st, int tile_down, int tile_coarse) {
  if (!st) return make_status(HMP_ERR_INVALID_VALUE, "stitcher is null");
  if (st->status.code != HMP_OK) return st->status;
  const hmp::Plan& p = st->plan;
  if (p.levels < 2) return make_status(HMP_OK, "");  // no pyramid tiles to choose
  const int align = 1 << (p.levels - 1);
  if ((tile_down != 32 && tile_down != 64) || tile_down % align != 0)
    return make_status(HMP_ERR_INVALID_VALUE, "tile_down must be 32 or 64 and a multiple of 2^(levels-1)");
  if (tile_coarse != 32 || (tile_coarse * 2) % align != 0)
    return make_status(HMP_ERR_INVALID_VALUE, "tile_coarse must be 32");
  const int cap = p.n > 3 ? st->down_cap_for(tile_down) : 0;
  if (hmp::pyr_down_smem(cap > 0 ? cap : p.n, tile_down) > 227 * 1024)
    return make_status(HMP_ERR_NOT_SUPPORTED, "pyramid tile does not fit in shared memory");
  st->tile_down = tile_down;
  st->down_residency = st->default_residency();
  st->down_cap = cap;
  st->tile_coarse = tile_coarse;
  st->coarse_smem = st->coarse_smem_for(tile_coarse);
  return make_status(HMP_OK, "");
}

HMP_API hmp_status hmp_stitcher_set_timing(hmp_stitcher* st, int enable) {
  if (!st) return make_status(HMP_ERR_INVALID_VALUE, "stitcher is null");
  const cudaError_t e = st->timing_enable(enable);
  if (e != cudaSuccess) return cuda_status(e, "timing events");
  return ok_status();
}

HMP_API hmp_status hmp_stitcher_dump_pyramid(hmp_stitcher* st, const char* directory, void* stream) {
  if (!st) return make_status(HMP_ERR_INVALID_VALUE, "stitcher is null");
  if (st->status.code != HMP_OK) return st->status;
  return st->dump_pyramid(directory, static_cast<cudaStream_t>(stream));
}

HMP_API hmp_status hmp_stitcher_get_timing(hmp_stitcher* st, hmp_kernel_timing* out) {
  if (!st || !out) return make_status(HMP_ERR_INVALID_VALUE, "null argument");
  const cudaError_t e = st->timing_collect(out);
  if (e != cudaSuccess) return cuda_status(e, "timing events");
  return ok_status();
}

HMP_API hmp_status hmp_plan_copy_blocks(const hmp_config* cfg, int* grid, uint8_t* classes, size_t capacity) {
  if (!cfg || !grid) return make_status(HMP_ERR_INVALID_VALUE, "null argument");
  hmp::Plan p;
  std::string msg;
  int rc = HMP_OK;
  try {
    rc = hmp::build_plan(*cfg, p, msg);
  } catch (const std::bad_alloc&) {
    return make_status(HMP_ERR_MEMORY_ALLOCATION, "out of host memory");
  }
  if (rc != HMP_OK) return make_status(rc, msg);
  for (int i = 0; i < 4; ++i) grid[i] = 0;
  if (p.levels < 2) return ok_status();
  hmp::CopyPlan c;
  try {
    hmp::plan_copy_blocks(p, std::max(32, 1 << (p.levels - 1)), std::max(32, 1 << (p.levels - 2)), c);
  } catch (const std::bad_alloc&) {
    return make_status(HMP_ERR_MEMORY_ALLOCATION, "out of host memory");
  }
  if (!c.usable) return ok_status();
  grid[0] = c.fx0 + p.blend.x;
  grid[1] = c.fy0 + p.blend.y;
  grid[2] = c.nfx;
  grid[3] = c.nfy;
  if (classes) {
    if (capacity < c.block_class.size()) return make_status(HMP_ERR_INVALID_VALUE, "classes buffer too small");
    std::memcpy(classes, c.block_class.data(), c.block_class.size());
  }
  return ok_status();
}

HMP_API hmp_status hmp_plan_geometry(const hmp_config* cfg, int* canvas_w, int* canvas_h, int* out9) {
  if (!cfg) return make_status(HMP_ERR_INVALID_VALUE, "config is null");
  hmp::Plan p;
  std::string msg;
  const int rc = hmp::plan_geometry(*cfg, p, msg);
  if (rc != HMP_OK) return make_status(rc, msg);
  if (canvas_w) *canvas_w = p.canvas_w;
  if (canvas_h) *canvas_h = p.canvas_h;
  if (out9) {
    const int v[9] = {p.blend.x, p.blend.y, p.blend.w, p.blend.h, p.write.x, p.write.y, p.write.w, p.write.h, p.levels};
    std::memcpy(out9, v, sizeof(v));
  }
  return ok_status();
}

}  // extern "C"
