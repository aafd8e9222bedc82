// hmp_pyramid.cu -- host side of the fused Laplacian-pyramid blend: shared-memory attributes,
// dispatch of the kernel instantiations (hmp_pyramid_kernels.cuh) and their launches, and the
// pyramid dump's plain kernels.
#include "hmp_pyramid_kernels.cuh"

namespace hmp {
namespace {

template <int NMAX, typename Store, int T, bool L = false, bool W = false>
void set_down_attr() {
  cudaFuncSetAttribute(pyr_down_kernel<NMAX, Store, T, L, W>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
}

template <int RULE, int NMAX, typename Store, int T, bool L = false, bool W = false>
void set_up_attr() {
  cudaFuncSetAttribute(pyr_coarse_kernel<RULE, NMAX, Store, T, L, W>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       227 * 1024);
}

template <typename Store, int T>
void set_down_attrs() {
  set_down_attr<2, Store, T>();
  set_down_attr<2, Store, T, true>();
  set_down_attr<2, Store, T, true, true>();
  set_down_attr<3, Store, T>();
  set_down_attr<3, Store, T, false, true>();
  set_down_attr<8, Store, T>();
  set_down_attr<8, Store, T, false, true>();
  cudaFuncSetAttribute(pyr_down_n_kernel<Store, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
  cudaFuncSetAttribute(pyr_down_n_kernel<Store, T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
}

template <typename Store, int T>
void set_coarse_attrs() {
  set_up_attr<kRuleTwo, 2, Store, T>();
  set_up_attr<kRuleTwo, 2, Store, T, true>();
  set_up_attr<kRuleTwo, 2, Store, T, true, true>();
  set_up_attr<kRuleThree, 3, Store, T>();
  set_up_attr<kRuleThree, 3, Store, T, false, true>();
  set_up_attr<kRuleNway, 8, Store, T>();
  set_up_attr<kRuleNway, 8, Store, T, false, true>();
  cudaFuncSetAttribute(pyr_coarse_n_kernel<Store, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
  cudaFuncSetAttribute(pyr_coarse_n_kernel<Store, T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
}

template <typename Store, int T, bool W>
void down_dispatch_w(const PyrArgs& a, dim3 grid, size_t smem, cudaStream_t stream) {
  smem = std::max(smem, size_t(a.down_smem_floor));
  if (a.n <= 2 && (a.tiles != nullptr || W))
    pyr_down_kernel<2, Store, T, true, W><<<grid, 256, smem, stream>>>(a);
  else if (a.n <= 2)
    pyr_down_kernel<2, Store, T><<<grid, 256, smem, stream>>>(a);
  else if (a.n == 3)
    pyr_down_kernel<3, Store, T, false, W><<<grid, 256, smem, stream>>>(a);
  else if (a.slots_cap > 0)
    pyr_down_n_kernel<Store, T, W><<<grid, 256, std::max(pyr_down_smem(a.slots_cap, T), size_t(a.down_smem_floor)), stream>>>(
        a);
  else
    pyr_down_kernel<8, Store, T, false, W><<<grid, 256, smem, stream>>>(a);
}

// The gated fallback (a.gate set) runs the walking instantiations.
template <typename Store, int T>
void down_dispatch(const PyrArgs& a, dim3 grid, size_t smem, cudaStream_t stream) {
  if (a.gate != nullptr)
    down_dispatch_w<Store, T, true>(a, grid, smem, stream);
  else
    down_dispatch_w<Store, T, false>(a, grid, smem, stream);
}

// Launches a pyramid kernel; with a.pdl as a programmatic dependent of the kernel before it on
// the stream (the kernel waits for that kernel's results with grid_dep_wait).
template <typename Kern>
void launch_pyr(Kern k, dim3 grid, size_t smem, cudaStream_t stream, const PyrArgs& a) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = grid;
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = a.pdl ? 1 : 0;
  cudaLaunchKernelEx(&cfg, k, a);
}

template <typename Store, int T, bool W>
void coarse_dispatch_w(const PyrArgs& a, int rule, dim3 grid, size_t smem, cudaStream_t stream) {
  if (rule == kRuleTwo && (a.tiles != nullptr || W))
    launch_pyr(pyr_coarse_kernel<kRuleTwo, 2, Store, T, true, W>, grid, smem, stream, a);
  else if (rule == kRuleTwo)
    launch_pyr(pyr_coarse_kernel<kRuleTwo, 2, Store, T>, grid, smem, stream, a);
  else if (rule == kRuleThree)
    launch_pyr(pyr_coarse_kernel<kRuleThree, 3, Store, T, false, W>, grid, smem, stream, a);
  else if (a.coarse_cap > 0)
    launch_pyr(pyr_coarse_n_kernel<Store, T, W>, grid, smem, stream, a);
  else
    launch_pyr(pyr_coarse_kernel<kRuleNway, 8, Store, T, false, W>, grid, smem, stream, a);
}

template <typename Store, int T>
void coarse_dispatch(const PyrArgs& a, int rule, dim3 grid, size_t smem, cudaStream_t stream) {
  if (a.gate != nullptr)
    coarse_dispatch_w<Store, T, true>(a, rule, grid, smem, stream);
  else
    coarse_dispatch_w<Store, T, false>(a, rule, grid, smem, stream);
}

template <typename Store, bool P0M, bool W>
void fine_dispatch2(const PyrArgs& a, int rule, dim3 grid, size_t smem, cudaStream_t stream) {
  if (rule == kRuleTwo && (a.tiles != nullptr || W))
    launch_pyr(pyr_fine_kernel<kRuleTwo, 2, Store, P0M, true, W>, grid, smem, stream, a);
  else if (rule == kRuleTwo)
    launch_pyr(pyr_fine_kernel<kRuleTwo, 2, Store, P0M>, grid, smem, stream, a);
  else if (rule == kRuleThree)
    launch_pyr(pyr_fine_kernel<kRuleThree, 3, Store, P0M, false, W>, grid, smem, stream, a);
  else
    launch_pyr(pyr_fine_kernel<kRuleNway, 8, Store, P0M, false, W>, grid, smem, stream, a);
}

template <typename Store, bool W>
void fine_dispatch_w(const PyrArgs& a, int rule, dim3 grid, cudaStream_t stream) {
  const size_t smem = a.levels > 1 ? size_t(kFineTA) * (sizeof(float4) + size_t(a.n) * sizeof(Store)) : 0;
  if (rule == kRuleNway && a.use_p0 && a.fine_cap > 0 && a.levels > 1)
    launch_pyr(pyr_fine_n_kernel<Store, W>, grid,
               size_t(kFineTA) * (sizeof(float4) + size_t(a.fine_cap) * sizeof(Store)), stream, a);
  else if (a.use_p0)
    fine_dispatch2<Store, true, W>(a, rule, grid, smem, stream);
  else
    fine_dispatch2<Store, false, W>(a, rule, grid, smem, stream);
}

template <typename Store>
void fine_dispatch(const PyrArgs& a, int rule, dim3 grid, cudaStream_t stream) {
  if (a.gate != nullptr)
    fine_dispatch_w<Store, true>(a, rule, grid, stream);
  else
    fine_dispatch_w<Store, false>(a, rule, grid, stream);
}

// ---- Pyramid dump (hmp_stitcher_dump_pyramid): the levels the fused kernels never store, each
// materialised by a plain kernel with the same device functions, for inspection only. ----

// Gaussian level 0 of slot k over the blend region: the level-0 gather of pyr_down.
__global__ void dump_level0_kernel(const __grid_constant__ PyrArgs a, int k, float4* out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, b = blockIdx.z;
  const int lw0 = a.lw[0], lh0 = a.lh[0];
  if (x >= lw0) return;
  const PlaneDev& P = a.slot[k];
  const int rx = x - P.x0, ry = y - P.y0;
  uint32_t e = 0xFFFFFFFFu;
  int o = P.owner != nullptr ? 0xFF : k;
  if ((unsigned)rx < (unsigned)P.w && (unsigned)ry < (unsigned)P.h) {
    e = __ldg(P.map + (long long)ry * P.map_pitch + rx);
    if (P.owner != nullptr) o = int(__ldg(P.owner + (long long)ry * P.owner_pitch + rx));
  }
  uint32_t fill;
  const uchar4* sp = slot_src<kDevMaxImages>(a, k, o, e, b, a.opaque != 0, fill);
  out[((long long)b * lh0 + y) * lw0 + x] = sp ? to_f4(__ldg(sp)) : u32_to_f4(fill);
}

template <typename Store>
__global__ void dump_widen_kernel(const Store* in, long long n, float4* out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = load_level(in + i);
}

// Laplacian: colour minus the alpha-aware upsample of the next level, the level's alpha.
__global__ void dump_lap_kernel(const float4* hi, int hw, int hh, const float4* lo, int lw, int lh, float4* lap) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, b = blockIdx.z;
  if (x >= hw) return;
  const long long i = ((long long)b * hh + y) * hw + x;
  const float4 g = hi[i];
  const float3 up = up_alpha(lo + (long long)b * lw * lh, lw, 0, 0, lw, lh, x, y);
  lap[i] = make_float4(g.x - up.x, g.y - up.y, g.z - up.z, g.w);
}

// Two-image blend of one level: mask values m (levels >= 1) or the level-0 seam weights.
__global__ void dump_blend2_kernel(const float4* l0, const float4* l1, const float* m, const uint8_t* m0, int m0_pitch,
                                   int w, int h, float4* out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, b = blockIdx.z;
  if (x >= w) return;
  const long long i = ((long long)b * h + y) * w + x;
  const float mv = m ? m[(long long)y * w + x] : float(m0[(long long)y * m0_pitch + x]);
  out[i] = blend_two(l0[i], l1[i], mv);
}

// Reconstruction: the alpha-aware upsample of the next level's reconstruction plus the blend.
__global__ void dump_recon_kernel(const float4* lo, int lw, int lh, const float4* bl, int w, int h, float4* out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, b = blockIdx.z;
  if (x >= w) return;
  const long long i = ((long long)b * h + y) * w + x;
  const float4 v = bl[i];
  const float3 up = up_alpha(lo + (long long)b * lw * lh, lw, 0, 0, lw, lh, x, y);
  out[i] = make_float4(up.x + v.x, up.y + v.y, up.z + v.z, v.w);
}

dim3 dump_grid(int w, int h, int batch) { return dim3((w + 255) / 256, h, batch); }

}  // namespace

size_t residency_smem(int ctas_per_sm) {
  if (ctas_per_sm <= 0) return 0;
  int dev = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess)
    per_sm = 228 * 1024;
  // One CTA more than the cap must not fit: (cap + 1) * (s + 1 KB) > per_sm, s in 128-byte units.
  const size_t s = (size_t(per_sm) / size_t(ctas_per_sm + 1) + 128) / 128 * 128 - 1024;
  return std::min<size_t>(s, 227 * 1024);
}

size_t pyr_down_smem(int n, int tile) {
  const int t2 = tile / 4;
  return size_t(n) * (size_t(tile) * tile * sizeof(uint32_t) + size_t(t2 * t2) * sizeof(float4));
}

size_t pyr_coarse_smem(int n, int k, int tile1, int levels, int storage) {
  const int sb = storage == 1 ? int(sizeof(half4)) : int(sizeof(float4));
  return size_t(coarse_layout(n, k, tile1, levels, sb).total);
}

cudaError_t kernels_init() {
  set_down_attrs<float4, 32>();
  set_down_attrs<half4, 32>();
  set_down_attrs<float4, 64>();
  set_down_attrs<half4, 64>();
  set_coarse_attrs<float4, 32>();
  set_coarse_attrs<half4, 32>();
  fallback_init();
  return cudaGetLastError();
}

cudaError_t launch_pyr_down(const PyrArgs& a, int storage, dim3 grid, cudaStream_t stream) {
  const size_t smem = pyr_down_smem(a.n, a.tile);
  if (a.tile == 32) {
    if (storage == 1)
      down_dispatch<half4, 32>(a, grid, smem, stream);
    else
      down_dispatch<float4, 32>(a, grid, smem, stream);
  } else if (a.tile == 64) {
    if (storage == 1)
      down_dispatch<half4, 64>(a, grid, smem, stream);
    else
      down_dispatch<float4, 64>(a, grid, smem, stream);
  } else {
    return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_pyr_coarse(const PyrArgs& a, int rule, int storage, dim3 grid, size_t smem, cudaStream_t stream) {
  if (a.tile == 32) {
    if (storage == 1)
      coarse_dispatch<half4, 32>(a, rule, grid, smem, stream);
    else
      coarse_dispatch<float4, 32>(a, rule, grid, smem, stream);
  } else {
    return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_pyr_fine(const PyrArgs& a, int rule, int storage, dim3 grid, cudaStream_t stream) {
  if (storage == 1)
    fine_dispatch<half4>(a, rule, grid, stream);
  else
    fine_dispatch<float4>(a, rule, grid, stream);
  return cudaGetLastError();
}

cudaError_t launch_dump_level0(const PyrArgs& a, int k, float4* out, int batch, cudaStream_t stream) {
  dump_level0_kernel<<<dump_grid(a.lw[0], a.lh[0], batch), 256, 0, stream>>>(a, k, out);
  return cudaGetLastError();
}

cudaError_t launch_dump_widen(const void* level, int storage, long long n, float4* out, cudaStream_t stream) {
  const unsigned blocks = unsigned((n + 255) / 256);
  if (storage == 1)
    dump_widen_kernel<half4><<<blocks, 256, 0, stream>>>(static_cast<const half4*>(level), n, out);
  else
    dump_widen_kernel<float4><<<blocks, 256, 0, stream>>>(static_cast<const float4*>(level), n, out);
  return cudaGetLastError();
}

cudaError_t launch_dump_lap(const float4* hi, int hw, int hh, const float4* lo, int lw, int lh, float4* lap, int batch,
                            cudaStream_t stream) {
  dump_lap_kernel<<<dump_grid(hw, hh, batch), 256, 0, stream>>>(hi, hw, hh, lo, lw, lh, lap);
  return cudaGetLastError();
}

cudaError_t launch_dump_blend2(const float4* l0, const float4* l1, const float* m, const uint8_t* m0, int m0_pitch, int w,
                               int h, float4* out, int batch, cudaStream_t stream) {
  dump_blend2_kernel<<<dump_grid(w, h, batch), 256, 0, stream>>>(l0, l1, m, m0, m0_pitch, w, h, out);
  return cudaGetLastError();
}

cudaError_t launch_dump_recon(const float4* lo, int lw, int lh, const float4* bl, int w, int h, float4* out, int batch,
                              cudaStream_t stream) {
  dump_recon_kernel<<<dump_grid(w, h, batch), 256, 0, stream>>>(lo, lw, lh, bl, w, h, out);
  return cudaGetLastError();
}

}  // namespace hmp
