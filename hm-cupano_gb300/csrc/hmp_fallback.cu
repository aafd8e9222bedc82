// hmp_fallback.cu -- the copy-block fallback as one launch (copy-block mode of hmp_stitcher.cu).
//
// Copy blocks are exact only while every source pixel in their supports has alpha != 0; the canvas
// gather and pyr_fine check that and set a flag. Most calls leave it clear, so the fallback must
// cost as little as possible then: one thread of fallback_gate_kernel reads the flag after the
// frame's other kernels and returns. When it is set, the thread clears it and tail-launches the
// dense chain (pyr_down, pyr_coarse, pyr_fine over every tile of the write rect, the instantiations
// the plain path uses), which recomputes the whole write rect after the gather wrote its copy
// blocks; tail launches run in order, each after the one before and after this grid, and the
// caller's stream continues only after the last.
//
// Device-side launches need relocatable device code, which raises the pyramid kernels' registers
// markedly, so this unit (-rdc=true) holds its own copies of the kernels (hmp_pyramid_kernels.cuh)
// for this rare path, and hmp_pyramid.cu's per-frame kernels stay whole-program compiled.
#include "hmp_pyramid_kernels.cuh"

namespace hmp {
namespace {

struct FallbackLaunch {
  dim3 down, coarse, fine;  // dense grids
  unsigned down_smem, coarse_smem, fine_smem;
  int rule, tile_down, tile_coarse;
};

template <typename Store, int T>
__device__ void tail_down(const PyrArgs& d, const FallbackLaunch& f) {
  if (d.n <= 2)
    pyr_down_kernel<2, Store, T><<<f.down, 256, f.down_smem, cudaStreamTailLaunch>>>(d);
  else if (d.n == 3)
    pyr_down_kernel<3, Store, T><<<f.down, 256, f.down_smem, cudaStreamTailLaunch>>>(d);
  else if (d.slots_cap > 0)
    pyr_down_n_kernel<Store, T><<<f.down, 256, f.down_smem, cudaStreamTailLaunch>>>(d);
  else
    pyr_down_kernel<8, Store, T><<<f.down, 256, f.down_smem, cudaStreamTailLaunch>>>(d);
}

template <typename Store, int T>
__device__ void tail_coarse(const PyrArgs& d, const FallbackLaunch& f) {
  if (f.rule == kRuleTwo)
    pyr_coarse_kernel<kRuleTwo, 2, Store, T><<<f.coarse, 256, f.coarse_smem, cudaStreamTailLaunch>>>(d);
  else if (f.rule == kRuleThree)
    pyr_coarse_kernel<kRuleThree, 3, Store, T><<<f.coarse, 256, f.coarse_smem, cudaStreamTailLaunch>>>(d);
  else if (d.coarse_cap > 0)
    pyr_coarse_n_kernel<Store, T><<<f.coarse, 256, f.coarse_smem, cudaStreamTailLaunch>>>(d);
  else
    pyr_coarse_kernel<kRuleNway, 8, Store, T><<<f.coarse, 256, f.coarse_smem, cudaStreamTailLaunch>>>(d);
}

template <typename Store, bool P0M>
__device__ void tail_fine2(const PyrArgs& d, const FallbackLaunch& f) {
  if (f.rule == kRuleTwo)
    pyr_fine_kernel<kRuleTwo, 2, Store, P0M><<<f.fine, 256, f.fine_smem, cudaStreamTailLaunch>>>(d);
  else if (f.rule == kRuleThree)
    pyr_fine_kernel<kRuleThree, 3, Store, P0M><<<f.fine, 256, f.fine_smem, cudaStreamTailLaunch>>>(d);
  else
    pyr_fine_kernel<kRuleNway, 8, Store, P0M><<<f.fine, 256, f.fine_smem, cudaStreamTailLaunch>>>(d);
}

template <typename Store>
__device__ void tail_fine(const PyrArgs& d, const FallbackLaunch& f) {
  if (f.rule == kRuleNway && d.use_p0 && d.fine_cap > 0 && d.levels > 1)
    pyr_fine_n_kernel<Store><<<f.fine, 256, f.fine_smem, cudaStreamTailLaunch>>>(d);
  else if (d.use_p0)
    tail_fine2<Store, true>(d, f);
  else
    tail_fine2<Store, false>(d, f);
}

template <typename Store>
__global__ void fallback_gate_kernel(const __grid_constant__ PyrArgs a, const FallbackLaunch f) {
  volatile int* g = a.gate;
  if (g[0] == 0) return;
  g[0] = 0;  // clear for the next call (the tail launches read no flag)
  PyrArgs d = a;
  d.gate = nullptr;
  d.alpha_flag = nullptr;
  d.tiles = nullptr;
  d.pdl = 0;
  if (d.levels > 1) {
    d.tile = f.tile_down;
    if (f.tile_down == 32)
      tail_down<Store, 32>(d, f);
    else
      tail_down<Store, 64>(d, f);
    d.tile = f.tile_coarse;
    tail_coarse<Store, 32>(d, f);
  }
  tail_fine<Store>(d, f);
}

template <typename Store, int T>
void set_attrs_tiles() {
  constexpr int kMax = 227 * 1024;
  cudaFuncSetAttribute(pyr_down_kernel<2, Store, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMax);
  cudaFuncSetAttribute(pyr_down_kernel<3, Store, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMax);
  cudaFuncSetAttribute(pyr_down_kernel<8, Store, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMax);
  cudaFuncSetAttribute(pyr_down_n_kernel<Store, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMax);
}

template <typename Store>
void set_attrs() {
  constexpr int kMax = 227 * 1024;
  set_attrs_tiles<Store, 32>();
  set_attrs_tiles<Store, 64>();
  cudaFuncSetAttribute(pyr_coarse_kernel<kRuleTwo, 2, Store, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMax);
  cudaFuncSetAttribute(pyr_coarse_kernel<kRuleThree, 3, Store, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMax);
  cudaFuncSetAttribute(pyr_coarse_kernel<kRuleNway, 8, Store, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMax);
  cudaFuncSetAttribute(pyr_coarse_n_kernel<Store, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMax);
  cudaFuncSetAttribute(pyr_fine_n_kernel<Store>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMax);
}

}  // namespace

cudaError_t fallback_init() {
  set_attrs<float4>();
  set_attrs<half4>();
  return cudaGetLastError();
}

cudaError_t launch_fallback_gate(const PyrArgs& a, int rule, int storage, int tile_down, int tile_coarse, dim3 down,
                                 dim3 coarse, dim3 fine, size_t coarse_smem, cudaStream_t stream) {
  if (a.gate == nullptr || (tile_down != 32 && tile_down != 64) || tile_coarse != 32) return cudaErrorInvalidValue;
  const size_t sb = storage == 1 ? sizeof(half4) : sizeof(float4);
  FallbackLaunch f{};
  f.down = down;
  f.coarse = coarse;
  f.fine = fine;
  f.rule = rule;
  f.tile_down = tile_down;
  f.tile_coarse = tile_coarse;
  // The plain path's shared-memory sizes for the same instantiations (hmp_pyramid.cu).
  const int down_n = a.n > 3 && a.slots_cap > 0 ? a.slots_cap : a.n;
  f.down_smem = unsigned(std::max(pyr_down_smem(down_n, tile_down), size_t(a.down_smem_floor)));
  f.coarse_smem = unsigned(coarse_smem);
  if (rule == kRuleNway && a.use_p0 && a.fine_cap > 0 && a.levels > 1)
    f.fine_smem = unsigned(size_t(kFineTA) * (sizeof(float4) + size_t(a.fine_cap) * sb));
  else
    f.fine_smem = unsigned(a.levels > 1 ? size_t(kFineTA) * (sizeof(float4) + size_t(a.n) * sb) : 0);
  if (storage == 1)
    fallback_gate_kernel<half4><<<1, 1, 0, stream>>>(a, f);
  else
    fallback_gate_kernel<float4><<<1, 1, 0, stream>>>(a, f);
  return cudaGetLastError();
}

}  // namespace hmp
