// cuda_stitch_pano.h -- header-only C++ drop-in for hm-cupano's stitcher classes, over the C ABI
// of libhmpano.so (include/hmpano.h).
//
// Keeps the reference's names and call shapes so that a caller of
//   hm::pano::cuda::CudaStitchPano<uchar4, float4>   (src/pano/cudaPano.h:68-115)
//   hm::pano::cuda::CudaStitchPano3<uchar4, float4>  (src/pano/cudaPano3.h:64-182)
//   hm::pano::cuda::CudaStitchPanoN<uchar4, float4>  (src/pano/cudaPanoN.h:80-146)
//   hm::CudaMat<T>                                   (src/pano/cudaMat.h:355-498)
//   CudaStatus / CudaStatusOr<T>                     (src/cuda/cudaStatus.h:12-198)
//   hm::pano::ControlMasks / ControlMasks3 / ControlMasksN (src/pano/controlMasks*.h)
// compiles against this header with the same code. Differences, all deliberate:
//   * ControlMasks hold HostImage<T> tables instead of cv::Mat (OpenCV is not a dependency);
//     when OpenCV is available, HostImage<T>::from_mat() converts a CV_16U / CV_8U matrix.
//   * process() never allocates: every buffer is allocated by the constructor, so the first
//     process() call can be captured in a CUDA graph too.
//   * T_compute = float4 is the reference default; T_compute = half4-style FP16 pyramid storage
//     is selected with the extra `storage` constructor argument (HMP_STORAGE_F16).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "hmpano.h"

#if defined(__has_include)
#if __has_include(<opencv2/core.hpp>)
#include <opencv2/core.hpp>
#define HMP_HAVE_OPENCV 1
#endif
#endif

// ---------------------------------------------------------------------------------------------
// CudaStatus / CudaStatusOr (global namespace, as in the reference)
// ---------------------------------------------------------------------------------------------
class CudaStatus {
 public:
  CudaStatus() : code_(cudaSuccess), message_("OK") {}
  CudaStatus(cudaError_t code) : code_(code), message_(code == cudaSuccess ? "OK" : cudaGetErrorString(code)) {}
  CudaStatus(cudaError_t code, std::string message) : code_(code) {
    message_ = code == cudaSuccess ? std::move(message) : std::string(cudaGetErrorString(code)) + ": " + message;
  }
  static CudaStatus FromC(const hmp_status& s) {
    CudaStatus r;
    r.code_ = static_cast<cudaError_t>(s.code);
    r.message_ = s.code == 0 ? "OK" : std::string(s.message);
    return r;
  }
  bool ok() const { return code_ == cudaSuccess; }
  cudaError_t code() const { return code_; }
  const std::string& message() const { return message_; }
  static CudaStatus OK() { return CudaStatus(); }
  static CudaStatus OkStatus() { return CudaStatus(); }
  void Update(const CudaStatus& o) {
    if (ok() && !o.ok()) *this = o;
  }

 private:
  cudaError_t code_;
  std::string message_;
};

template <typename T>
class CudaStatusOr {
 public:
  CudaStatusOr(T&& value) : status_(CudaStatus::OK()), value_(std::move(value)), has_value_(true) {}
  CudaStatusOr(const CudaStatus& status) : status_(status), has_value_(false) {
    if (status_.ok()) throw std::invalid_argument("CudaStatusOr: cannot construct OK status without a value.");
  }
  bool ok() const { return status_.ok(); }
  const CudaStatus& status() const { return status_; }
  T& ValueOrDie() {
    if (!ok()) throw std::runtime_error("CudaStatusOr: accessed value when status is not OK: " + status_.message());
    return value_;
  }
  T ConsumeValueOrDie() {
    if (!ok()) throw std::runtime_error("CudaStatusOr: consumed value when status is not OK: " + status_.message());
    has_value_ = false;
    return std::move(value_);
  }
  T& operator*() { return ValueOrDie(); }

 private:
  CudaStatus status_;
  T value_{};
  bool has_value_ = false;
};

#define CUDA_RETURN_IF_ERROR(expr) \
  do {                             \
    CudaStatus _status = (expr);   \
    if (!_status.ok()) {           \
      return _status;              \
    }                              \
  } while (0)

namespace hm {

// ---------------------------------------------------------------------------------------------
// CudaMat<T>: batched device image [B][H][pitch] (src/pano/cudaMat.h:355-498)
// ---------------------------------------------------------------------------------------------
template <typename T>
class CudaMat {
 public:
  CudaMat(int B, int W, int H) : rows_(H), cols_(W), batch_size_(B) {
    if (cudaMalloc(reinterpret_cast<void**>(&d_data_), size()) != cudaSuccess) d_data_ = nullptr;
  }
  // Non-owning view of existing device memory.
  CudaMat(T* dataptr, int B, int W, int H, int pitch = 0)
      : d_data_(dataptr), rows_(H), cols_(W), pitch_(pitch), batch_size_(B), owns_(false) {}
  CudaMat(const CudaMat&) = delete;
  CudaMat& operator=(const CudaMat&) = delete;
  ~CudaMat() {
    if (owns_ && d_data_) cudaFree(d_data_);
  }
  bool is_valid() const { return d_data_ != nullptr; }
  T* data() { return d_data_; }
  const T* data() const { return d_data_; }
  int width() const { return cols_; }
  int height() const { return rows_; }
  int batch_size() const { return batch_size_; }
  int channels() const { return sizeof(T) % 3 == 0 ? 3 : 4; }  // uchar3 / float3 vs uchar4 / float4
  int pitch() const { return pitch_ ? pitch_ : int(sizeof(T)) * cols_; }
  size_t size() const { return size_t(pitch()) * rows_ * batch_size_; }
  cudaError_t upload(const void* host, int batch_item = 0, cudaStream_t stream = 0) {
    return cudaMemcpy2DAsync(reinterpret_cast<char*>(d_data_) + size_t(batch_item) * pitch() * rows_, pitch(), host,
                             sizeof(T) * cols_, sizeof(T) * cols_, rows_, cudaMemcpyHostToDevice, stream);
  }
  cudaError_t download(void* host, int batch_item = 0, cudaStream_t stream = 0) const {
    return cudaMemcpy2DAsync(host, sizeof(T) * cols_,
                             reinterpret_cast<const char*>(d_data_) + size_t(batch_item) * pitch() * rows_, pitch(),
                             sizeof(T) * cols_, rows_, cudaMemcpyDeviceToHost, stream);
  }
  hmp_image c_image() const {
    return hmp_image{const_cast<T*>(d_data_), cols_, rows_, size_t(pitch())};
  }

 private:
  T* d_data_{nullptr};
  int rows_{0}, cols_{0};
  int pitch_{0};
  int batch_size_{0};
  bool owns_{true};
};

namespace pano {

// Host image standing in for the reference's cv::Mat tables (row-major, dense).
template <typename T>
struct HostImage {
  int cols = 0;
  int rows = 0;
  std::vector<T> data;
  bool empty() const { return data.empty(); }
#ifdef HMP_HAVE_OPENCV
  static HostImage from_mat(const cv::Mat& m) {
    HostImage h;
    h.cols = m.cols;
    h.rows = m.rows;
    h.data.resize(size_t(m.cols) * m.rows);
    for (int y = 0; y < m.rows; ++y) std::memcpy(&h.data[size_t(y) * m.cols], m.ptr<T>(y), sizeof(T) * m.cols);
    return h;
  }
#endif
};

struct SpatialTiff {
  float xpos{0};
  float ypos{0};
};

namespace detail {

// Reads a control directory through hmp_control_dir_load; false (with the reason on stderr, as
// the reference loaders print it) when a file is missing or invalid.
inline bool load_control_dir(const std::string& dir, int kind, int n_images, std::vector<HostImage<uint16_t>>& cols,
                             std::vector<HostImage<uint16_t>>& rows, HostImage<uint8_t>& seam,
                             std::vector<SpatialTiff>& positions) {
  hmp_control_dir* d = nullptr;
  const hmp_status s = hmp_control_dir_load(dir.c_str(), kind, n_images, &d);
  if (s.code != HMP_OK) {
    std::fprintf(stderr, "Unable to load control directory %s: %s\n", dir.c_str(), s.message);
    return false;
  }
  const auto copy = [](const auto* p, int w, int h, auto& img) {
    img.cols = w;
    img.rows = h;
    img.data.assign(p, p + size_t(w) * h);
  };
  cols.assign(size_t(d->n), {});
  rows.assign(size_t(d->n), {});
  positions.clear();
  for (int i = 0; i < d->n; ++i) {
    copy(d->map_x[i], d->map_width[i], d->map_height[i], cols[size_t(i)]);
    copy(d->map_y[i], d->map_width[i], d->map_height[i], rows[size_t(i)]);
    positions.push_back(SpatialTiff{d->xpos[i], d->ypos[i]});
  }
  copy(d->seam, d->seam_width, d->seam_height, seam);
  hmp_control_dir_free(d);
  return true;
}

}  // namespace detail

// Control data of a stitcher: the tables, the seam and the canvas positions. load() reads a
// control directory (mapping_000i{,_x,_y}.tif and seam_file.png, controlMasks.cpp:265-326).
struct ControlMasks {
  HostImage<uint16_t> img1_col, img1_row, img2_col, img2_row;
  HostImage<uint8_t> whole_seam_mask_image;  // inverted: 1 = image 1 (controlMasks.cpp:225-250)
  std::vector<SpatialTiff> positions;
  ControlMasks() = default;
  explicit ControlMasks(const std::string& game_dir) { (void)load(game_dir); }
  bool load(const std::string& game_dir) {
    std::vector<HostImage<uint16_t>> c, r;
    if (!detail::load_control_dir(game_dir, HMP_KIND_PANO2, 2, c, r, whole_seam_mask_image, positions)) return false;
    img1_col = std::move(c[0]);
    img2_col = std::move(c[1]);
    img1_row = std::move(r[0]);
    img2_row = std::move(r[1]);
    return is_valid();
  }
  bool is_valid() const {
    return !img1_col.empty() && !img1_row.empty() && !img2_col.empty() && !img2_row.empty() &&
           !whole_seam_mask_image.empty() && positions.size() == 2;
  }
};

struct ControlMasks3 {
  HostImage<uint16_t> img0_col, img0_row, img1_col, img1_row, img2_col, img2_row;
  HostImage<uint8_t> whole_seam_mask_image;  // labels 0..2
  std::vector<SpatialTiff> positions;
  ControlMasks3() = default;
  explicit ControlMasks3(const std::string& game_dir) { (void)load(game_dir); }
  bool load(const std::string& game_dir) {  // controlMasks3.cpp:219-300
    std::vector<HostImage<uint16_t>> c, r;
    if (!detail::load_control_dir(game_dir, HMP_KIND_PANO3, 3, c, r, whole_seam_mask_image, positions)) return false;
    img0_col = std::move(c[0]);
    img1_col = std::move(c[1]);
    img2_col = std::move(c[2]);
    img0_row = std::move(r[0]);
    img1_row = std::move(r[1]);
    img2_row = std::move(r[2]);
    return is_valid();
  }
  bool is_valid() const {
    return !img0_col.empty() && !img1_col.empty() && !img2_col.empty() && !whole_seam_mask_image.empty() &&
           positions.size() == 3;
  }
};

struct ControlMasksN {
  std::vector<HostImage<uint16_t>> img_col, img_row;
  HostImage<uint8_t> whole_seam_mask_indexed;  // labels 0..N-1
  std::vector<SpatialTiff> positions;
  ControlMasksN() = default;
  ControlMasksN(const std::string& dir, int n_images) { (void)load(dir, n_images); }
  bool load(const std::string& dir, int n_images) {  // controlMasksN.cpp:126-193
    return detail::load_control_dir(dir, HMP_KIND_PANON, n_images, img_col, img_row, whole_seam_mask_indexed,
                                    positions) &&
           is_valid();
  }
  bool is_valid() const {
    return !img_col.empty() && img_col.size() == img_row.size() && positions.size() == img_col.size() &&
           !whole_seam_mask_indexed.empty();
  }
};

namespace cuda {

// Pixel types of the reference's pipelines (CudaStitchPano*<T_pipeline, T_compute>): uchar4 is
// the fused per-frame path; uchar3, float4 and float3 run the level-by-level kernels.
template <typename T>
struct PixelTraits;
template <>
struct PixelTraits<uchar4> {
  static constexpr int kChannels = 4, kFormat = HMP_PIXEL_U8;
};
template <>
struct PixelTraits<uchar3> {
  static constexpr int kChannels = 3, kFormat = HMP_PIXEL_U8;
};
template <>
struct PixelTraits<float4> {
  static constexpr int kChannels = 4, kFormat = HMP_PIXEL_F32;
};
template <>
struct PixelTraits<float3> {
  static constexpr int kChannels = 3, kFormat = HMP_PIXEL_F32;
};

namespace detail {

// Owns an hmp_stitcher and implements the shared part of the three classes.
class StitcherBase {
 public:
  StitcherBase() = default;
  StitcherBase(const StitcherBase&) = delete;
  StitcherBase& operator=(const StitcherBase&) = delete;
  ~StitcherBase() {
    if (st_) hmp_stitcher_destroy(st_);
  }
  int canvas_width() const { return hmp_stitcher_canvas_width(st_); }
  int canvas_height() const { return hmp_stitcher_canvas_height(st_); }
  int batch_size() const { return batch_; }
  const CudaStatus status() const { return st_ ? CudaStatus::FromC(hmp_stitcher_status(st_)) : status_; }
  hmp_stitcher* handle() const { return st_; }

 protected:
  void create(int kind, int batch, int levels, const std::vector<const HostImage<uint16_t>*>& cols,
              const std::vector<const HostImage<uint16_t>*>& rows, const HostImage<uint8_t>& seam,
              const std::vector<SpatialTiff>& positions, bool minimize, bool fused, int storage, int channels,
              int pixel_format) {
    batch_ = batch;
    std::vector<hmp_remap> remaps(cols.size());
    for (size_t i = 0; i < cols.size(); ++i)
      remaps[i] = hmp_remap{cols[i]->data.data(), rows[i]->data.data(), cols[i]->cols, cols[i]->rows,
                            int(positions[i].xpos), int(positions[i].ypos)};
    hmp_config cfg{};
    cfg.kind = kind;
    cfg.n_images = int(cols.size());
    cfg.num_levels = levels;
    cfg.batch_size = batch;
    cfg.channels = channels;
    cfg.pixel_format = pixel_format;
    cfg.minimize_blend = minimize ? 1 : 0;
    cfg.fused = fused ? 1 : 0;
    cfg.storage = storage;
    cfg.filter = HMP_FILTER_REFBOX;
    cfg.remaps = remaps.data();
    cfg.seam = seam.data.data();
    cfg.seam_width = seam.cols;
    cfg.seam_height = seam.rows;
    status_ = CudaStatus::FromC(hmp_stitcher_create(&cfg, &st_));
  }

  template <typename Tp>
  CudaStatusOr<std::unique_ptr<CudaMat<Tp>>> run(const std::vector<const CudaMat<Tp>*>& inputs, cudaStream_t stream,
                                                 std::unique_ptr<CudaMat<Tp>>&& canvas) {
    if (!st_) return CudaStatus(status_.ok() ? cudaErrorInvalidValue : status_.code(), status_.message());
    CudaStatus sticky = status();
    if (!sticky.ok()) return sticky;
    if (!canvas) return CudaStatus(cudaErrorInvalidDevicePointer, "Canvas must be provided");
    std::vector<hmp_image> ins;
    for (const CudaMat<Tp>* m : inputs) {
      if (!m || m->batch_size() != batch_) return CudaStatus(cudaErrorInvalidValue, "Mismatched batch sizes");
      ins.push_back(m->c_image());
    }
    if (canvas->batch_size() != batch_) return CudaStatus(cudaErrorInvalidValue, "Canvas batch mismatch");
    const hmp_image cv = canvas->c_image();
    const hmp_status s = hmp_stitcher_process(st_, ins.data(), int(ins.size()), &cv, stream);
    if (s.code != 0) return CudaStatus::FromC(s);
    return std::move(canvas);
  }

  hmp_stitcher* st_ = nullptr;
  CudaStatus status_;
  int batch_ = 0;
};

}  // namespace detail

// Two-image stitcher (src/pano/cudaPano.h:68-115).
template <typename T_pipeline, typename T_compute>
class CudaStitchPano : public detail::StitcherBase {
 public:
  CudaStitchPano(int batch_size, int num_levels, const ControlMasks& control_masks, bool quiet = false,
                 bool minimize_blend = true, [[maybe_unused]] int max_output_width = 0, int storage = HMP_STORAGE_F32) {
    (void)quiet;
    if (!control_masks.is_valid()) {
      status_ = CudaStatus(cudaErrorFileNotFound, "Stitching masks were not able to be loaded");
      return;
    }
    create(HMP_KIND_PANO2, batch_size, num_levels, {&control_masks.img1_col, &control_masks.img2_col},
           {&control_masks.img1_row, &control_masks.img2_row}, control_masks.whole_seam_mask_image,
           control_masks.positions, minimize_blend, true, storage, PixelTraits<T_pipeline>::kChannels,
           PixelTraits<T_pipeline>::kFormat);
  }
  CudaStatusOr<std::unique_ptr<CudaMat<T_pipeline>>> process(const CudaMat<T_pipeline>& inputImage1,
                                                             const CudaMat<T_pipeline>& inputImage2,
                                                             cudaStream_t stream,
                                                             std::unique_ptr<CudaMat<T_pipeline>>&& canvas) {
    return run<T_pipeline>({&inputImage1, &inputImage2}, stream, std::move(canvas));
  }
  // Writes the soft-blend pyramid of the last process() under `directory` (cudaPano.h:101):
  // metadata.txt and float32 TIFF levels; see hmp_stitcher_dump_pyramid.
  CudaStatus dump_soft_blend_pyramid(const std::string& directory, cudaStream_t stream) const {
    if (!st_) return status();
    return CudaStatus::FromC(hmp_stitcher_dump_pyramid(st_, directory.c_str(), stream));
  }
};

// Three-image stitcher (src/pano/cudaPano3.h:64-182).
template <typename T_pipeline, typename T_compute>
class CudaStitchPano3 : public detail::StitcherBase {
 public:
  CudaStitchPano3(int batch_size, int num_levels, const ControlMasks3& control_masks, bool quiet = false,
                  bool fused = true, int storage = HMP_STORAGE_F32)
      : masks_(control_masks), levels_(num_levels), fused_(fused), storage_(storage) {
    (void)quiet;
    if (!control_masks.is_valid()) {
      status_ = CudaStatus(cudaErrorFileNotFound, "Stitching masks (3-image) were not able to be loaded");
      return;
    }
    create(HMP_KIND_PANO3, batch_size, num_levels,
           {&control_masks.img0_col, &control_masks.img1_col, &control_masks.img2_col},
           {&control_masks.img0_row, &control_masks.img1_row, &control_masks.img2_row},
           control_masks.whole_seam_mask_image, control_masks.positions, true, fused, storage,
           PixelTraits<T_pipeline>::kChannels, PixelTraits<T_pipeline>::kFormat);
  }
  // `fused` picks the remap per call, as in the reference (cudaPano3.h:101-107): the fused remap
  // (invalid entries leave pixels transparent) or the legacy remap + copy. The mode other than the
  // constructor's runs on a second stitcher, made on its first use.
  CudaStatusOr<std::unique_ptr<CudaMat<T_pipeline>>> process(const CudaMat<T_pipeline>& inputImage0,
                                                             const CudaMat<T_pipeline>& inputImage1,
                                                             const CudaMat<T_pipeline>& inputImage2,
                                                             cudaStream_t stream,
                                                             std::unique_ptr<CudaMat<T_pipeline>>&& canvas,
                                                             bool fused = true) {
    if (fused == fused_ || !st_)
      return run<T_pipeline>({&inputImage0, &inputImage1, &inputImage2}, stream, std::move(canvas));
    if (!other_) other_.reset(new CudaStitchPano3(batch_, levels_, masks_, true, fused, storage_));
    return other_->process(inputImage0, inputImage1, inputImage2, stream, std::move(canvas), fused);
  }

 private:
  ControlMasks3 masks_;
  int levels_ = 0;
  bool fused_ = true;
  int storage_ = HMP_STORAGE_F32;
  std::unique_ptr<CudaStitchPano3> other_;
};

// N-image stitcher, N in [2, 8] (src/pano/cudaPanoN.h:80-146).
template <typename T_pipeline, typename T_compute>
class CudaStitchPanoN : public detail::StitcherBase {
 public:
  CudaStitchPanoN(int batch_size, int num_levels, const ControlMasksN& control_masks, bool minimize_blend = true,
                  bool quiet = false, int storage = HMP_STORAGE_F32) {
    (void)quiet;
    if (!control_masks.is_valid()) {
      status_ = CudaStatus(cudaErrorFileNotFound, "Stitching masks (N-image) could not be loaded");
      return;
    }
    std::vector<const HostImage<uint16_t>*> cols, rows;
    for (size_t i = 0; i < control_masks.img_col.size(); ++i) {
      cols.push_back(&control_masks.img_col[i]);
      rows.push_back(&control_masks.img_row[i]);
    }
    create(HMP_KIND_PANON, batch_size, num_levels, cols, rows, control_masks.whole_seam_mask_indexed,
           control_masks.positions, minimize_blend, true, storage, PixelTraits<T_pipeline>::kChannels,
           PixelTraits<T_pipeline>::kFormat);
  }
  CudaStatusOr<std::unique_ptr<CudaMat<T_pipeline>>> process(const std::vector<const CudaMat<T_pipeline>*>& inputs,
                                                             cudaStream_t stream,
                                                             std::unique_ptr<CudaMat<T_pipeline>>&& canvas) {
    if (st_ && int(inputs.size()) != hmp_stitcher_info_n())
      return CudaStatus(cudaErrorInvalidValue, "inputs size != N");
    return run<T_pipeline>(inputs, stream, std::move(canvas));
  }

 private:
  int hmp_stitcher_info_n() const {
    hmp_stitcher_info info{};
    hmp_stitcher_get_info(st_, &info);
    return info.n_images;
  }
};

}  // namespace cuda
}  // namespace pano
}  // namespace hm
