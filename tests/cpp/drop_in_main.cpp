// drop_in_main.cpp -- exercises the C++ drop-in (include/hm/pano/cuda_stitch_pano.h) the way a
// caller of the reference's stitcher classes does: build ControlMasks in memory, construct the
// stitcher for the rig's kind, upload frames into CudaMat, process() with the canvas round trip,
// download the canvas. Test helper for tests/test_cpp_drop_in.py.
//
//   drop_in_main DIR   reads DIR/meta.txt and the raw tables/frames, writes DIR/canvas.bin
//
// meta.txt: "kind n levels batch minimize channels", then n lines "w h xpos ypos" (tables),
// "seam_w seam_h", then n lines "fw fh" (frames). Raw files: mapx_i.bin / mapy_i.bin (uint16),
// seam.bin (uint8), frame_i.bin (RGBA8 or RGB8 by `channels`, batch frames back to back). The
// three-image stitcher runs with the fused remap chosen per call (the reference's process(...,
// fused)): fused, then legacy, the legacy canvas written to canvas_legacy.bin.
#include <cstdio>
#include <fstream>
#include <iterator>
#include <memory>
#include <string>
#include <vector>

#include "hm/pano/cuda_stitch_pano.h"

using hm::CudaMat;
using hm::pano::HostImage;

template <typename T>
static bool read_raw(const std::string& path, std::vector<T>& out, size_t count) {
  std::ifstream f(path, std::ios::binary);
  out.resize(count);
  return bool(f.read(reinterpret_cast<char*>(out.data()), std::streamsize(count * sizeof(T))));
}

template <typename Tp>
static int run(const std::string& dir, std::ifstream& meta, int kind, int n, int levels, int batch, int minimize,
               int channels) {
  std::vector<HostImage<uint16_t>> cols(n), rows(n);
  std::vector<hm::pano::SpatialTiff> pos(n);
  for (int i = 0; i < n; ++i) {
    int w, h, x, y;
    meta >> w >> h >> x >> y;
    cols[i].cols = rows[i].cols = w;
    cols[i].rows = rows[i].rows = h;
    pos[i] = hm::pano::SpatialTiff{float(x), float(y)};
    if (!read_raw(dir + "/mapx_" + std::to_string(i) + ".bin", cols[i].data, size_t(w) * h) ||
        !read_raw(dir + "/mapy_" + std::to_string(i) + ".bin", rows[i].data, size_t(w) * h)) {
      std::fprintf(stderr, "cannot read tables %d\n", i);
      return 3;
    }
  }
  HostImage<uint8_t> seam;
  meta >> seam.cols >> seam.rows;
  if (!read_raw(dir + "/seam.bin", seam.data, size_t(seam.cols) * seam.rows)) return 3;
  std::vector<std::unique_ptr<CudaMat<Tp>>> frames;
  for (int i = 0; i < n; ++i) {
    int fw, fh;
    meta >> fw >> fh;
    std::vector<uint8_t> host;
    const size_t fb = size_t(fw) * fh * channels;
    if (!read_raw(dir + "/frame_" + std::to_string(i) + ".bin", host, size_t(batch) * fb)) return 3;
    frames.push_back(std::make_unique<CudaMat<Tp>>(batch, fw, fh));
    for (int b = 0; b < batch; ++b)
      if (frames.back()->upload(host.data() + size_t(b) * fb, b) != cudaSuccess) return 4;
  }

  cudaStream_t stream;
  if (cudaStreamCreate(&stream) != cudaSuccess) return 4;
  std::unique_ptr<hm::pano::cuda::detail::StitcherBase> holder;
  CudaStatusOr<std::unique_ptr<CudaMat<Tp>>> result(CudaStatus(cudaErrorInvalidValue, "unset"));
  CudaStatusOr<std::unique_ptr<CudaMat<Tp>>> legacy(CudaStatus(cudaErrorInvalidValue, "unset"));
  int cw = 0, ch = 0;
  if (kind == HMP_KIND_PANO2) {
    hm::pano::ControlMasks m;
    m.img1_col = cols[0], m.img1_row = rows[0], m.img2_col = cols[1], m.img2_row = rows[1];
    m.whole_seam_mask_image = seam;
    m.positions = pos;
    auto* p = new hm::pano::cuda::CudaStitchPano<Tp, float4>(batch, levels, m, true, minimize != 0);
    holder.reset(p);
    if (!p->status().ok()) return std::fprintf(stderr, "create: %s\n", p->status().message().c_str()), 5;
    cw = p->canvas_width(), ch = p->canvas_height();
    result = p->process(*frames[0], *frames[1], stream, std::make_unique<CudaMat<Tp>>(batch, cw, ch));
  } else if (kind == HMP_KIND_PANO3) {
    hm::pano::ControlMasks3 m;
    m.img0_col = cols[0], m.img0_row = rows[0], m.img1_col = cols[1], m.img1_row = rows[1];
    m.img2_col = cols[2], m.img2_row = rows[2];
    m.whole_seam_mask_image = seam;
    m.positions = pos;
    auto* p = new hm::pano::cuda::CudaStitchPano3<Tp, float4>(batch, levels, m, true);
    holder.reset(p);
    if (!p->status().ok()) return std::fprintf(stderr, "create: %s\n", p->status().message().c_str()), 5;
    cw = p->canvas_width(), ch = p->canvas_height();
    result = p->process(*frames[0], *frames[1], *frames[2], stream, std::make_unique<CudaMat<Tp>>(batch, cw, ch));
    legacy = p->process(*frames[0], *frames[1], *frames[2], stream, std::make_unique<CudaMat<Tp>>(batch, cw, ch),
                        /*fused=*/false);
    if (!legacy.ok()) return std::fprintf(stderr, "process: %s\n", legacy.status().message().c_str()), 6;
  } else {
    hm::pano::ControlMasksN m;
    m.img_col = cols, m.img_row = rows;
    m.whole_seam_mask_indexed = seam;
    m.positions = pos;
    auto* p = new hm::pano::cuda::CudaStitchPanoN<Tp, float4>(batch, levels, m, minimize != 0, true);
    holder.reset(p);
    if (!p->status().ok()) return std::fprintf(stderr, "create: %s\n", p->status().message().c_str()), 5;
    cw = p->canvas_width(), ch = p->canvas_height();
    std::vector<const CudaMat<Tp>*> ins;
    for (auto& f : frames) ins.push_back(f.get());
    result = p->process(ins, stream, std::make_unique<CudaMat<Tp>>(batch, cw, ch));
  }
  if (!result.ok()) return std::fprintf(stderr, "process: %s\n", result.status().message().c_str()), 6;
  const auto save = [&](CudaMat<Tp>& canvas, const std::string& name) -> bool {
    const size_t cb = size_t(cw) * ch * channels;
    std::vector<uint8_t> out(size_t(batch) * cb);
    for (int b = 0; b < batch; ++b)
      if (canvas.download(out.data() + size_t(b) * cb, b, stream) != cudaSuccess) return false;
    if (cudaStreamSynchronize(stream) != cudaSuccess) return false;
    std::ofstream(dir + "/" + name, std::ios::binary).write(reinterpret_cast<const char*>(out.data()),
                                                            std::streamsize(out.size()));
    return true;
  };
  if (!save(*result.ValueOrDie(), "canvas.bin")) return 7;
  if (kind == HMP_KIND_PANO3 && !save(*legacy.ValueOrDie(), "canvas_legacy.bin")) return 7;
  std::printf("ok %d %d\n", cw, ch);
  cudaStreamDestroy(stream);
  return 0;
}

int main(int argc, char** argv) {
  if (argc != 2) {
    std::fprintf(stderr, "usage: %s DIR\n", argv[0]);
    return 2;
  }
  const std::string dir = argv[1];
  std::ifstream meta(dir + "/meta.txt");
  int kind, n, levels, batch, minimize, channels;
  meta >> kind >> n >> levels >> batch >> minimize >> channels;
  return channels == 3 ? run<uchar3>(dir, meta, kind, n, levels, batch, minimize, 3)
                       : run<uchar4>(dir, meta, kind, n, levels, batch, minimize, 4);
}
