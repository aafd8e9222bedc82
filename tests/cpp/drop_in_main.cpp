// drop_in_main.cpp -- exercises the C++ drop-in (include/hm/pano/cuda_stitch_pano.h) the way a
// caller of the reference's stitcher classes does: build ControlMasks in memory, construct the
// stitcher for the rig's kind, upload frames into CudaMat, process() with the canvas round trip,
// download the canvas. Test helper for tests/test_cpp_drop_in.py.
//
//   drop_in_main DIR   reads DIR/meta.txt and the raw tables/frames, writes DIR/canvas.bin
//
// meta.txt: "kind n levels batch minimize", then n lines "w h xpos ypos" (tables), "seam_w seam_h",
// then n lines "fw fh" (frames). Raw files: mapx_i.bin / mapy_i.bin (uint16), seam.bin (uint8),
// frame_i.bin (RGBA8, batch frames back to back).
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

int main(int argc, char** argv) {
  if (argc != 2) {
    std::fprintf(stderr, "usage: %s DIR\n", argv[0]);
    return 2;
  }
  const std::string dir = argv[1];
  std::ifstream meta(dir + "/meta.txt");
  int kind, n, levels, batch, minimize;
  meta >> kind >> n >> levels >> batch >> minimize;
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
  std::vector<std::unique_ptr<CudaMat<uchar4>>> frames;
  for (int i = 0; i < n; ++i) {
    int fw, fh;
    meta >> fw >> fh;
    std::vector<uint8_t> host;
    if (!read_raw(dir + "/frame_" + std::to_string(i) + ".bin", host, size_t(batch) * fw * fh * 4)) return 3;
    frames.push_back(std::make_unique<CudaMat<uchar4>>(batch, fw, fh));
    for (int b = 0; b < batch; ++b)
      if (frames.back()->upload(host.data() + size_t(b) * fw * fh * 4, b) != cudaSuccess) return 4;
  }

  cudaStream_t stream;
  if (cudaStreamCreate(&stream) != cudaSuccess) return 4;
  std::unique_ptr<hm::pano::cuda::detail::StitcherBase> holder;
  CudaStatusOr<std::unique_ptr<CudaMat<uchar4>>> result(CudaStatus(cudaErrorInvalidValue, "unset"));
  int cw = 0, ch = 0;
  if (kind == HMP_KIND_PANO2) {
    hm::pano::ControlMasks m;
    m.img1_col = cols[0], m.img1_row = rows[0], m.img2_col = cols[1], m.img2_row = rows[1];
    m.whole_seam_mask_image = seam;
    m.positions = pos;
    auto* p = new hm::pano::cuda::CudaStitchPano<uchar4, float4>(batch, levels, m, true, minimize != 0);
    holder.reset(p);
    if (!p->status().ok()) return std::fprintf(stderr, "create: %s\n", p->status().message().c_str()), 5;
    cw = p->canvas_width(), ch = p->canvas_height();
    result = p->process(*frames[0], *frames[1], stream, std::make_unique<CudaMat<uchar4>>(batch, cw, ch));
  } else if (kind == HMP_KIND_PANO3) {
    hm::pano::ControlMasks3 m;
    m.img0_col = cols[0], m.img0_row = rows[0], m.img1_col = cols[1], m.img1_row = rows[1];
    m.img2_col = cols[2], m.img2_row = rows[2];
    m.whole_seam_mask_image = seam;
    m.positions = pos;
    auto* p = new hm::pano::cuda::CudaStitchPano3<uchar4, float4>(batch, levels, m, true);
    holder.reset(p);
    if (!p->status().ok()) return std::fprintf(stderr, "create: %s\n", p->status().message().c_str()), 5;
    cw = p->canvas_width(), ch = p->canvas_height();
    result = p->process(*frames[0], *frames[1], *frames[2], stream, std::make_unique<CudaMat<uchar4>>(batch, cw, ch));
  } else {
    hm::pano::ControlMasksN m;
    m.img_col = cols, m.img_row = rows;
    m.whole_seam_mask_indexed = seam;
    m.positions = pos;
    auto* p = new hm::pano::cuda::CudaStitchPanoN<uchar4, float4>(batch, levels, m, minimize != 0, true);
    holder.reset(p);
    if (!p->status().ok()) return std::fprintf(stderr, "create: %s\n", p->status().message().c_str()), 5;
    cw = p->canvas_width(), ch = p->canvas_height();
    std::vector<const CudaMat<uchar4>*> ins;
    for (auto& f : frames) ins.push_back(f.get());
    result = p->process(ins, stream, std::make_unique<CudaMat<uchar4>>(batch, cw, ch));
  }
  if (!result.ok()) return std::fprintf(stderr, "process: %s\n", result.status().message().c_str()), 6;
  std::unique_ptr<CudaMat<uchar4>> canvas = std::move(result.ValueOrDie());
  std::vector<uint8_t> out(size_t(batch) * cw * ch * 4);
  for (int b = 0; b < batch; ++b)
    if (canvas->download(out.data() + size_t(b) * cw * ch * 4, b, stream) != cudaSuccess) return 7;
  if (cudaStreamSynchronize(stream) != cudaSuccess) return 7;
  std::ofstream(dir + "/canvas.bin", std::ios::binary).write(reinterpret_cast<const char*>(out.data()),
                                                             std::streamsize(out.size()));
  std::printf("ok %d %d\n", cw, ch);
  cudaStreamDestroy(stream);
  return 0;
}
