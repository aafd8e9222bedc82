// Randomized configurations through the planner (hmp::build_plan: geometry, gather planes, seam
// padding, mask pyramid and classes), built with AddressSanitizer and UndefinedBehaviorSanitizer
// by tests/test_host_abi.py. Tables mix identity, in-range random and arbitrary entries (with the
// 65535 sentinel); seams may hold more labels than images; every kind, level count, batch,
// channel count, storage and filter. A configuration may be planned or rejected; any memory error
// or undefined behaviour aborts the process.
//
//   plan_fuzz <iterations> <seed>
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <string>
#include <vector>
#include "hmp_plan.h"

int main(int argc, char** argv) {
  const int iters = atoi(argv[1]);
  std::mt19937 rng(atoi(argv[2]));
  long ok = 0, bad = 0;
  for (int it = 0; it < iters; ++it) {
    const int kinds[3] = {HMP_KIND_PANON, HMP_KIND_PANO2, HMP_KIND_PANO3};
    const int kind = kinds[rng() % 3];
    const int n = kind == HMP_KIND_PANO2 ? 2 : kind == HMP_KIND_PANO3 ? 3 : 2 + int(rng() % 7);
    std::vector<std::vector<uint16_t>> mx(n), my(n);
    std::vector<hmp_remap> rm(n);
    int cw = 0, ch = 0;
    for (int i = 0; i < n; ++i) {
      const int w = 1 + int(rng() % 90), h = 1 + int(rng() % 60);
      const int sw = 1 + int(rng() % 80), sh = 1 + int(rng() % 60);
      mx[i].resize(size_t(w) * h);
      my[i].resize(size_t(w) * h);
      const int mode = int(rng() % 3);
      for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
          uint16_t a, b;
          if (mode == 0) { a = uint16_t(x % sw); b = uint16_t(y % sh); }
          else if (mode == 1) { a = uint16_t(rng() % (sw + 3)); b = uint16_t(rng() % (sh + 3)); }
          else { a = (rng() % 7 == 0) ? 65535 : uint16_t(rng() % 65536); b = (rng() % 7 == 0) ? 65535 : uint16_t(rng() % 65536); }
          mx[i][size_t(y) * w + x] = a;
          my[i][size_t(y) * w + x] = b;
        }
      const int xp = int(rng() % 80), yp = int(rng() % 20);
      rm[i] = hmp_remap{mx[i].data(), my[i].data(), w, h, xp, yp};
      cw = std::max(cw, xp + w);
      ch = std::max(ch, yp + h);
    }
    const int sw = std::max(1, cw - int(rng() % 3)), sh = std::max(1, ch - int(rng() % 3));
    std::vector<uint8_t> seam(size_t(sw) * sh);
    const int nl = kind == HMP_KIND_PANO2 ? 2 : n + (rng() % 4 == 0 ? 2 : 0);
    for (auto& v : seam) v = uint8_t(rng() % nl);
    hmp_config c{};
    c.kind = kind;
    c.n_images = n;
    c.num_levels = int(rng() % 8);
    c.batch_size = 1 + int(rng() % 3);
    c.channels = rng() % 4 == 0 ? 3 : 4;
    c.minimize_blend = int(rng() % 2);
    c.fused = int(rng() % 2);
    c.storage = c.channels == 4 && rng() % 3 == 0 ? HMP_STORAGE_F16 : HMP_STORAGE_F32;
    c.filter = c.channels == 4 && rng() % 4 == 0 ? HMP_FILTER_BINOMIAL5 : HMP_FILTER_REFBOX;
    c.remaps = rm.data();
    c.seam = seam.data();
    c.seam_width = sw;
    c.seam_height = sh;
    c.pixel_format = HMP_PIXEL_U8;
    hmp::Plan p;
    std::string msg;
    const int rc = hmp::build_plan(c, p, msg);
    if (rc == HMP_OK) ++ok; else ++bad;
  }
  printf("planned %ld rejected %ld\n", ok, bad);
  return 0;
}
