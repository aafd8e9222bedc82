// Loads a two-image control directory through the C++ drop-in (ControlMasks(dir)) and prints what
// the tests compare with the Python loader: sizes, positions and checksums of the tables and seam.
#include <cstdio>

#include "hm/pano/cuda_stitch_pano.h"

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  const hm::pano::ControlMasks m(argv[1]);
  if (!m.is_valid()) {
    std::printf("invalid\n");
    return 1;
  }
  unsigned long long sx = 0, sy = 0, ss = 0;
  for (uint16_t v : m.img1_col.data) sx = sx * 31 + v;
  for (uint16_t v : m.img2_row.data) sy = sy * 31 + v;
  for (uint8_t v : m.whole_seam_mask_image.data) ss = ss * 31 + v;
  std::printf("%d %d %d %d %g %g %g %g %llu %llu %llu\n", m.img1_col.cols, m.img1_col.rows, m.whole_seam_mask_image.cols,
              m.whole_seam_mask_image.rows, m.positions[0].xpos, m.positions[0].ypos, m.positions[1].xpos,
              m.positions[1].ypos, sx, sy, ss);
  return 0;
}
