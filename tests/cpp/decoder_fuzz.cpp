// Mutation fuzzer for the control-directory decoders (hmp_read_tiff_u16, hmp_read_seam_png),
// built with AddressSanitizer and UndefinedBehaviorSanitizer by tests/test_control_dir.py.
//
//   decoder_fuzz <iterations> <seed> <scratch file> <seed files...>
//
// Each iteration takes a seed file, applies one to eight random mutations (byte overwrite, bit
// flip, truncation, 32-bit overwrite, special byte), writes it to the scratch file and decodes
// it. A decoder may accept or reject the input; any memory error or undefined behaviour aborts
// the process through the sanitizers.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iterator>
#include <random>
#include <string>
#include <vector>

#include "hmpano.h"

static std::vector<uint8_t> slurp(const char* path) {
  std::ifstream f(path, std::ios::binary);
  return std::vector<uint8_t>((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
}

int main(int argc, char** argv) {
  if (argc < 5) {
    std::fprintf(stderr, "usage: decoder_fuzz <iterations> <seed> <scratch file> <seed files...>\n");
    return 2;
  }
  const long iters = std::atol(argv[1]);
  std::mt19937 rng(unsigned(std::atol(argv[2])));
  const std::string scratch = argv[3];
  std::vector<std::vector<uint8_t>> seeds;
  std::vector<bool> is_png;
  for (int i = 4; i < argc; ++i) {
    seeds.push_back(slurp(argv[i]));
    is_png.push_back(std::string(argv[i]).find(".png") != std::string::npos);
  }
  std::vector<uint8_t> out(size_t(1) << 24);
  long decoded = 0, rejected = 0;
  for (long it = 0; it < iters; ++it) {
    const size_t s = rng() % seeds.size();
    std::vector<uint8_t> b = seeds[s];
    const int mutations = 1 + int(rng() % 8);
    for (int m = 0; m < mutations && !b.empty(); ++m) {
      const size_t pos = rng() % b.size();
      switch (rng() % 5) {
        case 0: b[pos] = uint8_t(rng()); break;
        case 1: b[pos] ^= uint8_t(1u << (rng() % 8)); break;
        case 2: b.resize(pos); break;
        case 3: {
          const uint32_t v = rng();
          for (size_t k = 0; k < 4 && pos + k < b.size(); ++k) b[pos + k] = uint8_t(v >> (8 * k));
          break;
        }
        default: {
          static const uint8_t special[] = {0x00, 0xFF, 0x7F, 0x80};
          b[pos] = special[rng() % 4];
        }
      }
    }
    {
      std::ofstream f(scratch, std::ios::binary);
      f.write(reinterpret_cast<const char*>(b.data()), std::streamsize(b.size()));
    }
    int w = 0, h = 0, paletted = 0;
    const hmp_status st =
        is_png[s] ? hmp_read_seam_png(scratch.c_str(), &w, &h, &paletted, out.data(), out.size())
                  : hmp_read_tiff_u16(scratch.c_str(), &w, &h, reinterpret_cast<uint16_t*>(out.data()), out.size() / 2);
    if (st.code == HMP_OK)
      ++decoded;
    else
      ++rejected;
  }
  std::printf("decoded %ld rejected %ld\n", decoded, rejected);
  return 0;
}
