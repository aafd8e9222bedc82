/* Randomized stitches through the oracle (hmpo_stitch_f32 / hmpo_stitch_f64), built with
 * AddressSanitizer and UndefinedBehaviorSanitizer by tests/test_host_abi.py: every kind, level
 * count, batch, 3 or 4 channels, both filters, with tables that mix identity, in-range random and
 * arbitrary entries and frames smaller or larger than the tables expect. A configuration may run
 * or be rejected; any memory error or undefined behaviour aborts the process.
 *
 *   oracle_fuzz <iterations> <seed>
 */
#include <stdio.h>
#include <stdlib.h>
#include <stdint.h>
#include "hmp_oracle.h"

static unsigned long long s_state = 88172645463325252ull;
static unsigned rnd(void) { s_state ^= s_state << 13; s_state ^= s_state >> 7; s_state ^= s_state << 17; return (unsigned)(s_state >> 11); }

int main(int argc, char** argv) {
  int iters = atoi(argv[1]);
  s_state += (unsigned long long)atoi(argv[2]) * 0x9E3779B97F4A7C15ull;
  long ok = 0, bad = 0;
  for (int it = 0; it < iters; ++it) {
    int kind = 1 + rnd() % 3;
    int n = kind == 2 ? 2 : kind == 3 ? 3 : 2 + rnd() % 7;
    uint16_t* mx[8]; uint16_t* my[8]; int mw[8], mh[8], px[8], py[8];
    uint8_t* in[8]; int iw[8], ih[8];
    int cw = 0, chh = 0;
    int channels = rnd() % 4 == 0 ? 3 : 4;
    int batch = 1 + rnd() % 2;
    for (int i = 0; i < n; ++i) {
      int w = 1 + rnd() % 70, h = 1 + rnd() % 40;
      iw[i] = 1 + rnd() % 60; ih[i] = 1 + rnd() % 40;
      mw[i] = w; mh[i] = h;
      mx[i] = malloc(sizeof(uint16_t) * w * h); my[i] = malloc(sizeof(uint16_t) * w * h);
      int mode = rnd() % 3;
      for (int k = 0; k < w * h; ++k) {
        int x = k % w, y = k / w;
        if (mode == 0) { mx[i][k] = x % iw[i]; my[i][k] = y % ih[i]; }
        else if (mode == 1) { mx[i][k] = rnd() % (iw[i] + 3); my[i][k] = rnd() % (ih[i] + 3); }
        else { mx[i][k] = rnd() % 5 == 0 ? 65535 : rnd() % 65536; my[i][k] = rnd() % 5 == 0 ? 65535 : rnd() % 65536; }
      }
      px[i] = rnd() % 60; py[i] = rnd() % 15;
      if (px[i] + w > cw) cw = px[i] + w;
      if (py[i] + h > chh) chh = py[i] + h;
      size_t bytes = (size_t)batch * iw[i] * ih[i] * channels;
      in[i] = malloc(bytes);
      for (size_t b = 0; b < bytes; ++b) in[i][b] = rnd();
    }
    int sw = cw - (int)(rnd() % 3); if (sw < 1) sw = 1;
    int sh = chh - (int)(rnd() % 3); if (sh < 1) sh = 1;
    uint8_t* seam = malloc((size_t)sw * sh);
    int nl = kind == 2 ? 2 : n + (rnd() % 4 == 0 ? 2 : 0);
    for (int k = 0; k < sw * sh; ++k) seam[k] = rnd() % nl;
    hmpo_config c = {kind, n, (int)(rnd() % 8), batch, (int)(rnd() % 2), (int)(rnd() % 2),
                     channels == 4 && rnd() % 4 == 0 ? HMPO_FILTER_BINOMIAL5 : HMPO_FILTER_REFBOX,
                     (const uint16_t* const*)mx, (const uint16_t* const*)my, mw, mh, px, py, seam, sw, sh, channels};
    int W = 0, H = 0;
    int rc = hmpo_canvas_size(&c, &W, &H);
    if (rc == 0) {
      uint8_t* canvas = malloc((size_t)batch * W * H * channels + 1);
      rc = (it & 1) ? hmpo_stitch_f64(&c, (const uint8_t* const*)in, iw, ih, canvas)
                    : hmpo_stitch_f32(&c, (const uint8_t* const*)in, iw, ih, canvas);
      free(canvas);
    }
    if (rc == 0) ++ok; else ++bad;
    for (int i = 0; i < n; ++i) { free(mx[i]); free(my[i]); free(in[i]); }
    free(seam);
  }
  printf("stitched %ld rejected %ld\n", ok, bad);
  return 0;
}
