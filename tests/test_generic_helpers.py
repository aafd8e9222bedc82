"""The 3-channel reconstruction upsample of the generic kernels (up_taps, hm-cupano_gb300/csrc/
hmp_generic.cu) against the oracle's (up_taps3, oracle/hmp_oracle_body.h), on the CPU: both
functions are taken verbatim from their sources, compiled as host code with floating-point
contraction off (the kernel's translation unit is built with -fmad=false), and compared bit for
bit on random levels whose values are not dyadic fractions, where the summation order shows. The
separable form the Laplacian uses is compiled beside them to show the check can tell the orders
apart.
"""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]

HARNESS = r"""
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>
#include <algorithm>
struct float4 { float x, y, z, w; };
struct float3 { float x, y, z; };
static inline float3 make_float3(float a, float b, float c) { return float3{a, b, c}; }
using std::min;
@KERNEL@
@PLAIN@
@ORACLE@
int main() {
  std::mt19937 rng(7);
  std::uniform_real_distribution<float> U(-300.f, 300.f);
  long checked = 0, taps_differ = 0, plain_differ = 0;
  for (int trial = 0; trial < 200; ++trial) {
    const int lw = 1 + int(rng() % 40), lh = 1 + int(rng() % 30);
    const int hw = 2 * lw - int(rng() % 2), hh = 2 * lh - int(rng() % 2);
    std::vector<float4> lo(size_t(lw) * lh);
    for (auto& v : lo) {
      v = float4{U(rng) / 3.f, U(rng) / 7.f, U(rng) * 0.1f, 255.f};
      if (rng() % 5 == 0) v.x = -0.f;
    }
    for (int y = 0; y < hh; ++y)
      for (int x = 0; x < hw; ++x) {
        const float3 k = up_taps(lo.data(), lw, lh, x, y);
        const float3 p = up_plain(lo.data(), lw, lh, x, y);
        float o[3];
        oracle_up_taps3(reinterpret_cast<const float*>(lo.data()), lw, lh, x, y, o);
        ++checked;
        if (std::memcmp(&k.x, &o[0], 4) || std::memcmp(&k.y, &o[1], 4) || std::memcmp(&k.z, &o[2], 4)) ++taps_differ;
        if (p.x != o[0] || p.y != o[1] || p.z != o[2]) ++plain_differ;
      }
  }
  std::printf("%ld %ld %ld\n", checked, taps_differ, plain_differ);
  return 0;
}
"""


def _function(text: str, signature: str) -> str:
    start = text.index(signature)
    end = text.index("\n}\n", start) + 3
    return text[start:end]


def test_kernel_reconstruction_upsample_equals_the_oracle(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    cu = (REPO / "hm-cupano_gb300" / "csrc" / "hmp_generic.cu").read_text()
    body = (REPO / "oracle" / "hmp_oracle_body.h").read_text()
    kernel = _function(cu, "__device__ __forceinline__ float3 up_taps(").replace("__device__ __forceinline__",
                                                                                  "static inline")
    plain = _function(cu, "__device__ __forceinline__ float3 up_plain(").replace("__device__ __forceinline__",
                                                                                  "static inline")
    oracle = _function(body, "static inline void FN(up_taps3)(").replace("FN(up_taps3)", "oracle_up_taps3")
    oracle = oracle.replace("REAL", "float")
    src = tmp_path / "taps.cpp"
    src.write_text(HARNESS.replace("@KERNEL@", kernel).replace("@PLAIN@", plain).replace("@ORACLE@", oracle))
    exe = tmp_path / "taps"
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", str(src), "-o", str(exe)], check=True)
    checked, taps_differ, plain_differ = (int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True,
                                                                         check=True).stdout.split())
    assert checked > 100_000
    assert taps_differ == 0
    assert plain_differ > 0  # the separable order rounds differently on these values
