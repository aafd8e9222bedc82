"""The C++ drop-in header (include/hm/pano/cuda_stitch_pano.h) used as the reference's classes are.

tests/cpp/drop_in_main.cpp builds ControlMasks in memory, constructs CudaStitchPano /
CudaStitchPano3 / CudaStitchPanoN<uchar4, float4>, uploads frames into hm::CudaMat, calls
process() with the canvas round trip and downloads the canvas. On CPU the program must compile
and link against libhmpano.so; on a GPU its canvas must equal the FP32 oracle bit for bit.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parents[1]
PKG = REPO / "hm-cupano_gb300"
CUDA = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
EXE = PKG / "_build" / "drop_in_main"


def _compile() -> Path:
    import build as hmp_build

    lib = hmp_build.build()
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    EXE.parent.mkdir(exist_ok=True)
    cmd = [cxx, "-std=c++17", "-O1", "-Wall", str(REPO / "tests" / "cpp" / "drop_in_main.cpp"), "-I", str(REPO / "include"),
           "-I", str(CUDA / "include"), "-L", str(lib.parent), "-lhmpano", f"-Wl,-rpath,{lib.parent}",
           "-L", str(CUDA / "lib64"), "-lcudart", f"-Wl,-rpath,{CUDA / 'lib64'}", "-o", str(EXE)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return EXE


def test_cpp_drop_in_compiles_and_links():
    exe = _compile()
    assert exe.exists()


def _write_rig(d: Path, rig, frames, levels: int, batch: int, minimize: bool) -> None:
    lines = [f"{rig.kind} {rig.n} {levels} {batch} {int(minimize)} {frames[0].shape[-1]}"]
    for i in range(rig.n):
        h, w = rig.map_x[i].shape
        lines.append(f"{w} {h} {rig.pos_x[i]} {rig.pos_y[i]}")
        np.ascontiguousarray(rig.map_x[i], dtype=np.uint16).tofile(d / f"mapx_{i}.bin")
        np.ascontiguousarray(rig.map_y[i], dtype=np.uint16).tofile(d / f"mapy_{i}.bin")
    lines.append(f"{rig.seam.shape[1]} {rig.seam.shape[0]}")
    np.ascontiguousarray(rig.seam, dtype=np.uint8).tofile(d / "seam.bin")
    for i, f in enumerate(frames):
        lines.append(f"{f.shape[2]} {f.shape[1]}")
        np.ascontiguousarray(f).tofile(d / f"frame_{i}.bin")
    (d / "meta.txt").write_text("\n".join(lines) + "\n")


@pytest.mark.gpu
@pytest.mark.parametrize("channels", [4, 3])
@pytest.mark.parametrize("workload,kind,levels,batch", [
    ("pano2_1280x720_to_2200x800", 2, 6, 1),
    ("pano3_2704x1520_to_6000x1800", 3, 3, 2),
    ("panon8_2000x1500_to_9000x2400", 1, 4, 1),
])
def test_cpp_drop_in_matches_oracle(tmp_path, oracle_lib, workload, kind, levels, batch, channels):
    """CudaStitchPano*<uchar4, float4> and <uchar3, float3>; the three-image stitcher also runs its
    legacy remap per call (process(..., fused=false))."""
    from hmpano import synth

    exe = _compile()
    rig = synth.workload_rig(workload, seed=77, kind=kind, scale=0.25, oob_fraction=0.02)
    frames = [f[..., :channels].copy() for f in synth.rig_frames(rig, seed=5, batch=batch)]
    _write_rig(tmp_path, rig, frames, levels, batch, True)
    r = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    _, cw, ch = r.stdout.split()
    outputs = [("canvas.bin", True)] + ([("canvas_legacy.bin", False)] if kind == 3 else [])
    for name, fused in outputs:
        got = np.fromfile(tmp_path / name, dtype=np.uint8).reshape(batch, int(ch), int(cw), channels)
        want = oracle_lib.Stitch.from_rig(rig, levels, batch=batch, fused3=fused).run(frames)
        assert got.shape == want.shape
        assert np.array_equal(got, want), (name, int(np.abs(got.astype(int) - want.astype(int)).max()))
