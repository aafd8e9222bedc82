"""Byte models the benchmark reports beside its timings (host arithmetic only)."""
import importlib.util
import json
from pathlib import Path

REPO = Path(__file__).resolve().parents[1]


def _bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", REPO / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _info(levels, batch=1, mapped=4_000_000):
    cw, ch = 8500, 3300
    wr, br = (4018, 0, 482, 3300), (3954, 0, 610, 3300)
    a0 = wr[2] * wr[3] if levels else 0
    m0 = (cw * ch - a0) * (5 + 8 * batch) + (mapped * (4 + 4 * batch) + a0 * (1 + 4 * batch) if levels else 0)
    return {"m0_bytes": float(m0), "levels": levels, "canvas": (cw, ch), "write_rect": wr, "blend_rect": br}


def test_m1_equals_m0_for_the_hard_seam():
    b = _bench()
    info = _info(0)
    assert b.m1_bytes(info, 2, 1, "f32") == info["m0_bytes"]


def test_m1_adds_level0_again_and_the_levels():
    b = _bench()
    info = _info(6)
    mapped = 4_000_000
    w, h, lev32, lev16 = 610, 3300, 0, 0
    for _ in range(5):
        w, h = (w + 1) // 2, (h + 1) // 2
        lev32 += w * h * (2 * 2 * 16 + 2 * 16 + 4)
        lev16 += w * h * (2 * 2 * 8 + 2 * 8 + 4)
    assert b.m1_bytes(info, 2, 1, "f32") == info["m0_bytes"] + mapped * 8 + lev32
    assert b.m1_bytes(info, 2, 1, "f16") == info["m0_bytes"] + mapped * 8 + lev16


def test_frame_dram_needs_every_kernel():
    b = _bench()
    captured = json.loads((REPO / "profiles" / "traffic.json").read_text())
    prefix = "pano2_5120x2880_to_8500x3300/L6/f32"
    names = ["canvas_gather", "pyr_down", "pyr_coarse", "pyr_fine"]
    total = b.ncu_frame_bytes(captured, prefix, names)
    assert total == sum(captured[f"{prefix}/{k}"] for k in names)
    assert b.ncu_frame_bytes(captured, prefix, names + ["missing"]) is None
