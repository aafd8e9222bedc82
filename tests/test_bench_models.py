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


def test_clock_summary_keeps_the_timed_window_and_reasons():
    """nvidia-smi samples (index, sm, max sm, power, active, hw_slowdown, hw_thermal, sw_thermal,
    sw_power_cap) are kept only inside the timed window; the median SM clock, the largest maximum
    and every active throttle reason are reported."""
    b = _bench()
    s = b.ClockSampler(0)
    rows = [
        (0.5, "0, 1200, 2070, 500, 0x0, Not Active, Not Active, Not Active, Not Active"),
        (1.0, "0, 2070, 2070, 900, 0x0, Not Active, Not Active, Not Active, Not Active"),
        (1.1, "0, 2060, 2070, 950, 0x4, Not Active, Not Active, Not Active, Active"),
        (1.2, "0, 2070, 2070, 960, 0x0, Not Active, Not Active, Not Active, Not Active"),
        (1.3, "0, [N/A], 2070, 960, 0x0, Not Active"),  # a short or malformed line is skipped
        (3.0, "0, 900, 2070, 300, 0x40, Active, Not Active, Not Active, Not Active"),
    ]
    s.stamped = [(t, [v.strip() for v in line.split(",")]) for t, line in rows]
    s.mark(0.9, 2.0)
    out = s.summary()
    assert out["sm_mhz"] == 2070.0 and out["sm_max_mhz"] == 2070.0
    assert out["reasons"] == ["sw_power_cap"] and out["samples"] == 4
