#!/usr/bin/env python
"""Throughput of the GB300 stitching path on the production two-image workload.

Workload (the reference's headline case, README.md:1-7): two 5120x2880 RGBA frames remapped
through seeded cylindrical CV_16U tables onto an 8500x3300 canvas, 6-level Laplacian blend,
FP32 pyramid, uint8 pack; synthetic seeded inputs (no dataset). One step = one process() call
on one frame. Inputs are larger than L2: three frame/canvas sets rotate between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line. ``value`` is canvas Mpix/s over all ranks with inputs resident in HBM (the
pyramid kernels run concurrently with the canvas gather, as in production); ``e2e`` is the same
metric through the public API with pinned host frames copied in and the canvas copied out every
step; ``roofline`` is the dominant kernel's algorithmic bytes per launch over its CUDA-event
duration, taken in a pass where the stitcher runs its kernels one after another (so the time is
the kernel's own), against the measured HBM copy bandwidth; ``hbm_frac_frame`` is the frame's
compulsory bytes over the concurrent frame time. ``cpu_baseline`` is the oracle (a C port of the
reference's algorithm) on the host cores. ``--impl reference`` times that CPU implementation as
the reference arm. ``vs_baseline`` is fps over the reference's published 340 fps (RTX 4090, same
metric). ``batched`` is the multi-stream batched job (hmpano/batch.py): one CUDA graph per job,
frames per call and tiles autotuned, FP16 storage, against the plain per-frame path on the same
frames. ``serve`` is the serving sweep (hmpano/serve_bench.py): 12 seeded configurations,
Poisson arrivals at fractions of the saturation rate, p50/p99 latency, against the plain
per-frame path on the same request mix. Multi-GPU runs are independent replicas (weak scaling,
no collective on the data path).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO))
sys.path.insert(0, str(REPO / "hm-cupano_gb300"))

METRIC = "canvas Mpix/s & fps at 8500x3300 L=6; % HBM peak; p50/p99 serve latency"
WORKLOAD = "pano2_5120x2880_to_8500x3300"
N_SETS = 3
PUBLISHED_FPS = 340.0  # reference README: 2 images -> ~8500x3300, 6 levels, RTX 4090


def _peaks() -> tuple[float, str]:
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            d = json.loads(p.read_text())
            return float(d["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def m1_bytes(info: dict, n_images: int, batch: int, storage: str) -> float:
    """Bytes per process() of a level-materialised two-pass pyramid (the reference's structure):
    the compulsory bytes M0, plus level 0 gathered again for the reconstruction, plus, at every
    level >= 1, each image's Gaussian written and read once, the reconstruction written and read
    once (4 channels of `storage`) and the mask level read once (K floats: 1 for two images, else
    one per image). RGBA8 frames and canvas."""
    m0 = float(info["m0_bytes"])
    levels = int(info["levels"])
    if levels == 0:
        return m0
    cw, ch = info["canvas"]
    wr, br = info["write_rect"], info["blend_rect"]
    a0 = wr[2] * wr[3]
    # m0 = outside the write rect (5 + 8B per pixel) + mapped slot pixels (4 + 4B) + a0 (1 + 4B).
    level0 = m0 - (cw * ch - a0) * (5 + 8 * batch) - a0 * (1 + 4 * batch)
    s = 16 if storage == "f32" else 8
    k = 1 if n_images == 2 else n_images
    w, h, levels_bytes = br[2], br[3], 0.0
    for _ in range(1, levels):
        w, h = (w + 1) // 2, (h + 1) // 2
        levels_bytes += w * h * (batch * (2 * n_images * s + 2 * s) + 4 * k)
    return m0 + level0 + levels_bytes


def ncu_frame_bytes(traffic: dict, prefix: str, kernels) -> int | None:
    """DRAM bytes of one frame summed over its kernels' ncu captures (None unless all present)."""
    vals = [traffic.get(f"{prefix}/{k}") for k in kernels]
    return int(sum(vals)) if vals and all(v is not None for v in vals) else None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.samples: list[list[str]] = []
        self.stamped: list[tuple[float, list[str]]] = []
        self.window = (0.0, float("inf"))
        self._proc = None
        self._thr = None

    def _read(self):
        for line in self._proc.stdout:
            parts = [v.strip() for v in line.split(",")]
            if len(parts) >= 9:
                self.stamped.append((time.perf_counter(), parts))

    def __enter__(self):
        try:
            # Loop mode samples every 100 ms from one process (no per-sample start-up delay).
            self._proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                           "--format=csv,noheader,nounits", "-lms", "100"],
                                          stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._thr = threading.Thread(target=self._read, daemon=True)
            self._thr.start()
            time.sleep(0.15)  # first sample lands inside the timed region
        except Exception:
            self._proc = None
        return self

    def __exit__(self, *exc):
        if self._proc:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except Exception:
                self._proc.kill()
        if self._thr:
            self._thr.join(timeout=5)

    def mark(self, start: float, end: float) -> None:
        """Keep only the samples taken between start and end (host perf_counter)."""
        self.window = (start, end)

    def summary(self) -> dict:
        self.samples = [p for t, p in self.stamped if self.window[0] <= t <= self.window[1]]
        sm = [float(s[1]) for s in self.samples if len(s) >= 9 and s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if len(s) >= 9 and s[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            if len(s) < 9:
                continue
            for name, v in zip(names, s[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


CLOCK_PAD_S = 0.35


def pad_steps(step, stream, seconds: float) -> int:
    """Runs the bench step until `seconds` of wall time have passed (in chunks of 25 steps with a
    synchronize after each, outside any timed region); returns the number of steps."""
    import torch

    n = 0
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        with torch.cuda.stream(stream):
            for i in range(25):
                step(n + i)
        torch.cuda.synchronize()
        n += 25
    return n


def _concurrent_copies_s(dev, h_in, d_in, d_out, h_out) -> float:
    """Best of 5 (CUDA events) of one host-to-device copy and one device-to-host copy issued on
    two streams at once, in seconds."""
    import torch

    s_up, s_dn = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
    best = float("inf")
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        fork, done = torch.cuda.Event(), torch.cuda.Event()
        e0.record(s_up)
        fork.record(s_up)
        s_dn.wait_event(fork)
        with torch.cuda.stream(s_up):
            d_in.copy_(h_in, non_blocking=True)
        with torch.cuda.stream(s_dn):
            h_out.copy_(d_out, non_blocking=True)
        done.record(s_dn)
        s_up.wait_event(done)
        e1.record(s_up)
        torch.cuda.synchronize(dev)
        best = min(best, e0.elapsed_time(e1) / 1e3)
    return best


def host_link(dev, nbytes: int = 256 << 20) -> dict:
    """Pinned host <-> device copy bandwidth (GB/s, best of 5, CUDA events), the bound of the
    end-to-end number, whose every step copies its frames in and its canvas out: each direction
    alone, and each direction while the other runs (`both`; the link carries less per direction
    then, so this, not the one-way figures, bounds a pipeline that overlaps the two)."""
    import torch

    h = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
    h2 = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
    d = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    d2 = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    s = torch.cuda.Stream(dev)
    out = {}
    for name, dst, src in (("h2d", d, h), ("d2h", h, d)):
        best = float("inf")
        for _ in range(5):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(s):
                e0.record(s)
                dst.copy_(src, non_blocking=True)
                e1.record(s)
            torch.cuda.synchronize(dev)
            best = min(best, e0.elapsed_time(e1) / 1e3)
        out[name] = round(nbytes / best / 1e9, 1)
    out["both"] = round(nbytes / _concurrent_copies_s(dev, h, d, d2, h2) / 1e9, 1)
    return out


def step_copy_floor_ms(dev, in_bytes: int, out_bytes: int) -> float:
    """The copies of one end-to-end step alone: `in_bytes` host to device while `out_bytes` go
    device to host (ms, best of 5), the floor for a step whose copies overlap."""
    import torch

    h_in = torch.empty(in_bytes, dtype=torch.uint8).pin_memory()
    h_out = torch.empty(out_bytes, dtype=torch.uint8).pin_memory()
    d_in = torch.empty(in_bytes, dtype=torch.uint8, device=dev)
    d_out = torch.empty(out_bytes, dtype=torch.uint8, device=dev)
    return _concurrent_copies_s(dev, h_in, d_in, d_out, h_out) * 1e3


def _masks(rig):
    import hmpano

    pos = [hmpano.SpatialTiff(float(x), float(y)) for x, y in zip(rig.pos_x, rig.pos_y)]
    return hmpano.ControlMasks(rig.map_x[0], rig.map_y[0], rig.map_x[1], rig.map_y[1], rig.seam, pos)


def cpu_baseline(rig, frames, levels: int, seconds: float = 10.0) -> dict:
    """The oracle (C port of the reference algorithm) on all host cores, on a bounded sample:
    as many full frames as fit in about `seconds` of CPU time."""
    from oracle import oracle

    oracle.build()
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    st = oracle.Stitch.from_rig(rig, levels)
    t0 = time.perf_counter()
    st.run(frames)  # warm-up, also sizes the sample
    frames_sample = max(2, int(seconds / max(time.perf_counter() - t0, 1e-3)))
    t0 = time.perf_counter()
    for _ in range(frames_sample):
        st.run(frames)
    dt = (time.perf_counter() - t0) / frames_sample
    mpix = rig.canvas_w * rig.canvas_h / 1e6
    return {"value": round(mpix / dt, 2), "unit": "Mpix/s", "cores": oracle.get_threads(), "kind": "port",
            "sample": f"{frames_sample} full frames of {WORKLOAD} L={levels} FP32 after 1 warm-up, "
                      f"{dt * 1e3:.0f} ms/frame", "fps": round(1.0 / dt, 3)}


def cpu_baseline_stabilize(seconds: float = 8.0) -> dict:
    """The stabiliser oracle (C port of src/cuda/cudaStabilize.cu, one core) on the GPU leg's
    3840x2160 frame pair: as many runs as fit in about `seconds`."""
    from hmpano import stabilize_bench
    from oracle import oracle

    oracle.build()
    prev, nxt = stabilize_bench.frames(2160, 3840)
    st = oracle.Stabilize()
    t0 = time.perf_counter()
    st.run(prev, nxt)
    runs = max(2, int(seconds / max(time.perf_counter() - t0, 1e-3)))
    t0 = time.perf_counter()
    for _ in range(runs):
        st.run(prev, nxt)
    dt = (time.perf_counter() - t0) / runs
    return {"value": round(dt * 1e3, 2), "unit": "ms/frame", "cores": 1, "kind": "port",
            "sample": f"{runs} runs of the 3840x2160 pair after 1 warm-up"}


def reference_arm(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from hmpano import synth
    from oracle import oracle

    rig = synth.workload_rig(WORKLOAD, seed=1234)
    frames = synth.rig_frames(rig, seed=1)
    oracle.build()
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    st = oracle.Stitch.from_rig(rig, args.levels)
    for _ in range(args.warmup):
        st.run(frames)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        st.run(frames)
    dt = (time.perf_counter() - t0) / args.steps
    mpix = rig.canvas_w * rig.canvas_h / 1e6
    value = mpix / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "Mpix/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "fps": round(1.0 / dt, 4),
        "config": {"workload": WORKLOAD, "levels": args.levels, "storage": "f32", "batch": 1,
                   "canvas": f"{rig.canvas_w}x{rig.canvas_h}"},
        "cpu_baseline": {"value": round(value, 3), "unit": "Mpix/s", "cores": oracle.get_threads(), "kind": "port",
                         "sample": f"{args.steps} full frames after {args.warmup} warm-up"},
        "e2e": {"value": round(value, 3), "unit": "Mpix/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gpu_launches": 0,
    }
    print(json.dumps(line), flush=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--levels", type=int, default=6)
    ap.add_argument("--storage", default="f32")
    ap.add_argument("--batch", type=int, default=1, help="frames per process() call")
    ap.add_argument("--tile-down", type=int, default=0, help="pyramid down tile edge (32 or 64; 0 = default)")
    ap.add_argument("--filter", default="refbox", choices=["refbox", "binomial5"],
                    help="pyramid filter: the reference's 2x2 box / bilinear, or 5-tap binomial")
    ap.add_argument("--graph", action="store_true",
                    help="capture one process() per buffer set into a CUDA graph and replay it")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving sweep (p50/p99 latency)")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched multi-stream graph job")
    ap.add_argument("--no-variants", action="store_true", help="skip the other workloads' frame times")
    ap.add_argument("--no-stabilize", action="store_true", help="skip the frame stabiliser timings")
    ap.add_argument("--serve-seconds", type=float, default=1.0, help="arrival window per offered rate")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    if args.impl == "reference":
        reference_arm(args)
        return

    import numpy as np
    import torch

    import __graft_entry__

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    __graft_entry__.build()
    import hmpano
    from hmpano import _lib, replicas, synth

    reps = replicas.init("nccl")
    rank, world = reps.rank, reps.world

    rig = synth.workload_rig(WORKLOAD, seed=1234)
    B = args.batch
    host_frames = synth.rig_frames(rig, seed=1 + rank, batch=B)
    pano = hmpano.CudaStitchPano(B, args.levels, _masks(rig), quiet=True, storage=args.storage, filter=args.filter)
    if not pano.status.ok():
        raise SystemExit(f"stitcher: {pano.status}")
    if args.tile_down:
        pano.set_tiles(args.tile_down)
    info = pano.info()
    W, H = rig.canvas_w, rig.canvas_h
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(dev)
    sets = []
    for i in range(N_SETS):
        ins = [torch.from_numpy(np.roll(f, i, axis=2)).to(dev) for f in host_frames]
        canvas = torch.empty((B, H, W, 4), dtype=torch.uint8, device=dev)
        sets.append((ins, canvas))
    # Pre-marshalled C-ABI arguments: the timed loop is one C call per step.
    fn = _lib.lib().hmp_stitcher_process
    calls = []
    for ins, canvas in sets:
        imgs = (_lib.Image * 2)(*[hmpano.pano._image(t) for t in ins])
        cv = hmpano.pano._image(canvas)
        calls.append((imgs, cv))
    sptr = C.c_void_p(stream.cuda_stream)

    def step(i):
        imgs, cv = calls[i % N_SETS]
        s = fn(pano._handle, imgs, 2, C.byref(cv), sptr)
        if s.code:
            raise RuntimeError(s.message.decode())

    with torch.cuda.stream(stream):
        for i in range(args.warmup):
            step(i)
    torch.cuda.synchronize()
    pano.set_timing(True)
    reps.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    sampler = ClockSampler(local) if rank == 0 else None
    if sampler:
        sampler.__enter__()
    e0.record(stream)
    for i in range(args.steps):
        step(i)
    e1.record(stream)
    torch.cuda.synchronize()
    reps.barrier()
    ms = e0.elapsed_time(e1) / args.steps
    ktimes = pano.kernel_times()
    pano.set_timing(False)
    ms = reps.max_over_ranks(ms)
    mpix = W * H / 1e6

    # The headline pass: the same steps without per-kernel event records (instrumentation),
    # optionally replayed from a CUDA graph that holds one process() per buffer set.
    graph = None
    if args.graph:
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=stream):
            for k in range(N_SETS):
                step(k)
        torch.cuda.synchronize()
        for _ in range(2):
            graph.replay()
        torch.cuda.synchronize()
    torch.cuda.synchronize()
    # The clock record: nvidia-smi samples every 100 ms, and a short timed region (a few ms at
    # the default step counts) holds none. The same steps therefore run for at least
    # CLOCK_PAD_S before and after the timed region while the sampler runs, and the record
    # covers that window (the timed region inside it is unchanged: exactly K steps).
    t_region0 = time.perf_counter()
    pad_before = pad_steps(step, stream, CLOCK_PAD_S)
    torch.cuda.synchronize()
    e0.record(stream)
    if graph is not None:
        with torch.cuda.stream(stream):
            for _ in range(args.steps // N_SETS):
                graph.replay()
            for i in range(args.steps % N_SETS):
                step(i)
    else:
        for i in range(args.steps):
            step(i)
    e1.record(stream)
    torch.cuda.synchronize()
    pad_after = pad_steps(step, stream, CLOCK_PAD_S)
    t_region1 = time.perf_counter()
    if sampler:
        sampler.__exit__(None, None, None)
        sampler.mark(t_region0, t_region1)
    ms_plain = reps.max_over_ranks(e0.elapsed_time(e1) / args.steps)
    ms_instrumented = ms
    ms = ms_plain
    value = reps.job_rate(args.steps * B * mpix, ms * args.steps / 1e3)

    # Kernel attribution: a pass with the kernels serialised on one stream, so that each
    # kernel's event-timed duration is its own (feeds the roofline of the dominant kernel).
    k_serial = max(20, min(args.steps, 1000))
    pano.set_timing(True, serialize=True)
    with torch.cuda.stream(stream):
        for i in range(k_serial):
            step(i)
    torch.cuda.synchronize()
    ktimes_serial = pano.kernel_times()
    pano.set_timing(False)
    torch.cuda.synchronize()

    # End to end through the public API: every step copies its frames in from pinned host memory
    # and its canvas out to pinned host memory. Three buffer sets and three streams (copy-in,
    # stitch, copy-out) let step i+1's upload and step i-1's download overlap step i's stitch.
    e2e = None
    if not args.no_e2e:
        pinned_in = [torch.from_numpy(f).pin_memory() for f in host_frames]
        pinned_out = [torch.empty((B, H, W, 4), dtype=torch.uint8).pin_memory() for _ in range(N_SETS)]
        s_in, s_out = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
        ev_in = [torch.cuda.Event() for _ in range(N_SETS)]
        ev_st = [torch.cuda.Event() for _ in range(N_SETS)]
        ev_out = [torch.cuda.Event() for _ in range(N_SETS)]

        def e2e_step(t):
            k = t % N_SETS
            dins, dcanvas = sets[k]
            with torch.cuda.stream(s_in):
                if t >= N_SETS:
                    s_in.wait_event(ev_st[k])
                for d, h in zip(dins, pinned_in):
                    d.copy_(h, non_blocking=True)
                ev_in[k].record(s_in)
            with torch.cuda.stream(stream):
                stream.wait_event(ev_in[k])
                if t >= N_SETS:
                    stream.wait_event(ev_out[k])
                pano.process(dins[0], dins[1], dcanvas, stream=stream)
                ev_st[k].record(stream)
            with torch.cuda.stream(s_out):
                s_out.wait_event(ev_st[k])
                pinned_out[k].copy_(dcanvas, non_blocking=True)
                ev_out[k].record(s_out)

        k_e2e = max(12, min(args.steps, 60))
        for t in range(6):
            e2e_step(t)
        torch.cuda.synchronize()
        e0.record(s_in)
        for t in range(k_e2e):
            e2e_step(t + 6)
        e1.record(s_out)
        torch.cuda.synchronize()
        ms_e2e = e0.elapsed_time(e1) / k_e2e
        last = (k_e2e + 5) % N_SETS
        ok = bool(torch.equal(pinned_out[last], sets[last][1].cpu()))
        e2e = {"value": round(world * B * mpix / (ms_e2e / 1e3), 2), "unit": "Mpix/s",
               "h2d_bytes_per_step": int(sum(f.nbytes for f in host_frames)),
               "d2h_bytes_per_step": int(B * W * H * 4), "ms_per_step": round(ms_e2e, 4), "steps": k_e2e,
               "fps": round(world * B * 1e3 / ms_e2e, 1), "pipeline": "3 streams x 3 buffer sets",
               "output_check": ok}
        # Its bound: the step's copies alone, both directions at once as the pipeline runs them
        # (a direction carries less while the other runs, so the one-way rates understate it).
        link = host_link(dev)
        floor_ms = step_copy_floor_ms(dev, e2e["h2d_bytes_per_step"], e2e["d2h_bytes_per_step"])
        e2e["host_link_gbs"] = link
        e2e["copy_floor_ms_per_step"] = round(floor_ms, 4)
        e2e["frac_of_copy_floor"] = round(floor_ms / ms_e2e, 3)

    peak, peak_kind = _peaks()
    names = ["canvas_gather", "pyr_down", "pyr_coarse", "pyr_fine"]
    dom = max(names, key=lambda k: ktimes_serial[k][0])
    tot, cnt = ktimes_serial[dom]
    per_launch_ms = tot / max(cnt, 1)
    wr = info["write_rect"]
    canvas_px = W * H
    # 4 table bytes once per call (the entry carries the owner), 4 source + 4 canvas bytes per
    # frame of the batch.
    # Canvas pixels the gather writes: outside the write rect, plus the copy blocks inside it.
    gather_px = info["gather_pixels"]
    gather_bytes = gather_px * (4.0 + 8.0 * B)
    dom_bytes = {"canvas_gather": gather_bytes}.get(dom)
    achieved = dom_bytes / (per_launch_ms / 1e3) / 1e9 if dom_bytes else None
    traffic = frame_dram = None
    tp = REPO / "profiles" / "traffic.json"
    if tp.exists():
        try:
            prefix = f"{WORKLOAD}/L{args.levels}/{args.storage}"
            captured = json.loads(tp.read_text())
            traffic = captured.get(f"{prefix}/{dom}")
            if B == 1 and args.filter == "refbox":
                # The hard seam is the gather alone; a pyramid frame is all four kernels.
                frame_dram = ncu_frame_bytes(captured, prefix, names if info["levels"] > 1 else ["canvas_gather"])
        except Exception:
            traffic = frame_dram = None
    line = {
        "metric": METRIC,
        "value": round(value, 2),
        "unit": "Mpix/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms, 5),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": round(world * B * 1e3 / ms / PUBLISHED_FPS, 3) if args.storage == "f32" else None,
        "dtype": "f32" if args.storage == "f32" else "f16-storage/f32-arith",
        "data": "synthetic",
        "fps": round(world * B * 1e3 / ms, 1),
        "hbm_frac_frame": round(info["m0_bytes"] / (ms / 1e3) / (peak * 1e9), 4),
        "m0_bytes_per_step": int(info["m0_bytes"]),
        # The level-materialised model (every pyramid level through HBM) for comparison, and the
        # frame's DRAM bytes summed over its kernels' ncu captures (profiles/, each kernel alone).
        "m1_bytes_per_step": int(m1_bytes(info, 2, B, args.storage)),
        "ncu_dram_bytes_per_step": frame_dram,
        "ms_per_step_instrumented": round(ms_instrumented, 5),
        "config": {"workload": WORKLOAD, "levels": args.levels, "storage": args.storage, "batch": B,
                   "graph": bool(args.graph), "filter": args.filter,
                   "canvas": f"{W}x{H}", "blend_rect": list(info["blend_rect"]),
                   "l2": f"inputs larger than L2: {N_SETS} rotating frame/canvas sets",
                   "parallelism": f"replicas x{world}"},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1) if achieved else None,
                     "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4) if achieved else None,
                     "traffic": traffic, "peak_kind": peak_kind,
                     "bytes_per_launch": int(dom_bytes) if dom_bytes else None,
                     "ms_per_launch": round(per_launch_ms, 5),
                     "timing": f"CUDA events, {k_serial} steps with the kernels serialised on one stream"},
        "kernel_ms": {k: round(v[0] / max(v[1], 1), 5) for k, v in ktimes.items()},
        "kernel_ms_serialized": {k: round(v[0] / max(v[1], 1), 5) for k, v in ktimes_serial.items()},
        # Kernels launched in the headline timed region (every rank): each process() launches
        # exactly launches_per_process of this library's kernels (here 5: pyr_down, pyr_coarse,
        # pyr_fine over their work lists, canvas_gather, and the copy-block fallback's one-thread
        # gate, which returns at once unless a copy block's source alpha was 0).
        "gpu_launches": world * args.steps * int(info["launches_per_process"]),
        "e2e": e2e,
        "clocks": dict(sampler.summary(), window_s=round(t_region1 - t_region0, 3),
                       padding_steps=[pad_before, pad_after]) if sampler else None,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(rig, host_frames, args.levels)
    if not args.no_variants and world == 1:
        # The other named workloads alone: three-image 6000x1800 and eight-image 9000x2400 at 6
        # levels (FP32 and FP16), and the headline frame with FP16 storage, Binomial5, 0 levels.
        from hmpano import variants

        line["variants"] = variants.run(dev, max(50, min(args.steps, 300)), peak,
                                        only=[v[0] for v in variants.VARIANTS if v[0] != "pano2_l6_f32"])
    if not args.no_batched and world == 1:
        # Batched streaming job: 4 two-image + 4 three-image streams x 32 frames, FP16 storage, one
        # CUDA graph, frames per call and tiles autotuned.
        from hmpano import batch

        line["batched"] = batch.run(dev)
    if not args.no_serve and world == 1:
        # Serving mix on this GPU: 12 configurations, Poisson arrivals, 150 GB admission budget.
        from hmpano import serve_bench

        line["serve"] = serve_bench.sweep(dev, seconds=args.serve_seconds)
    if not args.no_stabilize and world == 1:
        # Frame stabiliser (Harris corners, Lucas-Kanade flow, warp) on a 3840x2160 float frame pair.
        from hmpano import stabilize_bench

        line["stabilize"] = stabilize_bench.run(dev, peak)
        if not args.no_cpu_baseline:
            line["stabilize"]["cpu_baseline"] = cpu_baseline_stabilize()
    if rank == 0:
        print(json.dumps(line), flush=True)
    reps.close()


if __name__ == "__main__":
    main()
