"""Serving benchmark: Poisson arrivals of stitch requests over a mix of seeded pano configurations,
served by hmp_server (continuous batching, resident stitchers, HBM-budget admission).

Also, per configuration of the mix alone (`python -m hmpano.serve_bench [--config SUBSTRING]`, with
hm-cupano_gb300 on the path and the library built): frame time on one stream and per-kernel
CUDA-event times from a pass with the kernels serialised.

The mix is 12 configurations: four seeded rigs (2 x 1280x720 -> 2200x800, 2 x 5120x2880 ->
8500x3300, 8 x 2000x1500 -> 9000x2400, 3 x 2704x1520 -> 6000x1800) at levels 0, 3 and 6. Each
request picks a configuration uniformly at random. Reported per offered rate: achieved canvas
Mpix/s and p50/p99 latency (observed completion - submission, host steady clock). Beside it, the
same request sequence through the plain per-frame path: one stitcher per configuration, one
request after another on one stream.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from . import _lib, pano, synth

RIGS = [
    ("pano2_1280x720_to_2200x800", 2),
    ("pano2_5120x2880_to_8500x3300", 2),
    ("panon8_2000x1500_to_9000x2400", 1),
    ("pano3_2704x1520_to_6000x1800", 3),
]
LEVELS = (0, 3, 6)


def _masks(kind: int, rig):
    pos = [pano.SpatialTiff(float(x), float(y)) for x, y in zip(rig.pos_x, rig.pos_y)]
    if kind == 2:
        return pano.ControlMasks(rig.map_x[0], rig.map_y[0], rig.map_x[1], rig.map_y[1], rig.seam, pos)
    if kind == 3:
        return pano.ControlMasks3(rig.map_x[0], rig.map_y[0], rig.map_x[1], rig.map_y[1], rig.map_x[2], rig.map_y[2],
                                  rig.seam, pos)
    return pano.ControlMasksN(list(rig.map_x), list(rig.map_y), rig.seam, pos)


def build_mix(device, seed: int = 4321, canvases_per_config: int = 4) -> list[dict]:
    """The 12 configurations with device-resident inputs and a few canvases each."""
    import torch

    mix = []
    for r, (workload, kind) in enumerate(RIGS):
        rig = synth.workload_rig(workload, seed=seed + r, kind=kind)
        frames = [torch.from_numpy(f).to(device) for f in synth.rig_frames(rig, seed=seed + 10 * r)]
        imgs = (_lib.Image * len(frames))(*[pano._image(t) for t in frames])
        for levels in LEVELS:
            canvases = [torch.empty((1, rig.canvas_h, rig.canvas_w, 4), dtype=torch.uint8, device=device)
                        for _ in range(canvases_per_config)]
            mix.append({"name": f"{workload}/L{levels}", "kind": kind, "rig": rig, "levels": levels, "frames": frames,
                        "imgs": imgs, "canvases": canvases, "cimgs": [pano._image(c) for c in canvases],
                        "mpix": rig.canvas_w * rig.canvas_h / 1e6, "masks": _masks(kind, rig)})
    torch.cuda.synchronize(device)
    return mix


class Served:
    """A StitchServer with every configuration of the mix registered and warmed up."""

    def __init__(self, mix: list[dict], budget_bytes: int, slots: int, per_config: int):
        self.mix = mix
        self.srv = pano.StitchServer(budget_bytes, slots=slots, max_instances_per_config=per_config)
        self.ids = [self.srv.add_config(m["kind"], m["masks"], m["levels"]) for m in mix]
        self._fn = _lib.lib().hmp_server_submit
        self._rid = C.c_longlong()
        for i, m in enumerate(mix):  # first instance of each configuration (planning, uploads)
            for k in range(per_config):
                self.submit(i, k)
        st = self.srv.drain(600000)
        if not st.ok():
            raise pano.CudaStatusError(st)

    def submit(self, i: int, k: int) -> None:
        m = self.mix[i]
        cv = m["cimgs"][k % len(m["cimgs"])]
        s = self._fn(self.srv._h, self.ids[i], m["imgs"], len(m["frames"]), C.byref(cv), C.byref(self._rid))
        if s.code:
            raise RuntimeError(s.message.decode())

    def run(self, picks: np.ndarray, arrivals_s: np.ndarray | None) -> dict:
        """Submit picks[i] at arrivals_s[i] (seconds from start; None = all at once), drain."""
        self.srv.reset_stats()
        t0 = time.perf_counter()
        for j, i in enumerate(picks):
            if arrivals_s is not None:
                t = arrivals_s[j]
                while time.perf_counter() - t0 < t:
                    pass
            self.submit(int(i), j)
        st = self.srv.drain(600000)
        if not st.ok():
            raise pano.CudaStatusError(st)
        s = self.srv.stats()
        span = max(s["span_ms"], 1e-6) / 1e3
        return {"requests": int(s["completed"]), "failed": int(s["failed"]),
                "achieved_mpix_s": round(s["canvas_mpix"] / span, 1), "achieved_rps": round(s["completed"] / span, 1),
                "p50_ms": round(s["p50_ms"], 4), "p99_ms": round(s["p99_ms"], 4), "mean_ms": round(s["mean_ms"], 4),
                "max_ms": round(s["max_ms"], 4), "max_in_flight": s["max_in_flight"],
                "evictions": int(s["instances_evicted"]), "resident_gb_peak": round(s["resident_bytes_peak"] / 1e9, 2)}

    def close(self) -> None:
        self.srv.close()


def plain_path(mix: list[dict], picks: np.ndarray, device) -> dict:
    """The same request sequence through the plain per-frame path: one stitcher per configuration,
    one process() after another on one stream."""
    import torch

    sts = []
    for m in mix:
        cls = {2: pano.CudaStitchPano, 3: pano.CudaStitchPano3}.get(m["kind"], pano.CudaStitchPanoN)
        st = cls(1, m["levels"], m["masks"], quiet=True)
        if not st.status.ok():
            raise pano.CudaStatusError(st.status)
        sts.append(st)
    stream = torch.cuda.Stream(device)
    fn = _lib.lib().hmp_stitcher_process
    sp = C.c_void_p(stream.cuda_stream)

    def go(seq):
        for j, i in enumerate(seq):
            m = mix[int(i)]
            s = fn(sts[int(i)]._handle, m["imgs"], len(m["frames"]), C.byref(m["cimgs"][j % len(m["cimgs"])]), sp)
            if s.code:
                raise RuntimeError(s.message.decode())

    go(picks[: min(len(picks), 24)])
    torch.cuda.synchronize(device)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    go(picks)
    e1.record(stream)
    torch.cuda.synchronize(device)
    sec = e0.elapsed_time(e1) / 1e3
    mpix = float(sum(mix[int(i)]["mpix"] for i in picks))
    del sts
    return {"requests": len(picks), "mpix_s": round(mpix / sec, 1), "rps": round(len(picks) / sec, 1)}


def sweep(device, budget_gb: float = 150.0, slots: int = 8, per_config: int = 2, seconds: float = 1.0,
          fractions=(0.25, 0.5, 0.75, 0.9), seed: int = 99) -> dict:
    """Saturation throughput, then Poisson arrivals at fractions of it; plain path beside."""
    mix = build_mix(device)
    rng = np.random.default_rng(seed)
    served = Served(mix, int(budget_gb * 1e9), slots, per_config)
    n_sat = 600
    sat = served.run(rng.integers(0, len(mix), n_sat), None)
    rates = []
    for f in fractions:
        rate = f * sat["achieved_rps"]
        n = max(50, int(rate * seconds))
        arrivals = np.cumsum(rng.exponential(1.0 / rate, n))
        r = served.run(rng.integers(0, len(mix), n), arrivals)
        r["offered_rps"] = round(rate, 1)
        r["load"] = f
        rates.append(r)
    served.close()
    plain = plain_path(mix, rng.integers(0, len(mix), n_sat), device)
    mid = min(rates, key=lambda r: abs(r["load"] - 0.75))
    return {"configs": len(mix), "budget_gb": budget_gb, "slots": slots, "instances_per_config": per_config,
            "saturation": sat, "plain_path": plain, "rates": rates,
            "p50_ms_at_75pct": mid["p50_ms"], "p99_ms_at_75pct": mid["p99_ms"],
            "speedup_vs_plain": round(sat["achieved_mpix_s"] / plain["mpix_s"], 3)}


def per_config(device, match: str = "", reps: int = 50, warmup: int = 5) -> list[dict]:
    """Each configuration of the mix alone: microseconds per frame (batch 1, one stream, CUDA
    events over `reps` frames) and per-kernel times from a serialised pass."""
    import torch

    out = []
    stream = torch.cuda.Stream(device)
    sp = C.c_void_p(stream.cuda_stream)
    fn = _lib.lib().hmp_stitcher_process
    for m in build_mix(device):
        if match not in m["name"]:
            continue
        cls = {2: pano.CudaStitchPano, 3: pano.CudaStitchPano3}.get(m["kind"], pano.CudaStitchPanoN)
        st = cls(1, m["levels"], m["masks"], quiet=True)
        if not st.status.ok():
            raise pano.CudaStatusError(st.status)

        def go(k):
            for j in range(k):
                s = fn(st._handle, m["imgs"], len(m["frames"]), C.byref(m["cimgs"][j % len(m["cimgs"])]), sp)
                if s.code:
                    raise RuntimeError(s.message.decode())

        go(warmup)
        torch.cuda.synchronize(device)
        st.set_timing(True, serialize=True)
        go(20)
        torch.cuda.synchronize(device)
        kt = st.kernel_times()
        st.set_timing(False)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        go(reps)
        e1.record(stream)
        torch.cuda.synchronize(device)
        us = e0.elapsed_time(e1) / reps * 1e3
        out.append({"config": m["name"], "us_per_frame": round(us, 1), "gpix_s": round(m["mpix"] / us * 1e3, 1),
                    "kernel_us_serialized": {k: round(v[0] / max(v[1], 1) * 1e3, 1) for k, v in kt.items()}})
        del st
    return out


if __name__ == "__main__":
    import argparse
    import json

    import torch

    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--config", default="", help="only configurations whose name contains this")
    ap.add_argument("--reps", type=int, default=50)
    args = ap.parse_args()
    for r in per_config(torch.device("cuda", 0), args.config, args.reps):
        print(json.dumps(r), flush=True)
