"""Batched streaming form: many frames of several independent streams with uneven canvas sizes,
the whole job replayed from one CUDA graph (the library's hmp_batch_* job), frames per call and
pyramid tiles chosen by an autotuner whose choice is cached in JSON.

The job: 4 two-image streams (2 x 5120x2880 -> 8500x3300) and 4 three-image streams
(3 x 2704x1520 -> 6000x1800), 32 consecutive frames each, 6 levels, FP16 pyramid storage with
FP32 arithmetic. Every stream has its own stitcher (batch = frames per call) and CUDA stream;
the graph holds each stream's calls in order, all streams forked from one root stream, so the
streams' kernels overlap on the GPU and one graph launch runs the whole job. Frames are seeded
synthetic frames, shifted per stream and frame.

The plain per-frame path for comparison runs the same frames one process() at a time (batch 1,
no graph) on one stream: FP32 level storage, the drop-in form the speed-up is quoted against, and
also with FP16 storage.
"""
from __future__ import annotations

import ctypes as C
import itertools
import json
import os
import time
from pathlib import Path

from . import _lib, pano, synth

JOB = [("pano2_5120x2880_to_8500x3300", 2)] * 4 + [("pano3_2704x1520_to_6000x1800", 3)] * 4
FRAMES = 32
CACHE = Path(os.environ.get("HMPANO_AUTOTUNE_CACHE", Path.home() / ".cache" / "hmpano" / "autotune.json"))


def _masks(kind: int, rig):
    pos = [pano.SpatialTiff(float(x), float(y)) for x, y in zip(rig.pos_x, rig.pos_y)]
    if kind == 2:
        return pano.ControlMasks(rig.map_x[0], rig.map_y[0], rig.map_x[1], rig.map_y[1], rig.seam, pos)
    return pano.ControlMasks3(rig.map_x[0], rig.map_y[0], rig.map_x[1], rig.map_y[1], rig.map_x[2], rig.map_y[2],
                              rig.seam, pos)


class Job:
    """Rigs and device-resident frames of the batched job (shared by every candidate)."""

    def __init__(self, device, levels: int = 6, storage: str = "f16", frames: int = FRAMES, seed: int = 77,
                 scale: float = 1.0):
        import torch

        self.device, self.levels, self.storage, self.frames = device, levels, storage, frames
        rigs = {}
        for w, kind in dict.fromkeys(JOB):
            rig = synth.workload_rig(w, seed=seed, kind=kind, scale=scale)
            base = [torch.from_numpy(f[0]).to(device) for f in synth.rig_frames(rig, seed=seed + 1)]
            rigs[w] = (rig, base)
        self.streams = []
        for s, (w, kind) in enumerate(JOB):
            rig, base = rigs[w]
            ins = [torch.stack([torch.roll(b, shifts=3 * s + 7 * f, dims=1) for f in range(frames)]) for b in base]
            self.streams.append({"workload": w, "kind": kind, "rig": rig, "inputs": ins, "masks": _masks(kind, rig),
                                 "mpix": rig.canvas_w * rig.canvas_h / 1e6})
        torch.cuda.synchronize(device)

    @property
    def mpix_total(self) -> float:
        return self.frames * sum(s["mpix"] for s in self.streams)

    def signature(self) -> str:
        import torch

        return f"{'+'.join(s['workload'] for s in self.streams)}/L{self.levels}/{self.storage}/" \
               f"{torch.cuda.get_device_name(self.device)}"


class Plan:
    """Stitchers (one per stream, `batch` frames per call) and the job as one native batch
    (hmp_batch_*: every stream's calls captured into one CUDA graph)."""

    def __init__(self, job: Job, batch: int, tile_down):
        """tile_down: one pyramid down-tile edge for every stream, or {kind: edge} per stream kind
        (2 = two-image, 3 = three-image); an edge may be an (edge, CTAs per SM) pair, which also
        caps the down kernel's residency (hmp_stitcher_set_down_residency)."""
        import torch

        if job.frames % batch:
            raise ValueError("frames per stream must be a multiple of the batch")
        self.job, self.batch, self.tile_down = job, batch, tile_down
        self.sts, self.canvases = [], []
        for s in job.streams:
            cls = pano.CudaStitchPano if s["kind"] == 2 else pano.CudaStitchPano3
            st = cls(batch, job.levels, s["masks"], quiet=True, storage=job.storage)
            if not st.status.ok():
                raise pano.CudaStatusError(st.status)
            self._apply(st, s["kind"])
            self.sts.append(st)
            h, w = s["rig"].canvas_h, s["rig"].canvas_w
            self.canvases.append([torch.empty((batch, h, w, 4), dtype=torch.uint8, device=job.device) for _ in range(2)])
        self.root = torch.cuda.Stream(job.device)
        self.graph = None
        self.rebuild()

    def _apply(self, st, kind: int) -> None:
        spec = self.tile_for(kind)
        tile, res = (spec, None) if isinstance(spec, int) else (int(spec[0]), int(spec[1]))
        st.set_tiles(tile)
        if res is not None:
            st.set_down_residency(res)

    def tile_for(self, kind: int):
        t = self.tile_down
        v = t[kind] if isinstance(t, dict) else t
        return int(v) if isinstance(v, (int, float, str)) else (int(v[0]), int(v[1]))

    def set_tiles(self, tile_down) -> None:
        """New tiles (one edge, or {kind: edge}); the graph is rebuilt."""
        self.tile_down = tile_down
        for st, s in zip(self.sts, self.job.streams):
            self._apply(st, s["kind"])
        self.rebuild()

    def rebuild(self) -> None:
        """A new batch of every stream's calls (after the stitchers' tiles change)."""
        self.graph = pano.Batch()
        for i, s in enumerate(self.job.streams):
            for k in range(self.job.frames // self.batch):
                ins = [t[k * self.batch:(k + 1) * self.batch] for t in s["inputs"]]
                self.graph.add(self.sts[i], ins, self.canvases[i][k % 2], stream_index=i)
        self.captured = False

    def capture(self) -> None:
        import torch

        self.graph.capture(self.root)  # one eager run (first-call work), then the capture
        torch.cuda.synchronize(self.job.device)
        self.captured = True

    def time(self, reps: int = 3) -> float:
        """Seconds per job (graph replay, CUDA events on the root stream)."""
        import torch

        if not self.captured:
            self.capture()
        self.graph.launch(self.root)
        torch.cuda.synchronize(self.job.device)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(self.root)
        for _ in range(reps):
            self.graph.launch(self.root)
        e1.record(self.root)
        torch.cuda.synchronize(self.job.device)
        return e0.elapsed_time(e1) / 1e3 / reps

    def last_canvases(self) -> list:
        """Each stream's canvas of its last frame (after a run)."""
        last = self.job.frames // self.batch - 1
        return [c[last % 2][-1] for c in self.canvases]


def autotune(job: Job, batches=(1, 2, 4, 8, 16), tiles=(32, 64), residencies=(0, 4), reps: int = 3,
             use_cache: bool = True) -> dict:
    """Time every frames-per-call candidate with every pyramid down-tile edge per stream kind
    (two-image and three-image streams choose theirs separately; with 64-pixel tiles each also
    tries each cap on the down kernel's CTAs per SM); keep and cache the fastest."""
    key = job.signature()
    cache = {}
    if use_cache and CACHE.exists():
        try:
            cache = json.loads(CACHE.read_text())
        except Exception:
            cache = {}
    if use_cache and key in cache:
        return dict(cache[key], cached=True)
    kinds = sorted({s["kind"] for s in job.streams})

    def options(kind):
        out = []
        for tile in tiles:
            for res in (residencies if tile == 64 else (0,)):
                out.append((tile, res))
        return out

    combos = [dict(zip(kinds, c)) for c in itertools.product(*[options(k) for k in kinds])]
    trials = []
    t0 = time.perf_counter()
    for b in batches:
        plan = None
        for combo in combos:
            if plan is None:
                plan = Plan(job, b, combo)
            else:
                plan.set_tiles(combo)
            sec = plan.time(reps)
            trials.append({"batch": b, "tile_down": {str(k): list(v) for k, v in combo.items()},
                           "fps": round(len(job.streams) * job.frames / sec, 1)})
        del plan
    best = max(trials, key=lambda t: t["fps"])
    result = {"batch": best["batch"], "tile_down": best["tile_down"], "fps": best["fps"], "trials": trials,
              "tuning_s": round(time.perf_counter() - t0, 1)}
    if use_cache:
        try:
            CACHE.parent.mkdir(parents=True, exist_ok=True)
            cache[key] = result
            CACHE.write_text(json.dumps(cache, indent=1))
        except OSError:
            pass
    return dict(result, cached=False)


def plain_path(job: Job, keep_last: bool = False, storage: str | None = None):
    """Seconds for the job through the plain per-frame path: batch 1, no graph, one stream, the
    job's level storage unless `storage` is given (with keep_last, also each stream's last
    canvas)."""
    import torch

    sts, cvs, cts = [], [], []
    for s in job.streams:
        cls = pano.CudaStitchPano if s["kind"] == 2 else pano.CudaStitchPano3
        st = cls(1, job.levels, s["masks"], quiet=True, storage=storage or job.storage)
        sts.append(st)
        cts.append(torch.empty((1, s["rig"].canvas_h, s["rig"].canvas_w, 4), dtype=torch.uint8, device=job.device))
        cvs.append(pano._image(cts[-1]))
    stream = torch.cuda.Stream(job.device)
    sp = C.c_void_p(stream.cuda_stream)
    fn = _lib.lib().hmp_stitcher_process
    calls = []
    for f in range(job.frames):
        for i, s in enumerate(job.streams):
            ins = [t[f:f + 1] for t in s["inputs"]]
            calls.append((i, (_lib.Image * len(ins))(*[pano._image(t) for t in ins]), len(ins)))

    def go():
        for i, imgs, n in calls:
            r = fn(sts[i]._handle, imgs, n, C.byref(cvs[i]), sp)
            if r.code:
                raise RuntimeError(r.message.decode())

    go()
    torch.cuda.synchronize(job.device)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    go()
    e1.record(stream)
    torch.cuda.synchronize(job.device)
    sec = e0.elapsed_time(e1) / 1e3
    return (sec, [c[0] for c in cts]) if keep_last else sec


def run(device, use_cache: bool = False) -> dict:
    """Autotune, then the batched job and the plain per-frame path on the same frames."""
    job = Job(device)
    tune = autotune(job, use_cache=use_cache)
    t = tune["tile_down"]
    plan = Plan(job, tune["batch"], {int(k): v for k, v in t.items()} if isinstance(t, dict) else t)
    sec = plan.time(5)
    plain_sec = plain_path(job, storage="f32")
    plain16_sec = plain_path(job, storage="f16")
    frames = len(job.streams) * job.frames
    return {"workload": "4 x pano2_5120x2880_to_8500x3300 + 4 x pano3_2704x1520_to_6000x1800, 32 frames each, L=6",
            "storage": job.storage, "batch": tune["batch"], "tile_down": tune["tile_down"], "graph": True,
            "fps": round(frames / sec, 1), "mpix_s": round(job.mpix_total / sec, 1),
            "plain_storage": "f32",
            "plain_fps": round(frames / plain_sec, 1), "plain_mpix_s": round(job.mpix_total / plain_sec, 1),
            "speedup_vs_plain": round(plain_sec / sec, 3),
            "plain_f16_fps": round(frames / plain16_sec, 1), "speedup_vs_plain_f16": round(plain16_sec / sec, 3),
            "autotune": tune}
