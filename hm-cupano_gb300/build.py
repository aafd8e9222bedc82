"""Build libhmpano.so (sm_103a) in-tree: hm-cupano_gb300/lib/libhmpano.so.

Each translation unit is compiled by nvcc in parallel, then linked into one shared library with
the CUDA runtime linked statically. The pyramid kernels are compiled with -fmad=false: the
reference rounds every product and sum separately, and fusing them would move results by an ulp
(and flip truncating uint8 packs).

    python hm-cupano_gb300/build.py [--force]
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
REPO = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "lib" / "libhmpano.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
          "-I", str(REPO / "include"), "-I", str(CSRC)]
UNITS = {
    "hmp_plan.cpp": ["-Xcompiler", "-ffp-contract=off"],
    "hmp_copyplan.cpp": [],
    "hmp_gather.cu": [],
    "hmp_pyramid.cu": ["-fmad=false"],
    "hmp_stitcher.cu": [],
    "hmp_noalloc.cu": ["-fmad=false"],
    "hmp_binomial.cu": ["-fmad=false"],
    "hmp_server.cpp": [],
    "hmp_control_dir.cpp": [],
    "hmp_generic.cu": ["-fmad=false"],
    "hmp_batch.cpp": [],
    "hmp_stabilize.cu": ["-fmad=false"],
    # Device-side (tail) launches need relocatable device code; only this unit has it, since it
    # raises the pyramid kernels' registers (it holds its own copies of them for the fallback).
    "hmp_fallback.cu": ["-fmad=false", "-rdc=true"],
}
RDC_UNITS = [u for u, extra in UNITS.items() if "-rdc=true" in extra]
HEADERS = ["hmp_plan.h", "hmp_copyplan.h", "hmp_device.cuh", "hmp_kernels.h", "hmp_blend.cuh", "hmp_admission.h",
           "hmp_pyramid_kernels.cuh"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _stale(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return True
    deps = [src, REPO / "include" / "hmpano.h"] + [CSRC / h for h in HEADERS]
    return any(d.stat().st_mtime > obj.stat().st_mtime for d in deps if d.exists())


def build(force: bool = False, verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    LIB.parent.mkdir(exist_ok=True)
    cc = nvcc()
    jobs = []
    for unit, extra in UNITS.items():
        src = CSRC / unit
        obj = BUILD / (unit + ".o")
        if force or _stale(obj, src):
            cmd = [cc, *ARCH, *COMMON, *extra, "-c", str(src), "-o", str(obj)]
            if unit.endswith(".cu") and os.environ.get("HMP_PTXAS_VERBOSE"):
                cmd += ["-Xptxas", "-v"]
            jobs.append((unit, cmd))

    def run(job):
        unit, cmd = job
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        return unit, r

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        results = list(ex.map(run, jobs))
    failed = [(u, r) for u, r in results if r.returncode != 0]
    for u, r in results:
        if r.stderr.strip() and (verbose or r.returncode != 0 or os.environ.get("HMP_PTXAS_VERBOSE")):
            print(f"--- {u}\n{r.stderr}", file=sys.stderr)
    if failed:
        raise RuntimeError(f"nvcc failed for {[u for u, _ in failed]}")
    objs = [str(BUILD / (u + ".o")) for u in UNITS]
    if jobs or force or not LIB.exists():
        # Device link of the relocatable units (with the device runtime), then the shared library.
        dlink = str(BUILD / "device_link.o")
        cmd = [cc, *ARCH, "-Xcompiler", "-fPIC", "-dlink", "-o", dlink,
               *[str(BUILD / (u + ".o")) for u in RDC_UNITS], "-lcudadevrt"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            print(r.stderr, file=sys.stderr)
            raise RuntimeError("device link failed")
        tmp = str(LIB) + ".tmp"
        cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, dlink, "-lcudadevrt"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            print(r.stderr, file=sys.stderr)
            raise RuntimeError("link failed")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-v", "--verbose", action="store_true")
    args = ap.parse_args()
    print(build(force=args.force, verbose=args.verbose))
