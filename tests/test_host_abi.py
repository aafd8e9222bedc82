"""Host-side checks of libhmpano.so that need no GPU: exported symbols, planning geometry
against the oracle, and configuration errors (which are rejected before any device work)."""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from helpers import masks_for_case, masks_for_rig

REPO = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def lib():
    import sys

    sys.path.insert(0, str(REPO / "hm-cupano_gb300"))
    import build as hmp_build
    from hmpano import _lib

    hmp_build.build()
    return _lib.lib()


def _declared_symbols():
    text = (REPO / "include" / "hmpano.h").read_text()
    return sorted(set(re.findall(r"HMP_API\s+[\w\s\*]+?\b(hmp_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol(lib):
    names = _declared_symbols()
    assert len(names) >= 10
    from hmpano import _lib

    for name in names:
        assert hasattr(lib, name), name
        assert name in _lib.SIGNATURES, f"{name} has no ctypes signature"


def test_version(lib):
    assert b"sm_103a" in lib.hmp_version()


def test_plan_geometry_matches_oracle(golden, oracle_lib):
    import hmpano

    for name in [str(n) for n in golden["names"]]:
        c = oracle_lib.load_golden_case(golden, name)
        g = hmpano.plan_geometry(c["kind"], masks_for_case(c), c["levels"], c["minimize"])
        st = oracle_lib.Stitch(c["kind"], c["map_x"], c["map_y"], c["pos_x"], c["pos_y"], c["seam"], c["levels"],
                               c["batch"], c["minimize"])
        assert g["canvas"] == (st.canvas_w, st.canvas_h), name
        if c["levels"] > 0:
            og = st.geometry()
            assert g["blend"] == og["blend"] and g["write"] == og["write"] and g["levels"] == og["levels"], name


@pytest.mark.parametrize("workload,kind,levels", [
    ("pano2_1280x720_to_2200x800", 2, 0),
    ("pano2_1280x720_to_2200x800", 2, 6),
    ("panon8_2000x1500_to_9000x2400", 1, 6),
    ("panon8_2000x1500_to_9000x2400", 1, 3),
    ("pano3_2704x1520_to_6000x1800", 3, 6),
])
def test_plan_geometry_matches_oracle_on_workloads(oracle_lib, workload, kind, levels):
    import hmpano
    from hmpano import synth

    rig = synth.workload_rig(workload, scale=0.25, kind=kind)
    g = hmpano.plan_geometry(kind, masks_for_rig(rig), levels)
    st = oracle_lib.Stitch.from_rig(rig, levels)
    assert g["canvas"] == (st.canvas_w, st.canvas_h)
    if levels:
        og = st.geometry()
        assert (g["blend"], g["write"], g["levels"]) == (og["blend"], og["write"], og["levels"])


def _create(lib, masks, kind, levels, batch=1, **kw):
    from hmpano import _lib
    from hmpano.pano import build_config

    cfg, keep = build_config(kind, masks, levels, batch, **kw)
    h = C.c_void_p()
    s = lib.hmp_stitcher_create(C.byref(cfg), C.byref(h))
    st = lib.hmp_stitcher_status(h)
    code = s.code
    assert st.code == code  # the error is also the stitcher's sticky status
    lib.hmp_stitcher_destroy(h)
    return code, s.message.decode()


def _two_image_masks(x2=200):
    import hmpano

    w, h = 400, 16
    mx = np.tile(np.arange(w, dtype=np.uint16), (h, 1))
    my = np.tile(np.arange(h, dtype=np.uint16)[:, None], (1, w))
    m = hmpano.ControlMasks(mx, my, mx, my, np.ones((h, w + x2), np.uint8),
                            [hmpano.SpatialTiff(0, 0), hmpano.SpatialTiff(x2, 0)])
    return m


def test_create_rejects_invalid_configurations(lib):
    from hmpano import _lib

    # no overlap between the two footprints (CanvasManager::updateMinimizeBlend)
    code, msg = _create(lib, _two_image_masks(x2=400), _lib.KIND_PANO2, 0)
    assert code == 1 and "overlap" in msg
    # blend strip of +/-128 px does not fit the canvas (x2 - 128 < 0)
    code, msg = _create(lib, _two_image_masks(x2=100), _lib.KIND_PANO2, 3)
    assert code == 1 and "strip" in msg
    # wrong image count for the two-image stitcher
    import hmpano

    m3 = hmpano.ControlMasksN([np.zeros((4, 4), np.uint16)] * 3, [np.zeros((4, 4), np.uint16)] * 3,
                              np.zeros((4, 4), np.uint8), [hmpano.SpatialTiff(0, 0)] * 3)
    code, _ = _create(lib, m3, _lib.KIND_PANO2, 0)
    assert code == 1
    # empty seam: masks not loaded (the reference's cudaErrorFileNotFound)
    m = _two_image_masks()
    m.whole_seam_mask_image = np.zeros((0, 0), np.uint8)
    code, msg = _create(lib, m, _lib.KIND_PANO2, 0)
    assert code == 301 and "masks" in msg
    # seam larger than the canvas
    m = _two_image_masks()
    m.whole_seam_mask_image = np.ones((64, 2000), np.uint8)
    code, _ = _create(lib, m, _lib.KIND_PANO2, 0)
    assert code == 1
    # too many images
    m9 = hmpano.ControlMasksN([np.zeros((4, 4), np.uint16)] * 9, [np.zeros((4, 4), np.uint16)] * 9,
                              np.zeros((4, 4), np.uint8), [hmpano.SpatialTiff(0, 0)] * 9)
    code, msg = _create(lib, m9, _lib.KIND_PANON, 0)
    assert code == 1 and "2..8" in msg
    # more pyramid levels than one fused pass supports
    w, h = 2048, 1024
    mx = np.tile(np.arange(w, dtype=np.uint16), (h, 1))
    my = np.tile(np.arange(h, dtype=np.uint16)[:, None], (1, w))
    mN = hmpano.ControlMasksN([mx, mx], [my, my], np.zeros((h, w), np.uint8), [hmpano.SpatialTiff(0, 0)] * 2)
    code, msg = _create(lib, mN, _lib.KIND_PANON, 9, minimize_blend=False)
    assert code == 801 and "levels" in msg
    # a batch whose level bytes would overflow (rejected before any sizing)
    code, msg = _create(lib, _two_image_masks(), _lib.KIND_PANO2, 3, batch=1 << 30)
    assert code == 1 and "65536" in msg
    # a position that puts the canvas beyond 2^20 pixels per side (rejected before any sizing)
    m = _two_image_masks()
    m.positions = [hmpano.SpatialTiff(0, 0), hmpano.SpatialTiff(float(1 << 21), 0)]
    code, msg = _create(lib, m, _lib.KIND_PANO2, 0)
    assert code == 801 and "2^20" in msg


def test_python_mirror_keeps_invalid_masks_as_status():
    import hmpano

    pano = hmpano.CudaStitchPano(1, 0, hmpano.ControlMasks(), quiet=True)
    assert not pano.status.ok() and pano.status.code == 301
    with pytest.raises(hmpano.CudaStatusError):
        pano.process(None, None)
    panoN = hmpano.CudaStitchPanoN(1, 0, hmpano.ControlMasksN(), quiet=True)
    assert not panoN.status.ok()


def test_python_mirror_takes_the_reference_constructor_arguments():
    """cupano's CudaStitchPano(batch, levels, masks, quiet, minimize_blend, max_output_width,
    backend, enable_cuda_graphs) and CudaStitchPanoN(batch, levels, masks, quiet, minimize_blend,
    backend, enable_cuda_graphs) (cupano/pano.py:127-138, 553-563), positionally and by name."""
    import hmpano

    p = hmpano.CudaStitchPano(1, 0, hmpano.ControlMasks(), True, True, 0, "triton", False)
    assert p.status.code == 301  # the masks' status, not a TypeError
    p = hmpano.CudaStitchPano(1, 0, hmpano.ControlMasks(), quiet=True, backend="auto", enable_cuda_graphs=True)
    assert p.status.code == 301
    n = hmpano.CudaStitchPanoN(1, 0, hmpano.ControlMasksN(), True, True, "auto", False)
    assert not n.status.ok()
    with pytest.raises(ValueError, match="Unsupported backend"):
        hmpano.pano._check_backend("torch")


def test_python_mirror_exports_the_reference_names():
    """Every name cupano exports (cupano/__init__.py) is importable from the mirror."""
    import hmpano

    for name in ("CanvasInfo", "ControlMasks", "ControlMasksN", "CudaStatus", "CudaStatusError", "CudaStitchPano",
                 "CudaStitchPanoN", "Rect", "SpatialTiff", "UNMAPPED_POSITION_VALUE"):
        assert hasattr(hmpano, name), name
    r = hmpano.Rect(2, 3, 10, 4).intersect(hmpano.Rect(8, 0, 10, 5))
    assert (r.x, r.y, r.width, r.height, r.right, r.bottom, r.empty) == (8, 3, 4, 2, 12, 5, False)
    assert hmpano.Rect(0, 0, 5, 5).intersect(hmpano.Rect(6, 0, 5, 5)).empty


def test_c_abi_rejects_bad_arguments_before_any_device_work(lib):
    """Argument errors come back as statuses with the reference's cudaError_t values, without a
    GPU: null handles, server options, batch-job rules (stitcher handles are only compared, never
    used, by hmp_batch_add)."""
    from hmpano import _lib

    info = _lib.StitcherInfo()
    assert lib.hmp_stitcher_get_info(None, C.byref(info)).code == 1
    assert lib.hmp_stitcher_process(None, None, 0, None, None).code == 1
    assert lib.hmp_stitcher_set_tiles(None, 64, 32).code == 1
    for mode in (0, 1, 2):
        assert lib.hmp_stitcher_set_copy_blocks(None, mode).code == 1
    assert lib.hmp_stitcher_set_down_residency(None, 4).code == 1
    assert lib.hmp_stitcher_status(None).code == 1
    assert lib.hmp_stitcher_canvas_width(None) == 0
    lib.hmp_stitcher_destroy(None)  # no-op

    srv = C.c_void_p()
    for budget, slots in ((0, 4), (1 << 30, 0), (1 << 30, 65)):
        opt = _lib.ServerOptions(budget, slots, 2)
        assert lib.hmp_server_create(C.byref(opt), C.byref(srv)).code == 1 and not srv

    b = C.c_void_p()
    assert lib.hmp_batch_create(C.byref(b)).code == 0 and b
    try:
        img = (_lib.Image * 2)()
        canvas = _lib.Image()
        st1, st2 = C.c_void_p(0x1000), C.c_void_p(0x2000)
        assert lib.hmp_batch_add(b, st1, img, 2, C.byref(canvas), 0).code == 0
        assert lib.hmp_batch_add(b, st1, img, 2, C.byref(canvas), 0).code == 0  # in order, same index
        s = lib.hmp_batch_add(b, st1, img, 2, C.byref(canvas), 1)  # one stitcher, two stream indices
        assert s.code == 1 and b"one stream index" in s.message
        assert lib.hmp_batch_add(b, st2, img, 2, C.byref(canvas), 1).code == 0
        assert lib.hmp_batch_add(b, st2, img, 2, C.byref(canvas), 256).code == 1
        assert lib.hmp_batch_add(b, st2, img, 0, C.byref(canvas), 1).code == 1
        assert lib.hmp_batch_add(b, None, img, 2, C.byref(canvas), 1).code == 1
    finally:
        lib.hmp_batch_destroy(b)  # nothing was captured: no CUDA objects to release
    assert lib.hmp_batch_capture(None, None).code == 1 and lib.hmp_batch_launch(None, None).code == 1

    d = C.POINTER(_lib.ControlDir)()
    assert lib.hmp_control_dir_load(b"/nonexistent", 99, 2, C.byref(d)).code == 1 and not d

    # The allocation-failure hook is host state only: set, read back through the counter, cleared.
    n = lib.hmp_debug_allocation_count()
    assert n >= 0
    lib.hmp_debug_fail_allocation(3)
    lib.hmp_debug_fail_allocation(0)
    assert lib.hmp_debug_allocation_count() == n


def test_noalloc_blend_rejects_bad_arguments_before_any_device_work(lib):
    """hmp_blend2_noalloc checks every argument before its first CUDA call, so fake non-null
    pointers are never dereferenced: each rejection is HMP_ERR_INVALID_VALUE with its message."""
    from hmpano import _lib

    def img(w, h, pitch=None, ptr=0x10000):
        return _lib.Image(C.c_void_p(ptr), w, h, pitch if pitch is not None else 4 * w)

    seam = C.c_void_p(0x20000)

    def call(a, b, o, seam_ptr=seam, seam_pitch=64, levels=3, batch=1):
        return lib.hmp_blend2_noalloc(C.byref(a) if a is not None else None, C.byref(b) if b is not None else None,
                                      seam_ptr, seam_pitch, levels, batch, C.byref(o) if o is not None else None, None)

    good = img(64, 32)
    cases = [
        (dict(a=None, b=good, o=good), b"non-null RGBA8"),
        (dict(a=img(64, 32, ptr=0), b=good, o=good), b"non-null RGBA8"),
        (dict(a=img(64, 32, pitch=4 * 64 - 4), b=good, o=good), b"non-null RGBA8"),  # pitch below a row
        (dict(a=img(64, 32, pitch=4 * 64 + 2), b=good, o=good), b"non-null RGBA8"),  # pitch not a multiple of 4
        (dict(a=img(64, 32, ptr=0x10002), b=good, o=good), b"non-null RGBA8"),  # data not 4-byte aligned
        (dict(a=good, b=img(0, 32), o=good), b"non-null RGBA8"),
        (dict(a=good, b=good, o=None), b"non-null RGBA8"),
        (dict(a=img(65, 32), b=good, o=good), b"same size"),
        (dict(a=good, b=img(64, 31), o=good), b"same size"),
        (dict(a=img(70000, 2), b=img(70000, 2), o=img(70000, 2)), b"smaller than 65535"),
        (dict(a=good, b=good, o=good, seam_ptr=None), b"seam"),
        (dict(a=good, b=good, o=good, seam_pitch=63), b"seam"),
        (dict(a=good, b=good, o=good, seam_pitch=1 << 40), b"seam"),
        (dict(a=good, b=good, o=good, levels=0), b"num_levels"),
        (dict(a=good, b=good, o=good, levels=31), b"num_levels"),
        (dict(a=good, b=good, o=good, batch=0), b"batch_size"),
        (dict(a=good, b=good, o=good, batch=65537), b"batch_size"),
    ]
    for kw, msg in cases:
        s = call(**kw)
        assert s.code == 1 and msg in s.message, (kw, s.code, s.message)


def _sanitized_build(tmp_path, name, sources, compiler):
    import shutil
    import subprocess

    if shutil.which(compiler) is None:
        pytest.skip(f"no {compiler}")
    exe = tmp_path / name
    std = "-std=c++17" if compiler == "g++" else "-std=c11"
    r = subprocess.run([compiler, std, "-O1", "-g", "-fsanitize=address,undefined", "-fno-sanitize-recover=undefined",
                        "-I", str(REPO / "include"), "-I", str(REPO / "hm-cupano_gb300" / "csrc"),
                        "-I", str(REPO / "oracle"), *[str(s) for s in sources], "-lm", "-o", str(exe)],
                       capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip(f"no sanitizer runtime: {r.stderr.strip()[:200]}")
    return exe


def test_planner_under_sanitizers(tmp_path):
    """tests/cpp/plan_fuzz.cpp: thousands of random configurations through the planner built with
    AddressSanitizer and UndefinedBehaviorSanitizer; each is planned or rejected, none misbehaves."""
    import subprocess

    exe = _sanitized_build(tmp_path, "plan_fuzz", [REPO / "tests" / "cpp" / "plan_fuzz.cpp",
                                                   REPO / "hm-cupano_gb300" / "csrc" / "hmp_plan.cpp"], "g++")
    out = subprocess.run([str(exe), "3000", "5"], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    planned, rejected = (int(v) for v in out.stdout.split()[1::2])
    assert planned > 0 and rejected > 0


def test_oracle_under_sanitizers(tmp_path):
    """tests/cpp/oracle_fuzz.c: random stitches through the oracle (the parity checker) built with
    AddressSanitizer and UndefinedBehaviorSanitizer; each runs or is rejected, none misbehaves."""
    import subprocess

    exe = _sanitized_build(tmp_path, "oracle_fuzz", [REPO / "tests" / "cpp" / "oracle_fuzz.c",
                                                     REPO / "oracle" / "hmp_oracle.c"], "gcc")
    out = subprocess.run([str(exe), "1500", "3"], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    ran, rejected = (int(v) for v in out.stdout.split()[1::2])
    assert ran > 0 and rejected > 0


def test_plan_geometry_matches_oracle_on_random_configurations(oracle_lib):
    """The product's planner and the oracle agree on every random configuration: both reject it,
    or both give the same canvas, blend region, write region and effective level count."""
    import hmpano
    from helpers import masks_for

    rng = np.random.default_rng(2026)
    agreed = rejected = 0
    for _ in range(300):
        kind = int(rng.choice([1, 2, 3]))
        n = {2: 2, 3: 3}.get(kind, int(rng.integers(2, 9)))
        mx, my, px, py = [], [], [], []
        for _i in range(n):
            w, h = int(rng.integers(8, 400)), int(rng.integers(8, 120))
            mx.append(np.tile(np.arange(w, dtype=np.uint16), (h, 1)))
            my.append(np.tile(np.arange(h, dtype=np.uint16)[:, None], (1, w)))
            px.append(int(rng.integers(0, 300)))
            py.append(int(rng.integers(0, 40)))
        cw = max(x + m.shape[1] for x, m in zip(px, mx))
        ch = max(y + m.shape[0] for y, m in zip(py, mx))
        labels = 2 if kind == 2 else n
        seam = rng.integers(0, labels, (ch, cw)).astype(np.uint8)
        if rng.random() < 0.5:  # a few large regions instead of noise
            cuts = np.sort(rng.integers(0, cw, labels - 1))
            seam = np.searchsorted(cuts, np.arange(cw), side="right").astype(np.uint8)[None, :].repeat(ch, 0)
        levels = int(rng.integers(0, 8))
        minimize = bool(rng.integers(0, 2))
        try:
            g = hmpano.plan_geometry(kind, masks_for(kind, mx, my, px, py, seam), levels, minimize)
        except hmpano.CudaStatusError:
            g = None
        try:  # the oracle checks a configuration when it plans the stitch (at every level count)
            st = oracle_lib.Stitch(kind, mx, my, px, py, seam, levels, 1, minimize)
            og = st.geometry()
            canvas = (st.canvas_w, st.canvas_h)
        except ValueError:
            st = None
        if g is None or st is None:
            assert g is None and st is None, (kind, n, levels, minimize)
            rejected += 1
            continue
        assert g["canvas"] == canvas
        if levels:
            assert (g["blend"], g["write"], g["levels"]) == (og["blend"], og["write"], og["levels"]), \
                (kind, n, levels, minimize)
        agreed += 1
    assert agreed > 200


def test_c_abi_header_is_plain_c(tmp_path):
    """include/hmpano.h compiles as strict C99 and C++11 with every warning an error: any FFI that
    reads C headers (cgo, JNI, N-API, ctypes generators) can take it as is."""
    import shutil
    import subprocess

    src_c = tmp_path / "abi.c"
    src_c.write_text('#include "hmpano.h"\nint main(void) { hmp_config c = {0}; hmp_image i = {0}; (void)c; (void)i; '
                     'return hmp_version() == 0; }\n')
    src_cpp = tmp_path / "abi.cpp"
    src_cpp.write_text('#include "hmpano.h"\nint main() { hmp_config c{}; (void)c; return hmp_version() == nullptr; }\n')
    for cc, std, src in (("gcc", "-std=c99", src_c), ("g++", "-std=c++11", src_cpp)):
        if shutil.which(cc) is None:
            pytest.skip(f"no {cc}")
        r = subprocess.run([cc, std, "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", str(REPO / "include"),
                            "-fsyntax-only", str(src)], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


def test_copy_block_modes_from_the_python_mirror(monkeypatch):
    """set_copy_blocks(enable, opaque_frames) passes the C ABI's mode: 0 off, 1 on (checked),
    2 on for frames promised opaque; opaque_frames without enable stays off. A recording stand-in
    for the library takes the call, so no stitcher (and no GPU) is needed."""
    from hmpano import _lib, pano

    calls = []

    class FakeLib:
        def hmp_stitcher_set_copy_blocks(self, handle, mode):
            calls.append(mode)
            return _lib.Status(0, b"")

        def hmp_stitcher_destroy(self, handle):
            pass

    monkeypatch.setattr(_lib, "lib", lambda: FakeLib())
    st = object.__new__(pano._Stitcher)
    st._handle = C.c_void_p(1)  # never dereferenced: only the stand-in sees it
    try:
        for enable, opaque in ((False, False), (True, False), (True, True), (False, True)):
            st.set_copy_blocks(enable, opaque_frames=opaque)
        st.set_copy_blocks(True)
    finally:
        st._handle = C.c_void_p()  # so that no later destructor hands it to the real library
    assert calls == [0, 1, 2, 0, 1]
