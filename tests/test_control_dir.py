"""Control-directory loader (hmp_control_dir_load; the reference's ControlMasks*::load): its TIFF
and PNG decoders against files written independently from the format specifications
(tests/control_files.py), the seam and position rules of the reference loaders, and a synthetic
rig's control directory round trip. Host code only: no GPU.
"""
from __future__ import annotations

import struct
from pathlib import Path

import numpy as np
import pytest

import control_files as cf


@pytest.fixture(scope="module")
def hp():
    import hmpano

    hmpano.pano._lib.lib()  # fails loudly if libhmpano.so is missing
    return hmpano


# ---- PNG ----

def test_png_paletted_indices_every_filter(hp, tmp_path):
    rng = np.random.default_rng(1)
    idx = rng.integers(0, 9, (37, 53)).astype(np.uint8)
    idx[5:12, 3:40] = 4  # runs for the back-references of the deflate stream
    pal = rng.integers(0, 256, (9, 3))
    cf.write_png(tmp_path / "p.png", idx, color_type=3, palette=pal)
    out, paletted = hp.read_seam_png(tmp_path / "p.png")
    assert paletted
    np.testing.assert_array_equal(out, idx)


@pytest.mark.parametrize("depth", [1, 2, 4, 8, 16])
def test_png_grayscale_depths(hp, tmp_path, depth):
    rng = np.random.default_rng(depth)
    g = rng.integers(0, 1 << depth, (19, 29))
    cf.write_png(tmp_path / "g.png", g, color_type=0, bit_depth=depth)
    out, paletted = hp.read_seam_png(tmp_path / "g.png")
    assert not paletted
    if depth == 16:
        expect = g >> 8
    else:
        expect = g * 255 // ((1 << depth) - 1)
    np.testing.assert_array_equal(out, expect.astype(np.uint8))


def test_png_colour_to_grey_and_low_depth_palette(hp, tmp_path):
    rng = np.random.default_rng(3)
    rgb = rng.integers(0, 256, (11, 17, 3))
    cf.write_png(tmp_path / "c.png", rgb, color_type=2)
    out, paletted = hp.read_seam_png(tmp_path / "c.png")
    expect = (rgb[..., 0] * 4899 + rgb[..., 1] * 9617 + rgb[..., 2] * 1868 + 8192) >> 14
    assert not paletted
    np.testing.assert_array_equal(out, expect.astype(np.uint8))
    # A 4-bit paletted seam is not read as indices (the reference's index reader wants 8 bits):
    # it falls back to the grey of the palette colours.
    idx = rng.integers(0, 16, (9, 13))
    pal = rng.integers(0, 256, (16, 3))
    cf.write_png(tmp_path / "p4.png", idx, color_type=3, bit_depth=4, palette=pal)
    out, paletted = hp.read_seam_png(tmp_path / "p4.png")
    pc = pal[idx]
    assert not paletted
    np.testing.assert_array_equal(out, ((pc[..., 0] * 4899 + pc[..., 1] * 9617 + pc[..., 2] * 1868 + 8192) >> 14))


def _py_png_gray8(path: Path):
    """An independent decoder for 8-bit greyscale / paletted PNGs (zlib + the row filters)."""
    import struct
    import zlib

    b = path.read_bytes()
    pos, idat, hdr = 8, b"", None
    while pos < len(b):
        n = struct.unpack(">I", b[pos:pos + 4])[0]
        kind, data = b[pos + 4:pos + 8], b[pos + 8:pos + 8 + n]
        if kind == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", data)
        elif kind == b"IDAT":
            idat += data
        pos += 12 + n
    w, h, depth, color, _, _, inter = hdr
    if depth != 8 or color not in (0, 3) or inter:
        return None
    raw = zlib.decompress(idat)
    out = np.zeros((h, w), np.int64)
    prev = np.zeros(w, np.int64)
    for y in range(h):
        f, row = raw[y * (w + 1)], np.frombuffer(raw, np.uint8, w, y * (w + 1) + 1).astype(np.int64)
        cur = np.zeros(w, np.int64)
        for x in range(w):
            a = cur[x - 1] if x else 0
            c = prev[x - 1] if x else 0
            p = a + prev[x] - c
            pr = (0, a, prev[x], (a + prev[x]) >> 1,
                  a if abs(p - a) <= abs(p - prev[x]) and abs(p - a) <= abs(p - c) else
                  (prev[x] if abs(p - prev[x]) <= abs(p - c) else c))[f]
            cur[x] = (row[x] + pr) & 0xFF
        out[y], prev = cur, cur
    return out.astype(np.uint8)


def test_png_system_files_match_an_independent_decoder(hp):
    found = 0
    for p in sorted(Path("/usr/share").rglob("*.png"))[:200]:
        if p.stat().st_size > 200_000:
            continue
        ref = _py_png_gray8(p)
        if ref is None:
            continue
        out, _ = hp.read_seam_png(p)
        np.testing.assert_array_equal(out, ref, err_msg=str(p))
        found += 1
        if found >= 5:
            break
    if not found:
        pytest.skip("no 8-bit greyscale or paletted PNG on this machine")


# ---- TIFF ----

@pytest.mark.parametrize("compression", [1, 5, 8, 32773])
@pytest.mark.parametrize("predictor", [1, 2])
@pytest.mark.parametrize("big_endian", [False, True])
@pytest.mark.parametrize("layout", ["strips", "tiles"])
def test_tiff_u16(hp, tmp_path, compression, predictor, big_endian, layout):
    rng = np.random.default_rng(compression + 7 * predictor)
    img = (np.add.outer(np.arange(45) * 31, np.arange(70) * 7) + rng.integers(0, 3, (45, 70))).astype(np.uint16)
    img[10:20, :] = 65535  # unmapped rows (runs)
    kw = {"tile": 16} if layout == "tiles" else {"rows_per_strip": 7}
    cf.write_tiff(tmp_path / "m.tif", img, big_endian=big_endian, compression=compression, predictor=predictor, **kw)
    np.testing.assert_array_equal(hp.read_tiff_u16(tmp_path / "m.tif"), img)


def test_tiff_lzw_long_stream_with_clear_codes(hp, tmp_path):
    rng = np.random.default_rng(9)
    img = rng.integers(0, 65535, (200, 300)).astype(np.uint16)  # incompressible: the table fills and clears
    cf.write_tiff(tmp_path / "m.tif", img, compression=5, rows_per_strip=200)
    np.testing.assert_array_equal(hp.read_tiff_u16(tmp_path / "m.tif"), img)


def test_tiff_rejects_float_tables(hp, tmp_path):
    p = tmp_path / "f.tif"
    cf.write_tiff(p, np.zeros((4, 4), np.uint16))
    b = bytearray(p.read_bytes())
    # SampleFormat 1 -> 3 (IEEE float): tag 339 is stored inline
    at = bytes(b).index((339).to_bytes(2, "little") + (3).to_bytes(2, "little"))
    b[at + 8] = 3
    p.write_bytes(bytes(b))
    with pytest.raises(hp.CudaStatusError, match="16-bit unsigned"):
        hp.read_tiff_u16(p)


# ---- malformed and oversized files: errors or bounded work, never a crash ----

def _patch_tiff_tag(path: Path, tag: int, ttype: int, new_tag: int | None = None, new_value: int | None = None):
    b = bytearray(path.read_bytes())
    at = bytes(b).index(tag.to_bytes(2, "little") + ttype.to_bytes(2, "little"))
    if new_tag is not None:
        b[at:at + 2] = new_tag.to_bytes(2, "little")
    if new_value is not None:
        b[at + 8:at + 12] = new_value.to_bytes(4, "little")
    path.write_bytes(bytes(b))


def test_tiff_missing_width_is_an_error(hp, tmp_path):
    p = tmp_path / "m.tif"
    cf.write_tiff(p, np.zeros((4, 4), np.uint16))
    _patch_tiff_tag(p, 256, 4, new_tag=0x8123)  # ImageWidth renamed to an unknown private tag
    with pytest.raises(hp.CudaStatusError, match="256"):
        hp.read_tiff_u16(p)


def test_tiff_and_png_reject_huge_headers(hp, tmp_path):
    p = tmp_path / "m.tif"
    cf.write_tiff(p, np.zeros((4, 4), np.uint16))
    _patch_tiff_tag(p, 256, 4, new_value=1 << 30)
    with pytest.raises(hp.CudaStatusError, match="larger than") as e:
        hp.read_tiff_u16(p)
    assert e.value.status.code == 801
    q = tmp_path / "s.png"
    cf.write_png(q, np.zeros((4, 4), np.uint8), color_type=0)
    b = bytearray(q.read_bytes())
    b[16:24] = (0x7FFF0000).to_bytes(4, "big") + (0x7FFF0000).to_bytes(4, "big")  # IHDR width, height
    q.write_bytes(bytes(b))
    with pytest.raises(hp.CudaStatusError, match="larger than"):
        hp.read_seam_png(q)


@pytest.mark.parametrize("compression", [5, 8])
def test_tiff_strip_that_decodes_past_the_image_is_cut(hp, tmp_path, compression):
    """A strip whose stream holds far more than the image: the decoder stops at the strip's size
    (a 100 MB stream of zeros after the pixels costs nothing)."""
    import zlib

    img = np.arange(48, dtype=np.uint16).reshape(6, 8) * 997
    p = tmp_path / "m.tif"
    cf.write_tiff(p, img, compression=compression)
    raw = img.astype("<u2").tobytes() + bytes(100 << 20 if compression == 8 else 1 << 16)
    stream = zlib.compress(raw, 9) if compression == 8 else cf.lzw_encode(raw)
    b = p.read_bytes()
    old = zlib.compress(img.astype("<u2").tobytes()) if compression == 8 else cf.lzw_encode(img.astype("<u2").tobytes())
    assert b.endswith(old)
    p.write_bytes(b[: len(b) - len(old)] + stream)
    _patch_tiff_tag(p, 279, 4, new_value=len(stream))  # StripByteCounts
    np.testing.assert_array_equal(hp.read_tiff_u16(p), img)


def test_png_idat_that_decodes_past_the_image_is_cut(hp, tmp_path):
    import zlib

    rows = b"".join(b"\x00" + bytes([y * 10 + x for x in range(5)]) for y in range(3))
    ihdr = struct.pack(">IIBBBBB", 5, 3, 8, 0, 0, 0, 0)
    idat = zlib.compress(rows + bytes(100 << 20), 9)
    data = cf._png_chunk(b"IHDR", ihdr) + cf._png_chunk(b"IDAT", idat) + cf._png_chunk(b"IEND", b"")
    q = tmp_path / "s.png"
    q.write_bytes(b"\x89PNG\r\n\x1a\n" + data)
    out, _ = hp.read_seam_png(q)
    np.testing.assert_array_equal(out, np.array([[y * 10 + x for x in range(5)] for y in range(3)], np.uint8))


def test_loader_reports_a_bad_table_without_crashing(hp, tmp_path):
    rng = np.random.default_rng(5)
    mx, my = _rig_tables(rng, 2)
    seam = np.zeros((24, 60), np.uint8)
    seam[:, 30:] = 255
    cf.write_control_dir(tmp_path, mx, my, [(0, 0), (20, 0)], seam, paletted=False)
    _patch_tiff_tag(tmp_path / "mapping_0001_y.tif", 257, 4, new_tag=0x8124)  # ImageLength missing
    with pytest.raises(hp.CudaStatusError, match="257"):
        hp.load_control_dir(tmp_path, hp.pano._lib.KIND_PANO2)
    assert not hp.ControlMasks().load(tmp_path)


# ---- the loader's rules ----

def _rig_tables(rng, n, h=24, w=40):
    maps_x = [rng.integers(0, 600, (h, w)).astype(np.uint16) for _ in range(n)]
    maps_y = [rng.integers(0, 400, (h, w)).astype(np.uint16) for _ in range(n)]
    for m in maps_x:
        m[:2, :] = 65535
    return maps_x, maps_y


def test_two_image_directory(hp, tmp_path):
    rng = np.random.default_rng(5)
    mx, my = _rig_tables(rng, 2)
    pos = [(1300, 17), (1325, 5)]
    seam_file = np.where(rng.random((24, 65)) < 0.5, 0, 255).astype(np.uint8)
    cf.write_control_dir(tmp_path, mx, my, pos, seam_file, paletted=False, compression=5, predictor=2)
    m = hp.ControlMasks()
    assert m.load(tmp_path)
    np.testing.assert_array_equal(m.img1_col, mx[0])
    np.testing.assert_array_equal(m.img2_row, my[1])
    assert [(p.xpos, p.ypos) for p in m.positions] == [(0.0, 12.0), (25.0, 0.0)]
    # inverted: the smallest value is image 1 (1), the largest 0
    np.testing.assert_array_equal(m.whole_seam_mask_image, (seam_file == 0).astype(np.uint8))
    assert m.canvas_width() == 65 and m.canvas_height() == 36
    # the reference's constructor form, with a str or a path
    for arg in (str(tmp_path), tmp_path):
        m2 = hp.ControlMasks(arg)
        assert m2.is_valid()
        np.testing.assert_array_equal(m2.img1_col, mx[0])
        np.testing.assert_array_equal(m2.whole_seam_mask_image, m.whole_seam_mask_image)
    assert not hp.ControlMasks(str(tmp_path / "missing")).is_valid()


def test_n_image_labels_remapped_and_counted(hp, tmp_path):
    rng = np.random.default_rng(6)
    mx, my = _rig_tables(rng, 3)
    labels = rng.integers(0, 3, (24, 60))
    seam_file = np.array([10, 20, 30], np.uint8)[labels]
    cf.write_control_dir(tmp_path, mx, my, [(0, 0), (10, 0), (20, 0)], seam_file, paletted=True, compression=8)
    m = hp.ControlMasksN()
    assert m.load(tmp_path, 3)
    np.testing.assert_array_equal(m.whole_seam_mask_indexed, labels)
    assert not hp.ControlMasksN().load(tmp_path, 4)  # three classes for four images
    m2 = hp.ControlMasksN(str(tmp_path), 3)  # the reference's constructor form
    assert m2.is_valid()
    np.testing.assert_array_equal(m2.whole_seam_mask_indexed, labels)
    assert not hp.ControlMasksN(str(tmp_path)).is_valid()  # without n_images nothing is loaded


def test_three_image_seam_rules(hp, tmp_path):
    rng = np.random.default_rng(7)
    mx, my = _rig_tables(rng, 3)
    labels = rng.integers(0, 3, (24, 60)).astype(np.uint8)
    cf.write_control_dir(tmp_path / "ok", mx, my, [(0, 0), (10, 0), (20, 0)], labels, paletted=True)
    m = hp.ControlMasks3()
    assert m.load(tmp_path / "ok")
    np.testing.assert_array_equal(m.whole_seam_mask_image, labels)
    assert hp.ControlMasks3(tmp_path / "ok").is_valid()
    cf.write_control_dir(tmp_path / "grey", mx, my, [(0, 0), (10, 0), (20, 0)], labels, paletted=False)
    assert not hp.ControlMasks3().load(tmp_path / "grey")  # the three-image seam must be paletted


def test_missing_files(hp, tmp_path):
    assert not hp.ControlMasks().load(tmp_path)
    with pytest.raises(hp.CudaStatusError) as e:
        hp.load_control_dir(tmp_path, hp.pano._lib.KIND_PANO2)
    assert e.value.status.code == 301  # HMP_ERR_FILE_NOT_FOUND


def test_synthetic_rig_round_trip_plans_identically(hp, tmp_path):
    from hmpano import synth

    from helpers import masks_for_rig

    rig = synth.workload_rig("pano2_1280x720_to_2200x800", seed=31, kind=2, scale=0.25)
    seam_file = np.where(rig.seam == 1, 0, 255).astype(np.uint8)
    cf.write_control_dir(tmp_path, rig.map_x, rig.map_y, list(zip(rig.pos_x, rig.pos_y)), seam_file, paletted=False,
                         compression=5, predictor=2, rows_per_strip=16)
    loaded = hp.ControlMasks.from_directory(tmp_path)
    assert loaded.is_valid()
    direct = masks_for_rig(rig)
    for a in ("img1_col", "img1_row", "img2_col", "img2_row", "whole_seam_mask_image"):
        np.testing.assert_array_equal(getattr(loaded, a), getattr(direct, a), err_msg=a)
    assert hp.plan_geometry(2, loaded, 6) == hp.plan_geometry(2, direct, 6)


def test_cpp_drop_in_loads_the_same_directory(hp, tmp_path):
    """ControlMasks(dir) of the C++ drop-in header reads what the Python mirror reads."""
    import shutil
    import subprocess

    if shutil.which("g++") is None:
        pytest.skip("no g++")
    repo = Path(__file__).resolve().parents[1]
    lib = repo / "hm-cupano_gb300" / "lib"
    exe = tmp_path / "control_dir_main"
    cuda_inc = Path("/usr/local/cuda/include")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", str(repo / "include"), "-I", str(cuda_inc),
                    str(repo / "tests" / "cpp" / "control_dir_main.cpp"), "-L", str(lib), "-lhmpano",
                    f"-Wl,-rpath,{lib}", "-o", str(exe)], check=True)
    rng = np.random.default_rng(11)
    mx, my = _rig_tables(rng, 2)
    seam_file = np.where(rng.random((24, 65)) < 0.5, 3, 200).astype(np.uint8)
    cf.write_control_dir(tmp_path / "d", mx, my, [(40, 9), (65, 2)], seam_file, paletted=True, compression=32773)
    out = subprocess.run([str(exe), str(tmp_path / "d")], capture_output=True, text=True, check=True).stdout.split()
    m = hp.ControlMasks.from_directory(tmp_path / "d")

    def h(a):
        v = 0
        for x in np.asarray(a).reshape(-1).tolist():
            v = (v * 31 + x) % (1 << 64)
        return v

    expect = [m.img1_col.shape[1], m.img1_col.shape[0], m.whole_seam_mask_image.shape[1],
              m.whole_seam_mask_image.shape[0], m.positions[0].xpos, m.positions[0].ypos, m.positions[1].xpos,
              m.positions[1].ypos, h(m.img1_col), h(m.img2_row), h(m.whole_seam_mask_image)]
    assert [float(x) for x in out] == [float(x) for x in expect]


def test_decoders_survive_mutated_files_under_sanitizers(tmp_path):
    """tests/cpp/decoder_fuzz.cpp, built with AddressSanitizer and UndefinedBehaviorSanitizer around
    the decoders' own source, decodes thousands of randomly mutated TIFF and PNG files (written from
    the format specifications by control_files.py): each is accepted or rejected, and no memory
    error or undefined behaviour occurs."""
    import shutil
    import subprocess

    if shutil.which("g++") is None:
        pytest.skip("no g++")
    repo = Path(__file__).resolve().parents[1]
    exe = tmp_path / "decoder_fuzz"
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-g", "-fsanitize=address,undefined",
                        "-fno-sanitize-recover=undefined", "-I", str(repo / "include"),
                        str(repo / "tests" / "cpp" / "decoder_fuzz.cpp"),
                        str(repo / "hm-cupano_gb300" / "csrc" / "hmp_control_dir.cpp"), "-o", str(exe)],
                       capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip(f"no sanitizer runtime: {r.stderr.strip()[:200]}")
    seeds = tmp_path / "seeds"
    seeds.mkdir()
    rng = np.random.default_rng(0)
    img = rng.integers(0, 65535, (37, 53)).astype(np.uint16)
    for i, (comp, pred, be, kw) in enumerate([(c, p, b, k) for c in (1, 5, 8, 32773) for p in (1, 2)
                                               for b in (False, True) for k in ({"rows_per_strip": 7}, {"tile": 16})]):
        cf.write_tiff(seeds / f"t{i}.tif", img, big_endian=be, compression=comp, predictor=pred, **kw)
    cf.write_png(seeds / "p.png", rng.integers(0, 9, (37, 53)), color_type=3, palette=rng.integers(0, 256, (9, 3)))
    for depth in (1, 4, 8, 16):
        cf.write_png(seeds / f"g{depth}.png", rng.integers(0, 1 << depth, (19, 29)), color_type=0, bit_depth=depth)
    cf.write_png(seeds / "c.png", rng.integers(0, 256, (11, 17, 3)), color_type=2)
    files = sorted(str(p) for p in seeds.iterdir())
    env = dict(__import__("os").environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0")
    out = subprocess.run([str(exe), "6000", "2024", str(tmp_path / "scratch"), *files], capture_output=True, text=True,
                         env=env, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    decoded, rejected = (int(v) for v in out.stdout.split()[1::2])
    assert decoded > 0 and rejected > 0 and decoded + rejected == 6000
