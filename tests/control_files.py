"""Writers of control-directory files for the loader tests: PNG (zlib from the standard library,
every row filter) and TIFF (uncompressed, Deflate, PackBits, LZW; horizontal predictor; strips or
tiles; either byte order), written from the format specifications independently of the loader's
decoders.
"""
from __future__ import annotations

import struct
import zlib
from pathlib import Path

import numpy as np

# ---- PNG ----


def _png_chunk(kind: bytes, data: bytes) -> bytes:
    return struct.pack(">I", len(data)) + kind + data + struct.pack(">I", zlib.crc32(kind + data) & 0xFFFFFFFF)


def _paeth(a: int, b: int, c: int) -> int:
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    return a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)


def _filter_rows(rows: list[bytes], bpp: int) -> bytes:
    """Each row with filter type (row index mod 5): None, Sub, Up, Average, Paeth."""
    out = bytearray()
    prev = bytes(len(rows[0]))
    for y, row in enumerate(rows):
        f = y % 5
        enc = bytearray(len(row))
        for i, x in enumerate(row):
            a = row[i - bpp] if i >= bpp else 0
            b = prev[i]
            c = prev[i - bpp] if i >= bpp else 0
            pred = (0, a, b, (a + b) >> 1, _paeth(a, b, c))[f]
            enc[i] = (x - pred) & 0xFF
        out.append(f)
        out += enc
        prev = row
    return bytes(out)


def write_png(path: Path, samples: np.ndarray, color_type: int, bit_depth: int = 8, palette=None) -> None:
    """samples: [h, w] (grey / palette index) or [h, w, c] at `bit_depth`."""
    s = np.asarray(samples)
    h, w = s.shape[:2]
    c = 1 if s.ndim == 2 else s.shape[2]
    rows = []
    for y in range(h):
        v = s[y].reshape(-1).astype(np.int64)
        if bit_depth == 16:
            rows.append(v.astype(">u2").tobytes())
        elif bit_depth == 8:
            rows.append(v.astype(np.uint8).tobytes())
        else:  # packed, most significant bits first
            per = 8 // bit_depth
            padded = np.concatenate([v, np.zeros((-len(v)) % per, np.int64)]).reshape(-1, per)
            shifts = np.array([8 - bit_depth * (k + 1) for k in range(per)])
            rows.append((padded << shifts).sum(axis=1).astype(np.uint8).tobytes())
    bpp = max(1, c * bit_depth // 8)
    data = _png_chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, bit_depth, color_type, 0, 0, 0))
    if palette is not None:
        data += _png_chunk(b"PLTE", bytes(np.asarray(palette, np.uint8).reshape(-1)))
    raw = _filter_rows(rows, bpp)
    z = zlib.compress(raw, 9)
    data += _png_chunk(b"IDAT", z[: len(z) // 2]) + _png_chunk(b"IDAT", z[len(z) // 2:])  # split IDAT
    Path(path).write_bytes(b"\x89PNG\r\n\x1a\n" + data + _png_chunk(b"IEND", b""))


# ---- TIFF ----


def packbits_encode(data: bytes) -> bytes:
    out = bytearray()
    i, n = 0, len(data)
    while i < n:
        run = 1
        while i + run < n and run < 128 and data[i + run] == data[i]:
            run += 1
        if run >= 3:
            out += bytes([(257 - run) & 0xFF, data[i]])
            i += run
            continue
        j = i
        while j < n and j - i < 128 and not (j + 2 < n and data[j] == data[j + 1] == data[j + 2]):
            j += 1
        out.append(j - i - 1)
        out += data[i:j]
        i = j
    return bytes(out)


def lzw_encode(data: bytes) -> bytes:
    """TIFF LZW: codes MSB first, Clear = 256, EOI = 257, the width growing when the next code
    would not fit (the decoder, one entry behind, sees this as the early change)."""
    bits: list[int] = []

    def put(code: int, width: int) -> None:
        bits.extend((code >> (width - 1 - k)) & 1 for k in range(width))

    def reset():
        return {bytes([i]): i for i in range(256)}, 258, 9

    table, nxt, width = reset()
    put(256, width)
    w = b""
    for byte in data:
        wc = w + bytes([byte])
        if wc in table:
            w = wc
            continue
        put(table[w], width)
        table[wc] = nxt
        nxt += 1
        if nxt >= (1 << width) and width < 12:
            width += 1
        if nxt >= 4094:
            put(256, width)
            table, nxt, width = reset()
        w = bytes([byte])
    if w:
        put(table[w], width)
        nxt += 1
        if nxt >= (1 << width) and width < 12:
            width += 1
    put(257, width)
    bits.extend([0] * ((-len(bits)) % 8))
    return bytes(int("".join(map(str, bits[i:i + 8])), 2) for i in range(0, len(bits), 8))


def write_tiff(path: Path, img: np.ndarray | None, *, big_endian: bool = False, compression: int = 1,
               predictor: int = 1, rows_per_strip: int | None = None, tile: int | None = None,
               position=None, resolution=(1, 1)) -> None:
    """A single-IFD TIFF: `img` [h, w] uint16 (or None for a 1x1 image that only carries the
    position tags); position = ((xnum, xden), (ynum, yden)) in resolution units."""
    e = ">" if big_endian else "<"
    if img is None:
        img = np.zeros((1, 1), np.uint16)
    img = np.asarray(img, np.uint16)
    h, w = img.shape

    def encode(block: np.ndarray) -> bytes:
        v = block.astype(np.int64)
        if predictor == 2:
            v = np.concatenate([v[:, :1], np.diff(v, axis=1)], axis=1) & 0xFFFF
        raw = v.astype(e + "u2").tobytes()
        if compression == 1:
            return raw
        if compression in (8, 32946):
            return zlib.compress(raw)
        if compression == 32773:
            return packbits_encode(raw)
        if compression == 5:
            return lzw_encode(raw)
        raise ValueError(compression)

    blocks = []
    if tile:
        for ty in range(0, h, tile):
            for tx in range(0, w, tile):
                b = np.zeros((tile, tile), np.uint16)
                part = img[ty:ty + tile, tx:tx + tile]
                b[: part.shape[0], : part.shape[1]] = part
                blocks.append(encode(b))
    else:
        rps = rows_per_strip or h
        for y in range(0, h, rps):
            blocks.append(encode(img[y:y + rps]))
    tags: list[tuple[int, int, list]] = [
        (256, 4, [w]), (257, 4, [h]), (258, 3, [16]), (259, 3, [compression]), (262, 3, [1]), (277, 3, [1]),
        (284, 3, [1]), (339, 3, [1]),
    ]
    if predictor != 1:
        tags.append((317, 3, [predictor]))
    if tile:
        tags += [(322, 4, [tile]), (323, 4, [tile])]
    else:
        tags.append((278, 4, [rows_per_strip or h]))
    rat = [r if isinstance(r, tuple) else (int(r), 1) for r in resolution]
    tags += [(282, 5, [rat[0]]), (283, 5, [rat[1]]), (296, 3, [2])]
    if position is not None:
        tags += [(286, 5, [position[0]]), (287, 5, [position[1]])]
    off_tag, cnt_tag = (324, 325) if tile else (273, 279)
    tags += [(off_tag, 4, [0] * len(blocks)), (cnt_tag, 4, [len(b) for b in blocks])]
    tags.sort(key=lambda t: t[0])
    ifd_at = 8
    extra_at = ifd_at + 2 + 12 * len(tags) + 4
    size = {3: 2, 4: 4, 5: 8}

    def packed(t, vals):
        if t == 5:
            return b"".join(struct.pack(e + "II", *v) for v in vals)
        return b"".join(struct.pack(e + ("H" if t == 3 else "I"), v) for v in vals)

    # Lay out: header, IFD, out-of-line tag values, block data.
    extra = bytearray()
    layout = {}
    for tag, t, vals in tags:
        if size[t] * len(vals) > 4:
            layout[tag] = extra_at + len(extra)
            extra += packed(t, vals) if tag != off_tag else bytes(4 * len(vals))
    data_at = extra_at + len(extra)
    offsets, pos = [], data_at
    for b in blocks:
        offsets.append(pos)
        pos += len(b)
    if off_tag in layout:
        at = layout[off_tag] - extra_at
        extra[at:at + 4 * len(offsets)] = packed(4, offsets)
    out = bytearray((b"MM" if big_endian else b"II") + struct.pack(e + "HI", 42, ifd_at))
    out += struct.pack(e + "H", len(tags))
    for tag, t, vals in tags:
        vals = offsets if tag == off_tag else vals
        if tag in layout:
            out += struct.pack(e + "HHII", tag, t, len(vals), layout[tag])
        else:
            v = packed(t, vals)
            out += struct.pack(e + "HHI", tag, t, len(vals)) + v + bytes(4 - len(v))
    out += struct.pack(e + "I", 0)
    out += extra
    for b in blocks:
        out += b
    Path(path).write_bytes(bytes(out))


def write_control_dir(directory: Path, maps_x, maps_y, positions, seam_file: np.ndarray, *, paletted: bool,
                      resolution=150, **tiff_kw) -> None:
    """mapping_000i{,_x,_y}.tif for each table and seam_file.png. positions in pixels; stored as
    XPosition = x / resolution (a rational) with XResolution = resolution."""
    d = Path(directory)
    d.mkdir(parents=True, exist_ok=True)
    for i, (mx, my) in enumerate(zip(maps_x, maps_y)):
        write_tiff(d / f"mapping_{i:04d}_x.tif", mx, **tiff_kw)
        write_tiff(d / f"mapping_{i:04d}_y.tif", my, **tiff_kw)
        x, y = positions[i]
        write_tiff(d / f"mapping_{i:04d}.tif", None, position=((int(x), resolution), (int(y), resolution)),
                   resolution=((resolution, 1), (resolution, 1)))
    if paletted:
        pal = np.stack([np.arange(256), 255 - np.arange(256), (np.arange(256) * 7) % 256], axis=1)
        write_png(d / "seam_file.png", seam_file, color_type=3, palette=pal)
    else:
        write_png(d / "seam_file.png", seam_file, color_type=0)
