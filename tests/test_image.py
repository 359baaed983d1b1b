"""Headless image export (csg_image_write): PNG and PPM files decode back to the frame."""
from __future__ import annotations

import struct
import zlib

import numpy as np


def _read_png(data: bytes):
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w = 8, b"", None
    while pos < len(data):
        n, = struct.unpack(">I", data[pos:pos + 4])
        kind, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        crc, = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        assert zlib.crc32(kind + body) & 0xFFFFFFFF == crc
        if kind == b"IHDR":
            w, h, depth, ctype = struct.unpack(">IIBB", body[:10])
            assert depth == 8 and ctype == 6
        elif kind == b"IDAT":
            idat += body
        pos += 12 + n
    raw = zlib.decompress(idat)
    rows = np.frombuffer(raw, np.uint8).reshape(h, 1 + 4 * w)
    assert (rows[:, 0] == 0).all()
    return rows[:, 1:].reshape(h, w, 4)


def test_png_and_ppm_round_trip(csg, tmp_path):
    rng = np.random.default_rng(3)
    for w, h in ((1, 1), (7, 5), (300, 257)):  # 300x257 RGBA spans several stored blocks
        px = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
        frame = px.reshape(-1, 4).copy().view(np.uint32).reshape(-1)
        csg.write_image(tmp_path / "f.png", frame, w, h, "png")
        assert np.array_equal(_read_png((tmp_path / "f.png").read_bytes()), px)
        csg.write_image(tmp_path / "f.ppm", frame, w, h, "ppm")
        data = (tmp_path / "f.ppm").read_bytes()
        head = f"P6\n{w} {h}\n255\n".encode()
        assert data.startswith(head)
        rgb = np.frombuffer(data[len(head):], np.uint8).reshape(h, w, 3)
        assert np.array_equal(rgb, px[..., :3])


def test_image_rejects_bad_arguments(csg, tmp_path):
    lib = csg.lib()
    buf = np.zeros(4, np.uint32)
    assert lib.csg_image_write(None, buf.ctypes.data, 2, 2, 1) == csg.CSG_E_ARG
    assert lib.csg_image_write(str(tmp_path / "x.png").encode(), None, 2, 2, 1) == csg.CSG_E_ARG
    assert lib.csg_image_write(str(tmp_path / "x.png").encode(), buf.ctypes.data, 0, 2, 1) == csg.CSG_E_ARG
    assert lib.csg_image_write(str(tmp_path / "x.png").encode(), buf.ctypes.data, 2, 2, 7) == csg.CSG_E_ARG
    assert lib.csg_image_write(str(tmp_path / "no" / "dir.png").encode(), buf.ctypes.data, 2, 2, 1) == csg.CSG_E_ARG
