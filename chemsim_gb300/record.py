"""Frame recording from the headless colour map.

taktoa/chemsim's `record` (src/display.rs:157-185) steps a simulation, renders
every step into an RGBA image and appends it to a GIF encoder.  Here the frame
comes from lbm_render (the colour map of src/render.rs on the device) and is
written losslessly as one PNG file per frame.  PNG needs no palette
quantisation, and the zlib module of the standard library is its only
dependency.
"""
from __future__ import annotations

import struct
import zlib

import numpy as np


def _chunk(kind: bytes, data: bytes) -> bytes:
    return (struct.pack(">I", len(data)) + kind + data
            + struct.pack(">I", zlib.crc32(kind + data) & 0xFFFFFFFF))


def png_bytes(rgba: np.ndarray, level: int = 6) -> bytes:
    """An 8-bit RGBA PNG of an (h, w, 4) uint8 image (filter type 0 on every
    scanline)."""
    img = np.ascontiguousarray(rgba, dtype=np.uint8)
    if img.ndim != 3 or img.shape[2] != 4:
        raise ValueError("expected an (h, w, 4) RGBA image")
    h, w, _ = img.shape
    raw = np.empty((h, 1 + 4 * w), dtype=np.uint8)
    raw[:, 0] = 0
    raw[:, 1:] = img.reshape(h, 4 * w)
    ihdr = struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)
    return (b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", ihdr)
            + _chunk(b"IDAT", zlib.compress(raw.tobytes(), level)) + _chunk(b"IEND", b""))


def read_png(data: bytes) -> np.ndarray:
    """Decodes what png_bytes writes (8-bit RGBA, filter type 0)."""
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError("not a PNG file")
    pos, idat = 8, b""
    w = h = 0
    while pos < len(data):
        (n,) = struct.unpack(">I", data[pos:pos + 4])
        kind, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        if kind == b"IHDR":
            w, h, depth, ctype = struct.unpack(">IIBB", body[:10])
            if depth != 8 or ctype != 6:
                raise ValueError("only 8-bit RGBA is supported")
        elif kind == b"IDAT":
            idat += body
        pos += 12 + n
    raw = np.frombuffer(zlib.decompress(idat), dtype=np.uint8).reshape(h, 1 + 4 * w)
    if raw[:, 0].any():
        raise ValueError("only filter type 0 is supported")
    return raw[:, 1:].reshape(h, w, 4).copy()


def record(lattice, frames: int, path_pattern: str, steps_per_frame: int = 1, mode: int = 2,
           geometry_overlay: bool = True) -> list:
    """Steps `lattice` and writes one frame after every `steps_per_frame`
    steps, `frames` frames in all, to path_pattern.format(frame_index).
    Mode is a render mode (lbm.RENDER_*; default velocity).  Returns the
    paths written."""
    paths = []
    for k in range(frames):
        lattice.step(steps_per_frame)
        img = lattice.render(mode, geometry_overlay)
        path = path_pattern.format(k)
        with open(path, "wb") as fh:
            fh.write(png_bytes(img))
        paths.append(path)
    return paths
