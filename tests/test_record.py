"""PNG frames of the frame recorder (CPU: the writer and its reader)."""
import struct
import zlib

import numpy as np

from chemsim_gb300.record import png_bytes, read_png


def test_png_roundtrip_and_layout():
    rng = np.random.default_rng(0)
    img = rng.integers(0, 256, size=(7, 13, 4), dtype=np.uint8)
    data = png_bytes(img)
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    n, kind = struct.unpack(">I", data[8:12])[0], data[12:16]
    assert kind == b"IHDR" and n == 13
    w, h, depth, ctype = struct.unpack(">IIBB", data[16:26])
    assert (w, h, depth, ctype) == (13, 7, 8, 6)
    # every chunk's CRC covers its type and body
    assert struct.unpack(">I", data[29:33])[0] == zlib.crc32(data[12:29]) & 0xFFFFFFFF
    assert np.array_equal(read_png(data), img)
    assert data.endswith(b"IEND\xaeB`\x82")
