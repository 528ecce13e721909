"""geon_gb300.render.write_png on uint8 pixels (no GPU): a valid PNG whose
decoded scanlines are the input bytes."""
import struct
import zlib

import numpy as np


def read_png(path):
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, chunks = 8, []
    while pos < len(data):
        (n,) = struct.unpack(">I", data[pos:pos + 4])
        tag, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        (crc,) = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        assert crc == zlib.crc32(tag + body) & 0xFFFFFFFF
        chunks.append((tag, body))
        pos += 12 + n
    return chunks


def test_write_png_uint8_round_trip(tmp_path):
    from geon_gb300.render import write_png
    rng = np.random.default_rng(11)
    h, w = 37, 53
    img = rng.integers(0, 256, (h, w, 3), dtype=np.uint8)
    path = tmp_path / "x.png"
    write_png(str(path), img, w, h)
    chunks = read_png(path)
    assert [c[0] for c in chunks] == [b"IHDR", b"IDAT", b"IEND"]
    width, height, depth, ctype, comp, filt, inter = struct.unpack(">IIBBBBB", chunks[0][1])
    assert (width, height, depth, ctype, comp, filt, inter) == (w, h, 8, 2, 0, 0, 0)
    raw = zlib.decompress(chunks[1][1])
    rows = np.frombuffer(raw, dtype=np.uint8).reshape(h, 1 + 3 * w)
    assert np.all(rows[:, 0] == 0)  # filter type 0 on every scanline
    assert np.array_equal(rows[:, 1:].reshape(h, w, 3), img)
