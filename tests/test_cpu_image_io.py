"""Headless artefacts: the PNG writer's file parses (signature, chunk CRCs,
IHDR) and inflates (Python's zlib) back to the pixels written."""
import struct
import zlib

import numpy as np
import pytest

from refraktor_gb300 import librefrakt as lr


def _read_png(path):
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, chunks = 8, []
    while pos < len(data):
        (n,) = struct.unpack(">I", data[pos:pos + 4])
        typ = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        (crc,) = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        assert crc == zlib.crc32(typ + body) & 0xFFFFFFFF
        chunks.append((typ, body))
        pos += 12 + n
    return chunks


@pytest.mark.parametrize("w,h,c", [(1, 1, 3), (37, 5, 4), (300, 250, 3)])
def test_png_roundtrip(tmp_path, w, h, c):
    rng = np.random.default_rng(w * h * c)
    px = rng.integers(0, 256, size=(h, w, c), dtype=np.uint8)
    f = tmp_path / "x.png"
    lr.write_png(f, px)
    chunks = _read_png(f)
    assert [t for t, _ in chunks] == [b"IHDR", b"IDAT", b"IEND"]
    ww, hh, depth, ctype, comp, filt, lace = struct.unpack(">IIBBBBB", chunks[0][1])
    assert (ww, hh, depth, ctype, comp, filt, lace) == (w, h, 8, 6 if c == 4 else 2, 0, 0, 0)
    raw = zlib.decompress(chunks[1][1])
    rows = np.frombuffer(raw, dtype=np.uint8).reshape(h, 1 + w * c)
    assert np.all(rows[:, 0] == 0)
    np.testing.assert_array_equal(rows[:, 1:].reshape(h, w, c), px)


def test_png_rejects_bad_arguments(tmp_path):
    with pytest.raises(lr.RfkError):
        lr.write_png(tmp_path / "y.png", np.zeros((4, 4, 2), dtype=np.uint8))
