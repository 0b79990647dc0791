"""PNG output (srpImageWritePNG, behind srpGpuSaveFramebufferPNG): stored-block
PNGs read back by the suite's own PIL-free reader, chunk CRCs and the zlib
checksum verified. The writer is host code: the CPU test calls it through the
library's C ABI without touching the GPU."""
import ctypes
import struct
import zlib

import numpy as np
import pytest

from pngio import read_png


def _chunks(path):
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, out = 8, []
    while pos < len(data):
        (n,) = struct.unpack(">I", data[pos:pos + 4])
        kind, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        (crc,) = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        out.append((kind, body, crc))
        pos += 12 + n
    return out


@pytest.mark.parametrize("w,h", [(1, 1), (7, 3), (200, 100), (37, 600)])
def test_png_writer_round_trip(built_library, tmp_path, w, h):
    import srp_gb300
    L = srp_gb300.lib()
    L.srpImageWritePNG.restype = ctypes.c_int
    L.srpImageWritePNG.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
    rgba = np.random.default_rng(w * 1000 + h).integers(0, 256, size=(h, w, 4), dtype=np.uint8)
    path = tmp_path / "out.png"
    assert L.srpImageWritePNG(str(path).encode(), rgba.ctypes.data, w, h) == 1
    chunks = _chunks(path)
    assert [c[0] for c in chunks] == [b"IHDR", b"IDAT", b"IEND"]
    for kind, body, crc in chunks:
        assert zlib.crc32(kind + body) & 0xFFFFFFFF == crc, kind
    ihdr = struct.unpack(">IIBBBBB", chunks[0][1])
    assert ihdr == (w, h, 8, 6, 0, 0, 0)
    raw = np.frombuffer(zlib.decompress(chunks[1][1]), np.uint8).reshape(h, 1 + 4 * w)  # checks the Adler-32
    assert np.all(raw[:, 0] == 0)
    assert np.array_equal(raw[:, 1:].reshape(h, w, 4), rgba)
    assert np.array_equal(read_png(str(path)), rgba[..., :3])  # the suite's own reader


def test_png_writer_rejects_empty_image(built_library, tmp_path):
    import srp_gb300
    L = srp_gb300.lib()
    L.srpImageWritePNG.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
    assert L.srpImageWritePNG(str(tmp_path / "e.png").encode(), None, 0, 5) == 0


@pytest.mark.gpu
def test_save_framebuffer_png_matches_colour_plane(built_library, tmp_path):
    """A rendered frame saved as the reference's harness saves it: R, G, B of
    the packed colour, alpha 255."""
    import srp_gb300
    L = srp_gb300.lib()
    L.srpGpuSaveFramebufferPNG.restype = ctypes.c_int
    L.srpGpuSaveFramebufferPNG.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
    L.srpGpuSetFramebufferMode(srp_gb300.SRP_GPU_FB_DEVICE)
    sc = srp_gb300.Scene("sphere", 3, 0.5)
    try:
        sc.prepare()
        sc.render()
        path = tmp_path / "frame.png"
        assert L.srpGpuSaveFramebufferPNG(ctypes.c_void_p(sc.fb), str(path).encode()) == 0
        color, _, _ = sc.planes()
        w, h = sc.info.width, sc.info.height
        chunks = _chunks(path)
        raw = np.frombuffer(zlib.decompress(chunks[1][1]), np.uint8).reshape(h, 1 + 4 * w)
        img = raw[:, 1:].reshape(h, w, 4).astype(np.uint32)
        packed = (img[..., 0] << 24) | (img[..., 1] << 16) | (img[..., 2] << 8)
        assert np.array_equal(packed.reshape(-1), color & 0xFFFFFF00)
        assert np.all(img[..., 3] == 255)
        assert np.array_equal(read_png(str(path)).astype(np.uint32), img[..., :3])
        assert int(np.count_nonzero(color)) > 1000
    finally:
        sc.close()
