"""Minimal PNG decoder (stdlib zlib + numpy) for comparing the reference's
golden images; PIL is not available on every machine this suite runs on.
Supports 8-bit greyscale / RGB / RGBA / grey+alpha, non-interlaced."""
import struct
import zlib

import numpy as np


def read_png(path):
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n", "not a PNG"
    pos, idat = 8, []
    width = height = ctype = None
    while pos < len(data):
        (length,) = struct.unpack(">I", data[pos:pos + 4])
        kind = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + length]
        if kind == b"IHDR":
            width, height, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", body)
            assert depth == 8 and interlace == 0, "only 8-bit non-interlaced PNGs"
        elif kind == b"IDAT":
            idat.append(body)
        elif kind == b"IEND":
            break
        pos += 12 + length
    ch = {0: 1, 2: 3, 4: 2, 6: 4}[ctype]
    raw = np.frombuffer(zlib.decompress(b"".join(idat)), np.uint8).reshape(height, 1 + width * ch)
    out = np.zeros((height, width * ch), np.int32)
    for y in range(height):
        f, row = raw[y, 0], raw[y, 1:].astype(np.int32)
        up = out[y - 1] if y else np.zeros(width * ch, np.int32)
        if f == 0:
            cur = row
        elif f == 2:
            cur = (row + up) & 255
        else:
            cur = np.zeros(width * ch, np.int32)
            for i in range(width * ch):
                a = cur[i - ch] if i >= ch else 0
                b = up[i]
                c = up[i - ch] if i >= ch else 0
                if f == 1:
                    p = a
                elif f == 3:
                    p = (a + b) >> 1
                else:
                    pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                    p = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                cur[i] = (row[i] + p) & 255
        out[y] = cur
    img = out.reshape(height, width, ch).astype(np.uint8)
    if ch == 1:
        img = np.repeat(img, 3, axis=2)
    elif ch == 2:
        img = np.repeat(img[:, :, :1], 3, axis=2)
    return img[:, :, :3]
