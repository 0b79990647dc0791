"""Reader for the raw framebuffer dumps written by the scene runner
(srp_gb300/scenes/scene_main.c): "SRPD", width, height (u32), input hash,
fragment count (u64), then colour (u32), depth (f32) and stencil (u8) planes."""
import numpy as np


def read_dump(path):
    d = open(path, "rb").read()
    assert d[:4] == b"SRPD", "not a framebuffer dump"
    w, h = np.frombuffer(d[4:12], np.uint32)
    hsh, frags = np.frombuffer(d[12:28], np.uint64)
    n = int(w) * int(h)
    o = 28
    color = np.frombuffer(d[o:o + 4 * n], np.uint32).copy()
    o += 4 * n
    depth = np.frombuffer(d[o:o + 4 * n], np.uint32).copy()
    o += 4 * n
    stencil = np.frombuffer(d[o:o + n], np.uint8).copy()
    return {"width": int(w), "height": int(h), "hash": int(hsh), "fragments": int(frags),
            "color": color, "depth_bits": depth, "stencil": stencil}
