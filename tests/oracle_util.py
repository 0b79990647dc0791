"""Test-side helpers: run the CPU oracle and compare framebuffers."""
import json
import os
import subprocess
import tempfile

import numpy as np

from dumpio import read_dump

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def manifest():
    with open(os.path.join(GOLDEN, "manifest.json")) as f:
        return json.load(f)


def hash_cases():
    """Reference frames too large to store, kept as SHA-256 digests of their
    planes (tests/golden/hashes.json, written by make_golden.py)."""
    with open(os.path.join(GOLDEN, "hashes.json")) as f:
        return json.load(f)


def plane_digests(d):
    """SHA-256 of the colour, depth-bit and stencil planes, little-endian."""
    import hashlib
    return {k: hashlib.sha256(np.ascontiguousarray(d[k]).astype(d[k].dtype.newbyteorder("<")).tobytes()).hexdigest()
            for k in ("color", "depth_bits", "stencil")}


def load_golden(case):
    z = np.load(os.path.join(GOLDEN, case["name"] + ".npz"))
    return {"color": z["color"], "depth_bits": z["depth_bits"], "stencil": z["stencil"]}


def oracle_render(exe, scene, seed, scale):
    with tempfile.NamedTemporaryFile(suffix=".bin", delete=False) as t:
        path = t.name
    try:
        subprocess.check_call([exe, "render", scene, str(seed), repr(float(scale)), path])
        return read_dump(path)
    finally:
        os.unlink(path)


def channel_diff(a, b):
    """Largest per-channel difference between packed RGBA8 colour planes."""
    a = a.astype(np.uint32)
    b = b.astype(np.uint32)
    m = 0
    for sh in (24, 16, 8, 0):
        d = np.abs(((a >> sh) & 255).astype(np.int32) - ((b >> sh) & 255).astype(np.int32))
        m = max(m, int(d.max()) if d.size else 0)
    return m


def compare_planes(got, want, what=""):
    """Depth and stencil bit-exact, colour within 1/255 per channel (the
    tolerance of the reference's own image tests, tests/compare.py:8)."""
    dz = np.nonzero(got["depth_bits"] != want["depth_bits"])[0]
    ds = np.nonzero(got["stencil"] != want["stencil"])[0]
    assert dz.size == 0, f"{what}: depth differs at {dz.size} pixels, first {dz[:8]}"
    assert ds.size == 0, f"{what}: stencil differs at {ds.size} pixels, first {ds[:8]}"
    cd = channel_diff(got["color"], want["color"])
    assert cd <= 1, f"{what}: colour differs by {cd}/255"
