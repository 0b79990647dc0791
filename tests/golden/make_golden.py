"""Generate the golden fixtures under tests/golden/ from the reference itself.

Each case (scene, seed, scale) is rendered by the reference library built from
its own sources (oracle/_ref/ref_scenes, see oracle/Makefile) and by the CPU
oracle (oracle/_build/port_scenes); the two must agree bit for bit, and the
reference's planes (colour, depth, stencil), its input hash and the oracle's
fragment count are stored as compressed .npz files. Frames too large to store
(the 1920x1080 bench frame) keep SHA-256 digests of the reference's planes in
hashes.json instead. Run it where the reference sources are available:

    make -C oracle port ref && python tests/golden/make_golden.py [case names]

With names, only those cases are rendered again and merged into the manifest.
"""
import hashlib
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(HERE))
from dumpio import read_dump  # noqa: E402

CASES = [
    ("sphere", 1, 1.0), ("sphere", 7, 0.25),
    ("soup", 3, 0.004),
    ("clip_tris", 1, 1.0), ("clip_lines", 1, 1.0), ("points", 1, 1.0), ("interp", 1, 1.0),
    ("depth_ops", 1, 1.0), ("raster_rules", 1, 1.0), ("scissor", 1, 1.0), ("stencil", 1, 1.0),
    ("poly_modes", 1, 1.0), ("topologies", 1, 1.0), ("late_z", 1, 1.0), ("lit", 1, 1.0),
    ("varyings", 1, 1.0),
]
# stored as digests only: the 2M-triangle soup at 1920x1080 that bench.py times
HASH_CASES = [("soup", 1, 1.0)]


def case_name(scene, seed, scale):
    return f"{scene}_s{seed}_x{scale:g}".replace(".", "p")


def render(exe, scene, seed, scale, out):
    subprocess.check_call([exe, "render", scene, str(seed), repr(scale), out])
    return read_dump(out)


def plane_digests(d):
    return {k: hashlib.sha256(np.ascontiguousarray(d[k]).astype(d[k].dtype.newbyteorder("<")).tobytes()).hexdigest()
            for k in ("color", "depth_bits", "stencil")}


def main(only):
    ref = os.path.join(ROOT, "oracle", "_ref", "ref_scenes")
    port = os.path.join(ROOT, "oracle", "_build", "port_scenes")
    mpath = os.path.join(HERE, "manifest.json")
    old = {}
    if only and os.path.exists(mpath):
        with open(mpath) as f:
            old = {c["name"]: c for c in json.load(f)}
    manifest = []
    for scene, seed, scale in CASES:
        name = case_name(scene, seed, scale)
        if only and name not in only and scene not in only:
            if name in old:
                manifest.append(old[name])
            continue
        r = render(ref, scene, seed, scale, "/tmp/_golden_ref.bin")
        p = render(port, scene, seed, scale, "/tmp/_golden_port.bin")
        for k in ("color", "depth_bits", "stencil"):
            assert np.array_equal(r[k], p[k]), f"{scene}: oracle differs from the reference in {k}"
        assert r["hash"] == p["hash"]
        np.savez_compressed(os.path.join(HERE, name + ".npz"), color=r["color"], depth_bits=r["depth_bits"],
                            stencil=r["stencil"])
        manifest.append({"name": name, "scene": scene, "seed": seed, "scale": scale, "width": r["width"],
                         "height": r["height"], "input_hash": str(r["hash"]), "fragments": int(p["fragments"])})
        print(name, r["width"], r["height"], p["fragments"])
    with open(mpath, "w") as f:
        json.dump(manifest, f, indent=1)
    hpath = os.path.join(HERE, "hashes.json")
    hashes = []
    if os.path.exists(hpath):
        with open(hpath) as f:
            hashes = json.load(f)
    for scene, seed, scale in HASH_CASES:
        name = case_name(scene, seed, scale)
        if only and name not in only and scene not in only:
            continue
        r = render(ref, scene, seed, scale, "/tmp/_golden_ref.bin")
        p = render(port, scene, seed, scale, "/tmp/_golden_port.bin")
        for k in ("color", "depth_bits", "stencil"):
            assert np.array_equal(r[k], p[k]), f"{scene}: oracle differs from the reference in {k}"
        hashes = [h for h in hashes if h["name"] != name]
        hashes.append({"name": name, "scene": scene, "seed": seed, "scale": scale, "width": r["width"],
                       "height": r["height"], "input_hash": str(r["hash"]), "fragments": int(p["fragments"]),
                       "sha256": plane_digests(r)})
        print(name, r["width"], r["height"], p["fragments"], "(digests)")
    with open(hpath, "w") as f:
        json.dump(hashes, f, indent=1)


if __name__ == "__main__":
    main(set(sys.argv[1:]))
