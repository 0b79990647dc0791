"""Generate the golden fixtures under tests/golden/ from the reference itself.

Each case (scene, seed, scale) is rendered by the reference library built from
its own sources (oracle/_ref/ref_scenes, see oracle/Makefile) and by the CPU
oracle (oracle/_build/port_scenes); the two must agree bit for bit, and the
reference's planes (colour, depth, stencil), its input hash and the oracle's
fragment count are stored as compressed .npz files. Run it where the reference
sources are available:

    make -C oracle port ref && python tests/golden/make_golden.py
"""
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
]


def case_name(scene, seed, scale):
    return f"{scene}_s{seed}_x{scale:g}".replace(".", "p")


def render(exe, scene, seed, scale, out):
    subprocess.check_call([exe, "render", scene, str(seed), repr(scale), out])
    return read_dump(out)


def main():
    ref = os.path.join(ROOT, "oracle", "_ref", "ref_scenes")
    port = os.path.join(ROOT, "oracle", "_build", "port_scenes")
    manifest = []
    for scene, seed, scale in CASES:
        r = render(ref, scene, seed, scale, "/tmp/_golden_ref.bin")
        p = render(port, scene, seed, scale, "/tmp/_golden_port.bin")
        for k in ("color", "depth_bits", "stencil"):
            assert np.array_equal(r[k], p[k]), f"{scene}: oracle differs from the reference in {k}"
        assert r["hash"] == p["hash"]
        name = case_name(scene, seed, scale)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), color=r["color"], depth_bits=r["depth_bits"],
                            stencil=r["stencil"])
        manifest.append({"name": name, "scene": scene, "seed": seed, "scale": scale, "width": r["width"],
                         "height": r["height"], "input_hash": str(r["hash"]), "fragments": int(p["fragments"])})
        print(name, r["width"], r["height"], p["fragments"])
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1)


if __name__ == "__main__":
    main()
