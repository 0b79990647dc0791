"""Fixture for the reference's own 18 image tests (tests/scenes/**/*.c of the
reference, compared by its tests/compare.py at tolerance 1): the golden images
(tests/references/**/*.png) as RGB arrays, and the two input assets those
scenes load, as the reference loads them: the Utah teapot mesh through its
OBJ loader and the stone-wall texture through its stb_image with 3 channels
(both dumped by oracle/ref_assets.c). tests/refscenes.py restates the
scenes' call sequences; tests/test_refscenes.py renders them through the
oracle and the GPU library and compares with these images.

Run where the reference sources are available:

    python tests/golden/make_refimages.py
"""
import glob
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(HERE))
from pngio import read_png  # noqa: E402

REF = os.environ.get("SRP_REFERENCE", "/root/reference")


def main():
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "refassets", f"REF={REF}"])
    out = {}
    with tempfile.TemporaryDirectory() as d:
        subprocess.check_call([os.path.join(ROOT, "oracle", "_ref", "ref_assets"),
                               os.path.join(REF, "examples", "res", "objects", "utah_teapot.obj"),
                               os.path.join(REF, "examples", "res", "textures", "stoneWall.png"), d])
        t = open(os.path.join(d, "teapot.bin"), "rb").read()
        nv, ni = (int(x) for x in np.frombuffer(t[:16], np.uint64))
        out["teapot_vertices"] = np.frombuffer(t[16:16 + 32 * nv], np.float32).reshape(nv, 8).copy()
        out["teapot_indices"] = np.frombuffer(t[16 + 32 * nv:16 + 32 * nv + 4 * ni], np.uint32).copy()
        x = open(os.path.join(d, "texture.bin"), "rb").read()
        w, h = (int(v) for v in np.frombuffer(x[:8], np.int32))
        out["texture"] = np.frombuffer(x[8:8 + w * h * 3], np.uint8).reshape(h, w, 3).copy()
    goldens = sorted(glob.glob(os.path.join(REF, "tests", "references", "*", "*.png")))
    assert len(goldens) == 18, goldens
    for g in goldens:
        name = os.path.basename(os.path.dirname(g)) + "_" + os.path.basename(g)[:-4]
        img = read_png(g)
        assert img.shape[:2] == (512, 512), (name, img.shape)
        out["golden_" + name] = img[:, :, :3].astype(np.uint8)  # RGB; the harness forces alpha to 255
        print(name)
    np.savez_compressed(os.path.join(HERE, "refimages.npz"), **out)


if __name__ == "__main__":
    main()
