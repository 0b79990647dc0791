"""The CPU oracle (oracle/srp_port.c) against the reference: committed golden
fixtures rendered by the reference library, the reference's own 18 golden
images, and the exact chain used by the GPU raster. CPU only."""
import glob
import os
import subprocess

import numpy as np
import pytest

from oracle_util import manifest, load_golden, oracle_render, compare_planes, hash_cases, plane_digests

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("SRP_REFERENCE", "/root/reference")


@pytest.mark.parametrize("case", manifest(), ids=lambda c: c["name"])
def test_oracle_matches_reference_fixtures(oracle_exe, case):
    got = oracle_render(oracle_exe, case["scene"], case["seed"], case["scale"])
    assert str(got["hash"]) == case["input_hash"], "scene inputs differ from the fixture's"
    want = load_golden(case)
    for k in ("color", "depth_bits", "stencil"):
        assert np.array_equal(got[k], want[k]), f"{case['name']}: {k} differs from the reference"
    assert got["fragments"] == case["fragments"]


@pytest.mark.parametrize("case", hash_cases(), ids=lambda c: c["name"])
def test_oracle_matches_reference_digests(oracle_exe, case):
    """The full-size bench frame: the oracle's planes hash to the reference's."""
    got = oracle_render(oracle_exe, case["scene"], case["seed"], case["scale"])
    assert str(got["hash"]) == case["input_hash"], "scene inputs differ from the reference's"
    assert plane_digests(got) == case["sha256"]
    assert got["fragments"] == case["fragments"]


def test_chain_jump_is_exact(tmp_path):
    exe = str(tmp_path / "chain_test")
    subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-o", exe,
                           os.path.join(ROOT, "tests", "native", "chain_test.c"), "-lm"])
    for seed in (11, 12):
        out = subprocess.check_output([exe, "150000", str(seed)]).decode()
        assert out.startswith("ok"), out


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "tests", "references")),
                    reason="reference sources not present on this machine")
def test_reference_golden_images(tmp_path):
    """Build the reference's own test scenes against the reference library and
    against the oracle; the reference matches its golden PNGs within the
    tolerance of its tests (1/255), the oracle matches the reference exactly."""
    from pngio import read_png
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "refscenes", f"REF={REF}"])
    d = os.path.join(ROOT, "oracle", "_ref", "refscenes")
    goldens = sorted(glob.glob(os.path.join(REF, "tests", "references", "*", "*.png")))
    assert len(goldens) == 18
    for g in goldens:
        name = os.path.basename(os.path.dirname(g)) + "_" + os.path.basename(g)[:-4]
        imgs = {}
        for kind in ("ref", "port"):
            out = str(tmp_path / f"{kind}_{name}.png")
            subprocess.check_call([os.path.join(d, f"{kind}_{name}"), out], cwd=d,
                                  stdout=subprocess.DEVNULL)
            imgs[kind] = read_png(out).astype(int)
        gold = read_png(g).astype(int)
        assert np.abs(imgs["ref"] - gold).max() <= 1, name
        assert np.array_equal(imgs["port"], imgs["ref"]), name
