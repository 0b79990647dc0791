"""The reference's own 18 image tests (tests/scenes/**/*.c of kitrofimov/srp),
restated as srp API call sequences in tests/refscenes.py, rendered through
srp's C API by the CPU oracle (its shared build) and by the GPU library, and
compared with the reference's golden images at the tolerance of its own
comparator (tests/compare.py:8: every channel within 1). The GPU run is also
held to the oracle: depth and stencil bit-exact, colour within 1/255."""
import os
import subprocess

import numpy as np
import pytest

import refscenes
import srpapi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NAMES = sorted(refscenes.SCENES)


@pytest.fixture(scope="module")
def oracle_srp():
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "portlib"])
    s = srpapi.Srp(os.path.join(ROOT, "oracle", "_build", "libsrp_port.so"))
    yield s
    s.close()


@pytest.fixture(scope="module")
def gpu_srp(built_library):
    import srp_gb300
    L = srp_gb300.lib()
    # the reference's programs read the public planes after each draw
    L.srpGpuSetFramebufferMode(srp_gb300.SRP_GPU_FB_COHERENT)
    s = srpapi.Srp(srp_gb300.library_path())
    yield s
    s.close()
    assert L.srpGpuSynchronize() == 0


def max_channel_diff(a, b):
    return int(np.abs(a.astype(np.int32) - b.astype(np.int32)).max())


@pytest.mark.parametrize("name", NAMES)
def test_oracle_matches_reference_golden_image(oracle_srp, name):
    color, _, _ = refscenes.SCENES[name](oracle_srp)
    img = srpapi.rgb_image(color, refscenes.W, refscenes.H)
    assert max_channel_diff(img, refscenes.golden(name)) <= 1, name
    assert not oracle_srp.errors(), oracle_srp.errors()


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_gpu_matches_reference_golden_image(oracle_srp, gpu_srp, name):
    color, depth, stencil = refscenes.SCENES[name](gpu_srp)
    assert not gpu_srp.errors(), gpu_srp.errors()
    img = srpapi.rgb_image(color, refscenes.W, refscenes.H)
    assert max_channel_diff(img, refscenes.golden(name)) <= 1, name
    wc, wd, ws = refscenes.SCENES[name](oracle_srp)
    assert np.array_equal(depth.view(np.uint32), wd.view(np.uint32)), f"{name}: depth differs from the oracle"
    assert np.array_equal(stencil, ws), f"{name}: stencil differs from the oracle"
    assert max_channel_diff(img, srpapi.rgb_image(wc, refscenes.W, refscenes.H)) <= 1
