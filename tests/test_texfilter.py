"""Texture filtering, an addition to the reference (whose README.md:71-72
lists bilinear filtering and mipmapping as to do): known answers of the
oracle's restatement of srp/texture.h's definition, through the C API of
oracle/_build/libsrp_port.so. The device sampler is checked against it on
the GPU (scene texfilter in test_gpu_parity.py)."""
import ctypes
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NEAREST, BILINEAR, TRILINEAR = 0, 1, 2
REPEAT, CLAMP = 0, 1


@pytest.fixture(scope="module")
def port():
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "portlib"])
    L = ctypes.CDLL(os.path.join(ROOT, "oracle", "_build", "libsrp_port.so"))
    vp = ctypes.c_void_p
    L.srpNewTextureFromMemory.restype = vp
    L.srpNewTextureFromMemory.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_int]
    L.srpFreeTexture.argtypes = [vp]
    L.srpTextureSetFilter.argtypes = [vp, ctypes.c_int]
    L.srpTextureGetFilter.argtypes = [vp]
    L.srpTextureGetFilteredColor.argtypes = [vp, ctypes.c_float, ctypes.c_float, ctypes.POINTER(ctypes.c_float)]
    L.srpTextureGetFilteredColorLod.argtypes = [vp, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                                ctypes.POINTER(ctypes.c_float)]
    L.srpTextureMipLevels.argtypes = [ctypes.c_int, ctypes.c_int]
    return L


def texture(L, rgb, w, h, wx=REPEAT, wy=REPEAT):
    data = bytes(rgb)
    assert len(data) == w * h * 3
    return L.srpNewTextureFromMemory(data, w, h, 3, wx, wy)


def sample(L, t, u, v, lod=None):
    out = (ctypes.c_float * 4)()
    if lod is None:
        L.srpTextureGetFilteredColor(t, u, v, out)
    else:
        L.srpTextureGetFilteredColorLod(t, u, v, lod, out)
    return [round(x * 255.0, 3) for x in out[:3]]


def test_mip_levels(port):
    assert port.srpTextureMipLevels(1, 1) == 1
    assert port.srpTextureMipLevels(96, 64) == 7      # 96 48 24 12 6 3 1
    assert port.srpTextureMipLevels(5, 1) == 3        # 5 2 1
    assert port.srpTextureMipLevels(1024, 1024) == 11


def test_bilinear_blends_the_four_neighbours(port):
    # one row of three texels: x = 2u, so u = 0.25 falls half-way between texels 0 and 1
    t = texture(port, [0, 0, 0, 100, 10, 1, 200, 20, 2], 3, 1)
    try:
        assert port.srpTextureGetFilter(t) == NEAREST
        assert sample(port, t, 0.25, 0.5) == [100.0, 10.0, 1.0]   # the reference's nearest: round(0.5) = texel 1
        port.srpTextureSetFilter(t, BILINEAR)
        assert port.srpTextureGetFilter(t) == BILINEAR
        assert sample(port, t, 0.25, 0.5) == [50.0, 5.0, 0.5]
        assert sample(port, t, 0.5, 0.5) == [100.0, 10.0, 1.0]    # on a texel centre: the texel
        assert sample(port, t, 1.0, 0.5) == [200.0, 20.0, 2.0]    # last texel, its neighbour has weight 0
        # u wraps before filtering, as for the nearest texel
        assert sample(port, t, 1.25, 0.5) == sample(port, t, 0.25, 0.5)
    finally:
        port.srpFreeTexture(t)
    # 2 x 2: the +1 neighbour of the bottom-right texel wraps (repeat) or clamps
    rgb = [10, 0, 0, 20, 0, 0, 30, 0, 0, 40, 0, 0]
    for wrap, want in ((REPEAT, 25.0), (CLAMP, 25.0)):
        t = texture(port, rgb, 2, 2, wrap, wrap)
        try:
            port.srpTextureSetFilter(t, BILINEAR)
            # x = u, y = 1 - v: (0.5, 0.5) blends all four equally
            assert sample(port, t, 0.5, 0.5)[0] == want
        finally:
            port.srpFreeTexture(t)


def test_trilinear_levels_are_rounded_box_averages(port):
    # 2 x 2 -> level 1 is one texel: (a + b + c + d + 2) / 4 per channel
    rgb = [10, 1, 255, 21, 2, 255, 30, 3, 254, 40, 5, 254]
    t = texture(port, rgb, 2, 2)
    try:
        port.srpTextureSetFilter(t, TRILINEAR)
        assert sample(port, t, 0.3, 0.7, 1.0) == [25.0, 3.0, 255.0]   # (101+2)//4, (11+2)//4, (1018+2)//4
        assert sample(port, t, 0.9, 0.1, 7.5) == [25.0, 3.0, 255.0]   # clamped to the last level
        lvl0 = sample(port, t, 0.5, 0.5, 0.0)
        half = sample(port, t, 0.5, 0.5, 0.5)
        for a, b, c in zip(lvl0, half, [25.0, 3.0, 255.0]):
            assert abs(b - (a + c) / 2) < 1e-3                         # half-way between the two levels
        assert sample(port, t, 0.5, 0.5) == lvl0                       # srpTextureGetFilteredColor: level 0
        # a bilinear texture ignores the level of detail
        port.srpTextureSetFilter(t, BILINEAR)
        assert sample(port, t, 0.5, 0.5, 1.0) == lvl0
    finally:
        port.srpFreeTexture(t)


def test_unknown_filter_falls_back_to_nearest(port):
    t = texture(port, [1, 2, 3], 1, 1)
    try:
        port.srpTextureSetFilter(t, 7)
        assert port.srpTextureGetFilter(t) == NEAREST
    finally:
        port.srpFreeTexture(t)
