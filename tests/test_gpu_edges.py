"""Edge cases of the draw path on the GPU, through the C ABI: an index past
the vertex buffer (reported, framebuffer untouched), a fully culled draw, an
empty draw, a 1x1 framebuffer, and a batch whose pass meets a bad index
(every draw then reports on its own). The device framebuffer mode is used, so
that untouched means the device planes."""
import ctypes

import numpy as np
import pytest

from test_zz_no_alloc import Api, SRP_PRIM_TRIANGLES, assert_same, triangle_soup

pytestmark = pytest.mark.gpu


@pytest.fixture()
def api(built_library):
    a = Api()
    a.L.srpGpuSetFramebufferMode(1)
    yield a
    a.close()


def test_index_past_vertex_buffer_is_reported_and_draws_nothing(api):
    L = api.L
    rng = np.random.default_rng(5)
    tris = triangle_soup(rng, 500)
    vb = api.vertex_buffer(tris)
    idx = np.arange(tris.shape[0], dtype=np.uint32)
    idx[700] = tris.shape[0] + 3  # one index past the end
    ib = api.index_buffer(idx)
    fb = api.framebuffer(128, 96)
    before = api.planes(fb)
    api.messages.clear()
    L.srpDrawIndexBuffer(ib, vb, fb, ctypes.byref(api.prog), SRP_PRIM_TRIANGLES, 0, idx.size)
    errs = api.errors()
    assert errs and "out of range" in errs[-1][2], api.messages
    assert_same(api.planes(fb), before, "draw with a bad index")
    # the next draw is unaffected
    api.messages.clear()
    good = api.index_buffer(np.arange(tris.shape[0], dtype=np.uint32))
    L.srpDrawIndexBuffer(good, vb, fb, ctypes.byref(api.prog), SRP_PRIM_TRIANGLES, 0, tris.shape[0])
    assert not api.errors(), api.errors()
    assert int(np.count_nonzero(api.planes(fb)[0])) > 100
    assert L.srpGpuSynchronize() == 0


def test_fully_culled_and_empty_draws_leave_the_framebuffer(api):
    L = api.L
    L.srpRasterCullFace.argtypes = [ctypes.c_int]
    rng = np.random.default_rng(6)
    tris = triangle_soup(rng, 400)
    vb = api.vertex_buffer(tris)
    fb = api.framebuffer(160, 120)
    before = api.planes(fb)
    api.messages.clear()
    L.srpDrawVertexBuffer(vb, fb, ctypes.byref(api.prog), SRP_PRIM_TRIANGLES, 0, 0)  # empty
    L.srpRasterCullFace(3)  # SRP_FACE_FRONT_AND_BACK: the reference draws nothing
    L.srpDrawVertexBuffer(vb, fb, ctypes.byref(api.prog), SRP_PRIM_TRIANGLES, 0, tris.shape[0])
    L.srpRasterCullFace(0)  # SRP_FACE_NONE
    assert not api.errors(), api.errors()
    assert_same(api.planes(fb), before, "empty and culled draws")
    assert L.srpGpuSynchronize() == 0


def test_one_pixel_framebuffer(api):
    L = api.L
    verts = np.array([[-1, -1, 0, 1, 0, 0], [3, -1, 0, 0, 1, 0], [-1, 3, 0, 0, 0, 1]], dtype=np.float32)
    vb = api.vertex_buffer(verts)
    fb = api.framebuffer(1, 1)
    L.srpDrawVertexBuffer(vb, fb, ctypes.byref(api.prog), SRP_PRIM_TRIANGLES, 0, 3)
    color, depth, stencil = api.planes(fb)
    assert not api.errors(), api.errors()
    assert color.shape == (1,) and color[0] != 0
    assert L.srpGpuSynchronize() == 0


def test_batch_with_a_bad_index_reports_and_draws_the_rest(api):
    """A multi-draw pass meets an index past a vertex buffer: each draw of the
    pass is then issued on its own, the bad one reports, the others render as
    ordinary draws do."""
    import srp_gb300
    L = api.L
    L.srpGpuDrawBatch.argtypes = [ctypes.c_void_p, ctypes.c_size_t]
    rng = np.random.default_rng(8)
    n = 6
    draws = (srp_gb300.SRPGpuDraw * n)()
    fbs, refs = [], []
    for i in range(n):
        tris = triangle_soup(rng, 300)
        vb = api.vertex_buffer(tris)
        idx = np.arange(tris.shape[0], dtype=np.uint32)
        if i == 3:
            idx[10] = 10_000
        ib = api.index_buffer(idx)
        fb = api.framebuffer(96, 64)
        ref = api.framebuffer(96, 64)
        fbs.append(fb)
        refs.append((ib, vb, ref, idx.size))
        d = draws[i]
        d.indexBuffer, d.vertexBuffer, d.framebuffer = ib, vb, fb
        d.program = ctypes.addressof(api.prog)
        d.primitive, d.startIndex, d.count = SRP_PRIM_TRIANGLES, 0, idx.size
    api.messages.clear()
    L.srpGpuDrawBatch(ctypes.addressof(draws), n)
    errs = api.errors()
    assert len(errs) == 1 and "out of range" in errs[0][2], api.messages
    for i, (ib, vb, ref, cnt) in enumerate(refs):
        if i != 3:
            L.srpDrawIndexBuffer(ib, vb, ref, ctypes.byref(api.prog), SRP_PRIM_TRIANGLES, 0, cnt)
        assert_same(api.planes(fbs[i]), api.planes(ref), f"draw {i}")
    assert L.srpGpuSynchronize() == 0
