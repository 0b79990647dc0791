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


def test_framebuffer_work_between_overlapped_draws_keeps_its_place(api):
    """A depth fill and an asynchronous download queued between draws that
    overlap (front, resolve and shading on three streams) act at their place
    in submission order: the second draw sees the filled depth, and the
    download holds the planes after that draw, not after the one queued
    behind it. Overlap on and off give the same planes."""
    import srp_gb300
    L = api.L
    vp = ctypes.c_void_p
    L.srpGpuFramebufferFill.argtypes = [vp, ctypes.c_uint32, ctypes.c_float, ctypes.c_uint8, ctypes.c_uint]
    L.srpGpuFramebufferSyncAsync.argtypes = [vp]
    L.srpGpuSetDrawOverlap.argtypes = [ctypes.c_int]
    rng = np.random.default_rng(12)
    soups = [triangle_soup(rng, 3000) for _ in range(3)]
    results = []
    try:
        for overlap in (0, 1):
            L.srpGpuSetDrawOverlap(overlap)
            vbs = [api.vertex_buffer(t) for t in soups]
            fb = api.framebuffer(320, 240)
            for _ in range(2):
                L.srpFramebufferClear(fb)
                L.srpDrawVertexBuffer(vbs[0], fb, ctypes.byref(api.prog), SRP_PRIM_TRIANGLES, 0, soups[0].shape[0])
                L.srpGpuFramebufferFill(fb, 0, 0.25, 0, 2)  # depth plane only
                L.srpDrawVertexBuffer(vbs[1], fb, ctypes.byref(api.prog), SRP_PRIM_TRIANGLES, 0, soups[1].shape[0])
                L.srpGpuFramebufferSyncAsync(fb)
                L.srpDrawVertexBuffer(vbs[2], fb, ctypes.byref(api.prog), SRP_PRIM_TRIANGLES, 0, soups[2].shape[0])
            assert L.srpGpuSynchronize() == 0
            mid = srp_gb300.framebuffer_arrays(fb)
            end = api.planes(fb)
            assert not api.errors(), api.errors()
            results.append((mid, end))
    finally:
        L.srpGpuSetDrawOverlap(1)
    (mid0, end0), (mid1, end1) = results
    assert_same(mid1, mid0, "download between overlapped draws")
    assert_same(end1, end0, "planes after overlapped draws")
    # the download is not the final state: the third draw changed the image
    assert not np.array_equal(mid0[0], end0[0])
    # the fill took effect: pixels the second draw left alone hold its depth
    assert np.count_nonzero(mid0[1] == np.float32(0.25)) > 0


def test_batch_upload_of_a_repeated_buffer_keeps_the_last_copy(api):
    """srpGpuVertexBufferCopyDataBatchAsync given one buffer twice leaves it
    as two single calls would: holding the second copy."""
    L = api.L
    vp = ctypes.c_void_p
    L.srpGpuVertexBufferCopyDataBatchAsync.argtypes = [vp, vp, vp, vp, ctypes.c_size_t]
    rng = np.random.default_rng(14)
    a = np.ascontiguousarray(triangle_soup(rng, 800), dtype=np.float32)
    b = np.ascontiguousarray(triangle_soup(rng, 500), dtype=np.float32)
    vb = api.vertex_buffer(a)
    ref_vb = api.vertex_buffer(b)
    bufs = (vp * 2)(vb, vb)
    strides = (ctypes.c_size_t * 2)(a.shape[1] * 4, b.shape[1] * 4)
    sizes = (ctypes.c_size_t * 2)(a.nbytes, b.nbytes)
    datas = (vp * 2)(a.ctypes.data, b.ctypes.data)
    L.srpGpuVertexBufferCopyDataBatchAsync(ctypes.addressof(bufs), ctypes.addressof(strides), ctypes.addressof(sizes),
                                           ctypes.addressof(datas), 2)
    fb = api.framebuffer(256, 192)
    ref = api.framebuffer(256, 192)
    L.srpDrawVertexBuffer(vb, fb, ctypes.byref(api.prog), SRP_PRIM_TRIANGLES, 0, b.shape[0])
    L.srpDrawVertexBuffer(ref_vb, ref, ctypes.byref(api.prog), SRP_PRIM_TRIANGLES, 0, b.shape[0])
    got, want = api.planes(fb), api.planes(ref)
    assert not api.errors(), api.errors()
    assert_same(got, want, "repeated buffer in a batch upload")
    assert int(np.count_nonzero(want[0])) > 100
    assert L.srpGpuSynchronize() == 0
