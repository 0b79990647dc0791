"""srpGpuDrawBatch: scenes of the batched workload (one textured, lit mesh
each, framebuffers of different sizes) rendered by multi-draw passes must be
bit-identical to the same scenes drawn one by one with srpDrawIndexBuffer, and
match the CPU oracle. All calls go through the C API of libsrp_gb300.so."""
import ctypes

import numpy as np
import pytest

from oracle_util import oracle_render, compare_planes

pytestmark = pytest.mark.gpu

BASE = 11


def make_scenes(n, scale):
    import srp_gb300
    return [srp_gb300.Scene("bscene", srp_gb300.batch_seed(BASE, i), scale) for i in range(n)]


def sync_planes(srp_gb300, S, fb):
    S.srpGpuFramebufferSync(fb)
    c, d, s = srp_gb300.framebuffer_arrays(fb)
    return c, d.view(np.uint32), s


@pytest.mark.parametrize("mode", [1, 0], ids=["device", "coherent"])
def test_batch_matches_single_draws(built_library, mode):
    import srp_gb300
    L = srp_gb300.lib()
    S = srp_gb300.scenes()
    L.srpGpuSetFramebufferMode(mode)
    scenes = make_scenes(40, 0.25)
    try:
        want = []
        for sc in scenes:
            sc.prepare()
            sc.render()
            want.append(sync_planes(srp_gb300, S, sc.fb))
        fbs = []
        for sc in scenes:
            fb = S.srpNewFramebuffer(sc.info.width, sc.info.height)
            S.scenePrepareFramebuffer(sc.ptr, fb)
            fbs.append(fb)
        L.srpGpuResetStats()
        srp_gb300.render_batch(scenes, fbs)
        st = srp_gb300.SRPGpuStats()
        L.srpGpuGetStats(ctypes.byref(st))
        assert L.srpGpuSynchronize() == 0
        assert st.draws == len(scenes)
        drawn = 0
        for i, (sc, fb) in enumerate(zip(scenes, fbs)):
            got = sync_planes(srp_gb300, S, fb)
            for name, a, b in zip(("color", "depth", "stencil"), got, want[i]):
                bad = np.flatnonzero(a != b)
                assert bad.size == 0, f"scene {i}: {name} differs at {bad.size} pixels"
            drawn += int(np.count_nonzero(want[i][1] != np.float32(1.0).view(np.uint32)))
        assert drawn > 10000, "the batch should cover pixels"
    finally:
        for fb in locals().get("fbs", []):
            S.srpFreeFramebuffer(fb)
        for sc in scenes:
            sc.close()


def test_batch_shared_framebuffer_and_order(built_library):
    """Draws that share a framebuffer split the pass and keep their order."""
    import srp_gb300
    L = srp_gb300.lib()
    S = srp_gb300.scenes()
    L.srpGpuSetFramebufferMode(1)
    scenes = make_scenes(9, 0.2)
    try:
        order = [0, 1, 2, 2, 3, 4, 4, 4, 5]   # framebuffer of each draw
        fb_sizes = {}
        for k, sc in zip(order, scenes):
            fb_sizes.setdefault(k, (sc.info.width, sc.info.height))
        def fresh():
            out = {}
            for k, (w, h) in fb_sizes.items():
                fb = S.srpNewFramebuffer(w, h)
                S.scenePrepareFramebuffer(scenes[order.index(k)].ptr, fb)
                out[k] = fb
            return out
        ref = fresh()
        for k, sc in zip(order, scenes):
            S.sceneRender(sc.ptr, ref[k])
        got = fresh()
        srp_gb300.render_batch(scenes, [got[k] for k in order])
        assert L.srpGpuSynchronize() == 0
        for k in fb_sizes:
            a = sync_planes(srp_gb300, S, got[k])
            b = sync_planes(srp_gb300, S, ref[k])
            for name, x, y in zip(("color", "depth", "stencil"), a, b):
                assert np.array_equal(x, y), f"framebuffer {k}: {name} differs"
        for fb in list(ref.values()) + list(got.values()):
            S.srpFreeFramebuffer(fb)
    finally:
        for sc in scenes:
            sc.close()


@pytest.mark.parametrize("i", [0, 3, 7, 12, 21, 30])
def test_batch_scene_matches_oracle(built_library, oracle_exe, i):
    """Scenes of a batch against the oracle's rendering of the same scene."""
    import srp_gb300
    L = srp_gb300.lib()
    S = srp_gb300.scenes()
    L.srpGpuSetFramebufferMode(1)
    scenes = make_scenes(32, 0.25)
    try:
        fbs = [S.srpNewFramebuffer(sc.info.width, sc.info.height) for sc in scenes]
        for sc, fb in zip(scenes, fbs):
            S.scenePrepareFramebuffer(sc.ptr, fb)
        srp_gb300.render_batch(scenes, fbs)
        c, d, s = sync_planes(srp_gb300, S, fbs[i])
        want = oracle_render(oracle_exe, "bscene", srp_gb300.batch_seed(BASE, i), 0.25)
        assert want["hash"] == scenes[i].input_hash
        got = {"color": c, "depth_bits": d, "stencil": s, "width": scenes[i].info.width,
               "height": scenes[i].info.height}
        compare_planes(got, want, f"batch scene {i}")
        for fb in fbs:
            S.srpFreeFramebuffer(fb)
    finally:
        for sc in scenes:
            sc.close()


def test_autotune_keeps_results_exact(built_library):
    """The autotuner picks a resolve tuning; any tuning renders the same images."""
    import srp_gb300
    L = srp_gb300.lib()
    S = srp_gb300.scenes()
    L.srpGpuSetFramebufferMode(1)
    L.srpGpuGetTuning.argtypes = [ctypes.POINTER(srp_gb300.SRPGpuTuning)]
    L.srpGpuSetTuning.argtypes = [ctypes.POINTER(srp_gb300.SRPGpuTuning)]
    scenes = make_scenes(12, 0.3)
    default = srp_gb300.SRPGpuTuning()
    L.srpGpuGetTuning(ctypes.byref(default))
    try:
        fbs = [sc.fb for sc in scenes]

        def render():
            for sc in scenes:
                sc.prepare()
            srp_gb300.render_batch(scenes, fbs)
            return [sync_planes(srp_gb300, S, fb) for fb in fbs]

        want = render()
        for sc in scenes:
            sc.prepare()
        best = srp_gb300.autotune_batch(scenes, fbs, 1)
        assert best.heavyItems in (32, 64, 96, 192, 384) and 1 <= best.heavyCtasPerSM <= 3
        for tune in [(best.heavyItems, best.heavyCtasPerSM), (1, 1), (100000, 2)]:
            L.srpGpuSetTuning(ctypes.byref(srp_gb300.SRPGpuTuning(*tune)))
            got = render()
            for a, b in zip(got, want):
                for x, y in zip(a, b):
                    assert np.array_equal(x, y), tune
    finally:
        L.srpGpuSetTuning(ctypes.byref(default))
        for sc in scenes:
            sc.close()
    assert L.srpGpuSynchronize() == 0


def test_frame_autotuner_ends_and_keeps_results_exact(built_library):
    """The online frame autotuner ends 60 frames after its first call with a candidate tuning;
    the frames it renders meanwhile are the same as the default tuning's."""
    import srp_gb300
    L = srp_gb300.lib()
    S = srp_gb300.scenes()
    L.srpGpuSetFramebufferMode(1)
    L.srpGpuGetTuning.argtypes = [ctypes.POINTER(srp_gb300.SRPGpuTuning)]
    L.srpGpuSetTuning.argtypes = [ctypes.POINTER(srp_gb300.SRPGpuTuning)]
    scenes = make_scenes(4, 0.3)
    default = srp_gb300.SRPGpuTuning()
    L.srpGpuGetTuning(ctypes.byref(default))
    try:
        fbs = [sc.fb for sc in scenes]

        def render():
            for sc in scenes:
                sc.prepare()
            srp_gb300.render_batch(scenes, fbs)
            return [sync_planes(srp_gb300, S, fb) for fb in fbs]

        want = render()
        L.srpGpuAutotuneReset()
        frames = 0
        while True:
            got = render()
            for a, b in zip(got, want):
                for x, y in zip(a, b):
                    assert np.array_equal(x, y), frames
            frames += 1
            if not L.srpGpuAutotuneFrame():
                break
            assert frames <= 61
        assert frames == 61
        best = srp_gb300.SRPGpuTuning()
        L.srpGpuGetTuning(ctypes.byref(best))
        assert best.heavyItems in (32, 64, 96, 192, 384) and 1 <= best.heavyCtasPerSM <= 3
        assert L.srpGpuAutotuneFrame() == 0
    finally:
        L.srpGpuAutotuneReset()
        L.srpGpuSetTuning(ctypes.byref(default))
        for sc in scenes:
            sc.close()
    assert L.srpGpuSynchronize() == 0


@pytest.mark.parametrize("calls", ["per_buffer", "batch"])
def test_async_transfers_and_fill_batch_match_the_synchronous_path(built_library, calls):
    """Stream-ordered uploads, one batched framebuffer fill and stream-ordered
    downloads (one wait in all) give the images of the synchronous calls, with
    one call per buffer and with the Batch calls (gather kernels)."""
    import srp_gb300
    L = srp_gb300.lib()
    S = srp_gb300.scenes()
    L.srpGpuSetFramebufferMode(1)
    scenes = make_scenes(6, 0.3)
    try:
        fbs = [sc.fb for sc in scenes]
        for sc in scenes:
            sc.upload()
            sc.prepare()
        srp_gb300.render_batch(scenes, fbs)
        want = [sync_planes(srp_gb300, S, fb) for fb in fbs]
        # scribble over the device and host planes, then the asynchronous round trip
        for fb in fbs:
            S.srpGpuFramebufferFill(ctypes.c_void_p(fb), ctypes.c_uint32(0x12345678), ctypes.c_float(0.25),
                                    ctypes.c_uint8(7), 7)
            v = ctypes.cast(fb, ctypes.POINTER(srp_gb300.FramebufferView)).contents
            ctypes.memset(v.color, 0xAB, 4 * v.size)
            ctypes.memset(v.depth, 0xAB, 4 * v.size)
            ctypes.memset(v.stencil, 0xAB, v.size)
        if calls == "batch":
            srp_gb300.upload_batch(scenes)
        else:
            for sc in scenes:
                sc.upload_async()
        srp_gb300.prepare_batch(scenes, fbs)
        srp_gb300.render_batch(scenes, fbs)
        if calls == "batch":
            srp_gb300.sync_batch(fbs)
        else:
            for sc in scenes:
                sc.sync_async()
        # framebuffer work queued right behind the downloads waits for them
        for fb in fbs:
            S.srpGpuFramebufferFill(ctypes.c_void_p(fb), ctypes.c_uint32(0x12345678), ctypes.c_float(0.25),
                                    ctypes.c_uint8(7), 7)
        assert L.srpGpuSynchronize() == 0
        for fb, w in zip(fbs, want):
            c, d, st = srp_gb300.framebuffer_arrays(fb)
            for x, y in zip((c, d.view(np.uint32), st), w):
                assert np.array_equal(x, y)
    finally:
        for sc in scenes:
            sc.close()
    assert L.srpGpuSynchronize() == 0


def test_overlapped_passes_match_serial_passes(built_library):
    """A batch of more than 1024 draws runs as several passes whose front
    stages overlap the previous pass's resolve and shading (two scratch sets);
    its images equal those of the same batch drawn with every stage on one
    stream, also when the graphs are replayed."""
    import srp_gb300
    L = srp_gb300.lib()
    S = srp_gb300.scenes()
    L.srpGpuSetFramebufferMode(1)
    scenes = make_scenes(1100, 0.1)
    try:
        fbs = [sc.fb for sc in scenes]

        def render():
            srp_gb300.prepare_batch(scenes, fbs)
            srp_gb300.render_batch(scenes, fbs)
            return [sync_planes(srp_gb300, S, fb) for fb in fbs]

        L.srpGpuSetDrawOverlap(0)
        want = render()
        L.srpGpuSetDrawOverlap(1)
        for _ in range(2):
            got = render()
            for i, (a, b) in enumerate(zip(got, want)):
                for x, y in zip(a, b):
                    assert np.array_equal(x, y), i
        # gathered downloads: one kernel per pass, each after its own pass,
        # into host arrays scribbled over first
        for fb in fbs:
            v = ctypes.cast(fb, ctypes.POINTER(srp_gb300.FramebufferView)).contents
            ctypes.memset(v.color, 0xAB, 9 * v.size)
        srp_gb300.prepare_batch(scenes, fbs)
        srp_gb300.render_batch(scenes, fbs)
        srp_gb300.sync_batch(fbs)
        assert L.srpGpuSynchronize() == 0
        for i, (fb, b) in enumerate(zip(fbs, want)):
            c, d, st = srp_gb300.framebuffer_arrays(fb)
            for x, y in zip((c, d.view(np.uint32), st), b):
                assert np.array_equal(x, y), i
    finally:
        L.srpGpuSetDrawOverlap(1)
        for sc in scenes:
            sc.close()
    assert L.srpGpuSynchronize() == 0


def test_async_uploads_into_buffers_earlier_draws_read(built_library):
    """Stream-ordered uploads do not wait for earlier draws: every draw call
    returns only after its setup has read the vertex and index buffers. Three
    frames drawn from one vertex buffer and one index buffer, each refilled
    with srpGpu*CopyDataAsync before its draw, with one srpGpuSynchronize at
    the end, give the images of the synchronous calls."""
    import srp_gb300
    import srpapi as A
    L = srp_gb300.lib()
    L.srpGpuVertexBufferCopyDataAsync.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_void_p]
    L.srpGpuIndexBufferCopyDataAsync.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t, ctypes.c_void_p]
    L.srpGpuFramebufferSyncAsync.argtypes = [ctypes.c_void_p]
    L.srpGpuFramebufferSync.argtypes = [ctypes.c_void_p]
    rng = np.random.default_rng(77)
    n, W, H = 20000, 640, 360
    frames = []
    for _ in range(3):
        centre = rng.uniform(-1.1, 1.1, size=(n, 1, 3))
        verts = np.concatenate([(centre + rng.uniform(-0.06, 0.06, size=(n, 3, 3))).reshape(-1, 3),
                                rng.uniform(0, 1, size=(3 * n, 3))], axis=1).astype(np.float32)
        frames.append((verts, rng.permutation(3 * n).astype(np.uint32)))
    srp = A.Srp(srp_gb300.library_path())
    L.srpGpuSetFramebufferMode(srp_gb300.SRP_GPU_FB_DEVICE)
    try:
        srp.srpDepthTest(True)
        u = A.StdUniform()
        u.model = u.view = u.projection = srp.mat4ConstructIdentity()
        u.passOffset, u.passCount = 3, 3
        sp = srp.program(u, "srpVsTransform", "srpFsVaryingColor", [(3, A.FLOAT, A.INTERP_PERSPECTIVE)], 12)
        fbs = [srp.srpNewFramebuffer(W, H) for _ in frames]
        vb = srp.srpNewVertexBuffer()
        ib = srp.srpNewIndexBuffer()

        def draw(k):
            srp.srpFramebufferClear(fbs[k])
            srp.srpDrawIndexBuffer(ib, vb, fbs[k], ctypes.byref(sp), A.PRIM_TRIANGLES, 0, 3 * n)

        want = []
        for k, (verts, idx) in enumerate(frames):
            srp.srpVertexBufferCopyData(vb, 24, verts.nbytes, verts.ctypes.data)
            srp.srpIndexBufferCopyData(ib, A.UINT32, idx.nbytes, idx.ctypes.data)
            draw(k)
            L.srpGpuFramebufferSync(fbs[k])
            want.append(srp.planes(fbs[k]))
        for fb in fbs:
            srp.srpFramebufferClear(fb)
            L.srpGpuFramebufferSync(fb)
        for k, (verts, idx) in enumerate(frames):
            L.srpGpuVertexBufferCopyDataAsync(vb, 24, verts.nbytes, verts.ctypes.data)
            L.srpGpuIndexBufferCopyDataAsync(ib, A.UINT32, idx.nbytes, idx.ctypes.data)
            draw(k)
            L.srpGpuFramebufferSyncAsync(fbs[k])
        assert L.srpGpuSynchronize() == 0
        got = [srp.planes(fb) for fb in fbs]
        assert not srp.errors()
        srp.srpFreeVertexBuffer(vb)
        srp.srpFreeIndexBuffer(ib)
        for fb in fbs:
            srp.srpFreeFramebuffer(fb)
    finally:
        srp.close()
    for k, (a, b) in enumerate(zip(got, want)):
        assert int((b[1] != np.float32(-1.0)).sum()) > 20000, k
        for x, y in zip(a, b):
            assert np.array_equal(x, y), k
    assert not np.array_equal(want[0][0], want[1][0])
