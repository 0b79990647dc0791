"""srpGpuDrawFixedScratch, the draw that takes all of its scratch from one
fixed array in device memory, against the ordinary draw of the same inputs,
through the C ABI of libsrp_gb300.so.

The file is named so that pytest collects it last: it has to pass both on its
own in a fresh process (the first call then does the per-device set-up) and
after every other GPU test in the same process. Images must be bit-identical
to those of srpDrawIndexBuffer / srpDrawVertexBuffer, and the seeded scenes
drawn through it must match the reference's fixtures and the CPU oracle.
Callers that need it cannot have device memory allocated mid-frame, so one
test also checks that repeated calls leave the device's free memory as it
was."""
import ctypes
import glob
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SRP_FLOAT, SRP_UINT32 = 0, 8
SRP_INTERPOLATION_MODE_PERSPECTIVE = 0
SRP_PRIM_LINE_STRIP, SRP_PRIM_TRIANGLES = 2, 4


class VaryingInfo(ctypes.Structure):
    _fields_ = [("nItems", ctypes.c_size_t), ("type", ctypes.c_int), ("interpolationMode", ctypes.c_int)]


class VertexShader(ctypes.Structure):
    _fields_ = [("shader", ctypes.c_void_p), ("nVaryings", ctypes.c_size_t),
                ("varyingsInfo", ctypes.POINTER(VaryingInfo)), ("varyingsSize", ctypes.c_size_t)]


class FragmentShader(ctypes.Structure):
    _fields_ = [("shader", ctypes.c_void_p), ("mayOverwriteDepth", ctypes.c_bool)]


class ShaderProgram(ctypes.Structure):
    _fields_ = [("uniform", ctypes.c_void_p), ("vs", ctypes.POINTER(VertexShader)),
                ("fs", ctypes.POINTER(FragmentShader))]


class StdUniform(ctypes.Structure):
    """SRPStdUniform of srp/shaderlib.h."""
    _fields_ = [("model", ctypes.c_float * 16), ("view", ctypes.c_float * 16), ("projection", ctypes.c_float * 16),
                ("color", ctypes.c_float * 4), ("cameraPos", ctypes.c_float * 4),
                ("lightPos", ctypes.c_float * 64), ("lightColor", ctypes.c_float * 64), ("ambient", ctypes.c_float * 4),
                ("shininess", ctypes.c_float), ("marbleFrequency", ctypes.c_float), ("marbleGain", ctypes.c_float),
                ("depthScale", ctypes.c_float), ("depthBias", ctypes.c_float)] + \
               [(n, ctypes.c_uint32) for n in ("nLights", "marbleOctaves", "passOffset", "passCount", "normalOffset",
                                               "uvOffset", "extraOffset", "extraCount", "varyingOffset")] + \
               [("texelScale", ctypes.c_float), ("texture", ctypes.c_void_p)]


class Api:
    """The calls of this test, typed, plus a message log and a colour-varying
    shader program (srpVsTransform with identity matrices, srpFsVaryingColor)."""

    def __init__(self):
        import srp_gb300
        self.srp = srp_gb300
        L = srp_gb300.lib()
        vp = ctypes.c_void_p
        for name, res, args in [
            ("srpNewFramebuffer", vp, [ctypes.c_size_t, ctypes.c_size_t]),
            ("srpFreeFramebuffer", None, [vp]),
            ("srpFramebufferClear", None, [vp]),
            ("srpGpuFramebufferSync", None, [vp]),
            ("srpNewVertexBuffer", vp, []),
            ("srpFreeVertexBuffer", None, [vp]),
            ("srpVertexBufferCopyData", None, [vp, ctypes.c_size_t, ctypes.c_size_t, vp]),
            ("srpNewIndexBuffer", vp, []),
            ("srpFreeIndexBuffer", None, [vp]),
            ("srpIndexBufferCopyData", None, [vp, ctypes.c_int, ctypes.c_size_t, vp]),
            ("srpDrawVertexBuffer", None, [vp, vp, vp, ctypes.c_int, ctypes.c_size_t, ctypes.c_size_t]),
            ("srpDrawIndexBuffer", None, [vp, vp, vp, vp, ctypes.c_int, ctypes.c_size_t, ctypes.c_size_t]),
            ("srpGpuDrawFixedScratch", ctypes.c_int, [vp, vp, vp, vp, ctypes.c_int, ctypes.c_size_t, ctypes.c_size_t]),
            ("srpNewContext", None, [vp]),
            ("srpDepthTest", None, [ctypes.c_bool]),
        ]:
            f = getattr(L, name)
            f.restype, f.argtypes = res, args
        self.L = L
        ctx = ctypes.c_char.in_dll(L, "srpContext")
        L.srpNewContext(ctypes.addressof(ctx))
        self.messages = []
        self._cb = srp_gb300.MESSAGE_CALLBACK(
            lambda t, sev, fn, msg, user: self.messages.append((t, fn.decode(), msg.decode())))
        L.srpSetMessageCallback(srp_gb300.SRPMessageCallback(self._cb, None))
        L.srpDepthTest(True)
        u = StdUniform()
        for m in (u.model, u.view, u.projection):
            for i in range(4):
                m[5 * i] = 1.0
        u.passOffset, u.passCount = 3, 3
        self.uniform = u
        self.vinfo = (VaryingInfo * 1)(VaryingInfo(3, SRP_FLOAT, SRP_INTERPOLATION_MODE_PERSPECTIVE))
        self.vs = VertexShader(ctypes.cast(L.srpVsTransform, ctypes.c_void_p).value, 1, self.vinfo, 12)
        self.fs = FragmentShader(ctypes.cast(L.srpFsVaryingColor, ctypes.c_void_p).value, False)
        self.prog = ShaderProgram(ctypes.addressof(u), ctypes.pointer(self.vs), ctypes.pointer(self.fs))
        self.owned = []

    def errors(self):
        return [m for m in self.messages if m[0] == 0]  # SRP_MESSAGE_ERROR

    def framebuffer(self, w, h):
        fb = self.L.srpNewFramebuffer(w, h)
        assert fb, "srpNewFramebuffer failed"
        self.owned.append((self.L.srpFreeFramebuffer, fb))
        self.L.srpFramebufferClear(fb)
        return fb

    def vertex_buffer(self, verts):
        verts = np.ascontiguousarray(verts, dtype=np.float32)
        vb = self.L.srpNewVertexBuffer()
        self.owned.append((self.L.srpFreeVertexBuffer, vb))
        self.L.srpVertexBufferCopyData(vb, verts.shape[1] * 4, verts.nbytes, verts.ctypes.data)
        return vb

    def index_buffer(self, idx):
        idx = np.ascontiguousarray(idx, dtype=np.uint32)
        ib = self.L.srpNewIndexBuffer()
        self.owned.append((self.L.srpFreeIndexBuffer, ib))
        self.L.srpIndexBufferCopyData(ib, SRP_UINT32, idx.nbytes, idx.ctypes.data)
        return ib

    def planes(self, fb):
        self.L.srpGpuFramebufferSync(fb)
        c, d, s = self.srp.framebuffer_arrays(fb)
        return c, d.view(np.uint32), s

    def close(self):
        self.L.srpGpuSynchronize()
        for free, p in reversed(self.owned):
            free(p)
        self.owned = []
        # the ctypes thunk dies with this object: the library must not keep it
        self.L.srpSetMessageCallback(self.srp.SRPMessageCallback())


@pytest.fixture()
def api(built_library):
    a = Api()
    yield a
    a.close()


def triangle_soup(rng, n):
    """n small triangles, x/y in [-1.1, 1.1], z in [-1.1, 1.1] so that some
    are clipped; xyz then rgb per vertex."""
    centre = rng.uniform(-1.1, 1.1, size=(n, 1, 3))
    offs = rng.uniform(-0.06, 0.06, size=(n, 3, 3))
    pos = (centre + offs).reshape(-1, 3)
    rgb = rng.uniform(0.0, 1.0, size=(3 * n, 3))
    return np.concatenate([pos, rgb], axis=1)


def random_walk(rng, n):
    pos = np.cumsum(rng.uniform(-0.04, 0.04, size=(n, 3)), axis=0)
    pos = np.clip(pos, -0.95, 0.95)
    rgb = rng.uniform(0.0, 1.0, size=(n, 3))
    return np.concatenate([pos, rgb], axis=1)


def assert_same(a, b, what):
    for name, x, y in zip(("color", "depth", "stencil"), a, b):
        bad = np.flatnonzero(x != y)
        assert bad.size == 0, f"{what}: {name} differs at {bad.size} pixels (first {bad[:5]})"


@pytest.mark.parametrize("mode", [0, 1], ids=["coherent", "device"])
def test_fixed_scratch_matches_ordinary_draw(api, mode):
    """Two fixed-scratch draws in a row (indexed triangles, then a line strip
    over the first image) give exactly the images of the ordinary draws."""
    L = api.L
    L.srpGpuSetFramebufferMode(mode)
    rng = np.random.default_rng(20261204)
    W, H = 512, 384
    tris = triangle_soup(rng, 6000)
    perm = rng.permutation(tris.shape[0]).astype(np.uint32)
    tri_vb = api.vertex_buffer(tris[perm])
    tri_ib = api.index_buffer(np.argsort(perm).astype(np.uint32))
    walk = random_walk(rng, 3000)
    line_vb = api.vertex_buffer(walk)
    n_tri_idx, n_walk = tris.shape[0], walk.shape[0]

    ordinary = api.framebuffer(W, H)
    L.srpDrawIndexBuffer(tri_ib, tri_vb, ordinary, ctypes.byref(api.prog), SRP_PRIM_TRIANGLES, 0, n_tri_idx)
    want1 = api.planes(ordinary)
    L.srpDrawVertexBuffer(line_vb, ordinary, ctypes.byref(api.prog), SRP_PRIM_LINE_STRIP, 0, n_walk)
    want2 = api.planes(ordinary)
    assert not api.errors(), api.errors()

    fixed = api.framebuffer(W, H)
    rc1 = L.srpGpuDrawFixedScratch(tri_ib, tri_vb, fixed, ctypes.byref(api.prog), SRP_PRIM_TRIANGLES, 0, n_tri_idx)
    got1 = api.planes(fixed)
    rc2 = L.srpGpuDrawFixedScratch(None, line_vb, fixed, ctypes.byref(api.prog), SRP_PRIM_LINE_STRIP, 0, n_walk)
    got2 = api.planes(fixed)
    assert (rc1, rc2) == (0, 0), api.errors()
    assert not api.errors(), api.errors()
    assert L.srpGpuSynchronize() == 0

    drawn1 = int(np.count_nonzero(want1[1] != np.float32(-1.0).view(np.uint32)))
    assert drawn1 > 10000, "the triangle soup should cover a good part of the framebuffer"
    assert int(np.count_nonzero(want2[0] != want1[0])) > 1000, "the line strip should change the image"
    assert_same(got1, want1, "first call (indexed triangles)")
    assert_same(got2, want2, "second call (line strip)")


def test_fixed_scratch_rejects_oversized_draws(api):
    """Draws beyond the array are refused with a message and leave the
    framebuffer as it was; the next draw that fits is still exact."""
    L = api.L
    L.srpGpuSetFramebufferMode(1)
    rng = np.random.default_rng(7)
    W, H = 512, 384
    fb = api.framebuffer(W, H)
    before = api.planes(fb)

    # known before anything runs: per-vertex scratch for 1.2M vertices
    big_vb = api.vertex_buffer(np.zeros((1_200_000, 6), dtype=np.float32))
    rc = L.srpGpuDrawFixedScratch(None, big_vb, fb, ctypes.byref(api.prog), SRP_PRIM_TRIANGLES, 0, 3)
    errs = api.errors()
    assert rc == -1 and errs and "fixed scratch" in errs[-1][2], errs
    assert_same(api.planes(fb), before, "rejected draw (vertices)")

    # known after setup: 3000 half-screen triangles need ~5M tile entries
    half = np.array([[-1, -1], [1, -1], [-1, 1]], dtype=np.float32)
    n = 3000
    pos = np.tile(half, (n, 1))
    z = np.repeat(rng.uniform(-0.5, 0.5, size=n), 3)[:, None]
    verts = np.concatenate([pos, z, rng.uniform(0, 1, size=(3 * n, 3))], axis=1)
    vb = api.vertex_buffer(verts)
    api.messages.clear()
    rc = L.srpGpuDrawFixedScratch(None, vb, fb, ctypes.byref(api.prog), SRP_PRIM_TRIANGLES, 0, 3 * n)
    errs = api.errors()
    assert rc == -1 and errs and "tile entries" in errs[-1][2], errs
    assert_same(api.planes(fb), before, "rejected draw (tile entries)")

    # a draw that fits, after the rejected ones, matches the ordinary draw
    small = triangle_soup(rng, 2000)
    svb = api.vertex_buffer(small)
    ordinary = api.framebuffer(W, H)
    L.srpDrawVertexBuffer(svb, ordinary, ctypes.byref(api.prog), SRP_PRIM_TRIANGLES, 0, small.shape[0])
    api.messages.clear()
    rc = L.srpGpuDrawFixedScratch(None, svb, fb, ctypes.byref(api.prog), SRP_PRIM_TRIANGLES, 0, small.shape[0])
    assert rc == 0 and not api.errors(), api.errors()
    assert_same(api.planes(fb), api.planes(ordinary), "draw after rejections")
    assert L.srpGpuSynchronize() == 0


def test_fixed_scratch_between_overlapped_draws(api):
    """Ordinary draws overlap (the next draw's front stages beside the current
    draw's resolve); fixed-scratch draws interleaved with them, all into one
    framebuffer without waiting in between, give the image of the same
    sequence drawn strictly serially."""
    L = api.L
    L.srpGpuSetFramebufferMode(1)
    L.srpGpuSetDrawOverlap.argtypes = [ctypes.c_int]
    rng = np.random.default_rng(99)
    W, H = 512, 384
    tris = [api.vertex_buffer(triangle_soup(rng, 3000)) for _ in range(3)]
    walk = api.vertex_buffer(random_walk(rng, 2000))

    def sequence(fb):
        L.srpDrawVertexBuffer(tris[0], fb, ctypes.byref(api.prog), SRP_PRIM_TRIANGLES, 0, 9000)
        assert L.srpGpuDrawFixedScratch(None, walk, fb, ctypes.byref(api.prog), SRP_PRIM_LINE_STRIP, 0, 2000) == 0
        L.srpDrawVertexBuffer(tris[1], fb, ctypes.byref(api.prog), SRP_PRIM_TRIANGLES, 0, 9000)
        L.srpDrawVertexBuffer(walk, fb, ctypes.byref(api.prog), SRP_PRIM_LINE_STRIP, 0, 2000)
        assert L.srpGpuDrawFixedScratch(None, tris[2], fb, ctypes.byref(api.prog), SRP_PRIM_TRIANGLES, 0, 9000) == 0
        L.srpDrawVertexBuffer(tris[2], fb, ctypes.byref(api.prog), SRP_PRIM_LINE_STRIP, 0, 9000)
        return api.planes(fb)

    try:
        L.srpGpuSetDrawOverlap(0)
        want = sequence(api.framebuffer(W, H))
        L.srpGpuSetDrawOverlap(1)
        got = sequence(api.framebuffer(W, H))
        got2 = sequence(api.framebuffer(W, H))
    finally:
        L.srpGpuSetDrawOverlap(1)
    assert not api.errors(), api.errors()
    assert_same(got, want, "overlapped sequence")
    assert_same(got2, want, "overlapped sequence, graphs replayed")
    assert L.srpGpuSynchronize() == 0


# ------------------------------------------------- seeded scenes, oracle


def render_fixed(name, seed, scale):
    """One frame of a seeded scene with every draw through
    srpGpuDrawFixedScratch; returns the planes and the rejected-draw count."""
    import srp_gb300
    L, S = srp_gb300.lib(), srp_gb300.scenes()
    S.sceneUseFixedScratch.argtypes = [ctypes.c_int]
    S.sceneFixedScratchRejected.restype = ctypes.c_int
    L.srpGpuSetFramebufferMode(srp_gb300.SRP_GPU_FB_DEVICE)
    sc = srp_gb300.Scene(name, seed, scale)
    try:
        sc.prepare()
        S.sceneUseFixedScratch(1)
        try:
            sc.render()
            rejected = S.sceneFixedScratchRejected()
        finally:
            S.sceneUseFixedScratch(0)
        c, d, st = sc.planes()
        assert L.srpGpuSynchronize() == 0
        return {"color": c, "depth_bits": d.view(np.uint32), "stencil": st, "hash": int(sc.input_hash)}, rejected
    finally:
        sc.close()


# points, wireframe and point polygon modes, the late-depth resolve, large
# triangles with barycentric tables, every varying type, strips and fans
FIXED_SCENES = ["varyings", "poly_modes", "late_z", "points", "clip_tris", "raster_rules", "interp", "stencil",
                "topologies", "sphere"]
# draws a scene makes on purpose out of range, which both draws reject
EXPECTED_REJECTIONS = {"topologies": 1}


@pytest.mark.parametrize("scene", FIXED_SCENES)
def test_fixed_scratch_matches_reference_fixtures(built_library, scene):
    """Scenes whose every draw is a fixed-scratch draw equal the reference's
    own renderings (depth and stencil bit-exact, colour within 1/255)."""
    from oracle_util import manifest, load_golden, compare_planes
    cases = [c for c in manifest() if c["scene"] == scene]
    assert cases
    for case in cases:
        got, rejected = render_fixed(case["scene"], case["seed"], case["scale"])
        assert rejected == EXPECTED_REJECTIONS.get(scene, 0)
        assert str(got["hash"]) == case["input_hash"]
        compare_planes(got, load_golden(case), case["name"] + " (fixed scratch)")


@pytest.mark.parametrize("scene,scale", [("varyings", 1.0), ("poly_modes", 1.0), ("late_z", 1.0), ("clip_lines", 1.0),
                                         ("soup", 0.03)])
def test_fixed_scratch_matches_oracle(built_library, oracle_exe, scene, scale):
    from oracle_util import oracle_render, compare_planes
    want = oracle_render(oracle_exe, scene, 4, scale)
    got, rejected = render_fixed(scene, 4, scale)
    assert rejected == 0
    assert got["hash"] == want["hash"]
    compare_planes(got, want, f"{scene} seed 4 (fixed scratch)")


def cudart():
    """The CUDA runtime as a shared library, for cudaMemGetInfo and stream
    capture (the GPU library links its own static copy)."""
    cands = ["libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"]
    cands += glob.glob("/usr/local/lib/python3*/dist-packages/nvidia/cu13/lib/libcudart.so.13")
    for c in cands:
        try:
            return ctypes.CDLL(c)
        except OSError:
            continue
    pytest.fail("no libcudart shared library found")


def free_device_bytes(rt):
    free, total = ctypes.c_size_t(), ctypes.c_size_t()
    assert rt.cudaMemGetInfo(ctypes.byref(free), ctypes.byref(total)) == 0
    return free.value


def test_fixed_scratch_allocates_nothing(built_library):
    """After a first pass (which loads the array's device image), further
    fixed-scratch frames of several scenes leave the device's free memory
    exactly as it was: no call allocates or frees device memory."""
    import srp_gb300
    L, S = srp_gb300.lib(), srp_gb300.scenes()
    S.sceneUseFixedScratch.argtypes = [ctypes.c_int]
    S.sceneFixedScratchRejected.restype = ctypes.c_int
    rt = cudart()
    L.srpGpuSetFramebufferMode(srp_gb300.SRP_GPU_FB_DEVICE)
    scs = [srp_gb300.Scene(n, 6, x) for n, x in (("varyings", 1.0), ("poly_modes", 1.0), ("late_z", 1.0),
                                                   ("soup", 0.03), ("clip_lines", 1.0))]
    try:
        frees = []
        for rep in range(3):
            for sc in scs:
                sc.prepare()
            assert L.srpGpuSynchronize() == 0
            frees.append(free_device_bytes(rt))
            S.sceneUseFixedScratch(1)
            try:
                for sc in scs:
                    sc.render()
                assert S.sceneFixedScratchRejected() == 0
            finally:
                S.sceneUseFixedScratch(0)
            assert L.srpGpuSynchronize() == 0
            frees.append(free_device_bytes(rt))
        # the first pass may load the array's device image; none after it moves memory
        assert len(set(frees[1:])) == 1, frees
    finally:
        for sc in scs:
            sc.close()


def test_fixed_scratch_large_triangles(api):
    """A few triangles covering the whole framebuffer go through the
    barycentric-table path of large primitives; the images equal the
    ordinary draw's."""
    L = api.L
    L.srpGpuSetFramebufferMode(1)
    rng = np.random.default_rng(31)
    W, H = 640, 480
    n = 12
    pos = rng.uniform(-3.0, 3.0, size=(3 * n, 2))
    z = np.repeat(rng.uniform(-0.9, 0.9, size=n), 3)[:, None] + rng.uniform(-0.05, 0.05, size=(3 * n, 1))
    verts = np.concatenate([pos, z, rng.uniform(0, 1, size=(3 * n, 3))], axis=1)
    vb = api.vertex_buffer(verts)
    ordinary, fixed = api.framebuffer(W, H), api.framebuffer(W, H)
    L.srpDrawVertexBuffer(vb, ordinary, ctypes.byref(api.prog), SRP_PRIM_TRIANGLES, 0, 3 * n)
    assert L.srpGpuDrawFixedScratch(None, vb, fixed, ctypes.byref(api.prog), SRP_PRIM_TRIANGLES, 0, 3 * n) == 0
    want, got = api.planes(ordinary), api.planes(fixed)
    assert not api.errors(), api.errors()
    assert int(np.count_nonzero(want[1] != np.float32(-1.0).view(np.uint32))) > W * H // 2
    assert_same(got, want, "full-screen triangles")


def test_fixed_scratch_ignores_learned_shading(built_library):
    """With learned shading set, the ordinary draw shades with the network,
    while the fixed-scratch draw runs the program's own shader: its image is
    the plain draw's."""
    import srp_gb300
    L, S = srp_gb300.lib(), srp_gb300.scenes()
    vp = ctypes.c_void_p
    L.srpGpuMlpCreate.restype = vp
    L.srpGpuMlpCreate.argtypes = [ctypes.c_uint64, ctypes.c_size_t]
    L.srpGpuMlpFree.argtypes = [vp]
    L.srpGpuSetLearnedShading.argtypes = [vp, vp, ctypes.c_float, ctypes.c_uint32]
    S.sceneUseFixedScratch.argtypes = [ctypes.c_int]
    S.sceneFixedScratchRejected.restype = ctypes.c_int
    L.srpGpuSetFramebufferMode(srp_gb300.SRP_GPU_FB_DEVICE)
    marble = ctypes.cast(L.srpFsMarble, vp)
    net = L.srpGpuMlpCreate(3, 1 << 10)
    sc = srp_gb300.Scene("msoup", 12, 0.03)
    try:
        sc.prepare()
        sc.render()
        plain = [a.copy() for a in sc.planes()]
        L.srpGpuSetLearnedShading(marble, net, 0.0, 16)
        sc.prepare()
        sc.render()
        learned = sc.planes()
        sc.prepare()
        S.sceneUseFixedScratch(1)
        try:
            sc.render()
            assert S.sceneFixedScratchRejected() == 0
        finally:
            S.sceneUseFixedScratch(0)
        fixed = sc.planes()
    finally:
        L.srpGpuSetLearnedShading(None, None, 0.0, 0)
        sc.close()
        L.srpGpuMlpFree(net)
    assert L.srpGpuSynchronize() == 0
    assert (learned[0] != plain[0]).any(), "the untrained network should change the colours"
    for a, b in zip(fixed, plain):
        assert np.array_equal(a, b)


def test_fixed_scratch_refuses_stream_capture(api):
    """A call while the library's stream is being captured is rejected before
    anything is queued: the capture ends with an empty graph and stays valid,
    and the framebuffer is unchanged."""
    L = api.L
    rt = cudart()
    L.srpGpuSetFramebufferMode(1)
    rng = np.random.default_rng(5)
    vb = api.vertex_buffer(triangle_soup(rng, 200))
    fb = api.framebuffer(256, 192)
    before = api.planes(fb)
    stream = ctypes.c_void_p()
    assert rt.cudaStreamCreateWithFlags(ctypes.byref(stream), 1) == 0  # cudaStreamNonBlocking
    graph = ctypes.c_void_p()
    nodes = ctypes.c_size_t(1)
    try:
        L.srpGpuSetStream(stream)
        assert rt.cudaStreamBeginCapture(stream, 2) == 0  # cudaStreamCaptureModeRelaxed
        rc = L.srpGpuDrawFixedScratch(None, vb, fb, ctypes.byref(api.prog), SRP_PRIM_TRIANGLES, 0, 600)
        assert rt.cudaStreamEndCapture(stream, ctypes.byref(graph)) == 0
        assert rt.cudaGraphGetNodes(graph, None, ctypes.byref(nodes)) == 0
    finally:
        if graph.value:
            rt.cudaGraphDestroy(graph)
        L.srpGpuSetStream(None)
        rt.cudaStreamSynchronize(stream)
        rt.cudaStreamDestroy(stream)
    errs = api.errors()
    assert rc == -1 and errs and "captured" in errs[-1][2], errs
    assert nodes.value == 0
    assert_same(api.planes(fb), before, "rejected during capture")
    # the next call outside a capture draws as usual
    api.messages.clear()
    assert L.srpGpuDrawFixedScratch(None, vb, fb, ctypes.byref(api.prog), SRP_PRIM_TRIANGLES, 0, 600) == 0
    assert not api.errors(), api.errors()
    assert L.srpGpuSynchronize() == 0
