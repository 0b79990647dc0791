"""GPU draw path against the reference (committed fixtures rendered by the
reference library) and against the CPU oracle at other seeds and full size.
Coverage, depth and stencil must be bit-exact; colour within 1/255 per
channel. Every call goes through the srp C API of libsrp_gb300.so."""
import numpy as np
import pytest

from oracle_util import manifest, load_golden, oracle_render, compare_planes, hash_cases, plane_digests

pytestmark = pytest.mark.gpu


def gpu_render(name, seed, scale):
    import srp_gb300
    c, d, s, w, h, st, hsh = srp_gb300.render_scene(name, seed, scale)
    return {"color": c, "depth_bits": d.view("uint32"), "stencil": s, "width": w, "height": h,
            "fragments": int(st.fragments), "hash": int(hsh), "stats": st}


@pytest.mark.parametrize("case", manifest(), ids=lambda c: c["name"])
def test_gpu_matches_reference_fixture(built_library, case):
    got = gpu_render(case["scene"], case["seed"], case["scale"])
    assert str(got["hash"]) == case["input_hash"], "scene inputs differ from the fixture's"
    compare_planes(got, load_golden(case), case["name"])
    assert got["fragments"] == case["fragments"]


SEEDED = [(n, seed, scale) for n, scale in [
    ("sphere", 0.5), ("soup", 0.02), ("clip_tris", 1.0), ("clip_lines", 1.0), ("points", 1.0),
    ("interp", 1.0), ("depth_ops", 1.0), ("raster_rules", 1.0), ("scissor", 1.0), ("stencil", 1.0),
    ("poly_modes", 1.0), ("topologies", 1.0), ("late_z", 1.0), ("lit", 1.0), ("varyings", 1.0),
    ("texfilter", 1.0)]
    for seed in (2, 5)]


@pytest.mark.parametrize("scene,seed,scale", SEEDED)
def test_gpu_matches_oracle(built_library, oracle_exe, scene, seed, scale):
    want = oracle_render(oracle_exe, scene, seed, scale)
    got = gpu_render(scene, seed, scale)
    assert got["hash"] == want["hash"]
    compare_planes(got, want, f"{scene} seed {seed}")
    assert got["fragments"] == want["fragments"]


@pytest.mark.parametrize("scene,seed", [("sphere", 11), ("soup", 1)])
def test_full_size_configs_match_oracle(built_library, oracle_exe, scene, seed):
    """The two single-frame configurations at full size: UV sphere 512x512 and
    the ~2M-triangle soup at 1920x1080 with lines and points."""
    want = oracle_render(oracle_exe, scene, seed, 1.0)
    got = gpu_render(scene, seed, 1.0)
    compare_planes(got, want, f"{scene} full size")
    assert got["fragments"] == want["fragments"]


@pytest.mark.parametrize("case", hash_cases(), ids=lambda c: c["name"])
def test_full_size_bench_frame_matches_reference_digests(built_library, oracle_exe, case):
    """The frame bench.py times, against digests of the reference's own
    rendering: depth and stencil hash to the reference's planes; colour is
    within 1/255 of the oracle, whose colour plane hashes to the reference's."""
    got = gpu_render(case["scene"], case["seed"], case["scale"])
    assert str(got["hash"]) == case["input_hash"], "scene inputs differ from the reference's"
    dg = plane_digests(got)
    assert dg["depth_bits"] == case["sha256"]["depth_bits"], "depth differs from the reference's"
    assert dg["stencil"] == case["sha256"]["stencil"], "stencil differs from the reference's"
    assert got["fragments"] == case["fragments"]
    if dg["color"] != case["sha256"]["color"]:
        want = oracle_render(oracle_exe, case["scene"], case["seed"], case["scale"])
        assert plane_digests(want)["color"] == case["sha256"]["color"]
        compare_planes(got, want, case["name"])


@pytest.mark.parametrize("scene,scale", [("soup", 0.02), ("lit", 1.0), ("stencil", 1.0)])
def test_graph_replay_matches_direct_launches(built_library, scene, scale):
    """A repeated draw replays its captured CUDA graphs; the images equal those
    of the same draws launched directly."""
    import srp_gb300
    L = srp_gb300.lib()
    S = srp_gb300.scenes()
    L.srpGpuSetFramebufferMode(srp_gb300.SRP_GPU_FB_DEVICE)
    sc = srp_gb300.Scene(scene, 9, scale)
    try:
        frames = []
        for graphs in (1, 1, 0):
            L.srpGpuSetDrawGraphs(graphs)
            sc.prepare()
            sc.render()
            frames.append(sc.planes())
        assert L.srpGpuSynchronize() == 0
        for f in frames[1:]:
            for a, b in zip(f, frames[0]):
                assert np.array_equal(a, b)
    finally:
        L.srpGpuSetDrawGraphs(1)
        sc.close()


@pytest.mark.gpu
@pytest.mark.parametrize("scene,scale", [("soup", 0.5), ("clip_tris", 1.0), ("topologies", 1.0), ("late_z", 1.0)])
def test_overlapped_draws_match_serial_draws(built_library, scene, scale):
    """Consecutive draws overlap (front stages of draw N+1 beside the resolve
    and shading of draw N, two scratch sets); frames rendered that way, with
    and without graph replay, equal the frames of strictly serial draws."""
    import srp_gb300
    L = srp_gb300.lib()
    L.srpGpuSetFramebufferMode(srp_gb300.SRP_GPU_FB_DEVICE)
    sc = srp_gb300.Scene(scene, 11, scale)
    try:
        frames = []
        for overlap, graphs in ((0, 0), (1, 0), (1, 1), (1, 1), (1, 1)):
            L.srpGpuSetDrawOverlap(overlap)
            L.srpGpuSetDrawGraphs(graphs)
            sc.prepare()
            sc.render()
            frames.append(sc.planes())
        # frames back to back, with no wait in between: each draw's resolve
        # and lambda tables may queue behind the previous draw's work while
        # the next fronts already run
        for graphs in (0, 1):
            L.srpGpuSetDrawGraphs(graphs)
            for _ in range(4):
                sc.prepare()
                sc.render()
            frames.append(sc.planes())
        assert L.srpGpuSynchronize() == 0
        for f in frames[1:]:
            for a, b in zip(f, frames[0]):
                assert np.array_equal(a, b)
    finally:
        L.srpGpuSetDrawOverlap(1)
        L.srpGpuSetDrawGraphs(1)
        sc.close()


TILE_COPY_DEFAULT = 0  # the library's default: no tile copies


@pytest.mark.parametrize("scene,scale", [("soup", 0.1), ("stencil", 1.0), ("points", 1.0), ("varyings", 1.0),
                                         ("sphere", 1.0), ("interp", 1.0)])
def test_tma_tile_copies_match_direct_access(built_library, scene, scale):
    """With the tile copies by TMA (the default) the light-tile resolve and
    the shading move their tiles through shared memory with 2-D tensor
    copies; with them off they read and write the pixels directly. The
    images are identical, including framebuffers whose edge tiles reach past
    the planes (sides not multiples of 8)."""
    import ctypes
    import srp_gb300
    L = srp_gb300.lib()
    L.srpGpuSetTileCopies.argtypes = [ctypes.c_uint]
    L.srpGpuSetFramebufferMode(srp_gb300.SRP_GPU_FB_DEVICE)
    sc = srp_gb300.Scene(scene, 23, scale)
    try:
        frames = []
        for on in (0, 7, 7, 1, 3, 4):
            L.srpGpuSetTileCopies(on)
            sc.prepare()
            sc.render()
            frames.append([a.copy() for a in sc.planes()])
        assert L.srpGpuSynchronize() == 0
        for f in frames[1:]:
            for a, b in zip(f, frames[0]):
                assert np.array_equal(a, b)
    finally:
        L.srpGpuSetTileCopies(TILE_COPY_DEFAULT)
        sc.close()


def test_tma_tile_copies_on_ragged_framebuffer(built_library):
    """A 300 x 203 framebuffer (width a multiple of 4 but not of 8, height not
    a multiple of 8): the right and bottom tiles' TMA boxes reach past the
    planes. Random triangles with depth test, drawn with and without the
    tile copies, give the same planes, and the oracle's."""
    import ctypes
    import os
    import subprocess
    import srp_gb300
    import srpapi as A
    L = srp_gb300.lib()
    L.srpGpuSetTileCopies.argtypes = [ctypes.c_uint]
    L.srpGpuSetFramebufferMode(srp_gb300.SRP_GPU_FB_COHERENT)
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    subprocess.check_call(["make", "-s", "-C", os.path.join(root, "oracle"), "portlib"])
    rng = np.random.default_rng(41)
    n = 3000
    centre = rng.uniform(-1.2, 1.2, size=(n, 1, 3))
    verts = np.concatenate([(centre + rng.uniform(-0.08, 0.08, size=(n, 3, 3))).reshape(-1, 3),
                            rng.uniform(0, 1, size=(3 * n, 3))], axis=1).astype(np.float32)

    def render(srp):
        srp.new_context()
        srp.srpDepthTest(True)
        u = A.StdUniform()
        u.model = u.view = u.projection = srp.mat4ConstructIdentity()
        u.passOffset, u.passCount = 3, 3
        sp = srp.program(u, "srpVsTransform", "srpFsVaryingColor", [(3, A.FLOAT, A.INTERP_PERSPECTIVE)], 12)
        fb = srp.srpNewFramebuffer(300, 203)
        vb = srp.vertex_buffer(verts)
        srp.srpFramebufferClear(fb)
        srp.srpDrawVertexBuffer(vb, fb, ctypes.byref(sp), A.PRIM_TRIANGLES, 0, 3 * n)
        planes = srp.planes(fb)
        srp.srpFreeVertexBuffer(vb)
        srp.srpFreeFramebuffer(fb)
        return planes

    gpu = A.Srp(srp_gb300.library_path())
    port = A.Srp(os.path.join(root, "oracle", "_build", "libsrp_port.so"))
    try:
        got = []
        for on in (7, 0):
            L.srpGpuSetTileCopies(on)
            got.append(render(gpu))
        want = render(port)
        assert not gpu.errors() and not port.errors()
    finally:
        L.srpGpuSetTileCopies(TILE_COPY_DEFAULT)
        gpu.close()
        port.close()
    for a, b in zip(got[0], got[1]):
        assert np.array_equal(a, b)
    assert int((want[1] != np.float32(-1.0)).sum()) > 10000
    compare_planes({"color": got[0][0], "depth_bits": got[0][1].view(np.uint32), "stencil": got[0][2]},
                   {"color": want[0], "depth_bits": want[1].view(np.uint32), "stencil": want[2]}, "300x203")
