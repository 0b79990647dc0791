"""Line draws binned as runs of steps in one tile: long lines in every
direction (a warp per line), short ones (a thread per line), lines ending on
the framebuffer's right and bottom edges (where the reference's pixel index
wraps to the next row), with and without a scissor rectangle cutting them,
on a framebuffer whose size is not a multiple of the tile. The GPU's planes
must equal the oracle's (depth and stencil bit-exact, colour within 1/255),
through the srp C API of both libraries."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from oracle_util import compare_planes

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
W, H = 301, 203


def line_vertices(rng, n):
    """n lines as (pos3, rgb3) vertex pairs in clip space (w = 1): a third
    long and crossing the screen, a third short, a third ending on an edge."""
    a = rng.uniform(-1.0, 1.0, size=(n, 2))
    b = a + rng.uniform(-0.08, 0.08, size=(n, 2))
    k = n // 3
    b[:k] = rng.uniform(-1.0, 1.0, size=(k, 2))                 # long, any direction
    edge = rng.integers(0, 4, size=n - 2 * k)
    e = b[2 * k:]
    e[edge == 0, 0] = 1.0                                        # right edge: x = W after the viewport map
    e[edge == 1, 1] = -1.0                                       # bottom edge
    e[edge == 2, 0] = -1.0
    e[edge == 3, 1] = 1.0
    z = rng.uniform(-0.9, 0.9, size=(n, 2))
    v = np.zeros((n, 2, 6), np.float32)
    v[:, 0, :2], v[:, 1, :2] = a, b
    v[:, :, 2] = z
    v[:, :, 3:] = rng.uniform(0, 1, size=(n, 2, 3))
    return v.reshape(-1, 6)


def render(srp, A, verts, scissor):
    srp.new_context()
    srp.srpDepthTest(True)   # the context's default compare op, against the cleared depth
    srp.srpStencilTest(True)
    srp.srpStencilFunc(A.COMPARE_ALWAYS, 0, 0xFF)
    srp.srpStencilOp(A.STENCIL_KEEP, A.STENCIL_KEEP, A.STENCIL_INCR)
    srp.srpStencilWriteMask(0xFF)
    if scissor:
        srp.srpScissorTest(True)
        srp.srpScissorOptions(37, 21, 190, 150)
    u = A.StdUniform()
    u.model = u.view = u.projection = srp.mat4ConstructIdentity()
    u.passOffset, u.passCount = 3, 3
    sp = srp.program(u, "srpVsTransform", "srpFsVaryingColor", [(3, A.FLOAT, A.INTERP_PERSPECTIVE)], 12)
    fb = srp.srpNewFramebuffer(W, H)
    vb = srp.vertex_buffer(verts)
    srp.srpFramebufferClear(fb)
    srp.srpDrawVertexBuffer(vb, fb, ctypes.byref(sp), A.PRIM_LINES, 0, len(verts))
    planes = srp.planes(fb)
    srp.srpFreeVertexBuffer(vb)
    srp.srpFreeFramebuffer(fb)
    return planes


@pytest.mark.parametrize("scissor", [False, True], ids=["no_scissor", "scissor"])
@pytest.mark.parametrize("seed", [3, 9])
def test_line_runs_match_oracle(built_library, scissor, seed):
    import srp_gb300
    import srpapi as A
    L = srp_gb300.lib()
    L.srpGpuSetFramebufferMode(srp_gb300.SRP_GPU_FB_COHERENT)
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "portlib"])
    verts = line_vertices(np.random.default_rng(seed), 3000)
    gpu = A.Srp(srp_gb300.library_path())
    port = A.Srp(os.path.join(ROOT, "oracle", "_build", "libsrp_port.so"))
    try:
        got = render(gpu, A, verts, scissor)
        want = render(port, A, verts, scissor)
        assert not gpu.errors() and not port.errors()
    finally:
        gpu.close()
        port.close()
    assert int((want[2] != 0).sum()) > 5000        # many pixels drawn, many of them more than once
    assert int((want[2] > 1).sum()) > 500
    compare_planes({"color": got[0], "depth_bits": got[1].view(np.uint32), "stencil": got[2]},
                   {"color": want[0], "depth_bits": want[1].view(np.uint32), "stencil": want[2]},
                   f"lines seed {seed} scissor {scissor}")
