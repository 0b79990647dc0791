"""Failure detection on the GPU, made to happen without a fault: every device
wait on another block or on the tensor cores is bounded, and a test can
withhold the signal one of them waits for (srpGpuSetWaitTest) with a short
limit (srpGpuSetWaitLimit). The wait then runs out, the kernel records the
timeout and returns, and the host reports it through the message callback,
as the reference reports its errors (src/pipeline/draw.c:176-186: a message,
then the call returns). The context stays usable: the next draw is exact.
Also the grow-and-retry path of a draw whose (tile, primitive) pairs exceed
the buffers sized from the last draw's count."""
import ctypes

import numpy as np
import pytest

from oracle_util import oracle_render, compare_planes

pytestmark = pytest.mark.gpu

WAIT_TEST_SETUP, WAIT_TEST_LEARNED = 1, 2


class Messages:
    def __init__(self, srp_gb300, L):
        self.L, self.srp = L, srp_gb300
        self.log = []
        self._cb = srp_gb300.MESSAGE_CALLBACK(lambda t, sev, fn, msg, user: self.log.append((t, fn.decode(), msg.decode())))
        L.srpSetMessageCallback(srp_gb300.SRPMessageCallback(self._cb, None))

    def errors(self):
        return [m for m in self.log if m[0] == 0]

    def close(self):
        self.L.srpSetMessageCallback(self.srp.SRPMessageCallback())


@pytest.fixture()
def gpu(built_library):
    import srp_gb300
    L = srp_gb300.lib()
    L.srpGpuSetWaitLimit.argtypes = [ctypes.c_uint32]
    L.srpGpuSetWaitTest.argtypes = [ctypes.c_uint32]
    L.srpGpuSetEntryEstimate.argtypes = [ctypes.c_double]
    L.srpGpuSetFramebufferMode(srp_gb300.SRP_GPU_FB_DEVICE)
    m = Messages(srp_gb300, L)
    yield srp_gb300, L, m
    L.srpGpuSetWaitTest(0)
    L.srpGpuSetWaitLimit(0)
    m.close()
    assert L.srpGpuSynchronize() == 0


def frame(sc):
    sc.prepare()
    sc.render()
    return [a.copy() for a in sc.planes()]


@pytest.mark.parametrize("graphs", [1, 0])
def test_setup_wait_timeout_is_reported_and_draws_nothing(gpu, oracle_exe, graphs):
    """The ordered setup's first block withholds its prefix: the other blocks'
    look-back runs out, the draw reports the timeout and leaves the
    framebuffer as prepared; with the signal back the same draws are exact."""
    srp_gb300, L, msgs = gpu
    L.srpGpuSetDrawGraphs(graphs)
    sc = srp_gb300.Scene("soup", 21, 0.05)
    try:
        sc.prepare()
        prepared = [a.copy() for a in sc.planes()]
        L.srpGpuSetWaitLimit(1 << 14)
        L.srpGpuSetWaitTest(WAIT_TEST_SETUP)
        sc.render()
        got = [a.copy() for a in sc.planes()]
        errs = msgs.errors()
        # the triangle draw has many setup blocks; lines and points too
        assert errs and all("Ordered-compaction wait timed out" in e[2] for e in errs), errs
        for a, b in zip(got, prepared):
            assert np.array_equal(a, b), "a timed-out draw changed the framebuffer"
        L.srpGpuSetWaitTest(0)
        L.srpGpuSetWaitLimit(0)
        msgs.log.clear()
        c, d, s = frame(sc)
        assert not msgs.errors(), msgs.errors()
        want = oracle_render(oracle_exe, "soup", 21, 0.05)
        compare_planes({"color": c, "depth_bits": d.view(np.uint32), "stencil": s}, want, "draw after the timeout")
    finally:
        L.srpGpuSetDrawGraphs(1)
        sc.close()


def test_learned_wait_timeout_falls_back_to_the_shader(gpu):
    """Learned shading whose second layer's MMAs are withheld: its mbarrier
    wait runs out with no MMA in flight, the kernel releases its tensor
    memory, the draw reports the timeout and is shaded by its own shader
    (image equal to the plain draw's). A learned draw afterwards works."""
    srp_gb300, L, msgs = gpu
    vp = ctypes.c_void_p
    L.srpGpuMlpCreate.restype = vp
    L.srpGpuMlpCreate.argtypes = [ctypes.c_uint64, ctypes.c_size_t]
    L.srpGpuMlpFree.argtypes = [vp]
    L.srpGpuSetLearnedShading.argtypes = [vp, vp, ctypes.c_float, ctypes.c_uint32]
    marble = ctypes.cast(L.srpFsMarble, vp)
    net = L.srpGpuMlpCreate(5, 1 << 10)
    sc = srp_gb300.Scene("msoup", 5, 0.08)  # about 43,000 covered pixels
    try:
        plain = frame(sc)
        assert int((plain[1] != plain[1][0]).sum()) > 1000, "the scene should cover part of the framebuffer"
        L.srpGpuSetLearnedShading(marble, net, 0.0, 16)  # a 0 dB bar: no fallback for quality
        L.srpGpuSetWaitLimit(1 << 14)
        L.srpGpuSetWaitTest(WAIT_TEST_LEARNED)
        msgs.log.clear()
        timed_out = frame(sc)
        errs = msgs.errors()
        assert errs and "timed out" in errs[-1][2], errs
        for a, b in zip(timed_out, plain):
            assert np.array_equal(a, b), "the fallback should give the plain shader's image"
        # the tensor memory was released: the next learned draws run
        L.srpGpuSetWaitTest(0)
        L.srpGpuSetWaitLimit(0)
        msgs.log.clear()
        for _ in range(2):
            learned = frame(sc)
        assert not msgs.errors(), msgs.errors()
        assert np.array_equal(learned[1], plain[1]) and np.array_equal(learned[2], plain[2])
        assert (learned[0] != plain[0]).any(), "the network should colour the draw"
    finally:
        L.srpGpuSetLearnedShading(None, None, 0.0, 0)
        sc.close()
        L.srpGpuMlpFree(net)


@pytest.mark.parametrize("scene,scale", [("soup", 0.05), ("clip_lines", 1.0), ("sphere", 1.0)])
def test_pair_overflow_grows_and_retries(gpu, oracle_exe, scene, scale):
    """With the pair estimate at zero, every draw's binning overflows its
    buffers: the draw stops before its resolve, grows them and runs again,
    and the image is the oracle's."""
    srp_gb300, L, msgs = gpu
    sc = srp_gb300.Scene(scene, 17, scale)
    try:
        sc.prepare()
        L.srpGpuResetStats()
        L.srpGpuSetEntryEstimate(0.0)
        sc.render()
        c, d, s = [a.copy() for a in sc.planes()]
        st = srp_gb300.SRPGpuStats()
        L.srpGpuGetStats(ctypes.byref(st))
        assert st.drawRetries >= 1, "the draw should have overflowed and run again"
        assert not msgs.errors(), msgs.errors()
        want = oracle_render(oracle_exe, scene, 17, scale)
        compare_planes({"color": c, "depth_bits": d.view(np.uint32), "stencil": s}, want, f"{scene} after a retry")
    finally:
        sc.close()
