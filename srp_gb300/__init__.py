"""srp_gb300: the srp draw path on GB300 (sm_103a), behind srp's own C API.

The product is the shared library ``srp_gb300/lib/libsrp_gb300.so`` whose
exported symbols are the reference's public C API (include/srp/*.h) plus the
GPU additions of include/srp/gpu.h. This package only builds it and binds it
with ctypes for Python callers (tests, benchmarks). There is no CPU fallback:
when the library is missing or no GPU is present, calls that need the GPU fail
loudly.
"""
import ctypes
import os

import numpy as np

from .build import LIB, ROOT, build  # noqa: F401

_lib = None
_scenes = None

SRP_GPU_FB_COHERENT = 0
SRP_GPU_FB_DEVICE = 1


class SRPGpuStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in
                ("fragments", "primitives", "binEntries", "clipOverflows", "draws", "kernelLaunches", "drawRetries")]


class SRPGpuDraw(ctypes.Structure):
    _fields_ = [("indexBuffer", ctypes.c_void_p), ("vertexBuffer", ctypes.c_void_p),
                ("framebuffer", ctypes.c_void_p), ("program", ctypes.c_void_p), ("primitive", ctypes.c_int),
                ("startIndex", ctypes.c_size_t), ("count", ctypes.c_size_t)]


class SRPGpuTuning(ctypes.Structure):
    _fields_ = [("heavyItems", ctypes.c_uint32), ("heavyCtasPerSM", ctypes.c_uint32)]


class SceneInfo(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int), ("height", ctypes.c_int),
                ("inputTriangles", ctypes.c_size_t), ("inputLines", ctypes.c_size_t),
                ("inputPoints", ctypes.c_size_t), ("vertexBytes", ctypes.c_size_t),
                ("indexBytes", ctypes.c_size_t), ("textureBytes", ctypes.c_size_t),
                ("draws", ctypes.c_int), ("usesStencil", ctypes.c_int)]


STAGES = ("vertex", "setup", "bin", "resolve", "shade")


class SRPGpuProfile(ctypes.Structure):
    _fields_ = [("ms", ctypes.c_double * 5), ("launches", ctypes.c_uint64 * 5),
                ("resolveTiles", ctypes.c_uint64), ("resolveItems", ctypes.c_uint64)]


MESSAGE_CALLBACK = ctypes.CFUNCTYPE(None, ctypes.c_int, ctypes.c_int, ctypes.c_char_p, ctypes.c_char_p,
                                    ctypes.c_void_p)


class SRPMessageCallback(ctypes.Structure):
    _fields_ = [("func", MESSAGE_CALLBACK), ("userParameter", ctypes.c_void_p)]


def library_path():
    return os.path.join(LIB, "libsrp_gb300.so")


def lib():
    """The GPU library (C ABI). Raises if it has not been built."""
    global _lib
    if _lib is None:
        path = library_path()
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: run srp_gb300.build() (nvcc, sm_103a) first")
        L = ctypes.CDLL(path)
        L.srpGpuGetStats.argtypes = [ctypes.POINTER(SRPGpuStats)]
        L.srpGpuSetFramebufferMode.argtypes = [ctypes.c_int]
        L.srpGpuSetStream.argtypes = [ctypes.c_void_p]
        L.srpGpuGetStream.restype = ctypes.c_void_p
        L.srpGpuSynchronize.restype = ctypes.c_int
        L.srpSetMessageCallback.argtypes = [SRPMessageCallback]
        L.srpGpuGetProfile.argtypes = [ctypes.POINTER(SRPGpuProfile)]
        L.srpGpuSetProfiling.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def scenes():
    """The seeded scene library, driving the GPU library through the srp API."""
    global _scenes
    if _scenes is None:
        lib()  # the scene library resolves srp* (and srpContext) against it
        path = os.path.join(LIB, "libsrp_scenes_gpu.so")
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: run srp_gb300.build() first")
        S = ctypes.CDLL(path)
        S.sceneCreate.restype = ctypes.c_void_p
        S.sceneCreate.argtypes = [ctypes.c_char_p, ctypes.c_uint64, ctypes.c_double]
        S.sceneDestroy.argtypes = [ctypes.c_void_p]
        S.sceneGetInfo.argtypes = [ctypes.c_void_p, ctypes.POINTER(SceneInfo)]
        S.sceneInputHash.restype = ctypes.c_uint64
        S.sceneInputHash.argtypes = [ctypes.c_void_p]
        S.sceneUpload.argtypes = [ctypes.c_void_p]
        S.scenePrepareFramebuffer.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        S.sceneRender.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        S.sceneNames.restype = ctypes.POINTER(ctypes.c_char_p)
        S.srpNewFramebuffer.restype = ctypes.c_void_p
        S.srpNewFramebuffer.argtypes = [ctypes.c_size_t, ctypes.c_size_t]
        S.srpFreeFramebuffer.argtypes = [ctypes.c_void_p]
        S.srpGpuFramebufferSync.argtypes = [ctypes.c_void_p]
        S.sceneDrawDesc.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(SRPGpuDraw)]
        S.sceneBatchRender.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t,
                                       ctypes.POINTER(SRPGpuDraw)]
        S.sceneBatchAutotune.restype = ctypes.c_int
        S.sceneBatchAutotune.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t,
                                         ctypes.POINTER(SRPGpuDraw), ctypes.c_int, ctypes.POINTER(SRPGpuTuning)]
        _scenes = S
    return _scenes


def scene_names():
    S = scenes()
    out, p = [], S.sceneNames()
    i = 0
    while p[i]:
        out.append(p[i].decode())
        i += 1
    return out


class FramebufferView(ctypes.Structure):
    _fields_ = [("width", ctypes.c_size_t), ("height", ctypes.c_size_t), ("size", ctypes.c_size_t),
                ("color", ctypes.POINTER(ctypes.c_uint32)), ("depth", ctypes.POINTER(ctypes.c_float)),
                ("stencil", ctypes.POINTER(ctypes.c_uint8))]


def framebuffer_arrays(fb):
    """Copies of the host planes of an SRPFramebuffer* (after a sync)."""
    v = ctypes.cast(fb, ctypes.POINTER(FramebufferView)).contents
    n = v.size
    color = np.ctypeslib.as_array(v.color, shape=(n,)).copy()
    depth = np.ctypeslib.as_array(v.depth, shape=(n,)).copy()
    stencil = np.ctypeslib.as_array(v.stencil, shape=(n,)).copy()
    return color, depth, stencil


class Scene:
    """A seeded scene whose draws run on the GPU through the srp API."""

    def __init__(self, name, seed=1, scale=1.0):
        self.S = scenes()
        self.ptr = self.S.sceneCreate(name.encode(), seed, scale)
        if not self.ptr:
            raise ValueError(f"unknown scene {name}")
        self.info = SceneInfo()
        self.S.sceneGetInfo(self.ptr, ctypes.byref(self.info))
        self.name, self.seed, self.scale = name, seed, scale
        self.fb = self.S.srpNewFramebuffer(self.info.width, self.info.height)
        if not self.fb:
            raise RuntimeError("srpNewFramebuffer failed (no GPU?)")

    @property
    def input_hash(self):
        return self.S.sceneInputHash(self.ptr)

    def upload(self):
        self.S.sceneUpload(self.ptr)

    def upload_async(self):
        """upload() with srpGpu*CopyDataAsync: complete after srpGpuSynchronize."""
        self.S.sceneUploadAsync(self.ptr)

    def prepare(self):
        self.S.scenePrepareFramebuffer(self.ptr, self.fb)

    def render(self):
        self.S.sceneRender(self.ptr, self.fb)

    def sync(self):
        self.S.srpGpuFramebufferSync(self.fb)

    def sync_async(self):
        """sync() with srpGpuFramebufferSyncAsync: complete after srpGpuSynchronize."""
        self.S.srpGpuFramebufferSyncAsync(self.fb)

    def planes(self):
        self.sync()
        return framebuffer_arrays(self.fb)

    def close(self):
        if self.fb:
            self.S.srpFreeFramebuffer(self.fb)
            self.fb = None
        if self.ptr:
            self.S.sceneDestroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def batch_seed(base, i):
    """Seed of scene i of a batch: the scene generator's streams of seeds that
    differ by d are the same stream shifted by d draws, so batch scenes are
    spaced 2^32 draws apart."""
    return ((i + 1) << 32) + base


def render_batch(batch, fbs):
    """Render batch[i] (Scene objects of the batched workload, one draw each)
    into fbs[i] with one srpGpuDrawBatch call; fbs may repeat a framebuffer."""
    S = scenes()
    n = len(batch)
    sp = (ctypes.c_void_p * n)(*[sc.ptr for sc in batch])
    fp = (ctypes.c_void_p * n)(*fbs)
    scratch = (SRPGpuDraw * n)()
    S.sceneBatchRender(sp, fp, n, scratch)


def upload_batch(batch):
    """Scene.upload_async of every scene with the Batch copies (gather
    kernels, 256 scenes at a time): complete after srpGpuSynchronize."""
    S = scenes()
    n = len(batch)
    sp = (ctypes.c_void_p * n)(*[sc.ptr for sc in batch])
    S.sceneUploadBatchAsync(sp, ctypes.c_size_t(n))


def sync_batch(fbs):
    """srpGpuFramebufferSyncBatchAsync of the framebuffers: the host arrays
    are current after srpGpuSynchronize."""
    L = lib()
    n = len(fbs)
    fp = (ctypes.c_void_p * n)(*fbs)
    L.srpGpuFramebufferSyncBatchAsync(fp, ctypes.c_size_t(n))


def prepare_batch(batch, fbs):
    """Prepare the framebuffers of a batch in one srpGpuFramebufferFillBatch."""
    S = scenes()
    n = len(batch)
    sp = (ctypes.c_void_p * n)(*[sc.ptr for sc in batch])
    fp = (ctypes.c_void_p * n)(*fbs)
    S.scenePrepareBatch(sp, fp, ctypes.c_size_t(n))


def autotune_batch(batch, fbs, repeats=1):
    """srpGpuAutotune on the batch render_batch would draw; returns the chosen
    SRPGpuTuning (the framebuffers must be prepared again)."""
    S = scenes()
    n = len(batch)
    sp = (ctypes.c_void_p * n)(*[sc.ptr for sc in batch])
    fp = (ctypes.c_void_p * n)(*fbs)
    scratch = (SRPGpuDraw * n)()
    best = SRPGpuTuning()
    if S.sceneBatchAutotune(sp, fp, n, scratch, repeats, ctypes.byref(best)) != 0:
        raise RuntimeError("srpGpuAutotune failed")
    return best


def render_scene(name, seed=1, scale=1.0):
    """Render one frame of a scene on the GPU; returns (color, depth, stencil,
    width, height, stats, input_hash)."""
    L = lib()
    L.srpGpuSetFramebufferMode(SRP_GPU_FB_DEVICE)
    sc = Scene(name, seed, scale)
    try:
        sc.prepare()
        L.srpGpuResetStats()
        sc.render()
        c, d, s = sc.planes()
        st = SRPGpuStats()
        L.srpGpuGetStats(ctypes.byref(st))
        if L.srpGpuSynchronize() != 0:
            raise RuntimeError("GPU error during the draw")
        return c, d, s, sc.info.width, sc.info.height, st, sc.input_hash
    finally:
        sc.close()
