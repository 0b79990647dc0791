"""ctypes binding of srp's public C API (include/srp/*.h) for any library that
exports it: the GPU library (srp_gb300/lib/libsrp_gb300.so) or the CPU
oracle's shared build (oracle/_build/libsrp_port.so). A Python program written
against it makes the same calls, in the same order, as a C program against
the reference, which is how tests/refscenes.py restates the reference's own
image tests."""
import ctypes

import numpy as np

# enums (include/srp/buffer.h, context.h, type.h, texture.h, vertex.h)
PRIM_POINTS, PRIM_LINES, PRIM_LINE_STRIP, PRIM_LINE_LOOP, PRIM_TRIANGLES, PRIM_TRIANGLE_STRIP, PRIM_TRIANGLE_FAN = range(7)
PROVOKING_FIRST, PROVOKING_LAST = 0, 1
WINDING_CCW, WINDING_CW = 0, 1
FACE_NONE, FACE_FRONT, FACE_BACK, FACE_FRONT_AND_BACK = range(4)
POLYGON_FILL, POLYGON_LINE, POLYGON_POINT = range(3)
(COMPARE_NEVER, COMPARE_ALWAYS, COMPARE_LESS, COMPARE_LEQUAL, COMPARE_GREATER, COMPARE_GEQUAL, COMPARE_EQUAL,
 COMPARE_NOTEQUAL) = range(8)
(STENCIL_KEEP, STENCIL_ZERO, STENCIL_REPLACE, STENCIL_INCR, STENCIL_INCR_WRAP, STENCIL_DECR, STENCIL_DECR_WRAP,
 STENCIL_INVERT) = range(8)
FLOAT, DOUBLE, INT8, INT16, INT32, INT64, UINT8, UINT16, UINT32, UINT64 = range(10)
TW_REPEAT, TW_CLAMP_TO_EDGE = 0, 1
INTERP_PERSPECTIVE, INTERP_AFFINE, INTERP_FLAT = range(3)


class Mat4(ctypes.Structure):
    _fields_ = [("data", ctypes.c_float * 16)]


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
    """SRPStdUniform of srp/shaderlib.h, the uniform block of the built-in
    shaders."""
    _fields_ = [("model", Mat4), ("view", Mat4), ("projection", Mat4),
                ("color", ctypes.c_float * 4), ("cameraPos", ctypes.c_float * 4),
                ("lightPos", ctypes.c_float * 64), ("lightColor", ctypes.c_float * 64), ("ambient", ctypes.c_float * 4),
                ("shininess", ctypes.c_float), ("marbleFrequency", ctypes.c_float), ("marbleGain", ctypes.c_float),
                ("depthScale", ctypes.c_float), ("depthBias", ctypes.c_float)] + \
               [(n, ctypes.c_uint32) for n in ("nLights", "marbleOctaves", "passOffset", "passCount", "normalOffset",
                                               "uvOffset", "extraOffset", "extraCount", "varyingOffset")] + \
               [("texelScale", ctypes.c_float), ("texture", ctypes.c_void_p)]


class FramebufferView(ctypes.Structure):
    """The public part of SRPFramebuffer (include/srp/framebuffer.h)."""
    _fields_ = [("width", ctypes.c_size_t), ("height", ctypes.c_size_t), ("size", ctypes.c_size_t),
                ("color", ctypes.POINTER(ctypes.c_uint32)), ("depth", ctypes.POINTER(ctypes.c_float)),
                ("stencil", ctypes.POINTER(ctypes.c_uint8))]


MESSAGE_CALLBACK = ctypes.CFUNCTYPE(None, ctypes.c_int, ctypes.c_int, ctypes.c_char_p, ctypes.c_char_p,
                                    ctypes.c_void_p)


class MessageCallback(ctypes.Structure):
    _fields_ = [("func", MESSAGE_CALLBACK), ("userParameter", ctypes.c_void_p)]


_vp, _sz, _f, _b, _i, _u8 = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_float, ctypes.c_bool, ctypes.c_int, ctypes.c_uint8
_SIGNATURES = [
    ("srpNewContext", None, [_vp]),
    ("srpSetMessageCallback", None, [MessageCallback]),
    ("srpProvokingVertexMode", None, [_i]),
    ("srpRasterCullFace", None, [_i]),
    ("srpRasterFrontFace", None, [_i]),
    ("srpRasterPolygonMode", None, [_i]),
    ("srpRasterPointSize", None, [_f]),
    ("srpScissorTest", None, [_b]),
    ("srpScissorOptions", None, [_sz, _sz, _sz, _sz]),
    ("srpStencilTest", None, [_b]),
    ("srpStencilFunc", None, [_i, _u8, _u8]),
    ("srpStencilOp", None, [_i, _i, _i]),
    ("srpStencilWriteMask", None, [_u8]),
    ("srpDepthTest", None, [_b]),
    ("srpDepthWrite", None, [_b]),
    ("srpDepthCompareOp", None, [_i]),
    ("srpNewFramebuffer", _vp, [_sz, _sz]),
    ("srpFreeFramebuffer", None, [_vp]),
    ("srpFramebufferClear", None, [_vp]),
    ("srpNewVertexBuffer", _vp, []),
    ("srpFreeVertexBuffer", None, [_vp]),
    ("srpVertexBufferCopyData", None, [_vp, _sz, _sz, _vp]),
    ("srpNewIndexBuffer", _vp, []),
    ("srpFreeIndexBuffer", None, [_vp]),
    ("srpIndexBufferCopyData", None, [_vp, _i, _sz, _vp]),
    ("srpDrawVertexBuffer", None, [_vp, _vp, _vp, _i, _sz, _sz]),
    ("srpDrawIndexBuffer", None, [_vp, _vp, _vp, _vp, _i, _sz, _sz]),
    ("srpNewTexture", _vp, [ctypes.c_char_p, _i, _i]),
    ("srpFreeTexture", None, [_vp]),
    ("mat4ConstructIdentity", Mat4, []),
    ("mat4ConstructScale", Mat4, [_f, _f, _f]),
    ("mat4ConstructRotate", Mat4, [_f, _f, _f]),
    ("mat4ConstructTRS", Mat4, [_f] * 9),
    ("mat4ConstructView", Mat4, [_f] * 9),
    ("mat4ConstructPerspectiveProjection", Mat4, [_f] * 6),
    ("mat4MultiplyMat4", Mat4, [ctypes.POINTER(Mat4), ctypes.POINTER(Mat4)]),
]


class Srp:
    """The srp API of one library, typed, with a fresh context and a message
    log. `shader(name)` gives the address of an exported built-in shader."""

    def __init__(self, path):
        L = ctypes.CDLL(path)
        for name, res, args in _SIGNATURES:
            f = getattr(L, name)
            f.restype, f.argtypes = res, args
        self.L = L
        self.ctx = ctypes.c_char.in_dll(L, "srpContext")
        L.srpNewContext(ctypes.addressof(self.ctx))
        self.messages = []
        self._cb = MESSAGE_CALLBACK(lambda t, sev, fn, msg, user: self.messages.append((t, fn.decode(), msg.decode())))
        L.srpSetMessageCallback(MessageCallback(self._cb, None))
        self._keep = []

    def __getattr__(self, name):
        return getattr(self.L, name)

    def new_context(self):
        """srpNewContext(&srpContext), keeping the message callback."""
        self.L.srpNewContext(ctypes.addressof(self.ctx))
        self.L.srpSetMessageCallback(MessageCallback(self._cb, None))

    def shader(self, name):
        return ctypes.cast(getattr(self.L, name), ctypes.c_void_p).value

    def errors(self):
        return [m for m in self.messages if m[0] == 0]  # SRP_MESSAGE_ERROR

    def program(self, uniform, vs, fs, varyings=(), varyings_size=0, may_overwrite_depth=False):
        """An SRPShaderProgram; varyings is a list of (nItems, type, mode)."""
        info = (VaryingInfo * max(len(varyings), 1))(*[VaryingInfo(*v) for v in varyings])
        v = VertexShader(self.shader(vs), len(varyings), info if varyings else None, varyings_size)
        f = FragmentShader(self.shader(fs), may_overwrite_depth)
        p = ShaderProgram(ctypes.addressof(uniform) if uniform is not None else None, ctypes.pointer(v),
                          ctypes.pointer(f))
        self._keep += [info, v, f, p, uniform]
        return p

    def vertex_buffer(self, data):
        """srpVertexBufferCopyData of a structured or 2-D numpy array (one row
        per vertex)."""
        data = np.ascontiguousarray(data)
        vb = self.L.srpNewVertexBuffer()
        stride = data.dtype.itemsize if data.ndim == 1 else data.dtype.itemsize * data.shape[1]
        self.L.srpVertexBufferCopyData(vb, stride, data.nbytes, data.ctypes.data)
        self._keep.append(data)
        return vb

    def index_buffer(self, itype, idx):
        idx = np.ascontiguousarray(idx)
        ib = self.L.srpNewIndexBuffer()
        self.L.srpIndexBufferCopyData(ib, itype, idx.nbytes, idx.ctypes.data)
        self._keep.append(idx)
        return ib

    @staticmethod
    def planes(fb):
        """Copies of the public colour, depth and stencil arrays."""
        v = ctypes.cast(fb, ctypes.POINTER(FramebufferView)).contents
        n = v.size
        return (np.ctypeslib.as_array(v.color, shape=(n,)).copy(),
                np.ctypeslib.as_array(v.depth, shape=(n,)).copy(),
                np.ctypeslib.as_array(v.stencil, shape=(n,)).copy())

    def close(self):
        # the ctypes thunk dies with this object: the library must not keep it
        self.L.srpSetMessageCallback(MessageCallback())
        self._keep = []


def rgb_image(color, width, height):
    """The colour plane as an RGB image, top row first, as the reference's test
    harness writes it (tests/utils/save.c:3-34: R<<24 | G<<16 | B<<8 | A)."""
    c = color.reshape(height, width)
    return np.stack([(c >> 24) & 255, (c >> 16) & 255, (c >> 8) & 255], axis=-1).astype(np.uint8)
