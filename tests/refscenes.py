"""The reference's own 18 image tests (kitrofimov/srp tests/scenes/**/*.c),
restated as srp API call sequences over tests/srpapi.py, so that they run
through any library exporting srp's C API: the CPU oracle's shared build and
the GPU library. Each function makes the calls of the scene's main() in the
same order, with the same vertex data, index data, matrices and state, and
returns the framebuffer's planes; tests/test_refscenes.py compares the colour
plane with the reference's golden image at the tolerance of its
tests/compare.py:8 (1 per channel).

The scenes' shaders are host functions, which a GPU cannot call; each is
replaced by the built-in shader of srp/shaderlib.h that computes the same
thing:
  - vertexShader: clip = projection * view * model * (position, 1), varyings
    copied from the vertex -> srpVsTransform (passOffset/passCount = the
    varying's words in the vertex); where a scene's shader applies fewer
    matrices (a model matrix only, a rotation only, none) the others are the
    identity, and where it takes no uniform (uniform = NULL) an identity
    uniform is passed;
  - the uint8 palette of interpolation/flat.c -> srpVsBytes + srpFsBytePalette;
  - colour = interpolated vec3, alpha 1 -> srpFsVaryingColor;
  - srpTextureGetFilteredColor(texture, uv) -> srpFsTexture;
  - colour from (id * 97, 57, 23) mod 255 / 255 (/ 2) -> srpFsPrimitiveMod
    with colour[0] = 1 (2);
  - constant white / red -> srpFsSolid.
The Utah teapot (examples/res/objects/utah_teapot.obj) and the stone-wall
texture (examples/res/textures/stoneWall.png) come from
tests/golden/refimages.npz, dumped by tests/golden/make_refimages.py as the
reference's own loaders produce them; the texture is handed to srpNewTexture
as a PPM file, since both libraries decode PPM.
"""
import ctypes
import math
import os
import tempfile

import numpy as np

import srpapi as A

HERE = os.path.dirname(os.path.abspath(__file__))
W = H = 512


def _assets():
    z = np.load(os.path.join(HERE, "golden", "refimages.npz"))
    return z


def _rad(x):
    """RAD(x) of examples/utility/rad.h: ((float) x / 180.) * M_PI, in double."""
    return (float(np.float32(x)) / 180.0) * math.pi


def _uniform(srp, model=None, view=None, projection=None, pass_offset=0, pass_count=0):
    u = A.StdUniform()
    ident = srp.mat4ConstructIdentity()
    u.model = model if model is not None else ident
    u.view = view if view is not None else ident
    u.projection = projection if projection is not None else ident
    u.passOffset, u.passCount = pass_offset, pass_count
    u.color[:] = [1.0, 1.0, 1.0, 1.0]
    return u


def _pos_color(rows):
    """Vertex { vec3 position; vec3 color; } (24 bytes, alignment 1)."""
    return np.array([list(p) + list(c) for p, c in rows], dtype=np.float32)


CUBE_EDGES_U8 = np.array([0, 1, 1, 2, 2, 3, 3, 0, 4, 5, 5, 6, 6, 7, 7, 4, 0, 4, 1, 5, 2, 6, 3, 7], np.uint8)
CUBE_CORNERS = [(-1, -1, -1), (1, -1, -1), (1, -1, 1), (-1, -1, 1), (-1, 1, -1), (1, 1, -1), (1, 1, 1), (-1, 1, 1)]

# textured cube of interpolation/{affine,perspective}.c and misc/stencil_test.c
UV_CUBE = np.array([
    [-1, -1, -1, 0, 0], [1, -1, -1, 1, 0], [1, 1, -1, 1, 1], [-1, 1, -1, 0, 1],
    [-1, 1, -1, 0, 0], [1, 1, -1, 1, 0], [1, 1, 1, 1, 1], [-1, 1, 1, 0, 1],
    [1, -1, 1, 0, 0], [-1, -1, 1, 1, 0], [-1, 1, 1, 1, 1], [1, 1, 1, 0, 1],
    [1, -1, 1, 0, 0], [1, -1, -1, 1, 0], [1, 1, -1, 1, 1], [1, 1, 1, 0, 1],
    [-1, -1, -1, 0, 0], [-1, -1, 1, 1, 0], [-1, 1, 1, 1, 1], [-1, 1, -1, 0, 1],
    [-1, -1, -1, 0, 0], [1, -1, -1, 1, 0], [1, -1, 1, 1, 1], [-1, -1, 1, 0, 1]], dtype=np.float32)
UV_CUBE_IDX = np.array([0, 1, 2, 0, 2, 3, 4, 5, 6, 4, 6, 7, 8, 9, 10, 8, 10, 11,
                        12, 15, 14, 12, 14, 13, 16, 18, 17, 16, 19, 18, 20, 23, 22, 20, 22, 21], np.uint8)


class Run:
    """One scene: its srp library, framebuffer and what it must free."""

    def __init__(self, srp):
        self.srp = srp
        srp.new_context()
        self.fb = None
        self.free = []

    def framebuffer(self):
        self.fb = self.srp.srpNewFramebuffer(W, H)
        assert self.fb, "srpNewFramebuffer failed"
        self.free.append((self.srp.srpFreeFramebuffer, self.fb))
        return self.fb

    def vb(self, data):
        vb = self.srp.vertex_buffer(data)
        self.free.append((self.srp.srpFreeVertexBuffer, vb))
        return vb

    def ib(self, itype, idx):
        ib = self.srp.index_buffer(itype, idx)
        self.free.append((self.srp.srpFreeIndexBuffer, ib))
        return ib

    def texture(self):
        tex = _assets()["texture"]
        h, w, _ = tex.shape
        with tempfile.NamedTemporaryFile(suffix=".ppm", delete=False) as f:
            f.write(b"P6\n%d %d\n255\n" % (w, h))
            f.write(tex.tobytes())
            path = f.name
        try:
            t = self.srp.srpNewTexture(path.encode(), A.TW_REPEAT, A.TW_REPEAT)
        finally:
            os.unlink(path)
        assert t, "srpNewTexture failed"
        self.free.append((self.srp.srpFreeTexture, t))
        return t

    def teapot(self):
        z = _assets()
        vb = self.vb(z["teapot_vertices"])  # OBJVertex: position, uv, normal (32 bytes)
        ib = self.ib(A.UINT32, z["teapot_indices"])
        return vb, ib, int(z["teapot_indices"].size)

    def finish(self):
        planes = self.srp.planes(self.fb)
        for f, p in reversed(self.free):
            f(p)
        return planes


def clipping_line(srp):
    r = Run(srp)
    data = _pos_color([(p, (1, 1, 1)) for p in CUBE_CORNERS])
    u = _uniform(srp, srp.mat4ConstructTRS(0, 0, 0, 0, 0.4, 0, 0.5, 0.5, 0.5),
                 srp.mat4ConstructView(0, 0, -1.5, 0, 0, 0, 1, 1, 1),
                 srp.mat4ConstructPerspectiveProjection(-1, 1, -1, 1, 1, 10), 3, 3)
    sp = srp.program(u, "srpVsTransform", "srpFsVaryingColor", [(3, A.FLOAT, A.INTERP_PERSPECTIVE)], 12)
    srp.srpDepthTest(True)
    fb = r.framebuffer()
    vb = r.vb(data)
    ib = r.ib(A.UINT8, CUBE_EDGES_U8)
    srp.srpFramebufferClear(fb)
    srp.srpDrawIndexBuffer(ib, vb, fb, ctypes.byref(sp), A.PRIM_LINES, 0, 24)
    return r.finish()


def _teapot_uniform(srp, ry, view_z):
    return _uniform(srp, srp.mat4ConstructRotate(_rad(-90), ry, 0),
                    srp.mat4ConstructView(0, 1.75, view_z, 0, 0, 0, 1, 1, 1),
                    srp.mat4ConstructPerspectiveProjection(-1, 1, -1, 1, 1, 10))


def clipping_point(srp):
    r = Run(srp)
    u = _teapot_uniform(srp, 0.3, -2)
    u.color[0] = 2.0  # fsPrimitive divides by 2
    white = _uniform(srp)
    white.model, white.view, white.projection = u.model, u.view, u.projection
    sp1 = srp.program(u, "srpVsTransform", "srpFsPrimitiveMod")
    sp2 = srp.program(white, "srpVsTransform", "srpFsSolid")
    srp.srpRasterPolygonMode(A.POLYGON_LINE)
    srp.srpRasterPointSize(3.0)
    srp.srpDepthTest(True)
    fb = r.framebuffer()
    vb, ib, n = r.teapot()
    srp.srpFramebufferClear(fb)
    srp.srpDrawIndexBuffer(ib, vb, fb, ctypes.byref(sp1), A.PRIM_TRIANGLES, 0, n)
    srp.srpDrawIndexBuffer(ib, vb, fb, ctypes.byref(sp2), A.PRIM_POINTS, 0, n)
    return r.finish()


def clipping_triangle(srp):
    r = Run(srp)
    u = _teapot_uniform(srp, 0.2, -4)
    sp = srp.program(u, "srpVsTransform", "srpFsPrimitiveMod")
    srp.srpRasterFrontFace(A.WINDING_CW)
    srp.srpRasterCullFace(A.FACE_BACK)
    srp.srpRasterPolygonMode(A.POLYGON_FILL)
    srp.srpDepthTest(True)
    fb = r.framebuffer()
    vb, ib, n = r.teapot()
    srp.srpFramebufferClear(fb)
    srp.srpDrawIndexBuffer(ib, vb, fb, ctypes.byref(sp), A.PRIM_TRIANGLES, 0, n)
    return r.finish()


def _textured_cube(srp, mode):
    r = Run(srp)
    u = _uniform(srp, srp.mat4ConstructRotate(2.5, 0.7, 0.5), srp.mat4ConstructView(0, 0, -3, 0, 0, 0, 1, 1, 1),
                 srp.mat4ConstructPerspectiveProjection(-1, 1, -1, 1, 1, 50), 3, 2)
    u.texture = r.texture()
    sp = srp.program(u, "srpVsTransform", "srpFsTexture", [(2, A.FLOAT, mode)], 8)
    srp.srpRasterFrontFace(A.WINDING_CCW)
    srp.srpRasterCullFace(A.FACE_BACK)
    srp.srpDepthTest(True)
    fb = r.framebuffer()
    vb = r.vb(UV_CUBE)
    ib = r.ib(A.UINT8, UV_CUBE_IDX)
    srp.srpFramebufferClear(fb)
    srp.srpDrawIndexBuffer(ib, vb, fb, ctypes.byref(sp), A.PRIM_TRIANGLES, 0, 36)
    return r.finish()


def interpolation_affine(srp):
    return _textured_cube(srp, A.INTERP_AFFINE)


def interpolation_perspective(srp):
    return _textured_cube(srp, A.INTERP_PERSPECTIVE)


def interpolation_flat(srp):
    r = Run(srp)
    # Vertex { vec3 position; uint8_t color; }: 13 bytes
    data = np.zeros(3, dtype=np.dtype([("p", "<f4", 3), ("c", "u1")]))
    data["p"] = [(-0.5, -0.5, 0.0), (0.5, -0.5, 0.0), (0.0, 0.5, 0.0)]
    data["c"] = [0, 1, 2]
    assert data.dtype.itemsize == 13
    u = _uniform(srp, pass_offset=12, pass_count=1)
    # the scene declares its one-byte varying block as 3 flat floats
    sp = srp.program(u, "srpVsBytes", "srpFsBytePalette", [(3, A.FLOAT, A.INTERP_FLAT)], 1)
    fb = r.framebuffer()
    srp.srpFramebufferClear(fb)
    vb = r.vb(data)
    srp.srpProvokingVertexMode(A.PROVOKING_FIRST)
    u.model = srp.mat4ConstructTRS(-0.5, 0, 0, 0, 0, 0, 0.5, 0.5, 0.5)
    srp.srpDrawVertexBuffer(vb, fb, ctypes.byref(sp), A.PRIM_TRIANGLES, 0, 3)
    srp.srpProvokingVertexMode(A.PROVOKING_LAST)
    u.model = srp.mat4ConstructTRS(0.5, 0, 0, 0, 0, 0, 0.5, 0.5, 0.5)
    srp.srpDrawVertexBuffer(vb, fb, ctypes.byref(sp), A.PRIM_TRIANGLES, 0, 3)
    return r.finish()


def misc_depth_test(srp):
    r = Run(srp)
    data = _pos_color([(p, (1, 1, 1)) for p in CUBE_CORNERS] + [
        ((-1, -1, -1), (1, 0, 0)), ((-1, 1, 1), (0, 1, 0)), ((1, 1, -1), (0, 0, 1)),
        ((-1, 1, -1), (1, 1, 0)), ((-1, -1, 1), (0, 1, 1)), ((1, -1, -1), (1, 0, 1))])
    u = _uniform(srp, srp.mat4ConstructTRS(0, 0, 0, 0, 0.3, 0, 0.5, 0.5, 0.5),
                 srp.mat4ConstructView(0, 0, -2, 0, 0, 0, 1, 1, 1),
                 srp.mat4ConstructPerspectiveProjection(-1, 1, -1, 1, 1, 10), 3, 3)
    sp = srp.program(u, "srpVsTransform", "srpFsVaryingColor", [(3, A.FLOAT, A.INTERP_PERSPECTIVE)], 12)
    srp.srpDepthTest(True)
    fb = r.framebuffer()
    vb = r.vb(data)
    ib = r.ib(A.UINT8, CUBE_EDGES_U8)
    srp.srpFramebufferClear(fb)
    srp.srpDrawIndexBuffer(ib, vb, fb, ctypes.byref(sp), A.PRIM_LINES, 0, 24)
    srp.srpDrawVertexBuffer(vb, fb, ctypes.byref(sp), A.PRIM_TRIANGLES, 8, 6)
    return r.finish()


def misc_rasterization_rules(srp):
    r = Run(srp)
    data = _pos_color([((-0.5, -0.5, 0), (1, 0, 0)), ((0.5, 0.5, 0), (0, 1, 0)), ((-0.5, 0.5, 0), (0, 0, 1)),
                       ((0.5, 0.5, 0), (1, 1, 0)), ((0.5, -0.5, 0), (1, 0, 1)), ((-0.5, -0.5, 0), (0, 1, 1))])
    u = _uniform(srp, srp.mat4ConstructRotate(0.0, 0.0, 1.5), pass_offset=3, pass_count=3)
    sp = srp.program(u, "srpVsTransform", "srpFsVaryingColor", [(3, A.FLOAT, A.INTERP_PERSPECTIVE)], 12)
    fb = r.framebuffer()
    vb = r.vb(data)
    srp.srpFramebufferClear(fb)
    srp.srpDrawVertexBuffer(vb, fb, ctypes.byref(sp), A.PRIM_TRIANGLES, 0, 6)
    return r.finish()


def misc_scissor_test(srp):
    r = Run(srp)
    data = _pos_color([((-0.5, -0.5, 0), (1, 0, 0)), ((0.5, -0.5, 0), (0, 1, 0)), ((0, 0.5, 0), (0, 0, 1))])
    u = _uniform(srp, pass_offset=3, pass_count=3)
    sp = srp.program(u, "srpVsTransform", "srpFsVaryingColor", [(3, A.FLOAT, A.INTERP_PERSPECTIVE)], 12)
    fb = r.framebuffer()
    srp.srpScissorTest(True)
    srp.srpScissorOptions(140, 220, 200, 150)
    vb = r.vb(data)
    srp.srpFramebufferClear(fb)
    srp.srpDrawVertexBuffer(vb, fb, ctypes.byref(sp), A.PRIM_TRIANGLES, 0, 3)
    return r.finish()


def misc_stencil_test(srp):
    r = Run(srp)
    u = _uniform(srp, srp.mat4ConstructRotate(0.7, 0.7, 0.7), srp.mat4ConstructView(0, 0, -3, 0, 0, 0, 1, 1, 1),
                 srp.mat4ConstructPerspectiveProjection(-1, 1, -1, 1, 1, 50), 3, 2)
    u.texture = r.texture()
    sp = srp.program(u, "srpVsTransform", "srpFsTexture", [(2, A.FLOAT, A.INTERP_PERSPECTIVE)], 8)
    srp.srpRasterFrontFace(A.WINDING_CCW)
    srp.srpRasterCullFace(A.FACE_BACK)
    srp.srpDepthTest(True)
    srp.srpStencilTest(True)
    fb = r.framebuffer()
    vb = r.vb(UV_CUBE)
    ib = r.ib(A.UINT8, UV_CUBE_IDX)
    srp.srpFramebufferClear(fb)
    srp.srpStencilOp(A.STENCIL_KEEP, A.STENCIL_KEEP, A.STENCIL_REPLACE)
    srp.srpStencilFunc(A.COMPARE_ALWAYS, 1, 0xFF)
    srp.srpStencilWriteMask(0xFF)
    srp.srpDrawIndexBuffer(ib, vb, fb, ctypes.byref(sp), A.PRIM_TRIANGLES, 0, 36)
    scale = srp.mat4ConstructScale(1.05, 1.05, 1.05)
    model = A.Mat4.from_buffer_copy(u.model)
    u.model = srp.mat4MultiplyMat4(ctypes.byref(scale), ctypes.byref(model))
    u.color[:] = [1.0, 0.0, 0.0, 1.0]  # singleColor
    sp2 = srp.program(u, "srpVsTransform", "srpFsSolid", [(2, A.FLOAT, A.INTERP_PERSPECTIVE)], 8)
    srp.srpStencilFunc(A.COMPARE_NOTEQUAL, 1, 0xFF)
    srp.srpStencilWriteMask(0x00)
    srp.srpDepthTest(False)
    srp.srpDrawIndexBuffer(ib, vb, fb, ctypes.byref(sp2), A.PRIM_TRIANGLES, 0, 36)
    return r.finish()


def _teapot_mode(srp, mode, point_size):
    r = Run(srp)
    u = _teapot_uniform(srp, 0.3, -6)
    sp = srp.program(u, "srpVsTransform", "srpFsPrimitiveMod")
    if mode is not None:
        srp.srpRasterPolygonMode(mode)
    if point_size is not None:
        srp.srpRasterPointSize(point_size)
    srp.srpDepthTest(True)
    fb = r.framebuffer()
    vb, ib, n = r.teapot()
    srp.srpFramebufferClear(fb)
    prim = A.PRIM_POINTS if mode is None else A.PRIM_TRIANGLES
    srp.srpDrawIndexBuffer(ib, vb, fb, ctypes.byref(sp), prim, 0, n)
    return r.finish()


def polygon_modes_line(srp):
    return _teapot_mode(srp, A.POLYGON_LINE, None)


def polygon_modes_point(srp):
    return _teapot_mode(srp, A.POLYGON_POINT, 2.0)


def primitives_points(srp):
    return _teapot_mode(srp, None, 2.0)


def _square_lines(srp, prim):
    r = Run(srp)
    data = _pos_color([((-0.5, -0.5, 0), (0, 0, 0)), ((-0.5, 0.5, 0), (0, 0, 0)), ((0.5, 0.5, 0), (0, 0, 0)),
                       ((0.5, -0.5, 0), (0, 0, 0))])
    sp = srp.program(_uniform(srp), "srpVsTransform", "srpFsSolid")
    fb = r.framebuffer()
    vb = r.vb(data)
    srp.srpFramebufferClear(fb)
    srp.srpDrawVertexBuffer(vb, fb, ctypes.byref(sp), prim, 0, 4)
    return r.finish()


def primitives_line_loop(srp):
    return _square_lines(srp, A.PRIM_LINE_LOOP)


def primitives_line_strip(srp):
    return _square_lines(srp, A.PRIM_LINE_STRIP)


def primitives_lines(srp):
    r = Run(srp)
    data = _pos_color([(p, (0, 0, 0)) for p in CUBE_CORNERS])
    u = _uniform(srp, srp.mat4ConstructTRS(0, 0, 0, 0, 0.3, 0, 0.5, 0.5, 0.5),
                 srp.mat4ConstructView(0, 0, -2, 0, 0, 0, 1, 1, 1),
                 srp.mat4ConstructPerspectiveProjection(-1, 1, -1, 1, 1, 10))
    sp = srp.program(u, "srpVsTransform", "srpFsSolid")
    fb = r.framebuffer()
    vb = r.vb(data)
    ib = r.ib(A.UINT8, CUBE_EDGES_U8)
    srp.srpFramebufferClear(fb)
    srp.srpDrawIndexBuffer(ib, vb, fb, ctypes.byref(sp), A.PRIM_LINES, 0, 24)
    return r.finish()


def _four_colored(srp, rows, prim):
    r = Run(srp)
    sp = srp.program(_uniform(srp, pass_offset=3, pass_count=3), "srpVsTransform", "srpFsVaryingColor",
                     [(3, A.FLOAT, A.INTERP_PERSPECTIVE)], 12)
    fb = r.framebuffer()
    vb = r.vb(_pos_color(rows))
    srp.srpFramebufferClear(fb)
    srp.srpDrawVertexBuffer(vb, fb, ctypes.byref(sp), prim, 0, 4)
    return r.finish()


def primitives_triangle_fan(srp):
    return _four_colored(srp, [((-0.5, -0.5, 0), (1, 0, 0)), ((-0.5, 0.5, 0), (0, 1, 0)),
                               ((0.5, 0.75, 0), (0, 0, 1)), ((0.5, -0.25, 0), (1, 1, 1))], A.PRIM_TRIANGLE_FAN)


def primitives_triangle_strip(srp):
    return _four_colored(srp, [((-0.5, -0.5, 0), (1, 0, 0)), ((0.5, 0, 0), (0, 1, 0)),
                               ((-0.5, 0, 0), (0, 0, 1)), ((0.5, 0.5, 0), (1, 1, 1))], A.PRIM_TRIANGLE_STRIP)


SCENES = {f.__name__: f for f in [
    clipping_line, clipping_point, clipping_triangle, interpolation_affine, interpolation_flat,
    interpolation_perspective, misc_depth_test, misc_rasterization_rules, misc_scissor_test, misc_stencil_test,
    polygon_modes_line, polygon_modes_point, primitives_line_loop, primitives_line_strip, primitives_lines,
    primitives_points, primitives_triangle_fan, primitives_triangle_strip]}


def golden(name):
    return _assets()["golden_" + name]
