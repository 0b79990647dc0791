"""The C-ABI library: it loads, exports every function the public headers
declare, and its host-side validation reports through the message callback
the way the reference does. No GPU work is issued here."""
import ctypes
import os
import re
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in ("context.h", "buffer.h", "framebuffer.h", "texture.h", "vec.h", "mat.h", "gpu.h", "shaderlib.h"):
        src = open(os.path.join(ROOT, "include", "srp", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b((?:srp|vec[234]|mat4)\w*)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_headers_declare_the_reference_api():
    names = declared_functions()
    for n in ("srpNewContext", "srpDrawIndexBuffer", "srpDrawVertexBuffer", "srpFramebufferClear",
              "srpStencilOpSeparate", "srpTextureGetFilteredColor", "mat4ConstructPerspectiveProjection",
              "vec3Normalize", "srpGpuFramebufferSync", "srpVsTransform"):
        assert n in names
    assert len(names) > 60


REF = os.environ.get("SRP_REFERENCE", "/root/reference")


def layout(include_dir, tmp_path, tag):
    exe = str(tmp_path / f"abi_{tag}")
    subprocess.check_call(["gcc", "-std=c2x", "-I", include_dir, "-o", exe,
                           os.path.join(ROOT, "tests", "native", "abi_layout.c")])
    return subprocess.check_output([exe]).decode()


def test_struct_layouts(tmp_path):
    """Every public struct's size, alignment and member offsets, and the
    public enums' values, as this library's headers define them."""
    out = layout(os.path.join(ROOT, "include"), tmp_path, "ours")
    lines = out.splitlines()
    assert len(lines) > 90
    assert "sizeof vec3 12 align 1" in lines  # packed: user vertex structs rely on it


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "include", "srp")),
                    reason="reference headers not present on this machine")
def test_struct_layouts_match_the_reference_headers(tmp_path):
    """The same probe compiled against the reference's own headers prints the
    same layouts, so a program built against the reference hands this
    library the bytes it expects."""
    assert layout(os.path.join(ROOT, "include"), tmp_path, "ours") == \
        layout(os.path.join(REF, "include"), tmp_path, "ref")


def test_library_exports_every_declared_symbol(built_library):
    out = subprocess.check_output(["nm", "-D", "--defined-only", built_library]).decode()
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing
    assert "srpContext" in exported


HOST_SCRIPT = r"""
import ctypes, sys
sys.path.insert(0, sys.argv[1])
import srp_gb300 as s
L = s.lib()
msgs = []
@s.MESSAGE_CALLBACK
def cb(t, sev, fn, msg, user):
    msgs.append((t, sev, fn.decode(), msg.decode()))
ctx = ctypes.c_void_p.in_dll(L, "srpContext")
L.srpNewContext.argtypes = [ctypes.c_void_p]
L.srpNewContext(ctypes.addressof(ctx))
L.srpNewVertexBuffer.restype = ctypes.c_void_p
L.srpNewIndexBuffer.restype = ctypes.c_void_p
L.srpSetMessageCallback(s.SRPMessageCallback(cb, None))
vb = ctypes.c_void_p(L.srpNewVertexBuffer())
data = (ctypes.c_float * 30)()
L.srpVertexBufferCopyData.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_void_p]
L.srpVertexBufferCopyData(vb, 12, 120, data)
L.srpDrawVertexBuffer.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t, ctypes.c_size_t]
L.srpDrawVertexBuffer(vb, None, None, 4, 8, 3)   # 8..10 of 10 vertices: out of range
L.srpDrawVertexBuffer(vb, None, None, 42, 0, 3)  # unknown primitive
L.srpDrawVertexBuffer(vb, None, None, 4, 0, 0)   # empty draw: nothing
L.srpRasterCullFace(3)                           # FRONT_AND_BACK: triangle draws are no-ops
L.srpDrawVertexBuffer(vb, None, None, 4, 0, 9)
ib = ctypes.c_void_p(L.srpNewIndexBuffer())
L.srpIndexBufferCopyData.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t, ctypes.c_void_p]
L.srpIndexBufferCopyData(ib, 4, 16, data)        # SRP_INT32 has no index size
for m in msgs:
    print("MSG", m)
"""


def test_host_validation_reports_like_the_reference(built_library):
    out = subprocess.check_output([sys.executable, "-c", HOST_SCRIPT, ROOT], cwd=ROOT).decode()
    msgs = [l for l in out.splitlines() if l.startswith("MSG")]
    assert any("checkOOB" in m and "indices 8-10 (size: 10)" in m for m in msgs), msgs
    assert any("drawBuffer" in m and "Unknown primitive type: 42" in m for m in msgs), msgs
    assert any("srpSizeofType" in m for m in msgs), msgs
    assert len(msgs) == 3, msgs


NO_GPU_SCRIPT = r"""
import ctypes, sys
sys.path.insert(0, sys.argv[1])
import srp_gb300 as s
L = s.lib()
msgs = []
@s.MESSAGE_CALLBACK
def cb(t, sev, fn, msg, user):
    msgs.append((t, sev, fn.decode(), msg.decode()))
ctx = ctypes.c_void_p.in_dll(L, "srpContext")
L.srpNewContext.argtypes = [ctypes.c_void_p]
L.srpNewContext(ctypes.addressof(ctx))
L.srpSetMessageCallback(s.SRPMessageCallback(cb, None))
L.srpNewFramebuffer.restype = ctypes.c_void_p
L.srpNewFramebuffer.argtypes = [ctypes.c_size_t, ctypes.c_size_t]
fb = L.srpNewFramebuffer(64, 48)
print("FB", fb)
for m in msgs:
    print("MSG", m)
"""


def test_without_a_gpu_the_library_reports_instead_of_falling_back(built_library):
    """No CPU fallback: where no GPU can be used, creating a framebuffer
    reports the CUDA error through the message callback and returns NULL."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    out = subprocess.check_output([sys.executable, "-c", NO_GPU_SCRIPT, ROOT], cwd=ROOT).decode()
    assert "FB None" in out, out
    msgs = [l for l in out.splitlines() if l.startswith("MSG")]
    assert any("srpNewFramebuffer" in m and "CUDA error" in m for m in msgs), msgs
