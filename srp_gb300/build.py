"""Build the GPU library (sm_103a) and its helper artifacts in-tree.

Outputs (all git-ignored):
  srp_gb300/lib/libsrp_gb300.so        the srp API on the GPU (C ABI)
  srp_gb300/lib/libsrp_scenes_gpu.so   seeded scenes driven through that API
  oracle/_build/port_scenes            the CPU oracle (test infrastructure)
  oracle/_ref/...                      the reference built from source, only
                                       where its sources are present
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "srp_gb300")
CSRC = os.path.join(PKG, "csrc")
LIB = os.path.join(PKG, "lib")
OBJ = os.path.join(PKG, "_build")
INC = os.path.join(ROOT, "include")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
CU_SOURCES = ["k_front.cu", "k_bin.cu", "k_raster.cu", "k_shade.cu", "k_mlp.cu", "srp_api.cu", "srp_fixed.cu",
              "srp_learned.cu"]
# Units whose device arithmetic must round exactly as the reference's fp32
# code (vertex transform, setup, barycentrics, depth): no multiply-add
# contraction there. Shading (colour, held to 1/255) and the network's
# training and inference kernels may contract.
CONTRACTED = {"k_shade.cu", "k_mlp.cu"}
C_SOURCES = ["srp_math.c", "imageio.c"]


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build srp_gb300")


def _have_zlib():
    return os.path.exists("/usr/include/zlib.h")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(INC, "srp", f) for f in os.listdir(os.path.join(INC, "srp"))]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs


def build(verbose=False, ptxas_info=False):
    os.makedirs(LIB, exist_ok=True)
    os.makedirs(OBJ, exist_ok=True)
    nvcc = _nvcc()
    zdef = ["-DSRP_HAVE_ZLIB"] if _have_zlib() else []
    zlib = ["-lz"] if _have_zlib() else []
    hdrs = _headers()
    jobs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src + ".o")
        if _stale(o, [s] + hdrs):
            fmad = [] if src in CONTRACTED else ["-fmad=false"]
            cmd = [nvcc, ARCH, "-O3", "-lineinfo", "-std=c++17", *fmad, "-Xcompiler", "-fPIC",
                   "-I", INC, "-I", CSRC, *zdef, "-c", s, "-o", o]
            if ptxas_info:
                cmd.insert(2, "-Xptxas=-v")
            jobs.append(cmd)
    for src in C_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src + ".o")
        if _stale(o, [s] + hdrs):
            jobs.append(["gcc", "-std=c11", "-O3", "-fPIC", "-ffp-contract=off", "-fno-fast-math",
                         "-I", INC, *zdef, "-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    objs = [os.path.join(OBJ, s + ".o") for s in CU_SOURCES + C_SOURCES]
    so = os.path.join(LIB, "libsrp_gb300.so")
    if _stale(so, objs):
        _run([nvcc, ARCH, "-shared", "-o", so, *objs, *zlib])
    scenes = os.path.join(LIB, "libsrp_scenes_gpu.so")
    ssrc = [os.path.join(PKG, "scenes", "scenes.c")]
    if _stale(scenes, ssrc + [so] + hdrs):
        cuda = os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
        _run(["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-DSCENES_GPU", "-I", INC,
              "-I", os.path.join(cuda, "include"), *ssrc, "-o", scenes, "-L", LIB, "-lsrp_gb300",
              "-Wl,-rpath,$ORIGIN", "-L", os.path.join(cuda, "lib64"), "-lcudart",
              "-Wl,-rpath," + os.path.join(cuda, "lib64"), "-lm"])
    return so


def reference_dir():
    """Where the reference's sources are read from (test infrastructure only):
    $SRP_REFERENCE, else the read-only checkout of the build machine."""
    return os.environ.get("SRP_REFERENCE", "/root/reference")


def build_oracle():
    """CPU oracle (always) and the reference build (only where its sources are)."""
    _run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"])
    ref = reference_dir()
    if os.path.isdir(os.path.join(ref, "src")):
        _run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={ref}"])


if __name__ == "__main__":
    build(verbose=True, ptxas_info="--ptxas" in sys.argv)
    build_oracle()
    print("built", os.path.join(LIB, "libsrp_gb300.so"))
