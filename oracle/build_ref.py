"""TEST INFRASTRUCTURE -- build oracle/_ref/libcgs_ref.so from the reference's own sources.

Compiles the reference's hot-path sources, unchanged and where they lie in the
reference tree, as host C++ with g++ against the from-scratch Ds stand-in
(oracle/ds_compat), together with oracle/ref_bridge.cpp (a C ABI over them)
and oracle/ref_host_cudart.cpp (host-memory CUDA runtime calls).  Nothing is
copied out of the reference tree; the library links the oracle's
libcgs_oracle.so for the deterministic perfect-hash displacement table (the
reference's GPU build cannot run without a GPU and is not deterministic).

The reference tree is read from $CGS_REFERENCE_ROOT (default /root/reference).
Where it is absent -- on a machine that only has this repository -- build()
returns None and the tests that need the library skip.

Run:  python oracle/build_ref.py
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT, "libcgs_ref.so")
COMPAT = os.path.join(HERE, "ds_compat")
CUDA_INC = os.environ.get("CUDA_HOME", "/usr/local/cuda") + "/include"

# The reference's sources on the ray--patch path (paths inside its tree).
REF_SOURCES = [
    "src/Spline_BezierClipping.cu",   # doBezierClipping, host and device clip loops
    "src/Spline_Subdivision.cu",      # doSubdivision, host and device
    "src/Spline.cu",                  # spline::normal
    "src/rt/BVH.cpp",                 # BVH::build / split / wrap / link / buildHashTable
    "src/rt/Primitive.cu",            # BezierSurface::buildBVH, rt::intersect, rt::normal
    "src/rt/Scene.cu",                # Transform matrices, Scene::buildBVH
    "src/rt/SoA.cpp",
    "src/rt/PBR.cu",                  # lightVector, lightColor
    "src/rt/CPURayTracer.cpp",        # the CPU renderer: tiles, trace, intersect, closestHit
    "src/rt/CUDAUtility.cpp",         # CUDA_CHECK, ManagedResource
    "src/Log.cpp",
]
OWN_SOURCES = [os.path.join(HERE, "ref_bridge.cpp"), os.path.join(HERE, "ref_host_cudart.cpp")]


def reference_root() -> str | None:
    root = os.environ.get("CGS_REFERENCE_ROOT", "/root/reference")
    return root if os.path.isfile(os.path.join(root, "src", "Spline_BezierClipping.cu")) else None


def _flags(root: str) -> list[str]:
    return ["-std=c++20", "-O2", "-ffp-contract=off", "-fPIC", "-include", os.path.join(COMPAT, "prelude.h"),
            "-I", COMPAT, "-I", CUDA_INC, "-I", os.path.join(CUDA_INC, "cccl"), "-I", os.path.join(root, "src"),
            "-I", os.path.join(root, "src", "rt")]


def _inputs(root: str) -> list[str]:
    own = OWN_SOURCES + [__file__]
    for d, _, fs in os.walk(COMPAT):
        own += [os.path.join(d, f) for f in fs]
    ref = [os.path.join(root, s) for s in REF_SOURCES]
    for sub in ("src", os.path.join("src", "rt")):
        ref += [os.path.join(root, sub, f) for f in os.listdir(os.path.join(root, sub)) if f.endswith(".h")]
    return own + ref


def build(force: bool = False) -> str | None:
    root = reference_root()
    if root is None:
        return None
    import oracle
    olib = oracle.build()
    newest = max(os.path.getmtime(f) for f in _inputs(root) + [olib])
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    os.makedirs(os.path.join(OUT, "obj"), exist_ok=True)
    flags = _flags(root)

    def compile_one(src: str) -> str:
        is_ref = src.startswith(root)
        name = os.path.relpath(src, root).replace(os.sep, "_") if is_ref else os.path.basename(src)
        obj = os.path.join(OUT, "obj", name + ".o")
        cmd = ["g++", *(["-x", "c++"] if src.endswith(".cu") else []), *flags, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError(f"g++ failed for {src}:\n{r.stderr[-4000:]}")
        return obj

    srcs = [os.path.join(root, s) for s in REF_SOURCES] + OWN_SOURCES
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + f".tmp{os.getpid()}"
    odir = os.path.dirname(olib)
    cmd = ["g++", "-shared", "-o", tmp, *objs, "-L", odir, "-l:" + os.path.basename(olib),
           "-Wl,-rpath," + odir, "-Wl,--no-undefined", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError(f"link failed:\n{r.stderr[-4000:]}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    sys.path.insert(0, os.path.dirname(HERE))
    print(build(force="--force" in sys.argv))
