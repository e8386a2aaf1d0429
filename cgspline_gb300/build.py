"""Build libcgspline_gb300.so in-tree with nvcc for sm_103a.

Each .cu under csrc/ compiles to an object in parallel, then one link step.
Host code is compiled with -ffp-contract=off so the host BVH build (centroids,
object bounds) rounds identically on x86-64 and aarch64.

build(fmad=False) builds the same sources with nvcc --fmad=false into
libcgspline_gb300_nofma.so: device arithmetic without multiply-add
contraction, rounding every product and sum as the reference's host code
does.  It is the parity build the tests compare bit for bit with the
reference; the product library is the contracted one.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libcgspline_gb300.so")
LIB_NOFMA = os.path.join(OUT_DIR, "libcgspline_gb300_nofma.so")
# load-bandwidth probes (L1, L2) for the roofline denominators; not part of the library
MEMBENCH_SRC = os.path.join(HERE, "membench", "membench.cu")
MEMBENCH_LIB = os.path.join(OUT_DIR, "libcgs_membench.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++20", "-O3", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off", "--expt-relaxed-constexpr",
              "-I", os.path.join(HERE, "..", "include")]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _newest_input() -> float:
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(HERE, "..", "include", "cgspline.h"),
                                                                 __file__]
    return max(os.path.getmtime(f) for f in files if os.path.isfile(f))


def build(force: bool = False, verbose: bool = False, fmad: bool = True) -> str:
    lib = LIB if fmad else LIB_NOFMA
    if not force and os.path.exists(lib) and os.path.getmtime(lib) >= _newest_input():
        return lib
    objdir = os.path.join(OUT_DIR, "obj" if fmad else "obj_nofma")
    os.makedirs(objdir, exist_ok=True)
    nv = nvcc()
    extra = [] if fmad else ["--fmad=false"]

    def compile_one(src):
        obj = os.path.join(objdir, os.path.basename(src) + ".o")
        cmd = [nv, *ARCH, *NVCC_FLAGS, *extra, "-c", src, "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        return obj, r.stderr

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        results = list(ex.map(compile_one, sources()))
    if verbose:
        for _, err in results:
            sys.stderr.write(err)
    tmp = lib + f".tmp{os.getpid()}"
    cmd = [nv, *ARCH, "-shared", "-o", tmp, *[o for o, _ in results], "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


def build_membench(force: bool = False) -> str:
    if not force and os.path.exists(MEMBENCH_LIB) and os.path.getmtime(MEMBENCH_LIB) >= os.path.getmtime(MEMBENCH_SRC):
        return MEMBENCH_LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = MEMBENCH_LIB + f".tmp{os.getpid()}"
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-shared", MEMBENCH_SRC, "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError(f"nvcc failed for {MEMBENCH_SRC}:\n{r.stderr}")
    os.replace(tmp, MEMBENCH_LIB)
    return MEMBENCH_LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
    print(build(force="--force" in sys.argv, fmad=False))
    print(build_membench(force="--force" in sys.argv))
