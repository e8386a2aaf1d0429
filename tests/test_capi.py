"""The C ABI library builds, loads and exports every symbol include/cgspline.h declares
(no compute calls: runs without a GPU)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", fn)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(cgs_[a-z0-9_]+)\s*\(", txt))
    return names


@pytest.fixture(scope="module")
def lib():
    import shutil
    if not shutil.which("nvcc") and not os.path.exists("/usr/local/cuda/bin/nvcc"):
        pytest.skip("nvcc not available")
    from cgspline_gb300 import build
    path = build.build()
    return ctypes.CDLL(path)


def test_exports_every_declared_symbol(lib):
    names = declared_symbols()
    assert len(names) >= 20
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from cgspline_gb300 import _capi
    bound = {n for n, _, _ in _capi.SIGNATURES}
    assert declared_symbols() <= bound | set(), declared_symbols() - bound


def test_status_strings_without_gpu(lib):
    lib.cgs_status_string.restype = ctypes.c_char_p
    assert lib.cgs_status_string(0) == b"ok"
    assert b"hash" in lib.cgs_status_string(5)
    lib.cgs_version.restype = ctypes.c_int
    assert lib.cgs_version() >= 1


def test_invalid_arguments_rejected_without_gpu(lib):
    # null scene / null outputs are rejected before any CUDA call
    assert lib.cgs_scene_create(None, 0) == 1
    assert lib.cgs_scene_destroy(None) == 1
    assert lib.cgs_bvh_build(None) == 1
    assert lib.cgs_render(None, None, 0, 0, None, None, 0, None, None) == 1


def test_python_mirror_checks_arrays_before_the_library(lib):
    """The Python mirror refuses wrongly shaped host arrays before it hands
    their pointers to the library (checks that hold under python -O)."""
    import numpy as np
    from cgspline_gb300 import rt, scenes
    tr = rt.RayTracer(rt.Options())
    cam = scenes.camera_c1()
    with pytest.raises(ValueError):
        tr.render_host(cam, None, 4, 4, out=(np.zeros((3, 4), np.uint32), None))
    with pytest.raises(ValueError):
        tr.render_host(cam, None, 4, 4, out=(np.zeros((4, 4), np.int64), None))
    with pytest.raises(ValueError):
        tr.render_host(cam, None, 4, 4, out=(np.zeros((4, 4), np.uint32), np.zeros((4, 4), np.float32)))
    with pytest.raises(ValueError):
        rt.GpuScene._intersect_host(None, np.zeros((6, 5), np.float32), rt.CLIP, rt.FP32, rt.DEFAULT_TOL, False,
                                    None)


def test_header_serves_a_c_caller(lib, tmp_path):
    """include/cgspline.h compiles as pedantic C99, and a C program links
    against the library and calls it (calls that need no GPU)."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    from cgspline_gb300 import build
    so = build.build()
    src = tmp_path / "caller.c"
    src.write_text(
        '#include <stdio.h>\n#include <string.h>\n#include "cgspline.h"\n'
        "int main(void)\n{\n"
        "    if (cgs_scene_destroy(NULL) != CGS_ERR_INVALID_ARGUMENT) return 1;\n"
        "    if (strlen(cgs_status_string(CGS_OK)) == 0) return 2;\n"
        '    printf("%s\\n", cgs_status_string(CGS_ERR_INVALID_ARGUMENT));\n'
        "    return 0;\n}\n")
    exe = tmp_path / "caller"
    libdir = os.path.dirname(so)
    name = os.path.basename(so)[3:-3]  # libNAME.so -> NAME
    subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", os.path.join(ROOT, "include"),
                    str(src), "-o", str(exe), "-L", libdir, "-l" + name, "-Wl,-rpath," + libdir], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    assert out.strip()
