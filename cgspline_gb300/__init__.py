"""cgspline_gb300 -- GB300 (sm_103a) ray--bicubic-patch path of MachSilva/cgspline.

Compute lives in libcgspline_gb300.so (CUDA kernels + C ABI, include/cgspline.h);
this package is the host-side mirror of the reference's call surface
(rt.py), the seeded synthetic scenes (scenes.py) and the build recipe
(build.py).
"""
from . import rt, scenes  # noqa: F401

__all__ = ["scenes", "rt", "build_library"]


def build_library(force: bool = False, verbose: bool = False) -> str:
    from . import build
    return build.build(force=force, verbose=verbose)
