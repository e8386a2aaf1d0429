"""TEST INFRASTRUCTURE -- the reference program's own hot path, built from its sources.

Loads oracle/_ref/libcgs_ref.so, which oracle/build_ref.py compiles from the
reference's unchanged sources (with the from-scratch Ds stand-in in
oracle/ds_compat and the C ABI of oracle/ref_bridge.cpp).  It exists only
where the reference tree is present; available() says whether it does.  Only
tests/ and tests/golden/make_golden.py use it, to pin the oracle's
restatement (cgs_oracle.cpp) to the reference itself.

The reference's perfect-hash build needs a GPU and is not deterministic; the
library takes its displacement tables from the oracle's deterministic
restatement and fills and uses the hash table with the reference's own code.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build_ref

_lib = None
_err = None


def lib():
    global _lib, _err
    if _lib is None and _err is None:
        try:
            path = build_ref.build()
        except Exception as e:  # a failed build is reported by available()
            _err = str(e)
            return None
        if path is None:
            _err = "reference tree not present"
            return None
        L = C.CDLL(path)
        P = C.c_void_p
        fp = np.ctypeslib.ndpointer(np.float32, flags="C")
        u32 = np.ctypeslib.ndpointer(np.uint32, flags="C")
        i32 = np.ctypeslib.ndpointer(np.int32, flags="C")
        L.ref_scene_new.restype = P
        L.ref_scene_free.argtypes = [P]
        L.ref_scene_add_surface.argtypes = [P, fp, C.c_uint32, u32, C.c_uint32]
        L.ref_scene_add_object.argtypes = [P, C.c_int, fp, fp, fp]
        L.ref_scene_set_lights.argtypes = [P, fp, C.c_uint32]
        L.ref_scene_set_env.argtypes = [P, fp, fp]
        L.ref_scene_build.argtypes = [P]
        L.ref_bvh_sizes.argtypes = [P, C.c_int, u32]
        L.ref_bvh_export.argtypes = [P, C.c_int, u32, u32, u32]
        L.ref_intersect.argtypes = [P, fp, C.c_uint64, C.c_int, fp, i32, C.c_int]
        L.ref_render.argtypes = [P, fp, C.c_uint32, C.c_uint32, C.c_int, C.c_float, C.c_int, P, P]
        L.ref_patch_intersect.argtypes = [fp, C.c_uint32, u32, fp, C.c_float, C.c_int, fp, fp]
        L.ref_patch_normal.argtypes = [fp, C.c_uint32, u32, C.c_uint32, u32, fp, fp, C.c_uint32, fp]
        L.ref_pack_srgb.argtypes = [fp, C.c_uint64, u32]
        _lib = L
    return _lib


def available() -> bool:
    return lib() is not None


def unavailable_reason() -> str | None:
    lib()
    return _err


CLIP, SUBDIV = 0, 1


class RefScene:
    """A scenes.Scene built by the reference's own code (rt::Scene, BVHs)."""

    def __init__(self, scene):
        L = lib()
        if L is None:
            raise RuntimeError(f"reference build unavailable: {_err}")
        self.h = L.ref_scene_new()
        for s in scene.surfaces:
            pts = np.ascontiguousarray(s.points, np.float32).reshape(-1, 4)
            idx = np.ascontiguousarray(s.indices, np.uint32).reshape(-1)
            if L.ref_scene_add_surface(self.h, pts, pts.shape[0], idx, idx.size) < 0:
                raise ValueError("bad surface")
        for ob in scene.objects:
            if ob.patch_material is not None:
                raise ValueError("the reference has one material per object")
            m = np.ascontiguousarray(ob.material.packed(), np.float32)
            if L.ref_scene_add_object(self.h, ob.surface, np.ascontiguousarray(ob.local2world, np.float32),
                                      np.ascontiguousarray(ob.world2local, np.float32), m) < 0:
                raise ValueError("bad object")
        if scene.lights:
            lt = np.concatenate([np.asarray(l.packed(), np.float32) for l in scene.lights])
            L.ref_scene_set_lights(self.h, lt, len(scene.lights))
        L.ref_scene_set_env(self.h, np.asarray(scene.background, np.float32), np.asarray(scene.ambient, np.float32))
        r = L.ref_scene_build(self.h)
        if r:
            raise RuntimeError(f"ref_scene_build failed ({r})")

    def close(self):
        if self.h:
            lib().ref_scene_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def bvh(self, which: int):
        L = lib()
        sz = np.zeros(3, np.uint32)
        if L.ref_bvh_sizes(self.h, which, sz):
            raise IndexError(which)
        nodes = np.zeros((int(sz[0]), 14), np.uint32)
        keys = np.zeros(int(sz[1]), np.uint32)
        ind = np.zeros(int(sz[2]), np.uint32)
        L.ref_bvh_export(self.h, which, nodes, keys, ind)
        return dict(nodes=nodes, keys=keys, indices=ind)

    def intersect(self, rays, any_hit=False, nthreads=None):
        rays = np.ascontiguousarray(rays, np.float32)
        n = rays.shape[1]
        of = np.zeros((3, n), np.float32)
        oi = np.zeros((2, n), np.int32)
        r = lib().ref_intersect(self.h, rays, n, int(any_hit), of, oi, nthreads or os.cpu_count() or 1)
        if r:
            raise RuntimeError(f"ref_intersect failed ({r})")
        if any_hit:
            return dict(hit=oi[0].astype(bool))
        return dict(t=of[0], u=of[1], v=of[2], patch=oi[0], object=oi[1])

    def render(self, camera, w, h, depth=1, eps=1e-4, nthreads=None, want_rgb=True):
        packed = np.zeros((h, w), np.uint32)
        rgb = np.zeros((h, w, 3), np.float32) if want_rgb else None
        r = lib().ref_render(self.h, camera.packed(), w, h, depth, eps, nthreads or os.cpu_count() or 1,
                             packed.ctypes.data_as(C.c_void_p),
                             rgb.ctypes.data_as(C.c_void_p) if rgb is not None else None)
        if r:
            raise RuntimeError(f"ref_render failed ({r})")
        return dict(packed=packed, rgb=rgb)


def patch_intersect(points, idx16, ray7, tol=2.0 ** -12, method=CLIP, t=np.inf, tmin=1.0):
    """One (ray, patch) pair through spline::doBezierClipping or
    spline::doSubdivision (host).  tmin / the ray's max are the ray interval
    the subdivision's box and triangle tests use (rt::intersect passes 1 and
    the ray's max)."""
    pts = np.ascontiguousarray(points, np.float32).reshape(-1, 4)
    r = np.asarray(ray7, np.float32)
    ray9 = np.array([*r[:6], tmin, r[6], 0.0], np.float32)
    tt = np.array([t], np.float32)
    uv = np.zeros(2, np.float32)
    hit = lib().ref_patch_intersect(pts, pts.shape[0], np.ascontiguousarray(idx16, np.uint32), ray9, tol, method,
                                    tt, uv)
    if hit < 0:
        raise ValueError("index out of range")
    return bool(hit), float(tt[0]), uv


def patch_normal(points, indices, patch, u, v):
    pts = np.ascontiguousarray(points, np.float32).reshape(-1, 4)
    idx = np.ascontiguousarray(indices, np.uint32).reshape(-1)
    patch = np.ascontiguousarray(patch, np.uint32)
    out = np.zeros((patch.size, 3), np.float32)
    r = lib().ref_patch_normal(pts, pts.shape[0], idx, idx.size // 16, patch, np.ascontiguousarray(u, np.float32),
                               np.ascontiguousarray(v, np.float32), patch.size, out)
    if r:
        raise ValueError("patch id out of range")
    return out


def pack_srgb(rgb):
    rgb = np.ascontiguousarray(rgb, np.float32)
    out = np.zeros(rgb.size // 3, np.uint32)
    lib().ref_pack_srgb(rgb.reshape(-1), out.size, out)
    return out.reshape(rgb.shape[:-1])
