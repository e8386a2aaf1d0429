"""TEST INFRASTRUCTURE -- the CPU oracle for the ray--bicubic-patch path.

Loads ``oracle/_build/libcgs_oracle.so`` (the restatement in cgs_oracle.cpp)
through ctypes.  Only tests/, __graft_entry__.smoke() and bench.py's
cpu_baseline / reference arm may import this package; the product in
cgspline_gb300/ never does.

Parity unpinned: the reference program cannot be compiled without its
un-vendored Ds submodule and holds no golden vectors, so the restatement is
pinned by analytic known-answer patches, the reference's BVH and hash
invariants and the agreement of its FP32 variants with its FP64 search.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libcgs_oracle.so")
SRC = os.path.join(HERE, "cgs_oracle.cpp")

CLIP_HOST, CLIP_DEVICE, SUBDIV = 0, 1, 2
# the precision form's clip: CLIP_DEVICE, with near-grazing candidates (ray
# within GRAZE_5 / GRAZE_30 of the plane of the patch diagonals, graze_sin of
# intersect) searched on an FP64-projected net with FP64 fat-line bounds to
# tolerance 2^-20
CLIP_GRAZE64 = 5
# the host clip with the true convex hull of the fat-line bounds in place of
# the reference's one-pass scan (oracle only: finds roots that scan drops);
# with precision FP64 the FP64 search clips with it too
CLIP_EXACT_HULL = 6


def set_graze_mode(mode: int):
    """The near-grazing test of CLIP_GRAZE64: 1 (default) the diagonals' and
    the nine control-net cells' normals, with silhouettes; 0 the diagonals'
    plane alone."""
    lib().ora_set_graze_mode(int(mode))


def set_graze64_ray(on: int):
    """CLIP_GRAZE64: project a near-grazing candidate from the object-space
    ray computed in double from the world ray (1, the default), or from the
    FP32 one (0)."""
    lib().ora_set_graze64_ray(int(on))
GRAZE_5, GRAZE_30 = 0.0871557427, 0.5
FP32, FP32_POLISH64, FP64 = 0, 1, 2


def build(force: bool = False) -> str:
    """Compile the restatement (g++, -ffp-contract=off so x86-64 and aarch64 agree)."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = ["g++", "-std=c++20", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-o", tmp, SRC, "-lpthread"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        P = C.c_void_p
        fp = np.ctypeslib.ndpointer(np.float32, flags="C")
        u32 = np.ctypeslib.ndpointer(np.uint32, flags="C")
        L.ora_scene_new.restype = P
        L.ora_scene_free.argtypes = [P]
        L.ora_scene_add_surface.argtypes = [P, fp, C.c_uint32, u32, C.c_uint32]
        L.ora_scene_add_object.argtypes = [P, C.c_int, fp, fp, fp, P, P, C.c_uint32]
        L.ora_scene_set_lights.argtypes = [P, P, C.c_uint32]
        L.ora_scene_set_env.argtypes = [P, fp, fp]
        L.ora_scene_build.argtypes = [P]
        L.ora_scene_set_split.argtypes = [P, C.c_int]
        L.ora_set_graze_sin.argtypes = [C.c_float]
        L.ora_philox.argtypes = [u32, C.c_uint32, C.c_uint32]
        L.ora_bvh_sizes.argtypes = [P, C.c_int, u32]
        L.ora_bvh_export.argtypes = [P, C.c_int, u32, u32, u32, u32, u32, u32]
        L.ora_hash_build.argtypes = [u32, C.c_uint32, u32, u32, C.c_uint32, u32, C.c_uint32]
        L.ora_intersect.argtypes = [P, fp, C.c_uint64, C.c_int, C.c_int, C.c_float, C.c_double, C.c_int,
                                    fp, np.ctypeslib.ndpointer(np.int32, flags="C"), P, C.c_int]
        L.ora_render.argtypes = [P, fp, C.c_uint32, C.c_uint32, C.c_int, C.c_float, C.c_int, C.c_float,
                                 P, P, P, C.c_int, P]
        L.ora_render_rows.argtypes = [P, fp, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int, C.c_float,
                                      C.c_int, C.c_float, P, P, P, C.c_int, P]
        L.ora_render_spp.argtypes = [P, fp, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int, C.c_float, C.c_int,
                                     C.c_float, C.c_int, P, P, C.c_int]
        L.ora_intersect_stats.argtypes = [P, fp, C.c_uint64, C.c_int, C.c_float, C.c_int, u32, C.c_int]
        L.ora_camera_rays.argtypes = [fp, C.c_uint32, C.c_uint32, fp]
        L.ora_patch_intersect.argtypes = [fp, u32, fp, C.c_float, C.c_int, P, P, P]
        L.ora_patch_subdiv_host.argtypes = [fp, u32, fp, C.c_float, P, P]
        L.ora_set_graze_mode.argtypes = [C.c_int]
        L.ora_set_graze64_ray.argtypes = [C.c_int]
        L.ora_patch_eval.argtypes = [fp, C.c_float, C.c_float, fp, fp]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class OracleScene:
    """A built scene (BVHs + perfect hashes) in the oracle."""

    def __init__(self, scene, split=0):
        """split: 0 the reference's BVH split axis (always y), 1 the longest
        axis of the elements' centroid box."""
        L = lib()
        self.scene = scene
        self.h = L.ora_scene_new()
        L.ora_scene_set_split(self.h, split)
        for s in scene.surfaces:
            pts = np.ascontiguousarray(s.points, np.float32)
            idx = np.ascontiguousarray(s.indices, np.uint32)
            r = L.ora_scene_add_surface(self.h, pts, pts.shape[0], idx, idx.size)
            if r < 0:
                raise ValueError(f"bad surface ({r})")
        self._keep = []
        for o in scene.objects:
            pm = mats = None
            nm = 0
            if o.patch_material is not None:
                pm = np.ascontiguousarray(o.patch_material, np.uint32)
                mats = np.ascontiguousarray(np.stack([m.packed() for m in o.materials]), np.float32)
                nm = len(o.materials)
                self._keep += [pm, mats]
            r = L.ora_scene_add_object(self.h, o.surface, np.ascontiguousarray(o.local2world, np.float32),
                                       np.ascontiguousarray(o.world2local, np.float32), o.material.packed(),
                                       _ptr(pm), _ptr(mats), nm)
            if r < 0:
                raise ValueError(f"bad object ({r})")
        if scene.lights:
            lights = np.ascontiguousarray(np.stack([l.packed() for l in scene.lights]), np.float32)
            L.ora_scene_set_lights(self.h, _ptr(lights), len(scene.lights))
        L.ora_scene_set_env(self.h, np.asarray(scene.background, np.float32), np.asarray(scene.ambient, np.float32))
        e = L.ora_scene_build(self.h)
        if e:
            raise RuntimeError(f"oracle scene build failed ({e})")

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.ora_scene_free(self.h)
            self.h = None

    def bvh(self, which: int):
        """which = surface index, or -1 for the top-level BVH."""
        L = lib()
        sz = np.zeros(5, np.uint32)
        if L.ora_bvh_sizes(self.h, which, sz):
            raise IndexError(which)
        nodes = np.zeros((int(sz[0]), 14), np.uint32)
        keys = np.zeros(int(sz[4]), np.uint32)
        ind = np.zeros(int(sz[1]), np.uint32)
        table = np.zeros(int(sz[2]), np.uint32)
        disp = np.zeros(int(sz[3]), np.uint32)
        par = np.zeros(4, np.uint32)
        L.ora_bvh_export(self.h, which, nodes, keys, ind, table, disp, par)
        return dict(nodes=nodes, keys=keys, indices=ind, table=table, disp=disp,
                    A=int(par[0]), B=int(par[1]), N=int(par[2]), mask=int(par[3]))

    def intersect(self, rays, method=CLIP_HOST, precision=FP32, tol=2.0 ** -12, tol64=1e-9, any_hit=False,
                  nthreads=None, counters=False, graze_sin=GRAZE_30):
        """graze_sin: the grazing margin of CLIP_GRAZE64 (GRAZE_5 restates the
        GPU's FP32_POLISH64 level, GRAZE_30 its FP32_GRAZE64 level)."""
        L = lib()
        L.ora_set_graze_sin(graze_sin)
        rays = np.ascontiguousarray(rays, np.float32)
        n = rays.shape[1]
        of = np.zeros((3, n), np.float32)
        oi = np.zeros((2, n), np.int32)
        cnt = np.zeros(8, np.uint64) if counters else None
        nt = nthreads or os.cpu_count() or 1
        r = L.ora_intersect(self.h, rays, n, method, precision, tol, tol64, int(any_hit), of, oi, _ptr(cnt), nt)
        if r:
            raise RuntimeError(f"ora_intersect failed ({r})")
        out = dict(t=of[0], u=of[1], v=of[2], patch=oi[0], object=oi[1])
        if counters:
            out["counters"] = dict(zip(["nodes", "leaves", "hash_lookups", "candidates", "clip_iterations",
                                        "pushes", "max_depth", "overflow"], [int(x) for x in cnt]))
        return out

    def intersect_stats(self, rays, method=CLIP_HOST, tol=2.0 ** -12, any_hit=False, nthreads=None):
        """Per-ray work: dict of (n,) arrays nodes, hash_lookups, candidates, iterations."""
        rays = np.ascontiguousarray(rays, np.float32)
        n = rays.shape[1]
        out = np.zeros((4, n), np.uint32)
        lib().ora_intersect_stats(self.h, rays, n, method, tol, int(any_hit), out, nthreads or os.cpu_count() or 1)
        return dict(nodes=out[0], hash_lookups=out[1], candidates=out[2], iterations=out[3])

    def render(self, camera, w, h, depth=1, eps=1e-4, method=CLIP_HOST, tol=2.0 ** -12, nthreads=None,
               want_rgb=True, want_packed=True):
        L = lib()
        rgb = np.zeros((h, w, 3), np.float32) if want_rgb else None
        packed = np.zeros((h, w), np.uint32) if want_packed else None
        counts = np.zeros(3, np.uint64)
        secs = np.zeros(1, np.float64)
        nt = nthreads or os.cpu_count() or 1
        r = L.ora_render(self.h, camera.packed(), w, h, depth, eps, method, tol, _ptr(rgb), _ptr(packed),
                         _ptr(counts), nt, _ptr(secs))
        if r:
            raise RuntimeError(f"ora_render failed ({r})")
        return dict(rgb=rgb, packed=packed, primary=int(counts[0]), bounce=int(counts[1]),
                    shadow=int(counts[2]), seconds=float(secs[0]))


    def render_spp(self, camera, w, h, spp, depth=1, eps=1e-4, method=CLIP_HOST, tol=2.0 ** -12, nthreads=None,
                   mc=False):
        """spp jittered samples per pixel, averaged (linear rgb and packed sRGB);
        mc: the Monte-Carlo bounce (Philox keyed by image sample and depth)."""
        L = lib()
        rgb = np.zeros((h, w, 3), np.float32)
        packed = np.zeros((h, w), np.uint32)
        nt = nthreads or os.cpu_count() or 1
        r = L.ora_render_spp(self.h, camera.packed(), w, h, spp, depth, eps, method, tol, int(mc), _ptr(rgb),
                             _ptr(packed), nt)
        if r:
            raise RuntimeError(f"ora_render_spp failed ({r})")
        return dict(rgb=rgb, packed=packed)

    def render_rows(self, camera, w, h, row0, row_step, depth=1, eps=1e-4, method=CLIP_HOST, tol=2.0 ** -12,
                    nthreads=None):
        """Render rows row0, row0+row_step, ... of a w x h frame (a bounded CPU sample)."""
        L = lib()
        rgb = np.zeros((h, w, 3), np.float32)
        counts = np.zeros(3, np.uint64)
        secs = np.zeros(1, np.float64)
        nt = nthreads or os.cpu_count() or 1
        r = L.ora_render_rows(self.h, camera.packed(), w, h, row0, row_step, depth, eps, method, tol, _ptr(rgb),
                              None, _ptr(counts), nt, _ptr(secs))
        if r:
            raise RuntimeError(f"ora_render_rows failed ({r})")
        return dict(rgb=rgb, primary=int(counts[0]), bounce=int(counts[1]), shadow=int(counts[2]),
                    seconds=float(secs[0]), threads=nt)


def philox(counter, key):
    """Philox4x32-10 of (counter[4], key[2]) -> 4 x uint32."""
    c = np.ascontiguousarray(counter, np.uint32).copy()
    lib().ora_philox(c, int(key[0]), int(key[1]))
    return c


def camera_rays(camera, w, h):
    rays = np.zeros((7, w * h), np.float32)
    lib().ora_camera_rays(camera.packed(), w, h, rays)
    return rays


def hash_build(keys):
    keys = np.ascontiguousarray(keys, np.uint32)
    n = keys.size
    par = np.zeros(5, np.uint32)
    cap_d = max(2, n)
    cap_t = n + 16 * max(4, int(np.float32(0.05) * np.float32(n))) + 16
    disp = np.zeros(cap_d, np.uint32)
    table = np.zeros(cap_t, np.uint32)
    e = lib().ora_hash_build(keys, n, par, disp, cap_d, table, cap_t)
    dsize = int(par[3]) + 1
    return dict(status=int(e), A=int(par[0]), B=int(par[1]), N=int(par[2]), mask=int(par[3]),
                trials=int(par[4]), disp=disp[:dsize], table=table[:int(par[2])])


def patch_intersect(points, idx16, ray7, tol=2.0 ** -12, method=CLIP_HOST, t=np.inf):
    tt = np.array([t], np.float32)
    uv = np.zeros(2, np.float32)
    st = np.zeros(4, np.uint64)
    hit = lib().ora_patch_intersect(np.ascontiguousarray(points, np.float32), np.ascontiguousarray(idx16, np.uint32),
                                    np.ascontiguousarray(ray7, np.float32), tol, method, _ptr(tt), _ptr(uv), _ptr(st))
    return bool(hit), float(tt[0]), uv, st


def patch_subdiv_host(points, idx16, ray7, threshold=2.0 ** -4, t=np.inf, tmin=1.0):
    """doSubdivision_host (src/Spline_Subdivision.cu:166-288) on one (ray,
    patch) pair: 3-D sub-net boxes, triangle hits below `threshold` in u and
    v.  The ray interval is [tmin, ray7[6]] (rt::intersect passes 1 and the
    ray's max)."""
    r = np.asarray(ray7, np.float32)
    ray9 = np.array([*r[:6], tmin, r[6], 0.0], np.float32)
    tt = np.array([t], np.float32)
    uv = np.zeros(2, np.float32)
    hit = lib().ora_patch_subdiv_host(np.ascontiguousarray(points, np.float32), np.ascontiguousarray(idx16, np.uint32),
                                      ray9, threshold, _ptr(tt), _ptr(uv))
    return bool(hit), float(tt[0]), uv


def patch_eval(net16x4, u, v):
    p = np.zeros(3, np.float32)
    n = np.zeros(3, np.float32)
    lib().ora_patch_eval(np.ascontiguousarray(net16x4, np.float32), u, v, p, n)
    return p, n
