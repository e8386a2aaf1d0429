"""Host-side mirror of the reference's rt:: / spline:: call surface over the C ABI.

Reference surface (paths relative to the MachSilva/cgspline root):
  rt::Scene + BVH::build / buildHashTable   src/rt/Scene.h:97-159, src/rt/BVH.cpp:9-38
  rt::RayTracer::render / running            src/rt/RayTracer.h:13-72, src/rt/RayTracer.cu:107-180
  rt::intersect / BVH::hashIntersect         src/rt/Primitive.cu:222-268, src/rt/BVH.h:178-350
  spline::doBezierClipping / doSubdivision   src/Spline.h:488-508
  rt::PerfectHashFunction::build / hash      src/rt/PerfectHashFunction.h:30-70

Device memory comes from torch tensors; the compute is libcgspline_gb300.so.
Errors raise CgsError with the library's status code (the reference aborts or
throws; here nothing crashes the process).
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import math

import numpy as np

from . import _capi
from ._capi import check

CLIP, SUBDIV = 0, 1
FP32, FP32_POLISH64, FP64, FP32_GRAZE64 = 0, 1, 2, 3
PLAIN, WAVEFRONT = 0, 1
SPLIT_REFERENCE, SPLIT_LONGEST, SPLIT_MIRROR = 0, 1, 2
MIRROR, MONTE_CARLO = 0, 1
DEFAULT_TOL = 2.0 ** -12


def _torch():
    import torch
    return torch


def _require(ok: bool, what: str):
    """Argument check that stays in force under python -O: the library gets
    raw pointers, so a wrong shape or type must stop here."""
    if not ok:
        raise ValueError(what)


def _stream_handle(stream):
    if stream is None:
        torch = _torch()
        return C.c_void_p(torch.cuda.current_stream().cuda_stream)
    if isinstance(stream, int):
        return C.c_void_p(stream)
    return C.c_void_p(stream.cuda_stream)


def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _np_ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _material(m) -> _capi.Material:
    return _capi.Material((C.c_float * 3)(*m.diffuse), (C.c_float * 3)(*m.specular), m.metalness, m.roughness)


class GpuScene:
    """Scenes resident on one GPU: surfaces, objects, lights, BVHs and hash tables.

    `scene` is one scenes.Scene or a list of them; scene k of a list becomes
    group k of the store (its own object-level BVH, lights and environment,
    sharing the patch and BVH arrays with the others).  lib_path selects the
    library build (the product build, or _capi.LIB_NOFMA_PATH for the parity
    build without multiply-add contraction)."""

    def __init__(self, scene, device: int = 0, build: bool = True, stream=None, split: int = SPLIT_REFERENCE,
                 lib_path: str = _capi.LIB_PATH):
        self.lib = _capi.load(lib_path)
        self.scenes = list(scene) if isinstance(scene, (list, tuple)) else [scene]
        self.scene = self.scenes[0]
        self.device = device
        h = C.c_void_p()
        check(self.lib.cgs_scene_create(C.byref(h), device), "cgs_scene_create")
        self.h = h
        self._keep = []
        self.surface_base = []
        check(self.lib.cgs_scene_set_bvh_split(self.h, split), "cgs_scene_set_bvh_split")
        for g, sc in enumerate(self.scenes):
            if g > 0:
                gid = C.c_uint32()
                check(self.lib.cgs_scene_add_group(self.h, C.byref(gid)), "cgs_scene_add_group")
                if gid.value != g:
                    raise RuntimeError(f"cgs_scene_add_group gave group {gid.value}, expected {g}")
            self._add(sc)
        if build:
            self.build(stream)

    @property
    def groups(self) -> int:
        return len(self.scenes)

    def _add(self, scene):
        first = None
        for s in scene.surfaces:
            pts = np.ascontiguousarray(s.points, np.float32)
            idx = np.ascontiguousarray(s.indices, np.uint32)
            sid = C.c_uint32()
            check(self.lib.cgs_scene_add_surface(self.h, _np_ptr(pts), pts.shape[0], _np_ptr(idx), idx.size,
                                                 C.byref(sid)), "cgs_scene_add_surface")
            first = sid.value if first is None else first
        base = first if first is not None else 0
        self.surface_base.append(base)
        for o in scene.objects:
            l2w = np.ascontiguousarray(o.local2world, np.float32)
            w2l = np.ascontiguousarray(o.world2local, np.float32)
            pm = mats = None
            nm = 0
            if o.patch_material is not None:
                pm = np.ascontiguousarray(o.patch_material, np.uint32)
                arr = (_capi.Material * len(o.materials))(*[_material(m) for m in o.materials])
                mats, nm = arr, len(o.materials)
                self._keep.append(arr)
            oid = C.c_uint32()
            check(self.lib.cgs_scene_add_object(self.h, base + o.surface, _np_ptr(l2w), _np_ptr(w2l),
                                                C.byref(_material(o.material)), _np_ptr(pm),
                                                C.cast(mats, C.c_void_p) if mats is not None else None, nm,
                                                C.byref(oid)), "cgs_scene_add_object")
        self.set_lights(scene.lights)
        bg = np.asarray(scene.background, np.float32)
        amb = np.asarray(scene.ambient, np.float32)
        check(self.lib.cgs_scene_set_environment(self.h, _np_ptr(bg), _np_ptr(amb)), "cgs_scene_set_environment")

    def set_lights(self, lights):
        """Lights of the group being added (the last group)."""
        arr = (_capi.Light * max(1, len(lights)))()
        for k, l in enumerate(lights):
            arr[k] = _capi.Light((C.c_float * 3)(*l.color), l.strength, (C.c_float * 3)(*l.position), l.range,
                                 (C.c_float * 3)(*l.direction), l.angle)
        check(self.lib.cgs_scene_set_lights(self.h, C.cast(arr, C.c_void_p), len(lights)), "cgs_scene_set_lights")

    # BVH::build for every surface and the object level, then the device
    # upload and BVH::buildHashTable (MainWindow::convertScene's order).
    def build(self, stream=None):
        check(self.lib.cgs_bvh_build(self.h), "cgs_bvh_build")
        check(self.lib.cgs_hash_build(self.h, _stream_handle(stream) if stream is not None else None),
              "cgs_hash_build")

    def close(self):
        if getattr(self, "h", None):
            self.lib.cgs_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def save(self, path: str):
        """Writes the built store to a scene blob (cgs_scene_save)."""
        check(self.lib.cgs_scene_save(self.h, str(path).encode()), "cgs_scene_save")

    @classmethod
    def load(cls, path: str, device: int = 0) -> "GpuScene":
        """A store read back from a scene blob (cgs_scene_load): no BVH or hash build."""
        obj = cls.__new__(cls)
        obj.lib = _capi.load()
        h = C.c_void_p()
        check(obj.lib.cgs_scene_load(C.byref(h), str(path).encode(), device), "cgs_scene_load")
        obj.h, obj.scenes, obj.scene, obj.device, obj._keep, obj.surface_base = h, [], None, device, [], []
        return obj

    @property
    def surfaces(self) -> int:
        """Surfaces in the store (each has its patch BVH)."""
        return sum(len(sc.surfaces) for sc in self.scenes)

    def nbvh(self) -> int:
        """BVHs in the store: one per surface and one object-level BVH per group."""
        return self.surfaces + self.groups

    def bvh_sizes(self, which: int):
        """(nodes, leaf-list words, table size, displacement size, keys) of BVH
        `which` (surface id, or -1-g for the object level of group g)."""
        sz = np.zeros(5, np.uint32)
        check(self.lib.cgs_bvh_sizes(self.h, which, _np_ptr(sz)), "cgs_bvh_sizes")
        return tuple(int(x) for x in sz)

    def footprint(self) -> int:
        b = C.c_uint64()
        check(self.lib.cgs_scene_footprint(self.h, C.byref(b)), "cgs_scene_footprint")
        return int(b.value)

    def bvh(self, which: int):
        """Export one BVH: which = surface id, or -1-g for the object level of group g."""
        sz = np.zeros(5, np.uint32)
        check(self.lib.cgs_bvh_sizes(self.h, which, _np_ptr(sz)), "cgs_bvh_sizes")
        nodes = np.zeros((int(sz[0]), 14), np.uint32)
        keys = np.zeros(int(sz[4]), np.uint32)
        ind = np.zeros(int(sz[1]), np.uint32)
        table = np.zeros(int(sz[2]), np.uint32)
        disp = np.zeros(int(sz[3]), np.uint32)
        par = np.zeros(4, np.uint32)
        check(self.lib.cgs_bvh_export(self.h, which, _np_ptr(nodes), _np_ptr(keys), _np_ptr(ind), _np_ptr(table),
                                      _np_ptr(disp), _np_ptr(par)), "cgs_bvh_export")
        return dict(nodes=nodes, keys=keys, indices=ind, table=table, disp=disp,
                    A=int(par[0]), B=int(par[1]), N=int(par[2]), mask=int(par[3]))

    def counters(self) -> dict:
        c = _capi.Counters()
        check(self.lib.cgs_scene_counters(self.h, C.byref(c)), "cgs_scene_counters")
        return {k: int(getattr(c, k)) for k, _ in _capi.Counters._fields_}

    # rt::intersect / BVH::hashIntersect over a batch of rays
    def intersect(self, rays, method=CLIP, precision=FP32, tol=DEFAULT_TOL, any_hit=False, stream=None, out=None,
                  group=None):
        """rays: (7, n) float32 torch CUDA tensor (ox oy oz dx dy dz tmax) or numpy array (host path);
        group: per-ray group ids (same kind as rays; None = group 0).
        Returns dict t, u, v, patch, object (patch = -1 on a miss)."""
        if isinstance(rays, np.ndarray):
            return self._intersect_host(rays, method, precision, tol, any_hit, stream, group)
        torch = _torch()
        _require(rays.is_cuda and rays.dtype == torch.float32 and rays.dim() == 2 and rays.shape[0] == 7,
                 "rays: a (7, n) float32 CUDA tensor")
        rays = rays.contiguous()
        n = rays.shape[1]
        if out is None:
            fo = torch.empty((3, n), dtype=torch.float32, device=rays.device)
            io = torch.empty((2, n), dtype=torch.int32, device=rays.device)
        else:
            fo, io = out
        gp = None
        if group is not None:
            group = group.to(device=rays.device, dtype=torch.int32).contiguous()
            _require(group.numel() == n, "group: one id per ray")
            gp = group.data_ptr()
        r = _capi.Rays(*[rays[k].data_ptr() for k in range(7)], gp)
        h = _capi.Hits(fo[0].data_ptr(), fo[1].data_ptr(), fo[2].data_ptr(), io[0].data_ptr(), io[1].data_ptr())
        check(self.lib.cgs_intersect(self.h, C.byref(r), n, method, precision, tol, int(any_hit), C.byref(h),
                                     _stream_handle(stream)), "cgs_intersect")
        return dict(t=fo[0], u=fo[1], v=fo[2], patch=io[0], object=io[1])

    def traverse(self, rays, any_hit=False, stream=None, group=None, lengths=None, copy_lengths=True):
        """cgs_traverse: the traversal kernel alone (the query engine's first
        collect pass, no clipping) over (7, n) device rays.  Returns the
        per-ray candidate-list lengths (int32 tensor; patches plus object
        markers, at most 64), or None with copy_lengths=False."""
        torch = _torch()
        _require(rays.is_cuda and rays.dtype == torch.float32 and rays.dim() == 2 and rays.shape[0] == 7,
                 "rays: a (7, n) float32 CUDA tensor")
        rays = rays.contiguous()
        n = rays.shape[1]
        if lengths is None and copy_lengths:
            lengths = torch.empty(n, dtype=torch.int32, device=rays.device)
        gp = None
        if group is not None:
            group = group.to(device=rays.device, dtype=torch.int32).contiguous()
            _require(group.numel() == n, "group: one id per ray")
            gp = group.data_ptr()
        r = _capi.Rays(*[rays[k].data_ptr() for k in range(7)], gp)
        check(self.lib.cgs_traverse(self.h, C.byref(r), n, int(any_hit), _ptr(lengths) if copy_lengths else None,
                                    _stream_handle(stream)), "cgs_traverse")
        return lengths if copy_lengths else None

    def _intersect_host(self, rays, method, precision, tol, any_hit, stream, group=None):
        rays = np.ascontiguousarray(rays, np.float32)
        _require(rays.ndim == 2 and rays.shape[0] == 7, "rays: a (7, n) float32 array")
        n = rays.shape[1]
        fo = np.zeros((3, n), np.float32)
        io = np.zeros((2, n), np.int32)
        gp = None
        if group is not None:
            group = np.ascontiguousarray(group, np.uint32)
            _require(group.size == n, "group: one id per ray")
            gp = group.ctypes.data
        r = _capi.Rays(*[rays[k].ctypes.data for k in range(7)], gp)
        h = _capi.Hits(fo[0].ctypes.data, fo[1].ctypes.data, fo[2].ctypes.data, io[0].ctypes.data, io[1].ctypes.data)
        check(self.lib.cgs_intersect_host(self.h, C.byref(r), n, method, precision, tol, int(any_hit), C.byref(h),
                                          _stream_handle(stream) if stream is not None else None),
              "cgs_intersect_host")
        return dict(t=fo[0], u=fo[1], v=fo[2], patch=io[0], object=io[1])


def do_bezier_clipping(scene: GpuScene, surface: int, rays, patch_ids, t=None, tol=DEFAULT_TOL, method=CLIP,
                       stream=None):
    """spline::doBezierClipping(hit, ray, buffer, patch, tol) for a batch of
    (ray, patch) pairs on the device.  t is hit.distance in/out (default inf).
    Returns (found[int32], t, u, v) torch tensors."""
    torch = _torch()
    n = rays.shape[1]
    dev = rays.device
    tt = torch.full((n,), math.inf, dtype=torch.float32, device=dev) if t is None else t.clone()
    u = torch.zeros(n, dtype=torch.float32, device=dev)
    v = torch.zeros(n, dtype=torch.float32, device=dev)
    found = torch.zeros(n, dtype=torch.int32, device=dev)
    pid = patch_ids.to(torch.int32).contiguous()
    r = _capi.Rays(*[rays[k].data_ptr() for k in range(7)], None)
    h = _capi.Hits(tt.data_ptr(), u.data_ptr(), v.data_ptr(), found.data_ptr(), None)
    check(scene.lib.cgs_patch_intersect(scene.h, surface, C.byref(r), _ptr(pid), n, method, tol, C.byref(h),
                                        _stream_handle(stream)), "cgs_patch_intersect")
    return found, tt, u, v


def normal(scene: GpuScene, surface: int, patch_ids, u, v, stream=None):
    """rt::normal (src/rt/Primitive.cu:270-275) for a batch: the unit normal of
    patch patch_ids[k] of `surface` at (u[k], v[k]), in the surface's space.
    Returns a (3, n) float32 tensor (zeros for a patch id past the surface)."""
    torch = _torch()
    pid = patch_ids.to(torch.int32).contiguous()
    uu, vv = u.to(torch.float32).contiguous(), v.to(torch.float32).contiguous()
    n = pid.numel()
    out = torch.empty((3, n), dtype=torch.float32, device=pid.device)
    check(scene.lib.cgs_patch_normal(scene.h, surface, _ptr(pid), _ptr(uu), _ptr(vv), n, _ptr(out),
                                     _stream_handle(stream)), "cgs_patch_normal")
    return out


@dataclasses.dataclass
class Options:
    """rt::RayTracer::Options (src/rt/RayTracer.h:26-34) plus the search method,
    precision and schedule of this implementation."""
    recursion_depth: int = 6
    eps: float = 1e-4
    flip_y: bool = False
    method: int = CLIP
    precision: int = FP32
    tol: float = DEFAULT_TOL
    schedule: int = WAVEFRONT
    sampling: int = MIRROR

    def c(self) -> _capi.RenderOptions:
        return _capi.RenderOptions(self.recursion_depth, self.eps, int(self.flip_y), self.method, self.precision,
                                   self.tol, self.schedule, self.sampling)


class Frame:
    """A device framebuffer of RGBA8 sRGB pixels (src/rt/Frame.h:263-328); the
    stride is aligned to `alignment` pixels as the reference's frames are."""

    def __init__(self, width: int, height: int, alignment: int = 32, device: int = 0, linear: bool = False):
        torch = _torch()
        self.width, self.height = width, height
        a = max(1, alignment)
        self.stride = (width + a - 1) // a * a
        self.data = torch.zeros((height, self.stride), dtype=torch.int32, device=f"cuda:{device}")
        self.linear = torch.zeros((height, width, 3), dtype=torch.float32, device=f"cuda:{device}") if linear else None

    def rgba(self):
        """(h, w, 4) uint8 numpy copy."""
        d = self.data[:, : self.width].contiguous().cpu().numpy().view(np.uint8)
        return d.reshape(self.height, self.width, 4)


@dataclasses.dataclass
class Request:
    """One render request of a batch: `spp` jittered samples per pixel of a
    width x height image of group `group`; outputs are device tensors
    (framebuffer (h, w) int32 packed RGBA8 sRGB, linear (h, w, 3) float32)."""
    group: int
    camera: object
    width: int
    height: int
    spp: int = 1
    recursion_depth: int = -1
    framebuffer: object = None
    linear: object = None

    @classmethod
    def alloc(cls, group, camera, width, height, spp=1, recursion_depth=-1, linear=False, device=0):
        torch = _torch()
        fb = torch.zeros((height, width), dtype=torch.int32, device=f"cuda:{device}")
        lin = torch.zeros((height, width, 3), dtype=torch.float32, device=f"cuda:{device}") if linear else None
        return cls(group, camera, width, height, spp, recursion_depth, fb, lin)

    def c(self) -> _capi.RenderRequest:
        return _capi.RenderRequest(self.group, camera_struct(self.camera), self.width, self.height, self.spp,
                                   self.recursion_depth,
                                   self.framebuffer.data_ptr() if self.framebuffer is not None else None,
                                   self.linear.data_ptr() if self.linear is not None else None)

    def rgba(self):
        d = self.framebuffer.contiguous().cpu().numpy().view(np.uint8)
        return d.reshape(self.height, self.width, 4)


def camera_struct(cam) -> _capi.Camera:
    return _capi.Camera((C.c_float * 4)(*cam.rotation), (C.c_float * 3)(*cam.position), (C.c_float * 3)(*cam.scale),
                        cam.fovy)


def camera_rays(camera, width: int, height: int, flip_y: bool = False, device: int = 0, stream=None):
    """Primary rays of a width x height frame (cgs_camera_rays): (7, w*h) float32 CUDA tensor."""
    torch = _torch()
    lib = _capi.load()
    rays = torch.empty((7, width * height), dtype=torch.float32, device=f"cuda:{device}")
    check(lib.cgs_camera_rays(C.byref(camera_struct(camera)), width, height, int(flip_y), _ptr(rays),
                              _stream_handle(stream)), "cgs_camera_rays")
    return rays


class RayTracer:
    """rt::RayTracer: asynchronous render of a resident scene into a device frame."""

    def __init__(self, options: Options | None = None):
        self.options = options or Options()
        self.lib = _capi.load()
        self._scene = None

    def render(self, frame: Frame, camera, scene: GpuScene, stream=None):
        self._scene = scene
        o = self.options.c()
        check(self.lib.cgs_render(scene.h, C.byref(camera_struct(camera)), frame.width, frame.height, C.byref(o),
                                  _ptr(frame.data), frame.stride, _ptr(frame.linear), _stream_handle(stream)),
              "cgs_render")

    def render_host(self, camera, scene: GpuScene, width: int, height: int, linear: bool = True, stream=None,
                    out=None):
        """Render into host memory (copies inside); returns (packed (h,w) uint32, linear (h,w,3) or None).
        out: (fb, lin) arrays to write into instead of new ones (e.g. views of pinned memory);
        lin may be None."""
        if out is not None:
            fb, lin = out
            _require(fb.dtype == np.uint32 and fb.shape == (height, width) and fb.flags.c_contiguous,
                     "out[0]: a C-contiguous (height, width) uint32 array")
            _require(lin is None or (lin.dtype == np.float32 and lin.shape == (height, width, 3)
                                     and lin.flags.c_contiguous),
                     "out[1]: None or a C-contiguous (height, width, 3) float32 array")
        else:
            fb = np.zeros((height, width), np.uint32)
            lin = np.zeros((height, width, 3), np.float32) if linear else None
        o = self.options.c()
        check(self.lib.cgs_render_host(scene.h, C.byref(camera_struct(camera)), width, height, C.byref(o),
                                       _np_ptr(fb), _np_ptr(lin),
                                       _stream_handle(stream) if stream is not None else None), "cgs_render_host")
        return fb, lin

    def render_batch(self, requests, scene: GpuScene, stream=None):
        """Render a list of Request objects of any groups of `scene` together
        (one wavefront for all of them, or one launch each with PLAIN)."""
        self._scene = scene
        arr = (_capi.RenderRequest * len(requests))()
        for k, q in enumerate(requests):
            arr[k] = q.c()
        o = self.options.c()
        check(self.lib.cgs_render_batch(scene.h, arr, len(requests), C.byref(o), _stream_handle(stream)),
              "cgs_render_batch")

    def running(self) -> bool:
        return bool(self._scene is not None and self.lib.cgs_render_running(self._scene.h))


class Server:
    """Continuous-batching request server over a resident GpuScene
    (cgs_server_*): render and ray-query requests of any groups, cut into
    chunks that fit a slot's share of `memory_budget`, batched and run on
    `slots` concurrent streams.  Options.schedule = PLAIN gives the
    one-request-per-launch baseline (one slot, the plain kernels)."""

    def __init__(self, scene: GpuScene, slots: int = 4, memory_budget: int = 16 << 30, max_batch_samples: int = 0,
                 max_batch_requests: int = 0, options: Options | None = None):
        self.lib = _capi.load()
        self.scene = scene
        self.options = options or Options()
        o = _capi.ServerOptions(slots, memory_budget, max_batch_samples, max_batch_requests, self.options.c())
        h = C.c_void_p()
        check(self.lib.cgs_server_create(C.byref(h), scene.h, C.byref(o)), "cgs_server_create")
        self.h = h
        self._keep = {}

    def submit_render(self, req: "Request") -> int:
        t = C.c_uint64()
        check(self.lib.cgs_server_submit_render(self.h, C.byref(req.c()), C.byref(t)), "cgs_server_submit_render")
        self._keep[t.value] = req
        return t.value

    def submit_query(self, group: int, rays, any_hit: bool = False, out=None):
        """rays: (7, n) float32 CUDA tensor.  Returns (ticket, hits dict of device tensors)."""
        torch = _torch()
        n = rays.shape[1]
        if out is None:
            fo = torch.empty((3, n), dtype=torch.float32, device=rays.device)
            io = torch.empty((2, n), dtype=torch.int32, device=rays.device)
        else:
            fo, io = out
        r = _capi.Rays(*[rays[k].data_ptr() for k in range(7)], None)
        h = _capi.Hits(fo[0].data_ptr(), fo[1].data_ptr(), fo[2].data_ptr(), io[0].data_ptr(), io[1].data_ptr())
        q = _capi.QueryRequest(group, n, int(any_hit), r, h)
        t = C.c_uint64()
        check(self.lib.cgs_server_submit_query(self.h, C.byref(q), C.byref(t)), "cgs_server_submit_query")
        self._keep[t.value] = (rays, fo, io)
        return t.value, dict(t=fo[0], u=fo[1], v=fo[2], patch=io[0], object=io[1])

    def wait(self, ticket: int, timeout: float = -1.0) -> dict:
        info = _capi.RequestInfo()
        st = self.lib.cgs_server_wait(self.h, ticket, timeout, C.byref(info))
        check(st, "cgs_server_wait")
        self._keep.pop(ticket, None)
        return {k: getattr(info, k) for k, _ in _capi.RequestInfo._fields_}

    def clock(self) -> float:
        return float(self.lib.cgs_server_clock(self.h))

    def stats(self) -> dict:
        s = _capi.ServerStats()
        check(self.lib.cgs_server_stats_get(self.h, C.byref(s)), "cgs_server_stats_get")
        return {k: getattr(s, k) for k, _ in _capi.ServerStats._fields_}

    def close(self):
        if getattr(self, "h", None):
            self.lib.cgs_server_destroy(self.h)
            self.h = None
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def engine_config() -> dict:
    """The query engine's runtime settings (cgs_engine_config_get)."""
    lib = _capi.load()
    c = _capi.EngineConfig()
    check(lib.cgs_engine_config_get(C.byref(c)), "cgs_engine_config_get")
    return {k: getattr(c, k) for k, _ in _capi.EngineConfig._fields_}


def set_engine_config(**kw):
    lib = _capi.load()
    cur = engine_config()
    cur.update(kw)
    c = _capi.EngineConfig(**cur)
    check(lib.cgs_engine_config_set(C.byref(c)), "cgs_engine_config_set")


def debug_fail_allocation(nth: int):
    """cgs_debug_fail_allocation: the nth growth of a working buffer from now
    on (1 = the next) reports out of memory on the host; 0 cancels."""
    check(_capi.load().cgs_debug_fail_allocation(int(nth)), "cgs_debug_fail_allocation")


def autotune(scene: GpuScene, requests, options: Options | None = None, repeats: int = 3, stream=None):
    """cgs_autotune_render: a coordinate descent over the engine settings on
    this batch (two rounds over the knobs, each timed `repeats` times); keeps
    the fastest.  Returns (settings dict, median ms)."""
    lib = _capi.load()
    arr = (_capi.RenderRequest * len(requests))()
    for k, q in enumerate(requests):
        arr[k] = q.c()
    o = (options or Options()).c()
    best = _capi.EngineConfig()
    ms = C.c_double()
    check(lib.cgs_autotune_render(scene.h, arr, len(requests), C.byref(o), repeats, C.byref(best), C.byref(ms),
                                  _stream_handle(stream)), "cgs_autotune_render")
    return {k: getattr(best, k) for k, _ in _capi.EngineConfig._fields_}, float(ms.value)


class PerfectHashFunction:
    """rt::PerfectHashFunction on the device (deterministic build)."""

    def __init__(self):
        self.lib = _capi.load()
        self.A = 31
        self.B = 19
        self.N = 0
        self.mask = 0
        self.disp = None
        self.table = None
        self.trials = 0

    @staticmethod
    def displacement_size(n: int) -> int:
        s = max(2, (n - 1) >> 1)
        return 1 << (s.bit_length() - 1)

    @staticmethod
    def table_capacity(n: int) -> int:
        step = max(4, int(np.float32(0.05) * np.float32(n)))
        return n + 15 * step

    def build(self, keys, stream=None) -> int:
        """keys: uint32 torch CUDA tensor (or numpy).  Returns 0 on success
        (the reference returns non-zero on failure)."""
        torch = _torch()
        if isinstance(keys, np.ndarray):
            keys = torch.from_numpy(keys.astype(np.uint32).view(np.int32)).cuda()
        n = keys.numel()
        dsz, tcap = self.displacement_size(n), self.table_capacity(n)
        disp = torch.zeros(dsz, dtype=torch.int32, device=keys.device)
        table = torch.zeros(tcap, dtype=torch.int32, device=keys.device)
        par = np.zeros(5, np.uint32)
        st = self.lib.cgs_perfect_hash_build(_ptr(keys), n, _ptr(disp), dsz, _ptr(table), tcap, _np_ptr(par),
                                             _stream_handle(stream))
        self.A, self.B, self.N, self.mask, self.trials = (int(x) for x in par)
        if st == 0:
            self.disp = disp.cpu().numpy().view(np.uint32).copy()
            self.table = table[: self.N].cpu().numpy().view(np.uint32).copy()
        return st

    def hash(self, key: int) -> int:
        return ((self.A * key + self.B + int(self.disp[key & self.mask])) & 0xFFFFFFFF) % self.N
