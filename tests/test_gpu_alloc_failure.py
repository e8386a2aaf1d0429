"""GPU tests of the out-of-memory paths: a working buffer that cannot grow
(injected on the host by cgs_debug_fail_allocation, which frees the old
buffer and reports out of memory without calling the allocator) fails its
call with CGS_ERR_OUT_OF_MEMORY, and the next calls on the same scene,
frame slot or server grow their buffers again and return the same results
as a scene that never failed.

Each injection fails one growth at a different point of the sequence (the
query engine's scratch; the first, a middle or the last of a render slot's
buffers; a server slot's query staging), so that every buffer that a failed
call freed is grown again before it is used.
"""
import numpy as np
import pytest

from cgspline_gb300 import scenes as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch
    return torch


@pytest.fixture(scope="module")
def rt():
    from cgspline_gb300 import rt
    return rt


@pytest.fixture(autouse=True)
def no_injection_after(rt):
    yield
    rt.debug_fail_allocation(0)


@pytest.fixture(scope="module")
def torus():
    return S.scene_c2(nu=32, nv=32)


def host(d):
    return {k: v if isinstance(v, np.ndarray) else v.cpu().numpy() for k, v in d.items()}


def same_hits(a, b):
    return all(np.array_equal(a[k], b[k]) for k in a)


# device rays grow the engine scratch only; host rays grow the ray staging,
# the two hit stagings and then the engine scratch, in that order
@pytest.mark.parametrize("where,nth", [("device", 1), ("host", 1), ("host", 3), ("host", 4)])
def test_query_scratch_grows_again(rt, torus, torch, where, nth):
    from cgspline_gb300 import _capi
    small = rt.camera_rays(S.camera_c2(), 64, 36)
    big = rt.camera_rays(S.camera_c2(), 320, 180)
    if where == "host":
        small, big = small.cpu().numpy(), big.cpu().numpy()
    fresh = rt.GpuScene(torus)
    want_small, want_big = host(fresh.intersect(small)), host(fresh.intersect(big))
    fresh.close()
    g = rt.GpuScene(torus)
    assert same_hits(host(g.intersect(small)), want_small)
    rt.debug_fail_allocation(nth)
    with pytest.raises(_capi.CgsError) as err:
        g.intersect(big)
    assert err.value.status == 3
    rt.debug_fail_allocation(0)
    # smaller than the capacity the scene held before the failure
    assert same_hits(host(g.intersect(small)), want_small)
    assert same_hits(host(g.intersect(big)), want_big)
    g.close()


@pytest.mark.parametrize("nth", [1, 3, 9, 17])
def test_render_slot_grows_again(rt, torus, torch, nth):
    from cgspline_gb300 import _capi
    opts = rt.Options(recursion_depth=1, precision=rt.FP32_POLISH64)
    cam = S.camera_c2()

    def frames(g, tr, sizes):
        out = []
        for w, h in sizes:
            f = rt.Frame(w, h)
            tr.render(f, cam, g)
            torch.cuda.synchronize()
            out.append(f.rgba())
        return out

    fresh = rt.GpuScene(torus)
    want_small, want_big = frames(fresh, rt.RayTracer(opts), [(64, 36), (320, 180)])
    fresh.close()
    g = rt.GpuScene(torus)
    tr = rt.RayTracer(opts)
    assert np.array_equal(frames(g, tr, [(64, 36)])[0], want_small)
    rt.debug_fail_allocation(nth)
    with pytest.raises(_capi.CgsError) as err:
        tr.render(rt.Frame(320, 180), cam, g)
    assert err.value.status == 3
    rt.debug_fail_allocation(0)
    small, big = frames(g, tr, [(64, 36), (320, 180)])
    assert np.array_equal(small, want_small)
    assert np.array_equal(big, want_big)
    g.close()


@pytest.mark.parametrize("nth", [1, 4])
def test_server_slot_grows_again(rt, torus, torch, nth):
    opts = rt.Options(recursion_depth=1, precision=rt.FP32_POLISH64)
    small = rt.camera_rays(S.camera_c2(), 64, 36)
    big = rt.camera_rays(S.camera_c2(), 320, 180)
    g = rt.GpuScene(torus)
    want_small = host(g.intersect(small, precision=rt.FP32_POLISH64))
    want_big = host(g.intersect(big, precision=rt.FP32_POLISH64))
    req = rt.Request.alloc(0, S.camera_c2(), 96, 54, spp=1, recursion_depth=1)
    tr = rt.RayTracer(rt.Options(recursion_depth=1, precision=rt.FP32_POLISH64, schedule=rt.WAVEFRONT))
    tr.render_batch([req], g)
    torch.cuda.synchronize()
    want_frame = req.rgba()

    sv = rt.Server(g, slots=1, memory_budget=4 << 30, options=opts)

    def query(rays):
        t, out = sv.submit_query(0, rays)
        return sv.wait(t, timeout=120.0), out

    info, out = query(small)
    assert info["status"] == 0 and same_hits(host(out), want_small)
    rt.debug_fail_allocation(nth)
    info, _ = query(big)
    assert info["status"] == 3
    rt.debug_fail_allocation(0)
    info, out = query(small)
    assert info["status"] == 0 and same_hits(host(out), want_small)
    # a render on the slot whose query buffers failed, then the big query
    r2 = rt.Request.alloc(0, S.camera_c2(), 96, 54, spp=1, recursion_depth=1)
    assert sv.wait(sv.submit_render(r2), timeout=120.0)["status"] == 0
    assert np.array_equal(r2.rgba(), want_frame)
    info, out = query(big)
    assert info["status"] == 0 and same_hits(host(out), want_big)
    sv.close()
    g.close()
