"""GPU tests of the request server (cgs_server_*): continuous batching of
render and ray-query requests over resident scene groups.

Bars: every request's result is bit-identical whether it runs alone or in a
mix of other requests, groups, sizes and chunkings, and equals the direct
entry points (cgs_render_batch, cgs_intersect) bit for bit; the plain
schedule equals the plain path; admission and argument errors are refused
on the host with their status codes, and the slots stay inside the budget.
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


@pytest.fixture(scope="module")
def store(rt):
    return rt.GpuScene([S.scene_c1(), S.scene_c2(nu=32, nv=32), S.scene_c4(3, max_patches=4096)])


def cams():
    return [S.camera_c1(), S.camera_c2(), S.camera_c4(3)[0]]


RENDERS = [(0, 64, 48, 1, 0), (1, 96, 54, 2, 1), (2, 80, 80, 1, 2), (1, 33, 21, 3, 1), (2, 120, 90, 1, 1),
           (0, 16, 200, 1, 1)]


def make_renders(rt):
    c = cams()
    return [rt.Request.alloc(g, c[g], w, h, spp=s, recursion_depth=d, linear=True) for g, w, h, s, d in RENDERS]


def query_rays(oracle_mod, torch):
    out = []
    for g, (cam, w, h) in enumerate([(S.camera_c1(), 40, 30), (S.camera_c2(), 64, 36), (S.camera_c4(3)[0], 50, 50)]):
        out.append((g, torch.from_numpy(oracle_mod.camera_rays(cam, w, h)).cuda(), g == 1))
    return out


def run_server(rt, torch, store, renders, queries, **kw):
    sv = rt.Server(store, **kw)
    tickets, qouts = [], []
    for r in renders:
        tickets.append(sv.submit_render(r))
    for g, rays, any_hit in queries:
        t, out = sv.submit_query(g, rays, any_hit=any_hit)
        tickets.append(t)
        qouts.append(out)
    infos = [sv.wait(t, timeout=120.0) for t in tickets]
    stats = sv.stats()
    sv.close()
    torch.cuda.synchronize()
    return infos, qouts, stats


def test_results_same_alone_and_in_mix(rt, store, oracle_mod, torch):
    opts = rt.Options(recursion_depth=1, precision=rt.FP32_POLISH64)
    queries = query_rays(oracle_mod, torch)
    # alone: one request at a time, one slot, no chunking limit
    alone_r, alone_q = [], []
    for spec in RENDERS:
        req = make_renders(rt)[RENDERS.index(spec)]
        run_server(rt, torch, store, [req], [], slots=1, options=opts)
        alone_r.append(req)
    for q in queries:
        _, outs, _ = run_server(rt, torch, store, [], [q], slots=1, options=opts)
        alone_q.append(outs[0])
    # in the mix: everything at once, 3 slots, small batches so requests are cut into row / ray chunks
    mix = make_renders(rt)
    infos, mix_q, stats = run_server(rt, torch, store, mix, queries, slots=3, max_batch_samples=3000, options=opts)
    assert all(i["status"] == 0 for i in infos)
    assert max(i["chunks"] for i in infos) > 1
    assert stats["finished"] == stats["submitted"] == len(mix) + len(queries)
    assert stats["batches"] >= 3 and stats["rays_traced"] > 0
    for a, b in zip(alone_r, mix):
        assert torch.equal(a.linear, b.linear) and torch.equal(a.framebuffer, b.framebuffer)
    for (g, rays, any_hit), a, b in zip(queries, alone_q, mix_q):
        assert torch.equal(a["patch"], b["patch"])
        if not any_hit:
            for k in ("t", "u", "v", "object"):
                assert torch.equal(a[k], b[k]), k
    # the direct entry points give the same bits
    direct = make_renders(rt)
    rt.RayTracer(opts).render_batch(direct, store)
    torch.cuda.synchronize()
    for a, b in zip(direct, mix):
        assert torch.equal(a.linear, b.linear)
    for (g, rays, any_hit), b in zip(queries, mix_q):
        grp = torch.full((rays.shape[1],), g, dtype=torch.int32, device="cuda")
        d = store.intersect(rays, precision=rt.FP32_POLISH64, any_hit=any_hit, group=grp)
        assert torch.equal(d["patch"], b["patch"])
        if not any_hit:
            assert torch.equal(d["t"], b["t"]) and torch.equal(d["object"], b["object"])


def test_plain_schedule_is_the_plain_path(rt, store, oracle_mod, torch):
    opts = rt.Options(recursion_depth=1, schedule=rt.PLAIN)
    reqs = make_renders(rt)
    infos, _, stats = run_server(rt, torch, store, reqs, [], slots=4, options=opts)
    assert all(i["chunks"] == 1 for i in infos)
    assert stats["batches"] == len(reqs)
    direct = make_renders(rt)
    rt.RayTracer(opts).render_batch(direct, store)
    torch.cuda.synchronize()
    for a, b in zip(direct, reqs):
        assert torch.equal(a.linear, b.linear)
    wf = make_renders(rt)
    run_server(rt, torch, store, wf, [], slots=2, options=rt.Options(recursion_depth=1))
    for a, b in zip(wf, reqs):
        assert (a.linear - b.linear).abs().max().item() < 1e-5
    # plain queries through the per-thread kernel agree with the engine
    queries = query_rays(oracle_mod, torch)
    _, pq, _ = run_server(rt, torch, store, [], queries, options=opts)
    _, eq, _ = run_server(rt, torch, store, [], queries, options=rt.Options())
    for (g, rays, any_hit), a, b in zip(queries, pq, eq):
        assert torch.equal(a["patch"] >= 0, b["patch"] >= 0)


def test_admission_and_argument_errors(rt, store, torch):
    from cgspline_gb300._capi import CgsError
    # a budget too small for a single sample is refused at creation
    with pytest.raises(CgsError) as e:
        rt.Server(store, slots=2, memory_budget=1024)
    assert e.value.status == 10
    sv = rt.Server(store, slots=2, memory_budget=64 << 20, max_batch_samples=1000)
    try:
        st = sv.stats()
        assert st["max_batch_samples"] == 1000
        # one row of 1200 samples cannot fit a 1000-sample batch: admission refused, nothing queued
        wide = rt.Request.alloc(0, S.camera_c1(), 600, 4, spp=2)
        with pytest.raises(CgsError) as e:
            sv.submit_render(wide)
        assert e.value.status == 10
        assert sv.stats()["rejected"] == 1 and sv.stats()["submitted"] == 0
        with pytest.raises(CgsError) as e:
            sv.submit_render(rt.Request.alloc(9, S.camera_c1(), 8, 8))
        assert e.value.status == 1
        with pytest.raises(CgsError) as e:
            sv.wait(12345, 0.0)
        assert e.value.status == 11
        ok = rt.Request.alloc(1, S.camera_c2(), 100, 30, spp=1, linear=True)
        t = sv.submit_render(ok)
        info = sv.wait(t, 60.0)
        assert info["status"] == 0 and info["chunks"] == 3
        assert info["submit_s"] <= info["start_s"] <= info["finish_s"]
        assert sv.stats()["peak_slot_bytes"] <= 64 << 20
    finally:
        sv.close()


def test_monte_carlo_same_alone_and_in_mix(rt, store, torch):
    """Monte-Carlo renders through the server: a request's random numbers are
    keyed by its own image sample and depth, so cutting it into row chunks and
    batching it with others changes no bit."""
    opts = rt.Options(recursion_depth=2, sampling=rt.MONTE_CARLO)
    specs = [(1, 96, 54, 3, 2), (2, 80, 60, 2, 1), (0, 64, 48, 4, 2)]
    c = cams()
    alone = []
    for g, w, h, s, d in specs:
        req = rt.Request.alloc(g, c[g], w, h, spp=s, recursion_depth=d, linear=True)
        run_server(rt, torch, store, [req], [], slots=1, options=opts)
        alone.append(req)
    mix = [rt.Request.alloc(g, c[g], w, h, spp=s, recursion_depth=d, linear=True) for g, w, h, s, d in specs]
    infos, _, _ = run_server(rt, torch, store, mix, [], slots=2, max_batch_samples=2500, options=opts)
    assert all(i["status"] == 0 for i in infos) and max(i["chunks"] for i in infos) > 1
    for a, b in zip(alone, mix):
        assert torch.equal(a.linear, b.linear) and torch.equal(a.framebuffer, b.framebuffer)
