"""Size-independent properties at the full headline size: the C2 torus
(16,384 patches) and all 2,073,600 primary rays of its 1920x1080 frame, the
size the benchmark runs, where lists park, passes resume and the inline
fallback takes over.

- Every engine setting (passes, block sizes, backtrack cache) gives the same
  hits: same hit/miss and patch (or an edge tie), t within 1e-6.
- A ray has a closest hit exactly when it has any hit (unbounded rays).
- The backtrack cache changes where a backtrack finds its node, not the walk:
  node and backtrack counts are equal with it on and off.
- The polished hits stay within 1e-5 of the FP32 hits they refine (t), on the
  same patch.
- Queries issued on two streams, which share the scene's engine scratch,
  each return their own rays' hits; so do host-staged queries from two
  threads.
"""
import numpy as np
import pytest

from cgspline_gb300 import scenes as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    import torch
    from cgspline_gb300 import rt
    g = rt.GpuScene(S.scene_c2())
    rays = rt.camera_rays(S.camera_c2(), 1920, 1080)
    yield rt, torch, g, rays
    g.close()


def host(d):
    return {k: v.cpu().numpy() for k, v in d.items()}


def same_hits(a, b):
    ha, hb = a["patch"] >= 0, b["patch"] >= 0
    assert np.array_equal(ha, hb)
    diff = ha & (a["patch"] != b["patch"])
    edge = lambda d: np.minimum.reduce([d["u"], 1 - d["u"], d["v"], 1 - d["v"]]) < 1e-5
    assert (edge(a)[diff] & edge(b)[diff]).all(), int(diff.sum())
    rel = np.abs(a["t"][ha] - b["t"][ha]) / a["t"][ha]
    assert rel.max(initial=0) <= 1e-6


def test_engine_settings_agree_at_full_size(setup):
    rt, torch, g, rays = setup
    base = rt.engine_config()
    got = {}
    try:
        for cfg in ({"passes": 2, "backtrack_cache": 1, "packet_width": 1},
                    {"passes": 1, "backtrack_cache": 0},
                    {"passes": 8, "collect_threads": 128, "resolve_threads": 128, "backtrack_cache": 1},
                    {"passes": 2, "backtrack_cache": 0, "packet_width": 1},
                    {"passes": 2, "backtrack_cache": 1, "packet_width": 8},
                    {"passes": 2, "backtrack_cache": 1, "queue_chunk": 16, "packet_width": 8},
                    {"passes": 1, "backtrack_cache": 1, "queue_chunk": 40, "packet_width": 32},
                    {"passes": 8, "backtrack_cache": 1, "queue_chunk": 8, "packet_width": 8, "ray_order": 1},
                    {"passes": 4, "backtrack_cache": 0, "queue_chunk": 32, "packet_width": 16,
                     "compressed_nodes": 1}):
            rt.set_engine_config(**{**base, **cfg})
            h = host(g.intersect(rays))
            c = g.counters()
            assert c["device_errors"] == 0
            got[tuple(sorted(cfg.items()))] = (h, c)
    finally:
        rt.set_engine_config(**base)
    runs = list(got.values())
    for h, _ in runs[1:]:
        same_hits(runs[0][0], h)
    (h1, c1) = got[(("backtrack_cache", 1), ("packet_width", 1), ("passes", 2))]
    (h0, c0) = got[(("backtrack_cache", 0), ("packet_width", 1), ("passes", 2))]
    for k in h1:
        assert np.array_equal(h1[k], h0[k]), k
    # the packet refill changes when a warp takes its rays, not which rays
    # park or what a ray meets: the same hits, bit for bit, and the same nodes
    hw, cw = got[(("backtrack_cache", 1), ("packet_width", 8), ("passes", 2))]
    for k in h1:
        assert np.array_equal(hw[k], h1[k]), k
    assert cw["nodes"] == c1["nodes"] and cw["hash_lookups"] == c1["hash_lookups"]
    assert c1["nodes"] == c0["nodes"] and c1["hash_lookups"] == c0["hash_lookups"]
    assert c0["hash_table_reads"] == c0["hash_lookups"] and c1["hash_table_reads"] < c1["hash_lookups"] // 100
    assert (runs[0][0]["patch"] >= 0).mean() > 0.2


def test_compressed_nodes_give_identical_hits(setup):
    """The traversal on the 32-byte compressed node mirror against the exact
    64-byte records: the same hits, bit for bit, on the full frame, closest
    and any hit, at FP32 and with the FP64 polish; the conservative boxes add
    a few node visits."""
    rt, torch, g, rays = setup
    base = rt.engine_config()
    out = {}
    try:
        for cq in (1, 0):
            rt.set_engine_config(compressed_nodes=cq)
            out[cq] = (host(g.intersect(rays)), g.counters(), host(g.intersect(rays, any_hit=True)),
                       host(g.intersect(rays, precision=rt.FP32_POLISH64)))
    finally:
        rt.set_engine_config(**base)
    (h1, c1, a1, p1), (h0, c0, a0, p0) = out[1], out[0]
    for k in h1:
        assert np.array_equal(h1[k], h0[k]), k
        assert np.array_equal(p1[k], p0[k]), k
    assert np.array_equal(a1["patch"] >= 0, a0["patch"] >= 0)
    assert c1["device_errors"] == 0 and c0["nodes"] <= c1["nodes"] <= 1.25 * c0["nodes"]


def test_closest_and_any_hit_agree_at_full_size(setup):
    rt, torch, g, rays = setup
    c = host(g.intersect(rays))
    a = host(g.intersect(rays, any_hit=True))
    assert np.array_equal(c["patch"] >= 0, a["patch"] >= 0)


def test_polish_refines_in_place_at_full_size(setup):
    rt, torch, g, rays = setup
    f = host(g.intersect(rays, precision=rt.FP32))
    p = host(g.intersect(rays, precision=rt.FP32_POLISH64))
    assert np.array_equal(f["patch"], p["patch"]) and np.array_equal(f["object"], p["object"])
    hit = f["patch"] >= 0
    rel = np.abs(f["t"][hit] - p["t"][hit]) / p["t"][hit]
    assert np.quantile(rel, 0.999) < 1e-5 and rel.max() < 1e-3


def test_queries_on_two_streams_keep_their_own_hits(setup):
    """A scene's queries share its engine scratch and counters: issued back to
    back on two streams, the second waits for the first, and each returns the
    hits of its own rays."""
    rt, torch, g, rays = setup
    a, b = rays[:, 0::2].contiguous(), rays[:, 1::2].contiguous()
    ref_a, ref_b = host(g.intersect(a)), host(g.intersect(b))
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    torch.cuda.synchronize()
    for _ in range(3):
        ha = g.intersect(a, stream=s1)
        hb = g.intersect(b, stream=s2)
        torch.cuda.synchronize()
        for ref, got in ((ref_a, host(ha)), (ref_b, host(hb))):
            for k in ref:
                assert np.array_equal(ref[k], got[k]), k
    assert g.counters()["device_errors"] == 0


def test_host_queries_from_two_threads_keep_their_own_hits(setup):
    """cgs_intersect_host stages rays and hits in buffers of the scene: two
    host threads querying one scene at once each get their own rays' hits."""
    import threading
    rt, torch, g, rays = setup
    hr = rays.cpu().numpy()
    parts = [np.ascontiguousarray(hr[:, 0::2]), np.ascontiguousarray(hr[:, 1::2][:, :500000])]
    refs = [g.intersect(p) for p in parts]
    got = [[], []]

    def work(i):
        for _ in range(3):
            got[i].append(g.intersect(parts[i]))

    threads = [threading.Thread(target=work, args=(i,)) for i in range(2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=120)
    for i in range(2):
        assert len(got[i]) == 3
        for h in got[i]:
            for k in refs[i]:
                assert np.array_equal(refs[i][k], h[k]), k


def test_render_host_into_caller_buffers(setup):
    """cgs_render_host into caller-owned (pinned) host arrays gives the same
    image as into fresh ones."""
    rt, torch, g, rays = setup
    tr = rt.RayTracer(rt.Options(recursion_depth=1))
    fb0, lin0 = tr.render_host(S.camera_c2(), g, 640, 360)
    fb = torch.empty((360, 640), dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
    lin = torch.empty((360, 640, 3), dtype=torch.float32, pin_memory=True).numpy()
    fb1, lin1 = tr.render_host(S.camera_c2(), g, 640, 360, out=(fb, lin))
    assert fb1 is fb and lin1 is lin
    assert np.array_equal(fb0, fb) and np.array_equal(lin0, lin)


def test_origin_last_keeps_any_hit_answers(setup):
    """Shadow rays from every primary hit of the frame toward the first light
    (origin offset 1e-4 along the light direction, bounded by the light's
    distance): searching the candidates whose leaf box holds the origin last
    gives the same any-hit answer for every ray, with no more clip
    iterations."""
    rt, torch, g, rays = setup
    h = g.intersect(rays)
    hit = h["patch"] >= 0
    P = rays[:3, hit] + rays[3:6, hit] * h["t"][hit]
    light = torch.tensor(S.scene_c2().lights[0].position, dtype=torch.float32, device=P.device)[:, None]
    L = light - P
    dist = L.norm(dim=0)
    L = L / dist
    shadow = torch.cat([P + 1e-4 * L, L, dist[None]], 0).contiguous()
    base = rt.engine_config()
    out = {}
    try:
        for ol in (0, 1):
            rt.set_engine_config(origin_last=ol)
            a = host(g.intersect(shadow, any_hit=True))
            out[ol] = (a["patch"] >= 0, g.counters())
    finally:
        rt.set_engine_config(**base)
    assert np.array_equal(out[0][0], out[1][0])
    assert 0.01 < out[0][0].mean() < 0.99
    assert out[1][1]["iterations"] <= out[0][1]["iterations"]
    assert out[0][1]["device_errors"] == 0 and out[1][1]["device_errors"] == 0
