"""GPU tests of scene groups (many resident scenes in one store) and batched
rendering through cgs_render_batch.

Bars: a group's BVHs and hash tables equal those of the same scene stored
alone (bit-exact); per-ray group queries agree with the oracle of each scene
as the single-scene queries do; a request rendered inside a batch of other
requests, groups and sizes is bit-identical to the same request rendered
alone; spp > 1 matches the oracle's jittered average within the single-sample
render tolerance.
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
def pair():
    return [S.scene_c1(), S.scene_c2(nu=32, nv=32)]


@pytest.fixture(scope="module")
def store(rt, pair):
    return rt.GpuScene(pair)


@pytest.fixture(scope="module")
def alone(rt, pair):
    return [rt.GpuScene(s) for s in pair]


@pytest.fixture(scope="module")
def oracles(oracle_mod, pair):
    return [oracle_mod.OracleScene(s) for s in pair]


CAMS = [S.camera_c1, S.camera_c2]


def test_group_bvhs_equal_single_scene_bvhs(store, alone, pair):
    for g in range(2):
        a = store.bvh(-1 - g)
        b = alone[g].bvh(-1)
        for k in ("nodes", "keys", "table", "disp"):
            assert np.array_equal(a[k], b[k]), (g, k)
        assert (a["A"], a["B"], a["N"], a["mask"]) == (b["A"], b["B"], b["N"], b["mask"])
        # object ids of group g are global: offset by the objects of earlier groups
        off = sum(len(p.objects) for p in pair[:g])
        ia, ib = a["indices"].astype(np.int64), b["indices"].astype(np.int64)
        leaf = ib != 0xFFFFFFFF
        assert np.array_equal(ia[leaf], ib[leaf] + off) and np.array_equal(ia[~leaf], ib[~leaf])
        base = store.surface_base[g]
        for s in range(len(pair[g].surfaces)):
            sa, sb = store.bvh(base + s), alone[g].bvh(s)
            for k in ("nodes", "keys", "indices", "table", "disp"):
                assert np.array_equal(sa[k], sb[k]), (g, s, k)


def test_grouped_queries_match_each_scene(store, alone, oracles, oracle_mod, pair, torch):
    rays = [oracle_mod.camera_rays(CAMS[g](), 96, 64) for g in range(2)]
    allr = np.concatenate(rays, axis=1)
    grp = np.concatenate([np.full(r.shape[1], g, np.uint32) for g, r in enumerate(rays)])
    # interleave the groups so that warps mix scenes
    perm = np.random.default_rng(5).permutation(allr.shape[1])
    res = store.intersect(torch.from_numpy(allr[:, perm]).cuda(), group=torch.from_numpy(grp[perm].view(np.int32)))
    res = {k: v.cpu().numpy() for k, v in res.items()}
    inv = np.argsort(perm)
    res = {k: v[inv] for k, v in res.items()}
    start = 0
    for g in range(2):
        n = rays[g].shape[1]
        one = {k: v.cpu().numpy() for k, v in alone[g].intersect(torch.from_numpy(rays[g]).cuda()).items()}
        part = {k: v[start:start + n] for k, v in res.items()}
        off = sum(len(p.objects) for p in pair[:g])
        for k in ("t", "u", "v", "patch"):
            assert np.array_equal(part[k], one[k]), (g, k)
        hit = one["object"] >= 0
        assert np.array_equal(part["object"][hit], one["object"][hit] + off)
        o = oracles[g].intersect(rays[g])
        assert np.array_equal(part["patch"] >= 0, o["patch"] >= 0)
        start += n
    # host entry point with per-ray groups gives the same
    h = store.intersect(allr[:, perm], group=grp[perm])
    h = {k: v[inv] for k, v in h.items()}
    for k in res:
        assert np.array_equal(h[k], res[k]), k


@pytest.mark.parametrize("schedule", [0, 1])
def test_request_same_alone_and_in_mix(rt, store, torch, schedule):
    specs = [(1, S.camera_c2(), 96, 54, 1, 1), (0, S.camera_c1(), 64, 64, 1, 0), (1, S.camera_c2(), 40, 30, 2, 2),
             (0, S.camera_c1(), 33, 17, 3, 1), (1, S.camera_c2(), 128, 72, 1, 0)]
    mix = [rt.Request.alloc(g, c, w, h, spp=s, recursion_depth=d, linear=True) for g, c, w, h, s, d in specs]
    tracer = rt.RayTracer(rt.Options(schedule=schedule))
    tracer.render_batch(mix, store)
    torch.cuda.synchronize()
    assert store.counters()["device_errors"] == 0
    for (g, c, w, h, s, d), q in zip(specs, mix):
        one = rt.Request.alloc(g, c, w, h, spp=s, recursion_depth=d, linear=True)
        tracer.render_batch([one], store)
        torch.cuda.synchronize()
        assert torch.equal(one.linear, q.linear), (g, w, h, s, d)
        assert torch.equal(one.framebuffer, q.framebuffer)


def test_batch_groups_match_single_scene_renders(rt, store, alone, torch):
    for g, cam in enumerate(CAMS):
        q = rt.Request.alloc(g, cam(), 80, 48, recursion_depth=1, linear=True)
        rt.RayTracer(rt.Options()).render_batch([q], store)
        torch.cuda.synchronize()
        fb, lin = rt.RayTracer(rt.Options(recursion_depth=1)).render_host(cam(), alone[g], 80, 48)
        assert np.array_equal(q.linear.cpu().numpy(), lin)


def test_schedules_agree_on_batches(rt, store, torch):
    specs = [(1, S.camera_c2(), 64, 36, 2, 1), (0, S.camera_c1(), 48, 48, 1, 1)]
    out = []
    for schedule in (0, 1):
        reqs = [rt.Request.alloc(g, c, w, h, spp=s, recursion_depth=d, linear=True) for g, c, w, h, s, d in specs]
        rt.RayTracer(rt.Options(schedule=schedule)).render_batch(reqs, store)
        torch.cuda.synchronize()
        out.append([r.linear.cpu().numpy() for r in reqs])
    for a, b in zip(*out):
        assert np.abs(a - b).max() < 1e-5


def test_spp_matches_oracle(rt, store, oracles, torch):
    q = rt.Request.alloc(1, S.camera_c2(), 96, 54, spp=4, recursion_depth=1, linear=True)
    rt.RayTracer(rt.Options()).render_batch([q], store)
    torch.cuda.synchronize()
    ro = oracles[1].render_spp(S.camera_c2(), 96, 54, 4, depth=1)
    err = np.abs(q.linear.cpu().numpy() - ro["rgb"])
    assert float(np.sqrt((err ** 2).mean())) < 5e-3
    assert (err.max(axis=-1) > 0.05).mean() < 2e-3


def test_invalid_batches_raise(rt, store, torch):
    from cgspline_gb300._capi import CgsError
    tracer = rt.RayTracer(rt.Options())
    bad_group = rt.Request.alloc(7, S.camera_c1(), 8, 8)
    with pytest.raises(CgsError) as e:
        tracer.render_batch([bad_group], store)
    assert e.value.status == 1
    zero_spp = rt.Request.alloc(0, S.camera_c1(), 8, 8)
    zero_spp.spp = 0
    with pytest.raises(CgsError):
        tracer.render_batch([zero_spp], store)
    with pytest.raises(CgsError):
        tracer.render_batch([], store)
    # per-ray groups live on the device: a ray of an unknown group is a miss and sets error bit 8
    rays = torch.zeros((7, 4), device="cuda")
    rays[3] = 1.0
    rays[6] = float("inf")
    res = store.intersect(rays, group=torch.tensor([0, 9, 1, 2], dtype=torch.int32))
    assert res["patch"].cpu().tolist()[1] == -1 and res["patch"].cpu().tolist()[3] == -1
    assert store.counters()["device_errors"] == 8


def test_union_scenes_batch_matches_oracle(rt, oracle_mod, torch):
    """Four seeded unions of cube-spheres and tori (the batching workload's
    generator, capped at 2,048 patches) in one store, rendered as one batch
    with one bounce, each against the oracle of its own scene."""
    scs = [S.scene_c4(i, max_patches=2048) for i in range(4)]
    store = rt.GpuScene(scs)
    cams = [S.camera_c4(i)[0] for i in range(4)]
    reqs = [rt.Request.alloc(i, cams[i], 72, 56, recursion_depth=1, linear=True) for i in range(4)]
    rt.RayTracer(rt.Options(precision=rt.FP32_POLISH64)).render_batch(reqs, store)
    torch.cuda.synchronize()
    assert store.counters()["device_errors"] == 0
    for i in range(4):
        ro = oracle_mod.OracleScene(scs[i]).render(cams[i], 72, 56, depth=1)
        err = np.abs(reqs[i].linear.cpu().numpy() - ro["rgb"])
        assert float(np.sqrt((err ** 2).mean())) < 5e-3, i
        assert (err.max(axis=-1) > 0.05).mean() < 5e-3, i


def test_camera_rays_match_oracle(rt, oracle_mod, torch):
    for cam, w, h in ((S.camera_c1(), 37, 23), (S.camera_c2(), 64, 36), (S.camera_c4(5)[0], 16, 16)):
        g = rt.camera_rays(cam, w, h).cpu().numpy()
        o = oracle_mod.camera_rays(cam, w, h)
        assert np.array_equal(g[:3], o[:3]) and np.isinf(g[6]).all()
        assert np.abs(g[3:6] - o[3:6]).max() < 1e-6  # a few ulps: FMA contraction differs


def test_engine_settings_and_autotune(rt, store, torch):
    """Every engine setting gives the same hits (the pass count only moves rays
    between the engine and its inline fallback); the autotuner picks one of
    the candidates and leaves it in force."""
    base = rt.engine_config()
    rays = rt.camera_rays(S.camera_c2(), 96, 64)
    grp = torch.ones(rays.shape[1], dtype=torch.int32, device="cuda")
    ref = {k: v.cpu().numpy() for k, v in store.intersect(rays, group=grp).items()}
    try:
        for passes, ct, rtn in ((1, 128, 64), (4, 256, 128), (8, 128, 128)):
            rt.set_engine_config(passes=passes, collect_threads=ct, resolve_threads=rtn)
            got = {k: v.cpu().numpy() for k, v in store.intersect(rays, group=grp).items()}
            assert np.array_equal(got["patch"] >= 0, ref["patch"] >= 0)
            hit = ref["patch"] >= 0
            assert np.abs(got["t"][hit] - ref["t"][hit]).max(initial=0) <= 1e-6 * ref["t"][hit].max(initial=1)
        from cgspline_gb300._capi import CgsError
        for bad in ({"passes": 9}, {"queue_chunk": 10}, {"queue_chunk": 72}, {"queue_chunk": 2}, {"queue_chunk": 0},
                    {"origin_last": 2},
                    {"packet_width": 0}, {"packet_width": 33}, {"ray_order": 2}):
            with pytest.raises(CgsError):
                rt.set_engine_config(**bad)
        reqs = [rt.Request.alloc(1, S.camera_c2(), 64, 36), rt.Request.alloc(0, S.camera_c1(), 32, 32)]
        cfg, ms = rt.autotune(store, reqs, rt.Options(recursion_depth=1), repeats=1)
        assert cfg == rt.engine_config() and ms > 0
        assert cfg["passes"] in (1, 2, 4, 8) and cfg["collect_threads"] in (128, 256)
        assert cfg["queue_chunk"] in (8, 16, 32, 64) and cfg["packet_width"] in (1, 8, 16)
        # a subdivision batch also tunes the subdivision levels per round
        cfg, ms = rt.autotune(store, reqs, rt.Options(recursion_depth=1, method=rt.SUBDIV), repeats=1)
        assert cfg == rt.engine_config() and ms > 0 and cfg["subdiv_levels"] in (1, 4, 16, 64)
    finally:
        rt.set_engine_config(**base)


@pytest.mark.parametrize("schedule", [0, 1])
def test_monte_carlo_matches_oracle(rt, store, oracles, torch, schedule):
    """The sampled path (GGX microfacet bounces, Philox keyed by image sample
    and depth) against the oracle's restatement with the same random numbers:
    paths only part where FP32 sin/cos or a clip result round differently."""
    q = rt.Request.alloc(1, S.camera_c2(), 96, 54, spp=2, recursion_depth=2, linear=True)
    rt.RayTracer(rt.Options(schedule=schedule, sampling=rt.MONTE_CARLO)).render_batch([q], store)
    torch.cuda.synchronize()
    ro = oracles[1].render_spp(S.camera_c2(), 96, 54, 2, depth=2, mc=True)
    err = np.abs(q.linear.cpu().numpy() - ro["rgb"])
    assert float(np.sqrt((err ** 2).mean())) < 1e-2
    assert (err.max(axis=-1) > 0.05).mean() < 2e-2


def test_monte_carlo_same_alone_and_in_mix(rt, store, torch):
    specs = [(1, S.camera_c2(), 64, 36, 3, 2), (0, S.camera_c1(), 40, 40, 2, 1), (1, S.camera_c2(), 33, 20, 1, 3)]
    tracer = rt.RayTracer(rt.Options(sampling=rt.MONTE_CARLO))
    mix = [rt.Request.alloc(g, c, w, h, spp=s, recursion_depth=d, linear=True) for g, c, w, h, s, d in specs]
    tracer.render_batch(mix, store)
    torch.cuda.synchronize()
    for (g, c, w, h, s, d), q in zip(specs, mix):
        one = rt.Request.alloc(g, c, w, h, spp=s, recursion_depth=d, linear=True)
        tracer.render_batch([one], store)
        torch.cuda.synchronize()
        assert torch.equal(one.linear, q.linear)
    plain = [rt.Request.alloc(g, c, w, h, spp=s, recursion_depth=d, linear=True) for g, c, w, h, s, d in specs]
    rt.RayTracer(rt.Options(sampling=rt.MONTE_CARLO, schedule=rt.PLAIN)).render_batch(plain, store)
    torch.cuda.synchronize()
    for a, b in zip(plain, mix):
        assert (a.linear - b.linear).abs().max().item() < 1e-5


@pytest.mark.parametrize("sampling", [0, 1])
def test_tiled_ray_order_gives_same_frames(rt, store, torch, sampling):
    """Primary rays queued in 8 x 4 pixel tiles instead of scanline order:
    the same frames, bit for bit (sizes that leave partial tiles, spp > 1,
    bounces, both bounce models)."""
    specs = [(1, S.camera_c2(), 93, 53, 1, 2), (0, S.camera_c1(), 37, 22, 3, 1), (1, S.camera_c2(), 8, 4, 2, 1),
             (1, S.camera_c2(), 5, 3, 1, 0), (0, S.camera_c1(), 64, 33, 1, 3)]
    base = rt.engine_config()
    out = {}
    try:
        for order in (0, 1):
            rt.set_engine_config(ray_order=order)
            reqs = [rt.Request.alloc(g, c, w, h, spp=s, recursion_depth=d, linear=True) for g, c, w, h, s, d in specs]
            rt.RayTracer(rt.Options(schedule=rt.WAVEFRONT, sampling=sampling)).render_batch(reqs, store)
            torch.cuda.synchronize()
            assert store.counters()["device_errors"] == 0
            out[order] = [(r.linear.clone(), r.framebuffer.clone()) for r in reqs]
    finally:
        rt.set_engine_config(**base)
    for spec, (la, fa), (lb, fb) in zip(specs, out[0], out[1]):
        assert torch.equal(la, lb) and torch.equal(fa, fb), spec[2:]


def test_scene_blob_round_trip(rt, pair, torch, tmp_path):
    """A saved and reloaded store has the same BVHs and hash tables bit for bit
    and gives the same hits and images; damaged or missing files are refused."""
    from cgspline_gb300._capi import CgsError
    scs = pair + [S.scene_c4(7, max_patches=2048)]
    a = rt.GpuScene(scs, split=rt.SPLIT_LONGEST)
    path = tmp_path / "store.cgsb"
    a.save(path)
    b = rt.GpuScene.load(path)
    nsurf = sum(len(s.surfaces) for s in scs)
    for which in list(range(nsurf)) + [-1, -2, -3]:
        x, y = a.bvh(which), b.bvh(which)
        for k in ("nodes", "keys", "indices", "table", "disp"):
            assert np.array_equal(x[k], y[k]), (which, k)
        assert (x["A"], x["B"], x["N"], x["mask"]) == (y["A"], y["B"], y["N"], y["mask"])
    rays = rt.camera_rays(S.camera_c4(7)[0], 64, 64)
    grp = torch.full((rays.shape[1],), 2, dtype=torch.int32, device="cuda")
    ra, rb = a.intersect(rays, group=grp), b.intersect(rays, group=grp)
    for k in ra:
        assert torch.equal(ra[k], rb[k]), k
    qa = rt.Request.alloc(1, S.camera_c2(), 48, 32, recursion_depth=1, linear=True)
    qb = rt.Request.alloc(1, S.camera_c2(), 48, 32, recursion_depth=1, linear=True)
    rt.RayTracer(rt.Options()).render_batch([qa], a)
    rt.RayTracer(rt.Options()).render_batch([qb], b)
    torch.cuda.synchronize()
    assert torch.equal(qa.linear, qb.linear)
    data = path.read_bytes()
    bad = tmp_path / "bad.cgsb"
    bad.write_bytes(data[: len(data) // 2])
    with pytest.raises(CgsError) as e:
        rt.GpuScene.load(bad)
    assert e.value.status == 1
    flipped = bytearray(data)
    flipped[4] ^= 0x5A  # the format version
    bad.write_bytes(bytes(flipped))
    with pytest.raises(CgsError) as e:
        rt.GpuScene.load(bad)
    assert e.value.status == 1
    with pytest.raises(CgsError) as e:
        rt.GpuScene.load(tmp_path / "missing.cgsb")
    assert e.value.status == 11
    # a BVH whose root's children point back up (a cycle the traversal would
    # walk for ever) or carry the wrong heap keys is refused before upload
    import struct
    s0 = scs[0].surfaces[0]
    nodes_at = 24 + 4 + s0.points.size * 4 + 4 + s0.indices.size * 4  # header, points, indices
    nnodes = struct.unpack_from("<I", data, nodes_at)[0]
    assert nnodes > 1
    root = nodes_at + 4  # 56-byte nodes: two boxes of 6 floats, then left, right
    left, right = struct.unpack_from("<II", data, root + 48)
    assert left == 1 and right > 1
    keys_at = nodes_at + 4 + 56 * nnodes + 4
    for at, value in ((root + 48, 0), (root + 52, 0), (keys_at + 4 * left, 5)):
        broken = bytearray(data)
        struct.pack_into("<I", broken, at, value)
        bad.write_bytes(bytes(broken))
        with pytest.raises(CgsError) as e:
            rt.GpuScene.load(bad)
        assert e.value.status == 1
    a.close()
    b.close()
