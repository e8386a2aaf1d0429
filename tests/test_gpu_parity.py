"""GPU parity: the CUDA path through the C ABI against the oracle on the same seeded inputs.

Bars: BVH topology and perfect-hash tables bit-exact; hit/miss and patch id
identical (a different patch id is allowed only when both hits lie within
1e-5 of a shared patch edge and their t agree to 1e-6 relative -- a tie);
t within 1e-5 relative, (u,v) within 1e-3 of the oracle's FP32 reference
semantics; after the FP64 polish t within 1e-5 relative of the FP64 oracle.
"""
import math

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
def c1_gpu(rt, c1_scene):
    return rt.GpuScene(c1_scene)


@pytest.fixture(scope="module")
def c2_small():
    return S.scene_c2(nu=32, nv=32)


@pytest.fixture(scope="module")
def c2_small_gpu(rt, c2_small):
    return rt.GpuScene(c2_small)


@pytest.fixture(scope="module")
def c2_small_oracle(oracle_mod, c2_small):
    return oracle_mod.OracleScene(c2_small)


def edge_tie(u, v, tol=1e-5):
    return (np.minimum.reduce([u, 1 - u, v, 1 - v]) < tol)


def compare_hits(g, o, t_rtol=1e-5, uv_atol=1e-3):
    gp, op = np.asarray(g["patch"]), np.asarray(o["patch"])
    assert np.array_equal(gp >= 0, op >= 0), f"hit/miss disagreements: {int(((gp >= 0) != (op >= 0)).sum())}"
    hit = op >= 0
    diff = hit & (gp != op)
    if diff.any():
        ties = edge_tie(np.asarray(g["u"])[diff], np.asarray(g["v"])[diff]) & \
            edge_tie(np.asarray(o["u"])[diff], np.asarray(o["v"])[diff])
        rel = np.abs(np.asarray(g["t"])[diff] - np.asarray(o["t"])[diff]) / np.asarray(o["t"])[diff]
        assert ties.all() and (rel < 1e-6).all(), f"{int(diff.sum())} patch-id disagreements"
    same = hit & (gp == op)
    rel = np.abs(np.asarray(g["t"])[same] - np.asarray(o["t"])[same]) / np.asarray(o["t"])[same]
    assert rel.max(initial=0) < t_rtol, rel.max()
    du = np.abs(np.asarray(g["u"])[same] - np.asarray(o["u"])[same])
    dv = np.abs(np.asarray(g["v"])[same] - np.asarray(o["v"])[same])
    assert max(du.max(initial=0), dv.max(initial=0)) < uv_atol
    return int(hit.sum()), int(diff.sum())


def to_host(d):
    return {k: v.cpu().numpy() for k, v in d.items()}


def test_bvh_and_hash_bit_exact(c1_gpu, c1_oracle):
    for which in (0, -1):
        g, o = c1_gpu.bvh(which), c1_oracle.bvh(which)
        for k in ("nodes", "keys", "indices", "table", "disp"):
            assert np.array_equal(g[k], o[k]), (which, k)
        assert (g["A"], g["B"], g["N"], g["mask"]) == (o["A"], o["B"], o["N"], o["mask"])


def test_bvh_and_hash_bit_exact_torus(c2_small_gpu, c2_small_oracle):
    g, o = c2_small_gpu.bvh(0), c2_small_oracle.bvh(0)
    for k in ("nodes", "keys", "indices", "table", "disp"):
        assert np.array_equal(g[k], o[k]), k
    assert (g["A"], g["B"], g["N"]) == (o["A"], o["B"], o["N"])


def test_store_hash_tables_bit_exact(rt, oracle_mod):
    """The batched store build (every BVH of up to 8,192 keys by one thread
    block, in one launch; larger ones by the multi-launch build) against the
    oracle, BVH by BVH: two union scenes (57 and 51 object surfaces, 13,144
    and 61,974 patches) and the full torus (one BVH of 32,767 keys)."""
    scenes = [S.scene_c4(17), S.scene_c4(5), S.scene_c2()]
    store = rt.GpuScene(scenes)
    base = obase = 0
    nbig = 0
    for g, sc in enumerate(scenes):
        o = oracle_mod.OracleScene(sc)
        for k in list(range(len(sc.surfaces))) + [-1]:
            gb = store.bvh(base + k if k >= 0 else -1 - g)
            ob = o.bvh(k)
            if k < 0:
                # an object-level BVH lists the store's object ids; the
                # oracle's scene numbers its objects from 0
                ind = gb["indices"].copy()
                ind[ind != 0xFFFFFFFF] -= obase
                gb["indices"] = ind
            for f in ("nodes", "keys", "indices", "table", "disp"):
                assert np.array_equal(gb[f], ob[f]), (g, k, f)
            assert (gb["A"], gb["B"], gb["N"], gb["mask"]) == (ob["A"], ob["B"], ob["N"], ob["mask"])
            nbig += gb["keys"].size > 8192
        base += len(sc.surfaces)
        obase += len(sc.objects)
    assert nbig >= 1
    store.close()


@pytest.mark.parametrize("n", [1, 2, 31, 1000, 8191, 8192, 8193, 32767, 65537, 1 << 20])
def test_perfect_hash_matches_oracle(rt, oracle_mod, n):
    keys = np.arange(1, n + 1, dtype=np.uint32)
    o = oracle_mod.hash_build(keys)
    h = rt.PerfectHashFunction()
    assert h.build(keys) == 0
    assert (h.A, h.B, h.N, h.mask) == (o["A"], o["B"], o["N"], o["mask"])
    assert np.array_equal(h.disp, o["disp"]) and np.array_equal(h.table, o["table"])


def test_c1_closest_hits(c1_gpu, c1_oracle, oracle_mod, torch):
    rays = oracle_mod.camera_rays(S.camera_c1(), 256, 256)
    o = c1_oracle.intersect(rays)
    g = to_host(c1_gpu.intersect(torch.from_numpy(rays).cuda()))
    nhit, nties = compare_hits(g, o)
    assert nhit > 40000
    assert c1_gpu.counters()["device_errors"] == 0


def test_c1_golden_on_gpu(c1_gpu, torch):
    import os
    gdn = np.load(os.path.join(os.path.dirname(__file__), "golden", "c1_golden.npz"))
    g = to_host(c1_gpu.intersect(torch.from_numpy(gdn["rays"]).cuda()))
    compare_hits(g, dict(t=gdn["t"], u=gdn["u"], v=gdn["v"], patch=gdn["patch"]))


def test_c1_host_entry_point_matches_device(c1_gpu, oracle_mod, torch):
    rays = oracle_mod.camera_rays(S.camera_c1(), 64, 64)
    a = c1_gpu.intersect(rays)  # numpy -> cgs_intersect_host (copies inside)
    b = to_host(c1_gpu.intersect(torch.from_numpy(rays).cuda()))
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def test_torus_closest_and_any(c2_small_gpu, c2_small_oracle, oracle_mod, torch):
    rays = oracle_mod.camera_rays(S.camera_c2(), 240, 135)
    o = c2_small_oracle.intersect(rays)
    g = to_host(c2_small_gpu.intersect(torch.from_numpy(rays).cuda()))
    compare_hits(g, o, t_rtol=1e-5, uv_atol=1e-3)
    oa = c2_small_oracle.intersect(rays, any_hit=True)
    ga = to_host(c2_small_gpu.intersect(torch.from_numpy(rays).cuda(), any_hit=True))
    assert np.array_equal(ga["patch"] >= 0, oa["patch"] >= 0)


def test_torus_polish_vs_fp64(rt, c2_small_gpu, c2_small_oracle, oracle_mod, torch):
    rays = oracle_mod.camera_rays(S.camera_c2(), 240, 135)
    o64 = c2_small_oracle.intersect(rays, precision=oracle_mod.FP64)
    g = to_host(c2_small_gpu.intersect(torch.from_numpy(rays).cuda(), precision=rt.FP32_POLISH64))
    gp, op = g["patch"], o64["patch"]
    assert np.array_equal(gp >= 0, op >= 0)
    both = (gp >= 0) & (gp == op)
    rel = np.abs(g["t"][both] - o64["t"][both]) / o64["t"][both]
    assert rel.max() <= 1e-5, rel.max()


def test_subdivision_agrees_with_clipping(rt, c1_gpu, c1_oracle, oracle_mod, torch):
    rays = oracle_mod.camera_rays(S.camera_c1(), 128, 128)
    o = c1_oracle.intersect(rays, method=oracle_mod.SUBDIV)
    g = to_host(c1_gpu.intersect(torch.from_numpy(rays).cuda(), method=rt.SUBDIV))
    compare_hits(g, o, t_rtol=1e-5, uv_atol=2e-3)


def test_subdivision_levels_per_round_give_identical_hits(rt, oracle_mod, torch):
    """The query engine runs subdivision searches resumably, subdiv_levels
    bisection levels per round of its clip kernel: every setting gives the
    same hits, bit for bit, as the one-search-per-call inline path (one pass
    of a one-entry list sends every ray to it)."""
    g = rt.GpuScene(S.scene_c2(nu=32, nv=32))
    rays = torch.from_numpy(oracle_mod.camera_rays(S.camera_c2(), 240, 135)).cuda()
    base = rt.engine_config()
    out = []
    try:
        for cfg in ({"subdiv_levels": 1}, {"subdiv_levels": 8}, {"subdiv_levels": 64},
                    {"passes": 1, "queue_chunk": 4, "subdiv_levels": 3}):
            rt.set_engine_config(**{**base, **cfg})
            out.append(to_host(g.intersect(rays, method=rt.SUBDIV)))
            assert g.counters()["device_errors"] == 0
        from cgspline_gb300._capi import CgsError
        for bad in (0, 65):
            with pytest.raises(CgsError):
                rt.set_engine_config(subdiv_levels=bad)
    finally:
        rt.set_engine_config(**base)
    assert (out[0]["patch"] >= 0).sum() > 1000
    for h in out[1:]:
        for k in ("t", "u", "v", "patch", "object"):
            assert np.array_equal(h[k], out[0][k]), k
    # at the precision form's level the FP64 grazing instance runs the
    # subdivision searches whole; the grazing test concerns clipping only, so
    # the polished hits equal those of FP32 + FP64 polish
    a = to_host(g.intersect(rays, method=rt.SUBDIV, precision=rt.FP32_GRAZE64))
    b = to_host(g.intersect(rays, method=rt.SUBDIV, precision=rt.FP32_POLISH64))
    for k in ("t", "u", "v", "patch", "object"):
        assert np.array_equal(a[k], b[k]), k
    g.close()


def test_patch_pairs_entry_point(rt, c1_gpu, c1_scene, oracle_mod, torch):
    rays = oracle_mod.camera_rays(S.camera_c1(), 32, 32)
    n = rays.shape[1]
    pids = np.arange(n, dtype=np.int32) % 16
    found, t, u, v = rt.do_bezier_clipping(c1_gpu, 0, torch.from_numpy(rays).cuda(), torch.from_numpy(pids).cuda())
    found, t = found.cpu().numpy(), t.cpu().numpy()
    s = c1_scene.surfaces[0]
    for k in range(0, n, 7):
        hit, to, uv, _ = oracle_mod.patch_intersect(s.points, s.indices[16 * pids[k]:16 * pids[k] + 16], rays[:, k],
                                                    method=oracle_mod.CLIP_DEVICE)
        assert bool(found[k]) == hit
        if hit:
            assert abs(t[k] - to) / to < 1e-5


@pytest.mark.parametrize("schedule", [0, 1])
def test_render_c1_matches_oracle(rt, c1_gpu, c1_oracle, schedule):
    cam = S.camera_c1()
    w = h = 128
    ro = c1_oracle.render(cam, w, h, depth=0)
    tracer = rt.RayTracer(rt.Options(recursion_depth=0, schedule=schedule))
    fb, lin = tracer.render_host(cam, c1_gpu, w, h)
    err = np.abs(lin - ro["rgb"])
    assert np.sqrt((err ** 2).mean()) < 1e-4
    assert err.max() < 1e-2


@pytest.mark.parametrize("schedule", [0, 1])
def test_render_torus_pbr_matches_oracle(rt, c2_small_gpu, c2_small_oracle, schedule):
    cam = S.camera_c2()
    w, h = 192, 108
    ro = c2_small_oracle.render(cam, w, h, depth=1)
    tracer = rt.RayTracer(rt.Options(recursion_depth=1, schedule=schedule))
    fb, lin = tracer.render_host(cam, c2_small_gpu, w, h)
    err = np.abs(lin - ro["rgb"])
    rmse = float(np.sqrt((err ** 2).mean()))
    # bounce rays start from FP32 hit points: a few silhouette pixels may differ
    assert rmse < 5e-3, rmse
    assert (err.max(axis=-1) > 0.05).mean() < 2e-3
    c = c2_small_gpu.counters()
    assert c["device_errors"] == 0 and c["rays"] >= w * h


def test_schedules_agree(rt, c2_small_gpu):
    cam = S.camera_c2()
    a = rt.RayTracer(rt.Options(recursion_depth=1, schedule=rt.PLAIN)).render_host(cam, c2_small_gpu, 160, 90)[1]
    b = rt.RayTracer(rt.Options(recursion_depth=1, schedule=rt.WAVEFRONT)).render_host(cam, c2_small_gpu, 160, 90)[1]
    assert np.abs(a - b).max() < 1e-5


def test_device_frame_and_busy_flag(rt, c1_gpu, torch):
    frame = rt.Frame(100, 60, alignment=32)
    assert frame.stride == 128
    tracer = rt.RayTracer(rt.Options(recursion_depth=0))
    tracer.render(frame, S.camera_c1(), c1_gpu)
    torch.cuda.synchronize()
    assert not tracer.running()
    img = frame.rgba()
    assert img.shape == (60, 100, 4) and (img[..., 3] == 255).all()


def test_long_runs_of_misses_do_not_end_the_query(c1_gpu, c1_oracle, oracle_mod, torch):
    # 64K rays that miss (pointing up, away from the heightfield) before the hitting ones:
    # persistent warps must keep fetching through them
    hit_rays = oracle_mod.camera_rays(S.camera_c1(), 128, 128)
    miss = hit_rays.copy()
    miss = np.repeat(miss, 4, axis=1)
    miss[5] = -miss[5]
    rays = np.ascontiguousarray(np.concatenate([miss, hit_rays], axis=1))
    o = c1_oracle.intersect(rays)
    g = to_host(c1_gpu.intersect(torch.from_numpy(rays).cuda()))
    assert (o["patch"][: miss.shape[1]] < 0).all()
    compare_hits(g, o)
    ga = to_host(c1_gpu.intersect(torch.from_numpy(rays).cuda(), any_hit=True))
    oa = c1_oracle.intersect(rays, any_hit=True)
    assert np.array_equal(ga["patch"] >= 0, oa["patch"] >= 0)


def test_longest_axis_split_bit_exact_and_same_hits(rt, c2_small, c2_small_gpu, oracle_mod, torch):
    """CGS_SPLIT_LONGEST: the BVHs and hash tables equal the oracle's
    longest-axis build bit for bit, and the hits equal the reference-split
    store's (t within 1e-6 relative where the patch differs only by a tie)."""
    g = rt.GpuScene(c2_small, split=rt.SPLIT_LONGEST)
    o = oracle_mod.OracleScene(c2_small, split=1)
    for which in (0, -1):
        a, b = g.bvh(which), o.bvh(which)
        for k in ("nodes", "keys", "indices", "table", "disp"):
            assert np.array_equal(a[k], b[k]), (which, k)
    rays = torch.from_numpy(oracle_mod.camera_rays(S.camera_c2(), 160, 90)).cuda()
    r1 = to_host(c2_small_gpu.intersect(rays))
    r2 = to_host(g.intersect(rays))
    assert np.array_equal(r1["patch"] >= 0, r2["patch"] >= 0)
    hit = r1["patch"] >= 0
    rel = np.abs(r1["t"][hit] - r2["t"][hit]) / r1["t"][hit]
    assert rel.max(initial=0) <= 1e-6
    assert (r1["patch"] != r2["patch"])[hit].mean() < 1e-3


@pytest.mark.parametrize("scene", ["torus", "union"])
def test_mirror_split_exports_reference_and_traverses_longest(rt, c2_small, torch, scene, tmp_path):
    """CGS_SPLIT_MIRROR: cgs_bvh_sizes / cgs_bvh_export give the reference
    topology and its hash table bit for bit (those of a reference-split
    store), while queries and renders run on the longest-axis build, so
    their results equal a longest-split store's bit for bit; a mirrored
    store saved and loaded again keeps both."""
    if scene == "torus":
        sc, cam = c2_small, S.camera_c2()
    else:
        sc, cam = S.scene_c4(3, max_patches=4096), S.camera_c4(3)[0]
    ref, lon, mir = (rt.GpuScene(sc, split=k) for k in (rt.SPLIT_REFERENCE, rt.SPLIT_LONGEST, rt.SPLIT_MIRROR))
    for which in list(range(len(sc.surfaces))) + [-1]:
        assert mir.bvh_sizes(which) == ref.bvh_sizes(which)
        a, b = mir.bvh(which), ref.bvh(which)
        for k in a:
            assert np.array_equal(a[k], b[k]), (which, k)
    rays = rt.camera_rays(cam, 160, 90)
    for any_hit in (False, True):
        a, b = to_host(mir.intersect(rays, any_hit=any_hit)), to_host(lon.intersect(rays, any_hit=any_hit))
        for k in a:
            assert np.array_equal(a[k], b[k]), (any_hit, k)
    frames = []
    for g in (mir, lon):
        f = rt.Frame(96, 54)
        rt.RayTracer(rt.Options(recursion_depth=1)).render(f, cam, g)
        torch.cuda.synchronize()
        frames.append(f.rgba())
    assert np.array_equal(frames[0], frames[1])
    mir.save(str(tmp_path / "mirror.cgs"))
    back = rt.GpuScene.load(str(tmp_path / "mirror.cgs"))
    for which in list(range(len(sc.surfaces))) + [-1]:
        a, b = back.bvh(which), ref.bvh(which)
        for k in a:
            assert np.array_equal(a[k], b[k]), ("loaded", which, k)
    a, b = to_host(back.intersect(rays)), to_host(lon.intersect(rays))
    for k in a:
        assert np.array_equal(a[k], b[k]), ("loaded", k)
    for g in (ref, lon, mir, back):
        g.close()


@pytest.mark.parametrize("split", [0, 1])
def test_union_scene_hits_match_oracle_across_list_chunks(rt, oracle_mod, torch, split):
    """A seeded union of 52 displaced cube-spheres and tori (3,258 patches):
    rays cross many objects, so their candidate lists fill and the engine
    parks and resumes them at every point of the object and leaf structure
    (a leaf's last patch, the marker that leaves an object, the step that
    enters the next).  With one, two and eight passes -- rays moving between
    the engine and its inline fallback -- every ray gets the oracle's hit:
    same hit/miss, same object, same patch or an edge tie, t within 1e-5.
    The backtrack cache changes where a backtrack finds its node, not which
    node: hits are bit-identical with it off, when every backtrack reads the
    perfect hash."""
    sc = S.scene_c4(54)
    g = rt.GpuScene(sc, split=split)
    o = oracle_mod.OracleScene(sc, split=split)
    rays = oracle_mod.camera_rays(S.camera_c4(54)[0], 192, 192)
    ref = o.intersect(rays, method=oracle_mod.CLIP_DEVICE)
    assert (ref["patch"] >= 0).mean() > 0.2
    base = rt.engine_config()
    got = {}
    try:
        for passes, cache in ((1, 1), (2, 1), (8, 1), (2, 0)):
            rt.set_engine_config(passes=passes, backtrack_cache=cache)
            h = to_host(g.intersect(torch.from_numpy(rays).cuda()))
            c = g.counters()
            assert c["device_errors"] == 0
            compare_hits(h, ref)
            hit = ref["patch"] >= 0
            assert np.array_equal(h["object"][hit], ref["object"][hit]), passes
            got[passes, cache] = (h, c)
    finally:
        rt.set_engine_config(**base)
    (a, ca), (b, cb) = got[2, 1], got[2, 0]
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    assert ca["nodes"] == cb["nodes"] and ca["hash_lookups"] == cb["hash_lookups"] > 0
    assert cb["hash_table_reads"] == cb["hash_lookups"] and ca["hash_table_reads"] < ca["hash_lookups"] // 2
    g.close()


def test_traversal_entry_point(rt, c2_small_gpu, oracle_mod, torch):
    """cgs_traverse runs the engine's first collect pass alone.  The scene
    has one object, and BVH::hashIntersect tests no root box, so every ray
    enters the object: its list holds the enter and leave markers, and a ray
    that hits a patch at least one patch between them (or its list is full
    and parked); a ray leaving the scene behind holds only the markers.
    Closest and any hit collect the same first-pass lists (both cull with
    the ray's extent only), and a query visits at least the pass's nodes."""
    cam = oracle_mod.camera_rays(S.camera_c2(), 160, 90)
    away = np.array([[0], [0], [50], [0], [0], [1], [np.inf]], np.float32)  # leaves the scene's box behind
    rays = torch.from_numpy(np.ascontiguousarray(np.concatenate([cam, away], axis=1))).cuda()
    hits = to_host(c2_small_gpu.intersect(rays))
    lc = c2_small_gpu.traverse(rays).cpu().numpy()
    nodes = c2_small_gpu.counters()["nodes"]
    la = c2_small_gpu.traverse(rays, any_hit=True).cpu().numpy()
    assert np.array_equal(lc, la)
    assert lc.min() >= 0 and lc.max() <= 64
    hit = hits["patch"] >= 0
    assert (lc[hit] >= 3).all()
    assert lc.min() >= 2 and lc[-1] == 2
    assert nodes > 0
    base = rt.engine_config()
    try:
        rt.set_engine_config(passes=8)
        c2_small_gpu.intersect(rays)
        assert c2_small_gpu.counters()["nodes"] >= nodes
    finally:
        rt.set_engine_config(**base)


def _edge_rays():
    """Rays at the edges of the slab test and the search: directions with
    exact zero components (infinite inverse) from origins exactly on patch
    and box planes (x or y = 0, 1, 2, 3, 4: 0 x inf = NaN inside the slab
    test), short and zero extents, rays along z (the reference's projection
    axes are degenerate for them: they miss), and rays cast sideways and from
    inside the field's box.  No ray lies in the surface: the field is 0 along
    its patch boundaries, so a ray along one of them at z = 0 meets a
    continuum of roots, of which the FP32 search may report any."""
    rays = []
    for x in (0.0, 0.5, 1.0, 2.0, 2.5, 3.0, 4.0):
        for y in (0.0, 1.0, 1.5, 3.0, 4.0):
            for d in ((0, 0.6, -0.8), (0, -0.6, -0.8), (0.6, 0, -0.8), (-0.6, 0, -0.8), (0, 0, -1)):
                for tmax in (np.inf, 2.0, 0.0):
                    rays.append((x, y, 2.0, *d, tmax))
    for z in (-0.2, 0.1, 0.3):
        for y in (0.0, 1.0, 2.2, 4.0):
            rays.append((-1.0, y, z, 1, 0, 0, np.inf))    # along +x
            rays.append((2.0, y, z, 0, 1, 0, np.inf))     # from inside the box along +y
            rays.append((2.0, 2.0, z, -1, 0, 0, np.inf))  # from inside along -x
    return np.ascontiguousarray(np.array(rays, np.float32).T)


def test_edge_rays_match_oracle(rt, c1_gpu, c1_oracle, torch):
    rays = _edge_rays()
    g = to_host(c1_gpu.intersect(torch.from_numpy(rays).cuda()))
    o = c1_oracle.intersect(rays)
    compare_hits(g, o)
    assert (g["patch"] >= 0).sum() > 50 and (g["patch"] < 0).sum() > 100
    zero = rays[6] == 0.0
    assert (g["patch"][zero] < 0).all()  # a zero extent hits nothing
    ga = to_host(c1_gpu.intersect(torch.from_numpy(rays).cuda(), any_hit=True))
    oa = c1_oracle.intersect(rays, any_hit=True)
    assert np.array_equal(ga["patch"] >= 0, oa["patch"] >= 0)
    assert c1_gpu.counters()["device_errors"] == 0


def test_empty_inputs(rt, c1_gpu, torch):
    """Zero rays are a no-op on every query entry point (their arrays may be
    null); an empty render batch is refused as an invalid argument."""
    from cgspline_gb300._capi import CgsError
    none = torch.empty((7, 0), dtype=torch.float32, device="cuda")
    h = c1_gpu.intersect(none)
    assert all(v.numel() == 0 for v in h.values())
    assert all(v.numel() == 0 for v in c1_gpu.intersect(none, any_hit=True).values())
    assert c1_gpu.traverse(none).numel() == 0
    assert c1_gpu.intersect(np.zeros((7, 0), np.float32))["patch"].size == 0
    with pytest.raises(CgsError) as e:
        rt.RayTracer(rt.Options()).render_batch([], c1_gpu)
    assert e.value.status == 1
    torch.cuda.synchronize()


def _rational_surface(seed=11):
    """Ten patches side by side along x: eight bumpy rational patches
    (homogeneous control points with weights in [0.5, 2]), one collapsed to a
    point and one whose control points lie on a line."""
    rng = np.random.default_rng(seed)
    nets = []
    for k in range(10):
        i, j = np.meshgrid(np.arange(4), np.arange(4), indexing="xy")
        x, y = k * 1.5 + i / 3.0, j / 3.0
        z = rng.normal(0.0, 0.3, (4, 4))
        w = rng.uniform(0.5, 2.0, (4, 4))
        if k == 8:
            x, y, z, w = np.full((4, 4), k * 1.5 + 0.5), np.full((4, 4), 0.5), np.zeros((4, 4)), np.ones((4, 4))
        if k == 9:
            x, y, z, w = k * 1.5 + i / 3.0 + j / 9.0, np.full((4, 4), 0.5), np.zeros((4, 4)), np.ones((4, 4))
        # homogeneous points (w x, w y, w z, w): the patch projects to x, y, z where w = 1
        nets.append(np.stack([x * w, y * w, z * w, w], axis=-1).reshape(16, 4))
    pts = np.concatenate(nets).astype(np.float32)
    return S.Surface(pts, np.arange(pts.shape[0], dtype=np.uint32))


def test_rational_and_degenerate_patches(rt, oracle_mod, torch):
    """Rational patches (non-unit weights) and degenerate ones (a point, a
    line) through the patch-pair entry point and the BVH query, against the
    oracle's device-structure search: the same found / missed decisions and t
    within 1e-5."""
    surf = _rational_surface()
    sc = S.Scene([surf], [S.Object(0, S.IDENTITY16.copy(), S.IDENTITY16.copy())],
                 [S.Light((1, 1, 1), 1.0, (0, 0, 5), 0.0, (0, 0, -1), 0.0)])
    g = rt.GpuScene(sc)
    rng = np.random.default_rng(5)
    n = 4000
    pids = rng.integers(0, 10, n).astype(np.int32)
    tx = pids * 1.5 + rng.uniform(-0.1, 1.1, n)
    ty = rng.uniform(-0.1, 1.1, n)
    d = np.stack([rng.uniform(-0.3, 0.3, n), rng.uniform(-0.3, 0.3, n), -np.ones(n)])
    d /= np.linalg.norm(d, axis=0)
    o = np.stack([tx, ty, np.full(n, 0.0)]) - 3.0 * d
    rays = np.ascontiguousarray(np.concatenate([o, d, np.full((1, n), np.inf)]).astype(np.float32))
    found, t, u, v = rt.do_bezier_clipping(g, 0, torch.from_numpy(rays).cuda(), torch.from_numpy(pids).cuda())
    found, t = found.cpu().numpy(), t.cpu().numpy()
    for k in range(n):
        hit, to, _, _ = oracle_mod.patch_intersect(surf.points, surf.indices[16 * pids[k]:16 * pids[k] + 16],
                                                    rays[:, k], method=oracle_mod.CLIP_DEVICE)
        assert bool(found[k]) == hit, k
        if hit:
            assert abs(t[k] - to) <= 1e-5 * to, k
    assert found[pids < 8].mean() > 0.3 and not found[pids == 8].any()
    q = to_host(g.intersect(torch.from_numpy(rays).cuda()))
    oq = oracle_mod.OracleScene(sc).intersect(rays, method=oracle_mod.CLIP_DEVICE)
    compare_hits(q, oq)
    assert g.counters()["device_errors"] == 0
    g.close()


@pytest.mark.parametrize("index", [2, 9, 21, 33])
@pytest.mark.parametrize("split", [0, 1])
def test_union_scenes_closest_and_any_match_oracle(rt, oracle_mod, torch, index, split):
    """More seeded unions (34-59 objects under random transforms), both BVH
    builds: closest hits equal the oracle's device-structure search (same
    object; same patch or an edge tie; t within 1e-5), any-hit decisions are
    identical, and the polished hits stay within 1e-5 of the FP64 oracle."""
    sc = S.scene_c4(index, max_patches=6000)
    g = rt.GpuScene(sc, split=split)
    o = oracle_mod.OracleScene(sc, split=split)
    rays = oracle_mod.camera_rays(S.camera_c4(index)[0], 128, 128)
    tr = torch.from_numpy(rays).cuda()
    h = to_host(g.intersect(tr))
    ref = o.intersect(rays, method=oracle_mod.CLIP_DEVICE)
    compare_hits(h, ref)
    hit = ref["patch"] >= 0
    assert np.array_equal(h["object"][hit], ref["object"][hit])
    ha = to_host(g.intersect(tr, any_hit=True))
    ra = o.intersect(rays, method=oracle_mod.CLIP_DEVICE, any_hit=True)
    assert np.array_equal(ha["patch"] >= 0, ra["patch"] >= 0)
    hp = to_host(g.intersect(tr, precision=rt.FP32_POLISH64))
    r64 = o.intersect(rays, precision=oracle_mod.FP64)
    same = (hp["patch"] >= 0) & (hp["patch"] == r64["patch"]) & (hp["object"] == r64["object"])
    assert same.sum() > 0.9 * (r64["patch"] >= 0).sum()
    rel = np.abs(hp["t"][same] - r64["t"][same]) / r64["t"][same]
    assert rel.max(initial=0) <= 1e-5
    assert g.counters()["device_errors"] == 0
    g.close()


def test_patch_normals_match_oracle(rt, torch, oracle_mod):
    """rt::normal through cgs_patch_normal on the heightfield and on rational
    patches, against the oracle's normal (src/SplineMat.h:178-187), and patch
    ids past the surface refused on the device (zero normal, error bit 16),
    as they are by the patch-pair entry point."""
    # the rational surface's patches 8 and 9 (a point, a line) have no normal:
    # their derivatives are parallel and the cross product is rounding noise
    for surf, regular in ((S.scene_c1().surfaces[0], 16), (_rational_surface(), 8)):
        sc = S.Scene([surf], [S.Object(0, S.IDENTITY16.copy(), S.IDENTITY16.copy())],
                     [S.Light((1, 1, 1), 1.0, (0, 0, 5), 0.0, (0, 0, -1), 0.0)])
        g = rt.GpuScene(sc)
        rng = np.random.default_rng(3)
        n = 500
        pids = rng.integers(0, regular, n).astype(np.int32)
        u, v = rng.uniform(0, 1, n).astype(np.float32), rng.uniform(0, 1, n).astype(np.float32)
        got = rt.normal(g, 0, torch.from_numpy(pids).cuda(), torch.from_numpy(u).cuda(),
                        torch.from_numpy(v).cuda()).cpu().numpy()
        nets = surf.patches()
        for k in range(n):
            _, nk = oracle_mod.patch_eval(nets[pids[k]], float(u[k]), float(v[k]))
            # FP32 normals of two evaluation orders (power basis without FMA in the
            # oracle, Bernstein form with FMA here) agree to a few 1e-5 on steep
            # rational patches
            assert np.abs(got[:, k] - nk).max() < 2e-4, k
        assert g.counters()["device_errors"] == 0
        bad = torch.tensor([0, surf.patch_count, surf.patch_count + 7], dtype=torch.int32, device="cuda")
        half = torch.full((3,), 0.5, device="cuda")
        out = rt.normal(g, 0, bad, half, half).cpu().numpy()
        assert np.abs(out[:, 1:]).max() == 0.0 and np.linalg.norm(out[:, 0]) > 0.5
        assert g.counters()["device_errors"] == 16
        rays = torch.zeros((7, 3), device="cuda")
        rays[5] = -1.0
        rays[6] = float("inf")
        found, t, _, _ = rt.do_bezier_clipping(g, 0, rays, bad)
        assert found.cpu().tolist()[1:] == [0, 0] and g.counters()["device_errors"] == 16
        g.close()
