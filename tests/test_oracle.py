"""CPU tests of the oracle: known-answer patches, BVH and hash
invariants of the reference (src/rt/BVH.cpp:9-124, src/rt/PerfectHashFunction.cu:486-503),
agreement between its FP32 variants and its FP64 truth, and determinism."""
import math

import numpy as np
import pytest

from cgspline_gb300 import scenes as S


def grid_patch(P00, P10, P01, P11):
    """Degree-elevated bilinear patch: control point (i,j) = bilinear(i/3, j/3)."""
    P00, P10, P01, P11 = (np.asarray(p, np.float64) for p in (P00, P10, P01, P11))
    pts = []
    for j in range(4):
        for i in range(4):
            u, v = i / 3.0, j / 3.0
            p = (1 - u) * (1 - v) * P00 + u * (1 - v) * P10 + (1 - u) * v * P01 + u * v * P11
            pts.append([*p, 1.0])
    return np.asarray(pts, np.float32)


def ray7(o, d):
    d = np.asarray(d, np.float64)
    d = d / np.linalg.norm(d)
    return np.asarray([*o, *d, np.inf], np.float32)


def test_planar_patch_known_answer(oracle_mod):
    # plane through (0,0,0) spanned by U=(1,0.2,0.1), V=(0.1,1,0.3): S(u,v) = uU + vV
    U, V = np.array([1.0, 0.2, 0.1]), np.array([0.1, 1.0, 0.3])
    pts = grid_patch([0, 0, 0], U, V, U + V)
    idx = np.arange(16, dtype=np.uint32)
    rng = S.SplitMix64(11)
    for _ in range(50):
        u, v = rng.uniform(2, 0.05, 0.95)
        target = u * U + v * V
        o = target + np.array([0.3, -0.2, 2.0]) * rng.uniform(1, 1.0, 3.0)[0]
        r = ray7(o, target - o)
        t_true = np.linalg.norm(target - o)
        for method in (oracle_mod.CLIP_HOST, oracle_mod.CLIP_DEVICE, oracle_mod.SUBDIV):
            hit, t, uv, _ = oracle_mod.patch_intersect(pts, idx, r, method=method)
            assert hit
            assert abs(t - t_true) / t_true < 1e-5
            assert abs(uv[0] - u) < 1e-4 and abs(uv[1] - v) < 1e-4


def test_bilinear_patch_known_answer(oracle_mod):
    # hyperbolic paraboloid z = (x - 0.5)(y - 0.5) over the unit square (a twisted bilinear patch)
    P00, P10, P01, P11 = [0, 0, 0.25], [1, 0, -0.25], [0, 1, -0.25], [1, 1, 0.25]
    pts = grid_patch(P00, P10, P01, P11)
    idx = np.arange(16, dtype=np.uint32)
    rng = S.SplitMix64(12)
    for _ in range(50):
        u, v = rng.uniform(2, 0.05, 0.95)
        target = np.array([u, v, (u - 0.5) * (v - 0.5)])
        o = target + np.array([0.1, 0.2, 3.0])
        r = ray7(o, target - o)
        t_true = np.linalg.norm(target - o)
        hit, t, uv, _ = oracle_mod.patch_intersect(pts, idx, r)
        assert hit
        assert abs(t - t_true) / t_true < 1e-5
        assert abs(uv[0] - u) < 2e-4 and abs(uv[1] - v) < 2e-4


def test_miss_and_behind(oracle_mod):
    pts = grid_patch([0, 0, 0], [1, 0, 0.1], [0, 1, 0.1], [1, 1, 0.2])
    idx = np.arange(16, dtype=np.uint32)
    # pointing away from the patch: the root is behind the origin (V.d <= 0 is rejected)
    hit, t, _, _ = oracle_mod.patch_intersect(pts, idx, ray7([0.5, 0.5, 2.0], [0, 0, 1]))
    assert not hit and math.isinf(t)
    # passing beside the patch
    hit, _, _, _ = oracle_mod.patch_intersect(pts, idx, ray7([3.0, 3.0, 2.0], [0, 0, -1]))
    assert not hit
    # a closer current hit.distance culls the root (onHit keeps t < hit.distance)
    hit, _, _, _ = oracle_mod.patch_intersect(pts, idx, ray7([0.5, 0.5, 2.0], [0.01, 0.02, -1]), t=0.5)
    assert not hit


def test_bvh_invariants(c1_oracle):
    b = c1_oracle.bvh(0)
    nodes, keys, ind = b["nodes"], b["keys"], b["indices"]
    P = 16
    assert nodes.shape[0] == 2 * P - 1 and keys.size == 2 * P - 1
    EMPTY = 0xFFFFFFFF
    leaves = 0
    seen = set()
    for i, nd in enumerate(nodes):
        left, right = int(nd[12]), int(nd[13])
        if left == EMPTY:
            leaves += 1
            assert ind[right] != EMPTY and ind[right + 1] == EMPTY  # one element per leaf
            seen.add(int(ind[right]))
        else:
            # pre-order layout: the left child follows its parent; heap keys
            assert left == i + 1
            assert keys[left] == 2 * keys[i] and keys[right] == 2 * keys[i] + 1
            box = nd[:12].view(np.float32)
            for child, off in ((left, 0), (right, 6)):
                cb = nodes[child][:12].view(np.float32)
                lo, hi = cb[0:3], cb[3:6]
                if nodes[child][12] != EMPTY:
                    lo = np.minimum(lo, cb[6:9]); hi = np.maximum(hi, cb[9:12])
                assert np.array_equal(box[off:off + 3], lo) and np.array_equal(box[off + 3:off + 6], hi)
    assert leaves == P and seen == set(range(P))
    assert keys[0] == 1


def test_perfect_hash_injective_and_deterministic(oracle_mod, c1_oracle):
    b = c1_oracle.bvh(0)
    keys = b["keys"]
    h = oracle_mod.hash_build(keys)
    assert h["status"] == 0
    assert h["A"] == b["A"] and h["B"] == b["B"] and h["N"] == b["N"]
    assert np.array_equal(h["table"], b["table"]) and np.array_equal(h["disp"], b["disp"])
    slots = ((h["A"] * keys.astype(np.uint64) + h["B"] + h["disp"][keys & h["mask"]]) & 0xFFFFFFFF) % h["N"]
    assert len(set(slots.tolist())) == keys.size
    assert np.array_equal(h["table"][slots], np.arange(keys.size))
    h2 = oracle_mod.hash_build(keys)
    assert all(np.array_equal(h[k], h2[k]) for k in ("disp", "table"))


@pytest.mark.parametrize("n", [1, 2, 3, 31, 1023, 4097, 65535, 200001])
def test_perfect_hash_sizes(oracle_mod, n):
    # heap keys of a complete-ish binary tree, as the BVH produces
    keys = np.arange(1, n + 1, dtype=np.uint32)
    h = oracle_mod.hash_build(keys)
    assert h["status"] == 0
    dsz = 1 << (max(2, (n - 1) >> 1).bit_length() - 1)
    assert h["disp"].size == dsz
    slots = ((h["A"] * keys.astype(np.uint64) + h["B"] + h["disp"][keys & h["mask"]]) & 0xFFFFFFFF) % h["N"]
    assert np.unique(slots).size == n


def test_hash_bucket_overflow_reported(oracle_mod):
    # 5 keys in one displacement bucket: the reference traps; the oracle reports status 1
    keys = np.array([8, 16, 24, 32, 40, 1, 2, 3, 4, 5, 6, 7], np.uint32)
    assert oracle_mod.hash_build(keys)["status"] == 1


def test_c1_variants_agree_with_fp64(oracle_mod, c1_oracle):
    rays = oracle_mod.camera_rays(S.camera_c1(), 128, 128)
    r = c1_oracle.intersect(rays)
    r64 = c1_oracle.intersect(rays, precision=oracle_mod.FP64)
    rd = c1_oracle.intersect(rays, method=oracle_mod.CLIP_DEVICE)
    hit = r["patch"] >= 0
    assert np.array_equal(hit, r64["patch"] >= 0)
    assert np.array_equal(r["patch"], r64["patch"])
    assert np.array_equal(r["patch"], rd["patch"])
    rel = np.abs(r["t"][hit] - r64["t"][hit]) / r64["t"][hit]
    assert rel.max() < 1e-5
    assert np.abs(rd["t"][hit] - r["t"][hit]).max() / r["t"][hit].min() < 1e-5


def test_c1_golden(c1_oracle, oracle_mod):
    """The restatement against committed vectors (tests/golden/make_golden.py)."""
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "c1_golden.npz"))
    sc = S.scene_c1()
    assert np.array_equal(sc.surfaces[0].points, g["points"])
    assert np.array_equal(sc.surfaces[0].indices, g["indices"])
    b = c1_oracle.bvh(0)
    for k in ("nodes", "keys", "indices", "table", "disp"):
        assert np.array_equal(b[k], g["bvh_" + k]), k
    rays = g["rays"]
    r = c1_oracle.intersect(rays)
    assert np.array_equal(r["patch"], g["patch"])
    hit = g["patch"] >= 0
    np.testing.assert_allclose(r["t"][hit], g["t"][hit], rtol=2e-6)
    np.testing.assert_allclose(r["u"][hit], g["u"][hit], atol=2e-5)
    np.testing.assert_allclose(r["v"][hit], g["v"][hit], atol=2e-5)


def test_render_c1_small(c1_oracle, oracle_mod):
    out = c1_oracle.render(S.camera_c1(), 64, 64, depth=0)
    assert out["primary"] == 64 * 64
    rgb = out["rgb"]
    assert np.isfinite(rgb).all() and 0.0 <= rgb.min() and rgb.max() <= 1.0
    # background pixels equal the background colour exactly; hits are lit
    assert (rgb.reshape(-1, 3) > 0.15).any()


def test_scene_generators_deterministic():
    a, b = S.torus_surface(nu=16, nv=16, seed=5), S.torus_surface(nu=16, nv=16, seed=5)
    assert np.array_equal(a.points, b.points) and np.array_equal(a.indices, b.indices)
    c = S.torus_surface(nu=16, nv=16, seed=6)
    assert not np.array_equal(a.points, c.points)
    # C0 across patch edges: neighbouring patches share their boundary points exactly
    nets = a.patches()
    nu = 16
    for p in range(nu * nu):
        q = (p // nu) * nu + (p % nu + 1) % nu  # next patch along u
        np.testing.assert_array_equal(nets[p].reshape(4, 4, 4)[:, 3], nets[q].reshape(4, 4, 4)[:, 0])


def test_generator_hash_size_lists(oracle_mod):
    """The grid sizes the scene generators avoid are exactly those whose BVH
    key sets the reference's hash cannot place in 16 trials (checked on the
    sizes up to 100 and on every listed size up to 140)."""
    from cgspline_gb300 import scenes as S
    for name, bad, patches, lo in (("torus", S.TORUS_NV_NO_HASH, lambda n: 2 * n * n, 3),
                                   ("sphere", S.SPHERE_N_NO_HASH, lambda n: 6 * n * n, 1)):
        sizes = set(range(lo, 101)) | {b for b in bad if b <= 140}
        for n in sorted(sizes):
            ok = oracle_mod.hash_build(S.bvh_keys(patches(n)))["status"] == 0
            assert ok == (n not in bad), (name, n)


def test_bvh_keys_match_oracle_topology(oracle_mod):
    from cgspline_gb300 import scenes as S
    sc = S.scene_c2(nu=8, nv=6)
    o = oracle_mod.OracleScene(sc)
    assert np.array_equal(o.bvh(0)["keys"], S.bvh_keys(48))


def test_grazing_variant_restatement(oracle_mod):
    """The oracle's precision-form clip (FP64 projection and fat-line bounds
    for near-grazing candidates, tolerance 2^-20) against its FP64 search on
    seeded grazing rays, and unchanged hits on camera rays."""
    from cgspline_gb300 import scenes as S
    sc = S.scene_c2(nu=16, nv=16)
    o = oracle_mod.OracleScene(sc)
    rays = S.grazing_rays(sc.surfaces[0], 4096, seed=21)
    ref = o.intersect(rays, precision=oracle_mod.FP64)
    g = o.intersect(rays, method=oracle_mod.CLIP_GRAZE64, precision=oracle_mod.FP32_POLISH64,
                    graze_sin=oracle_mod.GRAZE_30)
    f = o.intersect(rays, method=oracle_mod.CLIP_DEVICE, precision=oracle_mod.FP32_POLISH64)
    hm_g = ((g["patch"] >= 0) != (ref["patch"] >= 0)).mean()
    hm_f = ((f["patch"] >= 0) != (ref["patch"] >= 0)).mean()
    assert hm_g <= 2e-3 and hm_g < hm_f
    cam = oracle_mod.camera_rays(S.camera_c2(), 64, 36)
    a = o.intersect(cam, method=oracle_mod.CLIP_GRAZE64, precision=oracle_mod.FP32_POLISH64)
    b = o.intersect(cam, precision=oracle_mod.FP64)
    assert np.array_equal(a["patch"] >= 0, b["patch"] >= 0)


def test_grazing_test_catches_bumpy_patches(oracle_mod):
    """On the C2 torus (16,384 patches whose interior control points are
    displaced by about a patch width) a grazing ray can be tangent to a patch
    inside it while the plane of the patch's diagonals is far from the ray:
    the diagonals-only test sends that candidate to the plain FP32 search,
    which loses the root, and the ray reports a farther patch.  The precision
    form's test (the control-net cells' normals, and silhouettes) catches it:
    on 8,192 seeded grazing rays, far fewer hits on another patch than the
    FP64 search's (6 against 86) and far fewer beyond 1e-5 (11 against 108)."""
    from cgspline_gb300 import scenes as S
    sc = S.scene_c2()
    o = oracle_mod.OracleScene(sc)
    rays = S.grazing_rays(sc.surfaces[0], 8192, seed=21)
    ref = o.intersect(rays, precision=oracle_mod.FP64)
    out = {}
    try:
        for mode in (0, 1):
            oracle_mod.set_graze_mode(mode)
            g = o.intersect(rays, method=oracle_mod.CLIP_GRAZE64, precision=oracle_mod.FP32_POLISH64,
                            graze_sin=oracle_mod.GRAZE_30)
            both = (g["patch"] >= 0) & (ref["patch"] >= 0)
            rel = np.abs(g["t"][both] - ref["t"][both]) / ref["t"][both]
            out[mode] = (int((both & (g["patch"] != ref["patch"])).sum()), int((rel > 1e-5).sum()))
    finally:
        oracle_mod.set_graze_mode(1)
    assert out[1][0] <= 12 and out[1][0] * 5 <= out[0][0], out
    assert out[1][1] <= 20 and out[1][1] * 5 <= out[0][1], out


def test_longest_axis_split_same_hits(oracle_mod):
    """The longest-axis build changes only the tree: same hits, far fewer
    node visits than the reference's always-y split."""
    from cgspline_gb300 import scenes as S
    sc = S.scene_c2(nu=32, nv=32)
    a, b = oracle_mod.OracleScene(sc), oracle_mod.OracleScene(sc, split=1)
    rays = oracle_mod.camera_rays(S.camera_c2(), 96, 54)
    ra, rb = a.intersect(rays), b.intersect(rays)
    assert np.array_equal(ra["patch"] >= 0, rb["patch"] >= 0)
    hit = ra["patch"] >= 0
    assert np.abs(ra["t"][hit] - rb["t"][hit]).max() <= 1e-6 * ra["t"][hit].max()
    na = a.intersect_stats(rays)["nodes"].mean()
    nb = b.intersect_stats(rays)["nodes"].mean()
    assert nb < 0.3 * na
    assert not np.array_equal(a.bvh(0)["keys"], b.bvh(0)["keys"]) or a.bvh(0)["nodes"].shape != b.bvh(0)["nodes"].shape \
        or not np.array_equal(a.bvh(0)["nodes"], b.bvh(0)["nodes"])


def test_philox_known_answers(oracle_mod):
    """Philox4x32-10 of the Monte-Carlo path against the published
    known-answer vectors of the generator (Salmon et al., SC 2011)."""
    cases = [([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
             ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
             ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
              [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1])]
    for ctr, key, want in cases:
        assert [int(x) for x in oracle_mod.philox(ctr, key)] == want


def test_monte_carlo_render_restatement(oracle_mod):
    """The sampled path converges to a brightness near the mirror path's on a
    rough, mostly diffuse scene, and is a pure function of its inputs."""
    from cgspline_gb300 import scenes as S
    sc = S.scene_c2(nu=16, nv=16)
    o = oracle_mod.OracleScene(sc)
    a = o.render_spp(S.camera_c2(), 48, 27, 4, depth=2, mc=True)["rgb"]
    b = o.render_spp(S.camera_c2(), 48, 27, 4, depth=2, mc=True)["rgb"]
    m = o.render_spp(S.camera_c2(), 48, 27, 4, depth=2)["rgb"]
    assert np.array_equal(a, b)
    assert abs(float(a.mean()) - float(m.mean())) < 0.05


def test_exact_hull_recovers_roots_the_reference_scan_drops(oracle_mod):
    """The reference finds the fat-line range from a one-pass scan of the
    bound points (src/Spline_BezierClipping.cu:310-348 host, :655-693
    device).  On some nets its polygon leaves out part of the true convex
    hull, and the clip drops a root: the ray reports a farther surface.  On the
    32x32 torus, every ray where subdivision finds a closer hit than the clip
    gets it back from the exact-hull variant, whose hits lie on the surface;
    the exact hull loses no hit the scan finds.  The GPU path keeps the
    reference's scan, so it shares these misses with the oracle."""
    sc, cam = S.scene_c2(nu=32, nv=32), S.camera_c2()
    o = oracle_mod.OracleScene(sc)
    rays = oracle_mod.camera_rays(cam, 512, 512)
    rc = o.intersect(rays)
    rx = o.intersect(rays, method=oracle_mod.CLIP_EXACT_HULL)
    rs = o.intersect(rays, method=oracle_mod.SUBDIV)

    def closer(a, b):
        return (a["patch"] >= 0) & ((b["patch"] < 0) | (a["t"] < b["t"] * (1 - 1e-4)))

    dropped = closer(rs, rc)
    assert 0 < dropped.sum() < 1e-3 * (rc["patch"] >= 0).sum()
    assert not closer(rc, rx).any()
    assert not closer(rs, rx).any()
    assert closer(rx, rc)[dropped].all()
    # the FP64 search with either hull: the exact one finds every hit the
    # scan finds, and more
    x64 = o.intersect(rays, method=oracle_mod.CLIP_EXACT_HULL, precision=oracle_mod.FP64)
    r64 = o.intersect(rays, precision=oracle_mod.FP64)
    assert not closer(r64, x64).any() and closer(x64, r64).any()
    nets = sc.surfaces[0].patches().astype(np.float64)
    for i in np.nonzero(dropped)[0]:
        p = int(rx["patch"][i])
        point = S.eval_patches(nets[p:p + 1], np.array([rx["u"][i]]), np.array([rx["v"][i]]))[0][0]
        on_ray = rays[:3, i].astype(np.float64) + float(rx["t"][i]) * rays[3:6, i].astype(np.float64)
        assert np.linalg.norm(point - on_ray) < 1e-4 * float(rx["t"][i])
