"""The oracle pinned to the reference program itself (CPU).

tests/golden/*.npz hold outputs of the reference's own hot-path code,
compiled unchanged from its sources (oracle/build_ref.py, oracle/_ref); the
oracle must reproduce them bit for bit on every machine.  Where the
reference tree is present, the oracle is also compared live with that build:
BVHs (nodes, keys, leaf lists), closest and any hits through the reference's
CPURayTracer::intersect, frames through CPURayTracer::render / trace, and
single (ray, patch) pairs through spline::doBezierClipping,
spline::doSubdivision (host) and rt::normal.

Bar: bit-exact everywhere.
"""
import dataclasses

import numpy as np
import pytest

import golden_data as G
from cgspline_gb300 import scenes as S


def _ref():
    from oracle import ref
    return ref


needs_ref = pytest.mark.skipif(not _ref().available(), reason="reference tree not present")


@pytest.mark.parametrize("name", G.NAMES)
def test_oracle_reproduces_reference_fixture(oracle_mod, name):
    g = G.load(name)
    assert int(g["pinned_by_reference"]) == 1
    sc, cam = G.scene(name, g)
    o = oracle_mod.OracleScene(sc)
    rays = oracle_mod.camera_rays(cam, int(g["width"]), int(g["height"]))
    h = o.intersect(rays)
    for k in ("t", "u", "v", "patch", "object"):
        assert np.array_equal(h[k], g[k]), k
    a = o.intersect(rays, any_hit=True)
    assert np.array_equal(a["patch"] >= 0, g["any_hit"])
    f = o.render(cam, int(g["frame_width"]), int(g["frame_height"]), depth=int(g["depth"]))
    assert np.array_equal(f["packed"], g["frame_packed"])
    assert np.array_equal(f["rgb"], g["frame_rgb"])


def test_c1_fixture_is_pinned():
    import os
    g = np.load(os.path.join(G.GOLDEN, "c1_golden.npz"))
    assert int(g["pinned_by_reference"]) == 1


def _compare_scene(oracle_mod, sc, cam, w, h, fw=0, fh=0):
    R = _ref()
    r = R.RefScene(sc)
    o = oracle_mod.OracleScene(sc)
    for k in list(range(len(sc.surfaces))) + [-1]:
        rb, ob = r.bvh(k), o.bvh(k)
        for f in ("nodes", "keys", "indices"):
            assert np.array_equal(rb[f], ob[f]), (k, f)
    rays = oracle_mod.camera_rays(cam, w, h)
    hr, ho = r.intersect(rays), o.intersect(rays)
    for k in ("t", "u", "v", "patch", "object"):
        assert np.array_equal(hr[k], ho[k]), k
    assert np.array_equal(r.intersect(rays, any_hit=True)["hit"], o.intersect(rays, any_hit=True)["patch"] >= 0)
    if fw:
        fr, fo = r.render(cam, fw, fh, depth=1), o.render(cam, fw, fh, depth=1)
        assert np.array_equal(fr["packed"], fo["packed"])
        assert np.array_equal(fr["rgb"], fo["rgb"])
    return int((ho["patch"] >= 0).sum())


@needs_ref
def test_oracle_matches_reference_c1_and_torus(oracle_mod):
    assert _compare_scene(oracle_mod, S.scene_c1(), S.camera_c1(), 256, 256, 64, 64) > 50000
    sc, cam = G.torus32()
    assert _compare_scene(oracle_mod, sc, cam, 240, 135, 96, 54) > 8000


@needs_ref
@pytest.mark.parametrize("index", [0, 17])
def test_oracle_matches_reference_union_scene(oracle_mod, index):
    sc = S.scene_c4(index, max_patches=12000)
    assert _compare_scene(oracle_mod, sc, S.camera_c4(index)[0], 160, 160, 48, 48) > 1000


@needs_ref
@pytest.mark.parametrize("file", ["Test56.dl", "Test104.dl", "Teaset02.dl"])
def test_oracle_matches_reference_dl_scenes(oracle_mod, file):
    """The reference's own scene files beyond the stored fixtures: BVHs of
    every surface and of the object level, closest and any hits, a frame."""
    import os
    from cgspline_gb300 import dl
    root = os.environ.get("CGS_REFERENCE_ROOT", "/root/reference")
    sc, cam = dl.load_dl(os.path.join(root, "assets", "scenes", file))
    assert _compare_scene(oracle_mod, sc, cam, 160, 90, 64, 36) > 5000


@needs_ref
def test_oracle_matches_reference_full_c2_frame_rays(oracle_mod):
    """All 1920x1080 primary rays of the 16,384-patch torus."""
    sc = G.one_material(S.scene_c2())
    assert _compare_scene(oracle_mod, sc, S.camera_c2(), 1920, 1080) == 631561


@needs_ref
def test_oracle_matches_reference_on_single_patches(oracle_mod):
    """(ray, patch) pairs on the 32x32 torus: the hit patch and two random
    ones per camera ray, through spline::doBezierClipping and the host
    spline::doSubdivision (at its default 2^-4 threshold and at 2^-7), and
    rt::normal at random (patch, u, v)."""
    R = _ref()
    sc, cam = G.torus32()
    surf = sc.surfaces[0]
    rays = oracle_mod.camera_rays(cam, 48, 27)
    hits = oracle_mod.OracleScene(sc).intersect(rays)
    rng = np.random.default_rng(3)
    P = surf.patch_count
    n_sub = n_clip = 0
    for r in range(rays.shape[1]):
        ray = rays[:, r]
        pats = ([int(hits["patch"][r])] if hits["patch"][r] >= 0 else []) + [int(p) for p in rng.integers(0, P, 2)]
        for p in pats:
            idx = surf.indices[16 * p:16 * p + 16]
            a, b = oracle_mod.patch_intersect(surf.points, idx, ray), R.patch_intersect(surf.points, idx, ray)
            assert a[0] == b[0] and (not a[0] or (a[1] == b[1] and np.array_equal(a[2], b[2]))), (r, p)
            n_clip += a[0]
            for thr in (2.0 ** -4, 2.0 ** -7):
                a = oracle_mod.patch_subdiv_host(surf.points, idx, ray, thr)
                b = R.patch_intersect(surf.points, idx, ray, thr, method=R.SUBDIV)
                assert a[0] == b[0] and (not a[0] or (a[1] == b[1] and np.array_equal(a[2], b[2]))), (r, p, thr)
                n_sub += a[0]
    assert n_clip > 200 and n_sub > 300
    pidx = rng.integers(0, P, 2000).astype(np.uint32)
    u = rng.random(2000).astype(np.float32)
    v = rng.random(2000).astype(np.float32)
    nr = R.patch_normal(surf.points, surf.indices, pidx, u, v)
    no = np.stack([oracle_mod.patch_eval(surf.points[surf.indices[16 * p:16 * p + 16]], uu, vv)[1]
                   for p, uu, vv in zip(pidx, u, v)])
    assert np.array_equal(nr, no)


@needs_ref
def test_reference_srgb_pack_matches_oracle(oracle_mod):
    """The Ds stand-in's pack_sRGB and the oracle's packing agree on every
    channel value of a dense sweep."""
    R = _ref()
    c = np.linspace(-0.1, 1.1, 30001, dtype=np.float32)
    rgb = np.stack([c, c[::-1], np.roll(c, 7)], -1)
    sc = S.scene_c1()
    o = oracle_mod.OracleScene(sc)
    f = o.render(S.camera_c1(), 32, 32, depth=0)
    assert np.array_equal(R.pack_srgb(f["rgb"]), f["packed"])
    packed = R.pack_srgb(rgb)
    assert packed.dtype == np.uint32 and packed.shape == (c.size,)
    assert np.all((packed >> 24) == 255)


def test_one_material_keeps_geometry():
    sc = S.scene_c2(nu=8, nv=8)
    one = G.one_material(sc)
    assert all(o.patch_material is None for o in one.objects)
    assert G.scene_sha(dataclasses.replace(sc, objects=one.objects)) == G.scene_sha(one)
