"""GPU parity at the workloads' full sizes, against the oracle (which the CPU
tests hold bit-identical to the reference's own code on these scenes).

* C2: all 2,073,600 primary rays of the 1920x1080 frame on the 16,384-patch
  torus;
* C4: batching-workload scene 5 (61,974 patches, 51 objects), 768x768 rays;
* C5: serving-workload scene 26 (833,776 patches), 512x512 rays;
* C3: 2^20 seeded grazing rays on the C2 torus.

Bars.  The parity build (nvcc --fmad=false, the same sources) is
bit-identical to the oracle's restatement of the reference's GPU clip
structure on C2, C4 and C5 (t, u, v, patch and object of every ray) and on
all but 8 of the 2^20 grazing rays.  The product build (multiply-add
contraction) keeps every hit/miss decision of the reference's FP32 search;
its patch id and t differ only where contraction's rounding moves the FP32
search to another root: on at most 1e-4 of the hits, every other hit
within 1e-5 relative in t.  At FP32 + FP64 polish (the headline level) the
hits are held to the FP64 oracle: hit/miss disagreement at most 2e-5; at
most 1e-4 of the hits (C2, C4) or 1e-3 (the 833,776-patch C5 scene, whose
many small objects show more silhouettes) beyond 1e-5 relative in t,
counting hits on another patch than the FP64 search's.  On the grazing rays the
pure-FP64 GPU search matches the FP64 oracle's hit/miss decisions and t
bit for bit on hits of the same patch.
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


def host(d):
    return {k: v.cpu().numpy() for k, v in d.items()}


def identical(g, o):
    for k in ("t", "u", "v", "patch", "object"):
        assert np.array_equal(g[k], o[k]), (k, int((g[k] != o[k]).sum()))


def product_vs_reference(g, o, frac=1e-4):
    """Hit/miss identical; patch id and t (1e-5 relative) agree on all but
    `frac` of the hits."""
    gp, op = g["patch"], o["patch"]
    assert np.array_equal(gp >= 0, op >= 0), int(((gp >= 0) != (op >= 0)).sum())
    hit = op >= 0
    same = hit & (gp == op) & (g["object"] == o["object"])
    rel = np.abs(g["t"][same] - o["t"][same]) / o["t"][same]
    off = int((hit & ~same).sum()) + int((rel > 1e-5).sum())
    assert off <= frac * hit.sum(), (off, int(hit.sum()))
    return int(hit.sum()), off


def polish_vs_fp64(g, o64, hm_frac=2e-5, over_frac=1e-4):
    """Hit/miss within hm_frac; at most over_frac of the hits beyond 1e-5
    relative in t (a hit on another patch counts by its t)."""
    gp, op = g["patch"], o64["patch"]
    hm = float(((gp >= 0) != (op >= 0)).mean())
    assert hm <= hm_frac, hm
    both = (gp >= 0) & (op >= 0)
    rel = np.abs(g["t"][both] - o64["t"][both]) / o64["t"][both]
    assert (rel > 1e-5).sum() <= over_frac * both.sum(), int((rel > 1e-5).sum())


CASES = {  # scene, camera, rays, polish-vs-FP64 share of hits allowed beyond 1e-5
    "c2": (lambda: S.scene_c2(), lambda: S.camera_c2(), (1920, 1080), 1e-4),
    "c4_5": (lambda: S.scene_c4(5), lambda: S.camera_c4(5)[0], (768, 768), 1e-4),
    "c5_26": (lambda: S.scene_c5(26), lambda: S.camera_c5(26), (512, 512), 1e-3),
}


@pytest.mark.parametrize("case", list(CASES))
def test_fullsize_camera_rays(rt, torch, oracle_mod, case):
    from cgspline_gb300 import _capi
    make_scene, make_cam, (w, h), over = CASES[case]
    sc, cam = make_scene(), make_cam()
    rays_h = oracle_mod.camera_rays(cam, w, h)
    rays = torch.from_numpy(rays_h).cuda()
    o = oracle_mod.OracleScene(sc)
    oh = o.intersect(rays_h)
    od = o.intersect(rays_h, method=oracle_mod.CLIP_DEVICE)

    parity = rt.GpuScene(sc, lib_path=_capi.LIB_NOFMA_PATH)
    identical(host(parity.intersect(rays)), od)
    assert parity.counters()["device_errors"] == 0
    parity.close()

    g = rt.GpuScene(sc)
    nhit, _ = product_vs_reference(host(g.intersect(rays)), oh)
    assert nhit > 0.2 * w * h
    a = host(g.intersect(rays, any_hit=True))
    assert np.array_equal(a["patch"] >= 0, o.intersect(rays_h, any_hit=True)["patch"] >= 0)
    polish_vs_fp64(host(g.intersect(rays, precision=rt.FP32_POLISH64)), o.intersect(rays_h, precision=oracle_mod.FP64),
                   over_frac=over)
    assert g.counters()["device_errors"] == 0
    g.close()


def test_fullsize_grazing_rays(rt, torch, oracle_mod):
    """C3: 2^20 grazing rays.  The FP32 levels lose hits on such rays (the
    precision form's own measurement is the bench's precision leg); here the
    GPU search of each level is held to the oracle's restatement of it."""
    from cgspline_gb300 import _capi
    sc = S.scene_c2()
    rays_h = S.grazing_rays(sc.surfaces[0], 1 << 20, seed=3)
    rays = torch.from_numpy(rays_h).cuda()
    o = oracle_mod.OracleScene(sc)
    o64 = o.intersect(rays_h, precision=oracle_mod.FP64)
    g = rt.GpuScene(sc)
    g64 = host(g.intersect(rays, precision=rt.FP64))
    assert np.array_equal(g64["patch"] >= 0, o64["patch"] >= 0)
    both = (g64["patch"] >= 0) & (g64["patch"] == o64["patch"])
    assert (~both & (o64["patch"] >= 0)).sum() <= 4
    assert np.array_equal(g64["t"][both], o64["t"][both])
    # the precision form against the oracle's restatement of the same variant
    gg = host(g.intersect(rays, precision=rt.FP32_GRAZE64))
    og = o.intersect(rays_h, method=oracle_mod.CLIP_GRAZE64, precision=oracle_mod.FP32_POLISH64,
                     graze_sin=oracle_mod.GRAZE_30)
    assert float(((gg["patch"] >= 0) != (og["patch"] >= 0)).mean()) <= 1e-4
    # and against FP64: at most 2e-4 hit/miss disagreement (FP32 alone: ~5e-3)
    assert float(((gg["patch"] >= 0) != (o64["patch"] >= 0)).mean()) <= 2e-4
    assert g.counters()["device_errors"] & 1 == 0
    g.close()
    parity = rt.GpuScene(sc, lib_path=_capi.LIB_NOFMA_PATH)
    p = host(parity.intersect(rays))
    od = o.intersect(rays_h, method=oracle_mod.CLIP_DEVICE)
    differ = (p["patch"] != od["patch"]) | ((od["patch"] >= 0) & (p["t"] != od["t"]))
    assert int(differ.sum()) <= 8, int(differ.sum())
    parity.close()


def test_fullsize_shadow_rays(rt, torch, oracle_mod):
    """Shadow rays of the C2 torus (16,384 patches) from the hit points of a
    960x540 view toward two point lights: the any-hit engine, whose idle lanes
    take pending intervals of long clip searches at the end of a launch, gives
    the oracle's decisions on every ray -- the parity build against the
    restatement of the reference's GPU clip (identical), the product build
    (multiply-add contraction) on all but 1e-4 of the rays.  These rays leave
    the surface, many at grazing angles, where contraction alone moves a few
    near-tangent decisions."""
    from cgspline_gb300 import _capi
    sc = S.scene_c2()
    o = oracle_mod.OracleScene(sc)
    cam = oracle_mod.camera_rays(S.camera_c2(), 960, 540)
    h = o.intersect(cam)
    hit = h["patch"] >= 0
    P = cam[0:3, hit] + h["t"][hit] * cam[3:6, hit]
    shadow = []
    for light in ((4.0, 8.0, 6.0), (-6.0, 3.0, -2.0)):
        L = np.asarray(light, np.float32)[:, None] - P
        dist = np.linalg.norm(L, axis=0, keepdims=True)
        L = L / dist
        shadow.append(np.concatenate([P + 1e-4 * L, L, dist], 0))
    rays_h = np.ascontiguousarray(np.concatenate(shadow, 1), np.float32)
    rays = torch.from_numpy(rays_h).cuda()
    assert rays_h.shape[1] > 250_000
    od = o.intersect(rays_h, method=oracle_mod.CLIP_DEVICE, any_hit=True)
    oh = o.intersect(rays_h, any_hit=True)
    assert 0.05 < float((oh["patch"] >= 0).mean()) < 0.95
    parity = rt.GpuScene(sc, lib_path=_capi.LIB_NOFMA_PATH)
    p = host(parity.intersect(rays, any_hit=True))
    assert np.array_equal(p["patch"] >= 0, od["patch"] >= 0)
    assert parity.counters()["device_errors"] == 0
    parity.close()
    g = rt.GpuScene(sc)
    a = host(g.intersect(rays, any_hit=True))
    differ = int(((a["patch"] >= 0) != (od["patch"] >= 0)).sum())
    assert differ <= rays_h.shape[1] // 10_000, differ
    assert g.counters()["device_errors"] == 0
    g.close()
