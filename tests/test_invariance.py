"""Size-independent properties of the two-level intersection: moving a
scene's objects by a rigid motion or a uniform scale, and the rays with them,
keeps every hit (same hit/miss, same patch, u and v) and scales t by the scale
factor.  The oracle (CPU) here; the GPU path in test_gpu_invariance.py."""
import copy
import math

import numpy as np
import pytest

from cgspline_gb300 import scenes as S

MOTIONS = [((0.7, (1, 2, 3), (5.0, -3.0, 2.0)), 1.0),
           ((0.0, (0, 0, 1), (0.0, 0.0, 0.0)), 3.5),
           ((2.1, (0, 1, 0), (-1.0, 0.5, 4.0)), 0.25)]


def motion(angle, axis, t, s):
    """4x4 matrix s * R(axis, angle) followed by the translation t."""
    a = np.asarray(axis, np.float64)
    a /= np.linalg.norm(a)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    M = np.eye(4)
    M[:3, :3] = s * (np.eye(3) + math.sin(angle) * K + (1 - math.cos(angle)) * K @ K)
    M[:3, 3] = t
    return M


def moved_scene(scene, M):
    """The scene with M applied after every object's local-to-world matrix
    (column-major, as the objects store them)."""
    sc = copy.deepcopy(scene)
    for o in sc.objects:
        L = M @ np.asarray(o.local2world, np.float64).reshape(4, 4, order="F")
        o.local2world = L.reshape(16, order="F").astype(np.float32)
        o.world2local = np.linalg.inv(L).reshape(16, order="F").astype(np.float32)
    return sc


def moved_rays(rays, M, s):
    """(7, n) rays with M applied to the origins and the rotation to the unit
    directions (tmax unbounded)."""
    out = rays.astype(np.float64)
    out[:3] = M[:3, :3] @ out[:3] + M[:3, 3:4]
    out[3:6] = M[:3, :3] @ out[3:6] / s
    return out.astype(np.float32)


def check_same_hits(r0, r1, s):
    h0, h1 = r0["patch"] >= 0, r1["patch"] >= 0
    assert np.array_equal(h0, h1)
    assert np.array_equal(r0["patch"], r1["patch"])
    rel = np.abs(np.asarray(r1["t"])[h0] / s - np.asarray(r0["t"])[h0]) / np.asarray(r0["t"])[h0]
    assert rel.max(initial=0.0) < 1e-5
    # the moved rays are rounded to FP32, and a hit's (u, v) moves by about
    # that rounding over the cosine of the incidence angle: large only at
    # grazing hits
    duv = np.maximum(np.abs(np.asarray(r0["u"])[h0] - np.asarray(r1["u"])[h0]),
                     np.abs(np.asarray(r0["v"])[h0] - np.asarray(r1["v"])[h0]))
    assert np.quantile(duv, 0.999) < 1e-4 and duv.max() < 1e-3
    assert h0.mean() > 0.2


def cases():
    return [("heightfield", S.scene_c1(), S.camera_c1()), ("torus32", S.scene_c2(nu=32, nv=32), S.camera_c2())]


@pytest.mark.parametrize("k", range(len(MOTIONS)))
@pytest.mark.parametrize("which", [0, 1])
def test_oracle_hits_follow_the_motion(oracle_mod, which, k):
    name, sc, cam = cases()[which]
    (angle, axis, t), s = MOTIONS[k]
    M = motion(angle, axis, t, s)
    rays = oracle_mod.camera_rays(cam, 96, 96)
    for prec in (oracle_mod.FP32, oracle_mod.FP64):
        r0 = oracle_mod.OracleScene(sc).intersect(rays, precision=prec)
        r1 = oracle_mod.OracleScene(moved_scene(sc, M)).intersect(moved_rays(rays, M, s), precision=prec)
        check_same_hits(r0, r1, s)
