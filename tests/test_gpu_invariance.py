"""The motion property of test_invariance.py on the GPU path: moving a
scene's objects by a rigid motion or a uniform scale, and the rays with them,
keeps every hit (hit/miss, patch, u and v) and scales t by the scale factor,
at FP32 and with the FP64 polish."""
import numpy as np
import pytest

from test_invariance import MOTIONS, cases, check_same_hits, motion, moved_rays, moved_scene

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("k", range(len(MOTIONS)))
@pytest.mark.parametrize("which", [0, 1])
def test_gpu_hits_follow_the_motion(oracle_mod, which, k):
    import torch
    from cgspline_gb300 import rt
    name, sc, cam = cases()[which]
    (angle, axis, t), s = MOTIONS[k]
    M = motion(angle, axis, t, s)
    rays = oracle_mod.camera_rays(cam, 96, 96)
    g0, g1 = rt.GpuScene(sc), rt.GpuScene(moved_scene(sc, M))
    try:
        for prec in (rt.FP32, rt.FP32_POLISH64):
            r0 = g0.intersect(torch.from_numpy(rays).cuda(), precision=prec)
            r1 = g1.intersect(torch.from_numpy(moved_rays(rays, M, s)).cuda(), precision=prec)
            check_same_hits({k: v.cpu().numpy() for k, v in r0.items()},
                            {k: v.cpu().numpy() for k, v in r1.items()}, s)
        assert g0.counters()["device_errors"] == 0 and g1.counters()["device_errors"] == 0
    finally:
        g0.close()
        g1.close()
