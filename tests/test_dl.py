"""The .be loader and the .dl scene reader (host side), on synthetic files
written by the tests and, where the reference's assets are present, on the
reference's own scene files."""
import math
import os

import numpy as np
import pytest

from cgspline_gb300 import dl, scenes as S

# the reference tree's assets, where the tree is present (the teaset scene's
# geometry also lives in tests/golden/teaset_golden.npz for machines without it)
REF_ASSETS = os.path.join(os.environ.get("CGS_REFERENCE_ROOT", "/root/reference"), "assets")

SYNTH = """
// a synthetic scene in the reference's description language
let Gray = (0.5 0.5 0.5)
let Views = { Front: { position:(0 1 6) rotation:(-10 0 0) } }
Material { name:"Red" metalness:0.1 roughness:0.8 diffuse:From_sRGB(255 0 0) specular:(0.04 0.04 0.04) }
Material { name:"Metal" metalness:0.9 roughness:0.2 diffuse:Gray specular:(0.9 0.9 0.9) }
Surface { name:"field" file:"field.be" }
Surface { name:"ring" file:"ring.be" }
Scene
{
  environment:{ background:(0.2 0.2 0.25) ambient:(0.05 0.05 0.05) }
  view:Views.Front
  objects:
  [
    { name:"Floor" transform:{ position:(-2 0 -2) rotation:(0 0 0) scale:(1 1 1) }
      surface:{ model:Get("field") material:Get("Red") } }
    { name:"Group" transform:{ position:(0 1 0) rotation:(90 0 0) }
      objects:
      [
        { name:"Ring" transform:{ scale:(0.5 0.5 0.5) } surface:{ model:Get("ring") material:Get("Metal") } }
      ]
    }
    { name:"Lamp" transform:{ position:(3 4 5) } light:{ type:"point" color:*(40 (1 0.9 0.8)) } }
  ]
}
"""


@pytest.fixture(scope="module")
def synth_dir(tmp_path_factory):
    d = tmp_path_factory.mktemp("dl")
    S.save_be(S.heightfield(3, sigma=0.2, n=4), str(d / "field.be"))
    S.save_be(S.torus_surface(1.0, 0.3, 8, 6, 0.0, 4), str(d / "ring.be"))
    (d / "scene.dl").write_text(SYNTH)
    return d


def test_be_round_trip(tmp_path):
    s = S.torus_surface(nu=8, nv=6)
    S.save_be(s, str(tmp_path / "t.be"))
    r = S.load_be(str(tmp_path / "t.be"))
    assert np.array_equal(r.indices, s.indices) and np.abs(r.points - s.points).max() == 0.0
    with pytest.raises(ValueError):
        S.load_be("1\n" + ",".join(["1"] * 15) + ",9\n2\n0,0,0\n1,1,1\n")


def test_dl_synthetic_scene(synth_dir, oracle_mod):
    sc, cam = dl.load_dl(str(synth_dir / "scene.dl"))
    assert len(sc.surfaces) == 2 and len(sc.objects) == 2 and len(sc.lights) == 1
    floor, ring = sc.objects
    l2w = floor.local2world.reshape(4, 4).T
    assert np.allclose(l2w[:3, 3], (-2, 0, -2))
    # the ring: parent at (0,1,0) turned 90 degrees about x, scaled by 0.5
    R = ring.local2world.reshape(4, 4).T
    assert np.allclose(R[:3, 3], (0, 1, 0), atol=1e-6)
    assert np.allclose(R[:3, :3] @ np.array([0, 1, 0]), (0, 0, 0.5), atol=1e-6)
    assert np.allclose(ring.world2local.reshape(4, 4).T @ R, np.eye(4), atol=1e-5)
    assert ring.material.metalness == np.float32(0.9) and floor.material.diffuse[0] == 1.0
    li = sc.lights[0]
    assert np.allclose(li.position, (3, 4, 5)) and np.allclose(li.color, (40, 36, 32)) and li.angle > 1.57
    assert np.allclose(sc.background, (0.2, 0.2, 0.25))
    assert np.allclose(cam.position, (0, 1, 6)) and abs(cam.fovy - math.radians(60)) < 1e-6
    # the camera looks 10 degrees down the -z axis
    x, y, z, w = cam.rotation
    fwd = -np.array([2 * (x * z + w * y), 2 * (y * z - w * x), 1 - 2 * (x * x + y * y)])
    assert np.allclose(fwd, (0, -math.sin(math.radians(10)), -math.cos(math.radians(10))), atol=1e-6)
    o = oracle_mod.OracleScene(sc)
    hits = o.intersect(oracle_mod.camera_rays(cam, 64, 48))
    assert 0.05 < (hits["patch"] >= 0).mean() < 1.0


@pytest.mark.skipif(not os.path.isdir(REF_ASSETS), reason="reference assets not present")
@pytest.mark.parametrize("name", ["Teaset01", "Test32"])
def test_dl_reference_scenes(name, oracle_mod):
    sc, cam = dl.load_dl(os.path.join(REF_ASSETS, "scenes", f"{name}.dl"))
    assert len(sc.surfaces) == 4 and len(sc.objects) >= 4 and len(sc.lights) >= 1
    assert sorted(s.patch_count for s in sc.surfaces) == [4, 16, 26, 32]  # longwave, teaspoon, teacup, teapot
    o = oracle_mod.OracleScene(sc)
    r = o.render(cam, 48, 27, depth=1)
    assert (o.intersect(oracle_mod.camera_rays(cam, 48, 27))["patch"] >= 0).mean() > 0.5
    assert 0.02 < float(r["rgb"].mean()) < 0.9


@pytest.mark.gpu
def test_dl_scene_renders_on_gpu_like_oracle(synth_dir, oracle_mod):
    import torch
    from cgspline_gb300 import rt
    sc, cam = dl.load_dl(str(synth_dir / "scene.dl"))
    g = rt.GpuScene(sc)
    fb, lin = rt.RayTracer(rt.Options(recursion_depth=1)).render_host(cam, g, 96, 72)
    ro = oracle_mod.OracleScene(sc).render(cam, 96, 72, depth=1)
    err = np.abs(lin - ro["rgb"])
    assert float(np.sqrt((err ** 2).mean())) < 5e-3
    assert g.counters()["device_errors"] == 0
    g.close()
    torch.cuda.synchronize()
