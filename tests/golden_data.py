"""The reference-pinned golden fixtures of tests/golden/ and the scenes they
were computed on (tests/golden/make_golden.py writes them with the reference
program's own code)."""
import dataclasses
import hashlib
import os

import numpy as np

from cgspline_gb300 import scenes as S

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
NAMES = ("torus32", "union", "teaset", "test32", "test152")
# fixtures that store their scene (the reference's own .dl scenes)
STORED = ("teaset", "test32", "test152")


def load(name: str):
    return np.load(os.path.join(GOLDEN, f"{name}_golden.npz"))


def scene_sha(sc) -> str:
    """SHA-256 over every surface's points and indices and every object's
    surface, matrices and material."""
    h = hashlib.sha256()
    for s in sc.surfaces:
        h.update(np.ascontiguousarray(s.points, np.float32).tobytes())
        h.update(np.ascontiguousarray(s.indices, np.uint32).tobytes())
    for o in sc.objects:
        h.update(np.int32(o.surface).tobytes())
        h.update(np.ascontiguousarray(o.local2world, np.float32).tobytes())
        h.update(np.ascontiguousarray(o.world2local, np.float32).tobytes())
        h.update(np.ascontiguousarray(o.material.packed(), np.float32).tobytes())
    return h.hexdigest()


def one_material(sc):
    """The scene with per-patch materials dropped (the reference has one
    material per object)."""
    return dataclasses.replace(sc, objects=[dataclasses.replace(o, patch_material=None, materials=None)
                                            for o in sc.objects])


def torus32():
    return one_material(S.scene_c2(nu=32, nv=32)), S.camera_c2()


def union5():
    return S.scene_c4(5, max_patches=20000), S.camera_c4(5)[0]


def camera(packed):
    p = [float(x) for x in np.asarray(packed, np.float32)]
    return S.Camera(tuple(p[0:4]), tuple(p[4:7]), tuple(p[7:10]), p[10])


def stored_scene(g, name="teaset"):
    """The scene stored in a fixture of STORED."""
    surfaces = [S.Surface(g[f"surface{k}_points"], g[f"surface{k}_indices"]) for k in range(int(g["surfaces"]))]
    objects = []
    for row in g["objects"]:
        m = row[33:41]
        objects.append(S.Object(int(row[0]), row[1:17].copy(), row[17:33].copy(),
                                S.Material(tuple(m[0:3]), tuple(m[3:6]), float(m[6]), float(m[7]))))
    lights = [S.Light(tuple(l[0:3]), float(l[3]), tuple(l[4:7]), float(l[7]), tuple(l[8:11]), float(l[11]))
              for l in g["lights"]]
    return S.Scene(surfaces, objects, lights, tuple(float(x) for x in g["background"]),
                   tuple(float(x) for x in g["ambient"]), name=name)


def scene(name: str, g):
    """(scene, camera) of fixture `name`, checked against the fixture's SHA."""
    if name == "torus32":
        sc, _ = torus32()
    elif name == "union":
        sc, _ = union5()
    else:
        sc = stored_scene(g, name)
    if scene_sha(sc) != bytes(g["scene_sha"]).decode():
        raise AssertionError(f"{name}: the scene generator no longer gives the fixture's scene")
    return sc, camera(g["camera"])
