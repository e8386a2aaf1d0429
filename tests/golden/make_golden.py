"""Generate the committed golden vectors under tests/golden/ from the reference itself.

Every expected output in these files is computed by the reference program's
own hot-path code, compiled unchanged from its sources into oracle/_ref (see
oracle/build_ref.py), and checked here against the oracle's restatement
(oracle/cgs_oracle.cpp): the script refuses to write a file where the two
differ, and records "pinned_by_reference" = 1 in every file it writes.  The
reference tree must be present (it is not on the GPU machines, which use the
committed files).

  c1_golden.npz      the 4x4-patch heightfield (seed 1): scene, BVH, perfect
                     hash and closest hits of 128x128 camera rays (the inputs
                     are stored; the BVH and hash arrays are the oracle's,
                     the BVH checked equal to the reference's);
  torus32_golden.npz the displaced torus on a 32x32 patch grid (seed 2):
                     closest hits of 160x90 camera rays and a 64x36 frame
                     (depth 1, one material for the whole torus);
  union_golden.npz   union scene 5 of the batching workload at <= 20,000
                     patches (19,800 patches, 51 objects): closest and any
                     hits of 96x96 camera rays and a 64x64 frame;
  teaset_golden.npz  the reference's own teaset scene (assets/scenes/
                     Teaset01.dl with the .be surfaces it names): the scene's
                     surfaces, objects, light and camera, closest hits of
                     160x90 camera rays and a 96x54 frame;
  test32_golden.npz, test152_golden.npz
                     the reference's test scenes assets/scenes/Test32.dl and
                     Test152.dl (32 and 152 teaset pieces on the long-wave
                     floor, 11 and 51 lights), stored the same way: closest
                     and any hits of 160x90 camera rays and a 96x54 frame.

The seeded scenes are regenerated by the tests from cgspline_gb300.scenes;
each file stores a SHA-256 of the scene arrays so that a changed generator is
caught.  The teaset's geometry is stored in the file itself.

Run:  python tests/golden/make_golden.py [name ...]   (default: every file; names:
      c1 torus32 union teaset test32 test152)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import oracle  # noqa: E402
from golden_data import one_material, scene_sha, torus32, union5  # noqa: E402,F401
from oracle import ref as R  # noqa: E402
from cgspline_gb300 import scenes as S  # noqa: E402

REFERENCE_ROOT = os.environ.get("CGS_REFERENCE_ROOT", "/root/reference")


def dl_scene(file):
    from cgspline_gb300 import dl
    return dl.load_dl(os.path.join(REFERENCE_ROOT, "assets", "scenes", file))


def write_stored(name, sc, cam, size=(160, 90), frame=(96, 54)):
    """A fixture that stores its scene (surfaces, objects, lights, environment)."""
    print(f"{name}_golden.npz: {sc.patch_count} patches, {len(sc.objects)} objects, {len(sc.lights)} lights")
    out = reference_outputs(sc, cam, *size, *frame)
    geo = {}
    for k, s in enumerate(sc.surfaces):
        geo[f"surface{k}_points"] = s.points
        geo[f"surface{k}_indices"] = s.indices
    objs = np.array([[o.surface, *o.local2world, *o.world2local, *o.material.packed()] for o in sc.objects],
                    np.float32)
    lights = np.array([l.packed() for l in sc.lights], np.float32)
    np.savez_compressed(os.path.join(HERE, f"{name}_golden.npz"), surfaces=np.int32(len(sc.surfaces)), objects=objs,
                        lights=lights, background=np.asarray(sc.background, np.float32),
                        ambient=np.asarray(sc.ambient, np.float32), scene_sha=np.bytes_(scene_sha(sc)), **geo, **out)


def same_hits(a, b, keys=("t", "u", "v", "patch", "object")):
    return all(np.array_equal(a[k], b[k]) for k in keys)


def reference_outputs(sc, cam, w, h, fw, fh, depth=1):
    """Closest (and any) hits of w x h camera rays and an fw x fh frame, from
    the reference build; each checked equal to the oracle's."""
    r = R.RefScene(sc)
    o = oracle.OracleScene(sc)
    for k in list(range(len(sc.surfaces))) + [-1]:
        rb, ob = r.bvh(k), o.bvh(k)
        if not all(np.array_equal(rb[f], ob[f]) for f in ("nodes", "keys", "indices")):
            raise SystemExit(f"BVH {k}: reference and oracle differ")
    rays = oracle.camera_rays(cam, w, h)
    hr, ho = r.intersect(rays), o.intersect(rays)
    if not same_hits(hr, ho):
        raise SystemExit("closest hits: reference and oracle differ")
    ar, ao = r.intersect(rays, any_hit=True), o.intersect(rays, any_hit=True)
    if not np.array_equal(ar["hit"], ao["patch"] >= 0):
        raise SystemExit("any hits: reference and oracle differ")
    fr = r.render(cam, fw, fh, depth=depth)
    fo = o.render(cam, fw, fh, depth=depth)
    if not (np.array_equal(fr["packed"], fo["packed"]) and np.array_equal(fr["rgb"], fo["rgb"])):
        raise SystemExit("frames: reference and oracle differ")
    print(f"  {int((hr['patch'] >= 0).sum())} hits of {rays.shape[1]} rays; "
          f"{int(ar['hit'].sum())} blocked; frame {fw}x{fh}: reference == oracle")
    return dict(camera=cam.packed(), width=np.int32(w), height=np.int32(h), t=hr["t"], u=hr["u"], v=hr["v"],
                patch=hr["patch"], object=hr["object"], any_hit=ar["hit"], frame_width=np.int32(fw),
                frame_height=np.int32(fh), depth=np.int32(depth), frame_packed=fr["packed"], frame_rgb=fr["rgb"],
                pinned_by_reference=np.int32(1))


def write_c1():
    """C1: the inputs, BVH and hash in the file, checked against the reference."""
    sc = S.scene_c1()
    o = oracle.OracleScene(sc)
    r = R.RefScene(sc)
    b = o.bvh(0)
    rb = r.bvh(0)
    if not all(np.array_equal(rb[k], b[k]) for k in ("nodes", "keys", "indices")):
        raise SystemExit("C1 BVH: reference and oracle differ")
    rays = oracle.camera_rays(S.camera_c1(), 128, 128)
    hr, ho = r.intersect(rays), o.intersect(rays)
    if not same_hits(hr, ho):
        raise SystemExit("C1 hits: reference and oracle differ")
    np.savez_compressed(os.path.join(HERE, "c1_golden.npz"), points=sc.surfaces[0].points,
                        indices=sc.surfaces[0].indices, bvh_nodes=b["nodes"], bvh_keys=b["keys"],
                        bvh_indices=b["indices"], bvh_table=b["table"], bvh_disp=b["disp"],
                        hash_params=np.array([b["A"], b["B"], b["N"], b["mask"]], np.uint32), rays=rays,
                        t=hr["t"], u=hr["u"], v=hr["v"], patch=hr["patch"], pinned_by_reference=np.int32(1))
    print("c1_golden.npz: hits", int((hr["patch"] >= 0).sum()), "of", rays.shape[1], "(reference == oracle)")


def main():
    if not R.available():
        raise SystemExit(f"the reference build is needed: {R.unavailable_reason()}")
    # optional arguments: the fixture names to write (default: all)
    only = set(sys.argv[1:])

    if not only or "c1" in only:
        write_c1()

    for name, make, size, frame in (("torus32", torus32, (160, 90), (64, 36)),
                                    ("union", union5, (96, 96), (64, 64))):
        if only and name not in only:
            continue
        sc, cam = make()
        print(f"{name}_golden.npz: {sc.patch_count} patches, {len(sc.objects)} objects")
        out = reference_outputs(sc, cam, *size, *frame)
        np.savez_compressed(os.path.join(HERE, f"{name}_golden.npz"), scene_sha=np.bytes_(scene_sha(sc)), **out)

    for name, file in (("teaset", "Teaset01.dl"), ("test32", "Test32.dl"), ("test152", "Test152.dl")):
        if only and name not in only:
            continue
        write_stored(name, *dl_scene(file))


if __name__ == "__main__":
    main()
