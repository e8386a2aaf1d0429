"""Generate the committed golden vectors under tests/golden/.

c1_golden.npz: the 4x4-patch heightfield scene (seed 1), its BVH and perfect
hash, and closest hits of 128x128 camera rays, as computed by the oracle's
restatement of the reference host path (oracle/cgs_oracle.cpp).  When the
reference's own sources were compiled here (oracle/_ref, see
oracle/build_ref.py), the script also checks that they give the same BVH and
hits and records that in the file ("pinned_by_reference" = 1).

Run:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from cgspline_gb300 import scenes as S  # noqa: E402


def main():
    sc = S.scene_c1()
    o = oracle.OracleScene(sc)
    b = o.bvh(0)
    rays = oracle.camera_rays(S.camera_c1(), 128, 128)
    r = o.intersect(rays)
    pinned = 0
    try:
        from oracle import ref as R
        if R.available():
            rr = R.intersect_scene(sc, rays)
            rb = R.bvh_export(sc)
            same_bvh = all(np.array_equal(rb[k], b[k]) for k in ("nodes", "keys", "indices"))
            same_hits = np.array_equal(rr["patch"], r["patch"]) and np.array_equal(rr["t"], r["t"])
            pinned = int(same_bvh and same_hits)
            print("reference build agrees:", same_bvh, same_hits)
    except ImportError:
        pass
    np.savez_compressed(os.path.join(HERE, "c1_golden.npz"), points=sc.surfaces[0].points,
                        indices=sc.surfaces[0].indices, bvh_nodes=b["nodes"], bvh_keys=b["keys"],
                        bvh_indices=b["indices"], bvh_table=b["table"], bvh_disp=b["disp"],
                        hash_params=np.array([b["A"], b["B"], b["N"], b["mask"]], np.uint32), rays=rays,
                        t=r["t"], u=r["u"], v=r["v"], patch=r["patch"], pinned_by_reference=np.int32(pinned))
    print("wrote c1_golden.npz; hits", int((r["patch"] >= 0).sum()), "of", rays.shape[1])


if __name__ == "__main__":
    main()
