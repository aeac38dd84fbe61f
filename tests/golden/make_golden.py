"""Generates tests/golden/golden.npz (run here, where the reference is present).

Sources:
  * ref_*   -- the reference's own Core/random.cuh and Core/RayTracer.cu
               compiled for the host (oracle/_ref/libvenu_ref.so, built by
               `make -C oracle ref REF_ROOT=<reference checkout>`), run on the
               RTIOW scene;
  * gb_*    -- the oracle's GB300 arithmetic (oracle/_build/libvenu_oracle.so)
               on the same inputs, pinning the oracle across machines;
  * bvh_*   -- the oracle's host LBVH of the same scene.

Usage:  python tests/golden/make_golden.py [REF_ROOT]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import pyoracle  # noqa: E402

W, H, SPP = 48, 27, 4


def main(ref_root: str) -> None:
    pyoracle.build(ref_root=ref_root, with_ref=True)
    O = pyoracle.Oracle()
    R = pyoracle.RefBuild()
    out = {}
    pairs = np.array([(i, j) for i in (0, 1, 7, 1000, 123456, 2**31 + 5) for j in (0, 1, 2, 99, 2**32 - 1)],
                     np.uint32)
    out["rng_pairs"] = pairs
    out["rng_tea4"] = np.array([R.tea4(int(a), int(b)) for a, b in pairs], np.uint32)
    vals, states = R.rnd_stream(R.tea4(0, 1), 256)
    out["rng_rnd"] = vals
    out["rng_states"] = states

    spheres = O.scene_rtiow(0)
    cam = O.camera((13, 2, 3), (0, 0, 0), 20.0, W / H, 0.1, 10.0)
    out["scene"] = spheres.view(np.uint8).reshape(len(spheres), -1)
    out["camera"] = cam.view(np.uint8).reshape(-1)
    out["wh_spp"] = np.array([W, H, SPP], np.uint32)

    r0 = R.render(spheres, cam, W, H, SPP, subframe=0)
    out["ref_s0_accum"] = r0["accum"]
    out["ref_s0_image8"] = r0["image8"]
    prior = np.random.default_rng(7).random((W * H, 4)).astype(np.float32)
    r3 = R.render(spheres, cam, W, H, 2, subframe=3, accum=prior.copy())
    out["ref_s3_prior"] = prior
    out["ref_s3_accum"] = r3["accum"]
    out["ref_s3_image8"] = r3["image8"]

    for depth in (4, 50):
        g = O.render(spheres, cam, W, H, SPP, subframe=1, max_depth=depth, mode=pyoracle.MODE_GB300)
        out[f"gb_d{depth}_accum"] = g["accum"]
        out[f"gb_d{depth}_image8"] = g["image8"]
        out[f"gb_d{depth}_segments"] = np.array([g["segments"]], np.uint64)

    b = O.lbvh(spheres)
    out["bvh_keys"] = b["keys"]
    out["bvh_ids"] = b["ids"]
    out["bvh_nodes"] = b["nodes"].view(np.uint8).reshape(len(b["nodes"]), -1)
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **out)
    print("wrote", os.path.join(HERE, "golden.npz"), {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    if len(sys.argv) < 2 and not os.environ.get("VENU_REFERENCE_ROOT"):
        sys.exit("usage: make_golden.py <reference checkout> (or set VENU_REFERENCE_ROOT)")
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ["VENU_REFERENCE_ROOT"])
