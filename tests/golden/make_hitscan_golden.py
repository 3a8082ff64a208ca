"""Writes tests/golden/reference_hitscan.npz: the reference's own answers to
isInsideHitGeometry on the hitbox fixture scene (scenes.hitbox_scene).

The answers come from the reference's sutil/hitscanprocessing.cpp
(isPointWithinMesh), compiled unchanged by oracle/build_ref.py into
oracle/_ref/libref_hitscan.so and called on each hitbox's object-space
triangles and node transform (rounded to float, as the reference stores it)
for the points of scenes.hitbox_points().  Build the library first:

  python oracle/build_ref.py [checkout]
  python tests/golden/make_hitscan_golden.py
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "compound-ray_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import gltf_ref  # noqa: E402
import oracle  # noqa: E402
import scenes  # noqa: E402


def reference_answers():
    with tempfile.TemporaryDirectory() as tmp:
        ref = gltf_ref.load(scenes.hitbox_scene(os.path.join(tmp, "hitbox.gltf")))
    pts = scenes.hitbox_points()
    out = {"points": pts}
    for hb in ref.hitbox_meshes:
        xf = hb["xform"].astype(np.float32)
        out[hb["name"] + "__xform"] = xf
        out[hb["name"] + "__inside"] = oracle.ref_points_in_mesh(hb["tris"], xf, pts)
    return out


def main():
    out = reference_answers()
    np.savez_compressed(os.path.join(HERE, "reference_hitscan.npz"), **out)
    print("wrote", sorted(out))


if __name__ == "__main__":
    main()
