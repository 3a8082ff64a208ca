"""Generates tests/golden/reference_test_scene.npz from the reference checkout.

The reference's own fixture scenes data/test-scene/test-scene.gltf and
test-scene-sky.gltf (980 triangles of one material, uint16 indices; six
cameras, two of them compound eyes reading data/test-scene/test.eye and
test100.eye) are read with the oracle's glTF loader (oracle/gltf_ref.py) and
stored flattened, so that tests can rebuild them where the checkout is absent:
per variant the world-space triangles, colour records, shading kinds and miss
shader, and per compound camera its name, pose (position, local x/y/z axes),
projection and ommatidium records.

Usage: python tests/golden/make_reference_scene.py /path/to/compound-ray-checkout
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
import gltf_ref  # noqa: E402


def main(ref_root):
    out = {}
    for variant, name in (("plain", "test-scene.gltf"), ("sky", "test-scene-sky.gltf")):
        ref = gltf_ref.load(os.path.join(ref_root, "data", "test-scene", name))
        v, c, f = ref.arrays()
        out[variant + "__verts"] = v
        out[variant + "__colours"] = c
        out[variant + "__flags"] = f
        out[variant + "__miss"] = np.array(ref.miss)
        cams = [cam for cam in ref.cameras if cam["kind"] == "compound"]
        out[variant + "__cams"] = np.array([cam["name"] for cam in cams])
        for k, cam in enumerate(cams):
            key = "%s__cam%d" % (variant, k)
            out[key + "__pose"] = np.concatenate([cam["position"], cam["ls"].reshape(-1)]).astype(np.float32)
            out[key + "__omm"] = cam["omm"].astype(np.float32)
            out[key + "__projection"] = np.array(cam["projection"])
    np.savez_compressed(os.path.join(HERE, "reference_test_scene.npz"), **out)
    print("wrote", sorted(out))


if __name__ == "__main__":
    if len(sys.argv) < 2 and not os.environ.get("CR_REFERENCE_ROOT"):
        sys.exit("usage: %s <reference checkout> (or set CR_REFERENCE_ROOT)" % sys.argv[0])
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ["CR_REFERENCE_ROOT"])
