"""Generates tests/golden/reference_eyes.npz from the reference checkout.

Pins the .eye format against the reference's own Python reader: every .eye
file under data/ is read with python-examples/eyeRendererHelperFunctions.py's
readEyeFile (the reference code, imported from the checkout) and stored as
its row count, the first 32 records (float64, as that reader produces) and
the float64 sum of all values.  The reference's getIcoOmmatidia() (12
ommatidia on an icosahedron) is stored too; the GPU tests feed it through
setOmmatidia.

Usage: python tests/golden/make_golden.py /path/to/compound-ray-checkout
"""
import glob
import importlib.util
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref_root):
    spec = importlib.util.spec_from_file_location(
        "ref_helpers", os.path.join(ref_root, "python-examples", "eyeRendererHelperFunctions.py"))
    ref = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(ref)
    out = {}
    files = sorted(glob.glob(os.path.join(ref_root, "data", "eyes", "*.eye")) +
                   glob.glob(os.path.join(ref_root, "data", "test-scene", "*.eye")))
    names = []
    for path in files:
        rel = os.path.relpath(path, ref_root)
        omms = ref.readEyeFile(path)
        arr = np.array([list(o.position) + list(o.direction) + [o.acceptanceAngle, o.focalpointOffset] for o in omms],
                       np.float64)
        key = rel.replace("/", "__").replace("-", "_").replace(".", "_")
        names.append(rel)
        out[key + "__count"] = np.array(len(arr))
        out[key + "__head"] = arr[:32]
        out[key + "__sum"] = np.array(arr.sum(dtype=np.float64))
    ico = ref.getIcoOmmatidia()
    out["ico"] = np.array([list(o.position) + list(o.direction) + [o.acceptanceAngle, o.focalpointOffset] for o in ico],
                          np.float64)
    out["files"] = np.array(names)
    np.savez_compressed(os.path.join(HERE, "reference_eyes.npz"), **out)
    print("wrote", len(names), "eye files")


if __name__ == "__main__":
    if len(sys.argv) < 2 and not os.environ.get("CR_REFERENCE_ROOT"):
        sys.exit("usage: %s <reference checkout> (or set CR_REFERENCE_ROOT)" % sys.argv[0])
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ["CR_REFERENCE_ROOT"])
