"""Generates tests/golden/reference_test_renders.npz on a GPU.

Renders the reference's fixture scenes (rebuilt from reference_test_scene.npz
by scenes.fixture_scene) from each compound camera's own pose: insect-cam-1
(1000 ommatidia, test.eye) at 8 samples and insect-cam-2 (100 ommatidia,
test100.eye) at 32 samples, one recorded first frame each.  Stores per
(variant, camera) the random draws of every ray, the closest-hit triangle
ids, the rays themselves and the per-ommatidium RGB sums.  The CPU tests
replay the draws and rays through the oracle; the GPU tests re-render and
compare.

Usage (on a machine with the GPU and the built library):
    python tests/golden/make_reference_renders.py [out.npz]
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.join(HERE, "..", "..")
sys.path[:0] = [os.path.join(ROOT, "compound-ray_gb300"), os.path.join(ROOT, "oracle")]
import eyeRendererHelperFunctions as eh  # noqa: E402
import scenes  # noqa: E402

SPP = {1000: 8, 100: 32}


def render_all(lib, z, workdir):
    out = {}
    for variant in ("plain", "sky"):
        path = scenes.fixture_scene(z, variant, os.path.join(workdir, variant))
        for k, name in enumerate(z[variant + "__cams"]):
            eh.lastError(lib)
            lib.loadGlTFscene(path.encode())  # fresh streams for every camera
            if not lib.gotoCameraByName(str(name).encode()):
                raise RuntimeError("camera %s missing" % name)
            n = lib.getCurrentEyeOmmatidialCount()
            spp = SPP[n]
            lib.setCurrentEyeSamplesPerOmmatidium(spp)
            rec = eh.renderFrameRecorded(lib)
            err = eh.lastError(lib)
            if err:
                raise RuntimeError(err)
            key = "%s__cam%d" % (variant, k)
            out[key + "__spp"] = np.array(spp)
            out[key + "__draws"] = np.stack([rec["normalDraw"], rec["uniformDraw"]], axis=-1).astype(np.float32)
            out[key + "__origin"] = rec["origin"].astype(np.float32)
            out[key + "__direction"] = rec["direction"].astype(np.float32)
            out[key + "__hit"] = rec["hitId"].astype(np.int32)
            out[key + "__sums"] = eh.getOmmatidialColours(lib).astype(np.float32)
    return out


def main(dst):
    lib = eh.loadRenderer()
    lib.setVerbosity(False)
    z = np.load(os.path.join(HERE, "reference_test_scene.npz"))
    with tempfile.TemporaryDirectory() as d:
        out = render_all(lib, z, d)
    np.savez_compressed(dst, **out)
    print("wrote", dst)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(HERE, "reference_test_renders.npz"))
