"""The GPU renderer against the golden renders of the reference's fixture
scenes (see test_golden_renders.py): the same random draws and rays bit for
bit, the same closest hits, the per-ommatidium RGB within 1e-5 relative."""
import os

import numpy as np
import pytest

import eyeRendererHelperFunctions as eh
import scenes

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.mark.parametrize("variant", ["plain", "sky"])
def test_renderer_reproduces_golden_render(lib, tmp_path, variant):
    scene = np.load(os.path.join(GOLD, "reference_test_scene.npz"))
    rend = np.load(os.path.join(GOLD, "reference_test_renders.npz"))
    path = scenes.fixture_scene(scene, variant, str(tmp_path))
    for k, name in enumerate(scene[variant + "__cams"]):
        eh.lastError(lib)
        lib.loadGlTFscene(path.encode())
        assert lib.gotoCameraByName(str(name).encode())
        key = "%s__cam%d" % (variant, k)
        lib.setCurrentEyeSamplesPerOmmatidium(int(rend[key + "__spp"]))
        rec = eh.renderFrameRecorded(lib)
        assert eh.lastError(lib) == ""
        draws = np.stack([rec["normalDraw"], rec["uniformDraw"]], axis=-1)
        assert np.array_equal(draws, rend[key + "__draws"])
        assert np.array_equal(rec["origin"], rend[key + "__origin"])
        assert np.array_equal(rec["direction"], rend[key + "__direction"])
        assert np.array_equal(rec["hitId"], rend[key + "__hit"])
        want = rend[key + "__sums"]
        np.testing.assert_allclose(eh.getOmmatidialColours(lib), want, rtol=1e-5, atol=1e-7)
