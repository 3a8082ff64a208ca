"""Base colour textures on the GPU: the render kernel's bilinear filter
against the oracle (bit for bit) and against the CUDA texture unit in the
reference's sampler state; a textured scene rendered and checked ray by ray
against the oracle on the GPU's own rays."""
import numpy as np
import pytest

import eyeRendererHelperFunctions as eh
import gltf_ref
import oracle
import scenes
from test_gpu_parity import _check_frame, _load

pytestmark = pytest.mark.gpu

# The texture unit filters with 8-bit fractional weights; the renderer's
# filter restates that rule (axis weights rounded half up, corner weights
# rounded to 1/256).  It matches the unit exactly up to 2^-16 on most
# lookups; about 1% of two-axis lookups land one weight step (at most two
# 8-bit levels) away where the unit rounds a corner weight the other way.
HW_ATOL = 2.0 / 255.0
HW_MEAN_ATOL = 1e-4


def test_filter_against_oracle_and_texture_unit(lib):
    rng = np.random.default_rng(17)
    w, h = 37, 23
    img = rng.integers(0, 256, size=(h, w, 4), dtype=np.uint8)
    words = scenes.rgba_words(img)
    uv = np.concatenate([
        rng.uniform(-3, 3, size=(20000, 2)),
        # texel centres, edges, exact integers, tiny negatives, large values
        np.stack(np.meshgrid((np.arange(w) + 0.5) / w, (np.arange(h) + 0.5) / h), axis=-1).reshape(-1, 2),
        [[0, 0], [1, 1], [-1e-9, 1 - 1e-9], [1e-9, -1e-9], [100.25, -100.75], [0.5, 0.5]],
    ]).astype(np.float32)
    soft, hard = eh.compareTextureSampling(lib, words, w, h, uv)
    want = oracle.sample_texture(words, w, h, uv)
    assert np.array_equal(soft.view(np.uint32), want.view(np.uint32))
    err = np.abs(soft - hard)
    assert err.max() <= HW_ATOL, "renderer vs texture unit: max %.4g, mean %.4g" % (err.max(), err.mean())
    assert err.mean() <= HW_MEAN_ATOL, "renderer vs texture unit: mean %.4g" % err.mean()


def test_textured_scene_matches_oracle(lib, tmp_path):
    info = scenes.textured_scene(str(tmp_path))
    ref = gltf_ref.load(info["gltf"])
    v, c, f = ref.arrays()
    sc = oracle.OracleScene(v, c, f, ref.miss, textures=ref.textures())
    omm = [cam for cam in ref.cameras if cam["kind"] == "compound"][0]["omm"]
    _load(lib, info["gltf"], 32)
    lib.setCameraPose(0.0, 0.5, 0.0, 0.0, 0.0, 0.0)
    rec, _ = _check_frame(lib, sc, omm, 32, info["pose"])
    hit = rec["hitId"].reshape(-1)
    kinds = np.bincount(f[hit[hit >= 0]], minlength=3)
    assert (kinds > 0).all(), "every shading kind seen: %s" % kinds.tolist()
    # a second frame from another pose
    lib.setCameraPose(1.5, 0.9, -2.0, 0.0, 1.0, 0.0)
    ls = np.zeros(9, np.float32)
    lib.crGetCameraLocalSpace(ls)
    _check_frame(lib, sc, omm, 32, np.concatenate([eh.getCameraPosition(lib), ls]).astype(np.float32))
