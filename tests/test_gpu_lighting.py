"""The lighting-on closest-hit path (GGX/Smith with four point lights and
shadow rays) against the oracle on the GPU's own rays: hits bit for bit,
shadow decisions exactly (a flipped one would show as a whole light's
contribution), colours within LIT_RTOL; and the guards of the paths that
render with lighting off only."""
import numpy as np
import pytest

import eyeRendererHelperFunctions as eh
import gltf_ref
import oracle
import scenes
from test_gpu_parity import _load

pytestmark = pytest.mark.gpu

# The lit colour goes through powf, sqrtf and divisions that the reference
# build takes from fast-math intrinsics and the oracle from libm, on values
# of up to ~10 before the 1/spp scaling.
LIT_RTOL = 2e-4
LIT_ATOL = 2e-5


def test_lit_scene_matches_oracle(lib, tmp_path):
    info = scenes.lit_scene(str(tmp_path))
    ref = gltf_ref.load(info["gltf"])
    v, c, f = ref.arrays()
    sc = oracle.OracleScene(v, c, f, ref.miss, textures=ref.textures())
    light, pos, col = ref.lighting()
    sc.set_lighting(light, pos, col)
    omm = [cam for cam in ref.cameras if cam["kind"] == "compound"][0]["omm"]
    assert lib.crSetLighting(1) == 0
    try:
        _load(lib, info["gltf"], 16)
        for pose_args in ((0.0, 0.5, 0.0, 0.0, 0.0, 0.0), (2.0, 1.2, -1.5, 0.1, 0.8, 0.0)):
            lib.setCameraPose(*pose_args)
            rec = eh.renderFrameRecorded(lib)
            assert eh.lastError(lib) == ""
            org, dirs = rec["origin"].reshape(-1, 3), rec["direction"].reshape(-1, 3)
            hit, t, b1, b2 = sc.trace(org, dirs, np.repeat(omm[:, 7], 16))
            assert np.array_equal(hit, rec["hitId"].reshape(-1))
            want = sc.shade(dirs, hit, b1, b2)
            got = rec["rgb"].reshape(-1, 3)
            sky = (hit < 0)[:, None]
            err = np.abs(got - want)
            tol = LIT_RTOL * np.abs(want) + np.where(sky, 1e-5, LIT_ATOL)
            assert (err <= tol).all(), "lit colour: %d of %d rays out, max err %.3g" % ((err > tol).any(axis=1).sum(),
                                                                                    len(err), err.max())
            assert (want[~sky[:, 0]] > 0).any()  # something is lit
            sums = eh.getOmmatidialColours(lib)
            wsum = sc.render_rays(omm, 16, org, dirs)[0]
            assert np.allclose(sums, wsum, rtol=LIT_RTOL, atol=LIT_ATOL + 1e-5)
        # the learned and batched paths refuse to run lit
        assert lib.crDenoiserInit(1) == 0
        poses = np.stack([info["pose"]]).astype(np.float32)
        assert lib.crDenoiserAddTrainingPoses(poses, 1, 8, 16) == -1
        assert "lighting" in eh.lastError(lib)
    finally:
        lib.crSetLighting(0)
    # lighting off again: the plain shading
    _load(lib, info["gltf"], 16)
    rec = eh.renderFrameRecorded(lib)
    sc2 = oracle.OracleScene(v, c, f, ref.miss, textures=ref.textures())
    org, dirs = rec["origin"].reshape(-1, 3), rec["direction"].reshape(-1, 3)
    hit, t, b1, b2 = sc2.trace(org, dirs, np.repeat(omm[:, 7], 16))
    want = sc2.shade(dirs, hit, b1, b2)
    err = np.abs(rec["rgb"].reshape(-1, 3) - want)
    assert (err <= 1e-5 * np.abs(want) + np.where((hit < 0)[:, None], 1e-5, 1e-7)).all()
