"""The oracle against golden renders of the reference's own fixture scenes
(data/test-scene/test-scene{,-sky}.gltf with test.eye and test100.eye,
stored flattened in tests/golden/reference_test_scene.npz by
make_reference_scene.py; first frames recorded on a GB300 by
make_reference_renders.py into reference_test_renders.npz).  CPU only: the
oracle regenerates every ray from the stored draws, finds the stored closest
hits bit for bit on the stored rays, and sums the stored per-ommatidium RGB."""
import os

import numpy as np
import pytest

import oracle

GOLD = os.path.join(os.path.dirname(__file__), "golden")
RTOL, ATOL, SKY_ATOL, DIR_ATOL = 1e-5, 1e-7, 1e-5, 2e-6

CASES = [(v, k) for v in ("plain", "sky") for k in (0, 1)]


@pytest.fixture(scope="module")
def gold():
    return np.load(os.path.join(GOLD, "reference_test_scene.npz")), np.load(os.path.join(GOLD, "reference_test_renders.npz"))


@pytest.mark.parametrize("variant,cam", CASES)
def test_oracle_reproduces_golden_render(gold, variant, cam):
    scene, rend = gold
    sc = oracle.OracleScene(scene[variant + "__verts"], scene[variant + "__colours"], scene[variant + "__flags"],
                            int(scene[variant + "__miss"]))
    key = "%s__cam%d" % (variant, cam)
    omm = scene[key + "__omm"]
    pose = scene[key + "__pose"]
    spp = int(rend[key + "__spp"])
    N = len(omm)
    draws = rend[key + "__draws"].reshape(-1, 2)
    org = rend[key + "__origin"].reshape(-1, 3)
    dirs = rend[key + "__direction"].reshape(-1, 3)
    assert draws.shape == (N * spp, 2)
    # ray generation from the stored draws
    o2, d2 = oracle.gen_rays(omm, spp, pose, draws)
    np.testing.assert_allclose(d2, dirs, rtol=0, atol=DIR_ATOL)
    # origins are sums of terms as large as the camera position and the
    # ommatidium offsets: fused vs separate multiply-adds differ by ulps of those
    scale = np.abs(pose[:3]).max() + np.abs(omm[:, :3]).max() + 1.0
    np.testing.assert_allclose(o2, org, rtol=0, atol=1e-6 * scale)
    # closest hits on the stored rays, bit for bit
    hit, t, b1, b2 = sc.trace(org, dirs, np.repeat(omm[:, 7], spp))
    gh = rend[key + "__hit"].reshape(-1)
    assert np.array_equal(hit, gh)
    assert (gh >= 0).any() and (gh < 0).any()
    # per-ommatidium sums of the stored rays
    want = rend[key + "__sums"]
    got = sc.render_rays(omm, spp, org, dirs)[0]
    sky = (gh < 0).reshape(N, spp).mean(axis=1)[:, None]
    assert (np.abs(got - want) <= RTOL * np.abs(want) + ATOL + SKY_ATOL * sky).all()
