"""Spherical projections through the candidate grids against the exhaustive
search in index order (the reference's shaders.cu:412-640 loop): the same
image, pixel for pixel, for every spherical kind, including ties between
identical ommatidia, vectors of zero length, positions with x = +-0 for the
split projection and an ommatidium 0 whose angle is NaN."""
import ctypes

import numpy as np
import pytest

import eyeRendererHelperFunctions as eh
import scenes

pytestmark = pytest.mark.gpu

KINDS = ["spherical_positionwise", "spherical_orientationwise", "spherical_split_orientationwise",
         "spherical_orientationwise_ids", "spherical_positionwise_ids"]


def _set_ommatidia(lib, omm):
    """omm: (n, 8) float32 records (position, direction, acceptance, focal offset)."""
    omm = np.ascontiguousarray(omm, np.float32)
    lib.setOmmatidia.argtypes = [ctypes.c_void_p, ctypes.c_size_t]
    lib.setOmmatidia(omm.ctypes.data, len(omm))
    assert eh.lastError(lib) == ""


def _both(lib, kind, w, h):
    """The frame with each search; the eye's random streams restart before
    each render (a sample-count change resets them), so both frames project
    the same ommatidium colours."""
    frames = []
    lib.setCurrentEyeShaderName(kind.encode())
    eh.setRenderSize(lib, w, h)
    spp = lib.getCurrentEyeSamplesPerOmmatidium()
    try:
        for mode in (1, 0):
            assert lib.crSetProjectionSearch(mode) == 0
            lib.setCurrentEyeSamplesPerOmmatidium(spp + 1)
            lib.setCurrentEyeSamplesPerOmmatidium(spp)
            assert lib.renderFrame() >= 0, eh.lastError(lib)
            frames.append(eh.getFrame(lib, w, h).copy())
    finally:
        lib.crSetProjectionSearch(0)
    return frames


def _eye(rng, n, ties=0, zeros=0, xzero=0):
    d = rng.normal(size=(n, 3))
    pos = rng.normal(size=(n, 3)) * rng.uniform(1e-3, 2.0, size=(n, 1))
    if ties:
        src = rng.integers(0, n, size=ties)
        dst = rng.integers(0, n, size=ties)
        d[dst], pos[dst] = d[src], pos[src]
    if zeros:
        d[rng.integers(1, n, size=zeros)] = 0.0
        pos[rng.integers(1, n, size=zeros)] = 0.0
    if xzero:
        pos[rng.integers(1, n, size=xzero), 0] = 0.0
        pos[rng.integers(1, n, size=xzero), 0] = -0.0
    out = np.zeros((n, 8), np.float32)
    out[:, 0:3], out[:, 3:6], out[:, 6] = pos, d, 0.05
    return out


@pytest.mark.parametrize("kind", KINDS)
def test_grid_search_equals_exhaustive_small_eye(lib, small, kind):
    eh.lastError(lib)
    lib.loadGlTFscene(small["gltf"].encode())
    eh.gotoFirstCompoundEye(lib)
    lib.setCurrentEyeSamplesPerOmmatidium(8)
    a, b = _both(lib, kind, 160, 80)
    assert np.array_equal(a, b)
    assert len(np.unique(a.reshape(-1, 4), axis=0)) > 50


@pytest.mark.parametrize("kind", KINDS)
def test_grid_search_equals_exhaustive_awkward_eyes(lib, small, kind):
    eh.lastError(lib)
    lib.loadGlTFscene(small["gltf"].encode())
    eh.gotoFirstCompoundEye(lib)
    lib.setCurrentEyeSamplesPerOmmatidium(4)
    rng = np.random.default_rng(5)
    # ties, zero vectors, x = +-0 positions
    _set_ommatidia(lib, _eye(rng, 5000, ties=400, zeros=50, xzero=40))
    a, b = _both(lib, kind, 128, 64)
    assert np.array_equal(a, b)
    # a few ommatidia only: one grid cell
    _set_ommatidia(lib, _eye(rng, 7))
    a, b = _both(lib, kind, 64, 32)
    assert np.array_equal(a, b)
    # ommatidium 0 of zero length: its angle is NaN and every pixel keeps it
    e = _eye(rng, 300)
    e[0, 0:6] = 0.0
    _set_ommatidia(lib, e)
    a, b = _both(lib, kind, 64, 32)
    assert np.array_equal(a, b)
    if kind.endswith("_ids"):
        assert (a == 0).all()


def test_grid_search_equals_exhaustive_large_eye(lib, small):
    eh.lastError(lib)
    lib.loadGlTFscene(small["gltf"].encode())
    eh.gotoFirstCompoundEye(lib)
    lib.setCurrentEyeSamplesPerOmmatidium(1)
    rng = np.random.default_rng(9)
    d = scenes.fibonacci_sphere(60000) + rng.normal(scale=1e-3, size=(60000, 3))
    e = np.zeros((60000, 8), np.float32)
    e[:, 0:3], e[:, 3:6], e[:, 6] = d * 0.001, d, 0.01
    _set_ommatidia(lib, e)
    for kind in ("spherical_orientationwise_ids", "spherical_split_orientationwise"):
        a, b = _both(lib, kind, 256, 128)
        assert np.array_equal(a, b)
