"""Shared checks of the GPU parity tests: a recorded frame of the current
camera against the CPU oracle on the GPU's own rays.

Bars (the renderer's correctness contract):
  * hit triangle ids, hit distances and barycentrics: bit-exact against the
    oracle's float watertight search on the GPU's own rays;
  * disagreements with the independent double-precision search only for rays
    that pass within 1e-6 (barycentric) of a triangle edge;
  * ray generation from the same draws: within 2e-6 absolute per direction
    component (the GPU uses the fast sin/cos of the reference build);
  * per-ray shaded colour and per-ommatidium RGB: within 1e-5 relative
    (RTOL), with an absolute floor of 1e-7 for near-black channels, widened
    for sky-shaded rays by sky_tolerance: 1e-5 plus the miss shader's slope
    near the zenith times the y error of the fast-math normalisation (the
    reference build's fast normalise/asin against libm in the oracle).
"""
import numpy as np

import eyeRendererHelperFunctions as eh
import gltf_ref
import oracle

RTOL = 1e-5
ATOL = 1e-7
SKY_ATOL = 1e-5
DIR_ATOL = 2e-6
# simple_sky mixes two colours by m = asin(y) * 2 / pi of the normalised
# direction (shaders.cu:749-756); the colours differ by at most 0.45 per
# channel.  The GPU normalises and takes asin with the fast maths of the
# reference build, a few 1e-7 away from the oracle's libm in y, and
# d asin(y) / dy = 1 / sqrt(1 - y^2) magnifies that near the zenith, where
# asin moves by at most sqrt(2 dy) for a change dy of y.
SKY_DY = 4e-7


def sky_tolerance(dirs):
    """Per-ray bound for a sky-shaded sample: SKY_ATOL plus the miss shader's
    change for a y error of SKY_DY (the smaller of slope x SKY_DY and
    sqrt(2 SKY_DY))."""
    d = np.asarray(dirs, np.float64).reshape(-1, 3)
    y = d[:, 1] / np.maximum(np.linalg.norm(d, axis=1), 1e-30)
    dasin = np.minimum(SKY_DY / np.sqrt(np.maximum(1.0 - y * y, 1e-30)), np.sqrt(2.0 * SKY_DY))
    return SKY_ATOL + 0.45 * (2.0 / np.pi) * dasin


def _load(lib, path, spp):
    eh.lastError(lib)  # drop any message a previous test left behind
    lib.loadGlTFscene(path.encode())
    assert eh.lastError(lib) == ""
    eh.gotoFirstCompoundEye(lib)
    lib.setCurrentEyeSamplesPerOmmatidium(spp)


def _oracle(path):
    ref = gltf_ref.load(path)
    v, c, f = ref.arrays()
    cams = [c for c in ref.cameras if c["kind"] == "compound"]
    return ref, oracle.OracleScene(v, c, f, ref.miss), cams[0]["omm"]


def _check_frame(lib, sc, omm, spp, pose12):
    rec = eh.renderFrameRecorded(lib)
    N = len(omm)
    assert rec.shape == (N, spp)
    org = rec["origin"].reshape(-1, 3)
    dirs = rec["direction"].reshape(-1, 3)
    tmin = np.repeat(omm[:, 7], spp)

    # Ray generation from the GPU's own draws.
    draws = np.stack([rec["normalDraw"].reshape(-1), rec["uniformDraw"].reshape(-1)], axis=1)
    o2, d2 = oracle.gen_rays(omm, spp, pose12, draws)
    np.testing.assert_allclose(d2, dirs, rtol=0, atol=DIR_ATOL)
    np.testing.assert_allclose(o2, org, rtol=1e-6, atol=1e-7)

    # Closest hits on identical rays: bit-exact.
    hit, t, b1, b2 = sc.trace(org, dirs, tmin)
    gh = rec["hitId"].reshape(-1)
    assert np.array_equal(hit, gh), "hit ids differ on %d of %d rays" % ((hit != gh).sum(), len(gh))
    m = hit >= 0
    assert np.array_equal(t[m].view(np.uint32), rec["t"].reshape(-1)[m].view(np.uint32))
    assert np.array_equal(b1[m].view(np.uint32), rec["b1"].reshape(-1)[m].view(np.uint32))
    assert np.array_equal(b2[m].view(np.uint32), rec["b2"].reshape(-1)[m].view(np.uint32))

    # Independent double-precision search: only near-edge rays may differ.
    h64, t64, e32, e64 = sc.trace_f64(org, dirs, tmin, hit32=hit)
    diff = hit != h64
    near = (e32 < 1e-6) | (e64 < 1e-6)
    assert not (diff & ~near).any(), "fp32/fp64 disagree away from edges on %d rays" % (diff & ~near).sum()

    # Shading of the same hits.
    rgb = sc.shade(dirs, hit, b1, b2)
    miss = (hit < 0)[:, None]
    err = np.abs(rec["rgb"].reshape(-1, 3) - rgb)
    sky_tol = sky_tolerance(dirs)[:, None]
    assert (err <= RTOL * np.abs(rgb) + np.where(miss, sky_tol, ATOL)).all(), "per-ray colour max err %.3g" % err.max()

    # Per-ommatidium sums.
    got = eh.getOmmatidialColours(lib)
    want = sc.render_rays(omm, spp, org, dirs)[0]
    sky_bound = np.where(miss[:, 0], sky_tol[:, 0], 0.0).reshape(N, spp).mean(axis=1)[:, None]
    err = np.abs(got - want)
    tol = RTOL * np.abs(want) + ATOL + sky_bound
    assert (err <= tol).all(), "per-ommatidium colour: %d channels out of tolerance, max err %.3g" % (
        (err > tol).sum(), err.max())
    return rec, got
