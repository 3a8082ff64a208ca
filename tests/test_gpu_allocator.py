"""The learned sample allocator and the adaptive render: the adaptive kernel
(stratified Sobol'-net samples) against the oracle ray by ray; its estimates against the
plain render; minimum-sample labels; a trained allocator's adaptive render
against the 1024-sample plain render (error and rays); determinism and the
checkpoint round trip."""
import numpy as np
import pytest
import torch

import allocator_ref
import eyeRendererHelperFunctions as eh
import gltf_ref
import oracle
import scenes

pytestmark = pytest.mark.gpu

RTOL, ATOL, SKY_ATOL, DIR_ATOL = 1e-5, 1e-7, 1e-5, 2e-6


def _terrain(lib, tmp_path):
    info = scenes.terrain_scene(str(tmp_path), cells=128, extent=60.0, cones=300, n_omm=1500, poses=8)
    eh.lastError(lib)
    lib.loadGlTFscene(info["gltf"].encode())
    assert eh.lastError(lib) == ""
    eh.gotoFirstCompoundEye(lib)
    return info


def test_adaptive_kernel_matches_oracle(lib, small, small_ref):
    ref, sc = small_ref
    omm = ref.cameras[0]["omm"]
    eh.lastError(lib)
    lib.loadGlTFscene(small["gltf"].encode())
    eh.gotoFirstCompoundEye(lib)
    N, spp = len(omm), 64
    poses = np.stack([small["pose"], scenes.pose_rows(np.array([1.0, 0.7, -2.0]), 0.8)]).astype(np.float32)
    rec = np.zeros((2 * N * spp,), eh.RAY_RECORD_DTYPE)
    sums = np.zeros((2, N, 3), np.float32)
    assert lib.crAdaptiveRecord(poses, 2, spp, 7, rec.ctypes.data, sums) == 0, eh.lastError(lib)
    rec = rec.reshape(2, N * spp)
    # The draws: sample s of entry e is point s of the entry's digitally
    # shifted Sobol' net (seed 7), as oracle.net_draws restates it.
    nd, ud = oracle.net_draws(7, np.repeat(np.arange(2 * N), spp), np.tile(np.arange(spp), 2 * N))
    assert np.array_equal(rec["uniformDraw"].reshape(-1), ud)
    got = rec["normalDraw"].reshape(-1).astype(np.float64)
    # normcdfinvf under fast maths: close to float64 in the body of the
    # distribution, a few 1e-3 off far in the tails (its logarithm is the
    # fast approximation)
    body = np.abs(nd) < 3.0
    assert (np.abs(got - nd)[body] <= 4e-6 * np.maximum(1.0, np.abs(nd[body]))).all(), np.abs(got - nd)[body].max()
    assert np.abs(got - nd).max() <= 5e-3
    for p in range(2):
        r = rec[p]
        draws = np.stack([r["normalDraw"], r["uniformDraw"]], axis=1)
        o2, d2 = oracle.gen_rays(omm, spp, poses[p], draws)
        np.testing.assert_allclose(d2, r["direction"].reshape(-1, 3), rtol=0, atol=DIR_ATOL)
        org, dirs = r["origin"].reshape(-1, 3), r["direction"].reshape(-1, 3)
        hit, t, b1, b2 = sc.trace(org, dirs, np.repeat(omm[:, 7], spp))
        assert np.array_equal(hit, r["hitId"])
        want = sc.render_rays(omm, spp, org, dirs)[0]
        sky = (hit < 0).reshape(N, spp).mean(axis=1)[:, None]
        assert (np.abs(sums[p] - want) <= RTOL * np.abs(want) + ATOL + SKY_ATOL * sky).all()
    # the near-field cut changes no hit and no sum
    assert lib.crSetCutRadius(1.0 / 64) == 0
    try:
        rec2 = np.zeros_like(rec.reshape(-1))
        sums2 = np.zeros_like(sums)
        assert lib.crAdaptiveRecord(poses, 2, spp, 7, rec2.ctypes.data, sums2) == 0, eh.lastError(lib)
    finally:
        lib.crSetCutRadius(0.0)
    assert np.array_equal(rec2["hitId"], rec.reshape(-1)["hitId"])
    assert np.array_equal(sums2, sums)
    # neither do the kernel's occupancy (register budget) and refill schedule
    try:
        for blocks, sched in ((6, (16, 8)), (8, (32, 32))):
            assert lib.crSetAdaptiveOccupancy(blocks) == 0 and lib.crSetAdaptiveSchedule(*sched) == 0
            sums3 = np.zeros_like(sums)
            assert lib.crAdaptiveRecord(poses, 2, spp, 7, rec2.ctypes.data, sums3) == 0, eh.lastError(lib)
            assert np.array_equal(sums3, sums), blocks
    finally:
        lib.crSetAdaptiveOccupancy(5)
        lib.crSetAdaptiveSchedule(16, 16)
    assert lib.crSetAdaptiveOccupancy(7) == -1
    # normal / uniform draws look like N(0,1) / U(0,1], and each entry's 64
    # samples are stratified: one per 1/64 of the normal draw's distribution
    nd, ud = rec["normalDraw"].ravel(), rec["uniformDraw"].ravel()
    assert abs(nd.mean()) < 0.02 and abs(nd.std() - 1) < 0.02
    assert ud.min() > 0 and ud.max() <= 1 and abs(ud.mean() - 0.5) < 0.01
    from statistics import NormalDist
    cdf = np.vectorize(NormalDist().cdf)
    cells = np.floor(cdf(nd[:4 * spp].astype(np.float64)) * spp).astype(np.int64).reshape(4, spp)
    assert all(len(set(c.tolist())) == spp for c in cells)


def test_adaptive_estimate_matches_plain_render(lib, tmp_path):
    info = _terrain(lib, tmp_path)
    rng = np.random.default_rng(4)
    poses = scenes.random_poses(info["height_fn"], 3, rng, 20.0)
    n = lib.getCurrentEyeOmmatidialCount()
    rec = np.zeros((3 * n * 256,), eh.RAY_RECORD_DTYPE)
    a256 = np.zeros((3, n, 3), np.float32)
    assert lib.crAdaptiveRecord(poses, 3, 256, 11, rec.ctypes.data, a256) == 0, eh.lastError(lib)
    lib.setCurrentEyeSamplesPerOmmatidium(1024)
    p1024 = eh.renderPoses(lib, poses)
    lib.setCurrentEyeSamplesPerOmmatidium(32)
    p32 = eh.renderPoses(lib, poses)
    rmse = lambda a: float(np.sqrt(((a - p1024) ** 2).mean()))
    # 256 Philox samples sit between 32 and 1024 XORWOW samples
    assert rmse(a256) < 0.6 * rmse(p32), (rmse(a256), rmse(p32))


def test_allocator_labels_training_and_adaptive_render(lib, tmp_path):
    info = _terrain(lib, tmp_path)
    n = lib.getCurrentEyeOmmatidialCount()
    rng = np.random.default_rng(9)
    train = scenes.random_poses(info["height_fn"], 24, rng, 20.0)
    held = scenes.random_poses(info["height_fn"], 4, rng, 20.0)
    lib.crDenoiserRelease()  # no denoiser: entries the feature render covers keep its mean
    assert lib.crAllocatorInit(2) == 0
    thr = 1.0 / 512.0
    labels = np.zeros((24, n), np.uint16)
    for k in range(0, 24, 8):
        lab = np.zeros((8, n), np.uint16)
        assert lib.crAllocatorAddTrainingPoses(train[k:k + 8], 8, 8, thr, 8, lab.ctypes.data) == 0, eh.lastError(lib)
        labels[k:k + 8] = lab
    assert lib.crAllocatorTrainingRows() == 24 * n
    vals = set(np.unique(labels).tolist())
    assert vals <= {0, 4, 8, 16, 32, 64, 128, 256, 512, 1024}
    assert len(vals) >= 4  # the scene needs different counts in different places
    # labels follow the per-ommatidium sample spread: plain 8-sample std of
    # ommatidia labelled 4 or 8 is below that of ommatidia labelled >= 256
    lib.setCurrentEyeSamplesPerOmmatidium(8)
    # the spread proxy: |8-sample render - 1024-sample render|
    p8 = eh.renderPoses(lib, train[:8])
    lib.setCurrentEyeSamplesPerOmmatidium(1024)
    p1k = eh.renderPoses(lib, train[:8])
    err = np.abs(p8 - p1k).max(axis=2)
    lo, hi = labels[:8] <= 8, (labels[:8] >= 256) | (labels[:8] == 0)
    if lo.any() and hi.any():
        assert err[lo].mean() < err[hi].mean()
    loss = np.zeros(1500, np.float32)
    assert lib.crAllocatorTrain(1500, 4096, 1e-3, 5, loss.ctypes.data) == 0, eh.lastError(lib)
    assert loss[-50:].mean() < 0.5 * loss[:20].mean()

    dev = torch.device("cuda", torch.cuda.current_device())
    p16 = np.zeros((4, 16), np.float32)
    for k in range(4):
        p16[:, 4 * k:4 * k + 3] = held[:, 3 * k:3 * k + 3]
    d_poses = torch.from_numpy(p16).to(dev)
    out = torch.zeros((4, n, 3), dtype=torch.float32, device=dev)
    lev = torch.zeros((4, n), dtype=torch.uint8, device=dev)
    rays = eh.c_double(0.0)
    assert lib.crAdaptiveRenderPosesDevice(d_poses.data_ptr(), 4, 8, out.data_ptr(), lev.data_ptr(),
                                           eh.ctypes.byref(rays)) == 0, eh.lastError(lib)
    torch.cuda.synchronize()
    adaptive = out.cpu().numpy()
    levels = lev.cpu().numpy().astype(np.int64)
    assert set(np.unique(levels).tolist()) <= set(range(9)) | {0x88, 0xFF}
    spp_of = np.where(levels == 0xFF, 0, np.where(levels == 0x88, 1024, 4 << (levels & 0x7F)))
    assert abs(rays.value - (4 * n * 8 + spp_of.sum())) < 0.5
    assert rays.value < 0.5 * 4 * n * 1024  # far fewer rays than the plain 1024-sample render
    lib.setCurrentEyeSamplesPerOmmatidium(1024)
    plain = eh.renderPoses(lib, held)
    rmse = float(np.sqrt(((adaptive - plain) ** 2).mean()))
    print("labels", {int(v): int((labels == v).sum()) for v in np.unique(labels)},
          "levels", {int(v): int((levels == v).sum()) for v in np.unique(levels)},
          "rays/plain1024 %.4f rmse %.6f" % (rays.value / (4 * n * 1024), rmse))
    assert rmse <= 1.0 / 255.0, rmse

    # determinism: reloading restarts the feature and adaptive streams
    path = str(tmp_path / "alloc.bin")
    assert lib.crAllocatorSave(path.encode()) == 0
    assert lib.crAllocatorInit(77) == 0
    assert lib.crAllocatorLoad(path.encode()) == 0
    again = []
    for _ in range(2):
        lib.loadGlTFscene(info["gltf"].encode())
        eh.gotoFirstCompoundEye(lib)
        o2 = torch.zeros_like(out)
        assert lib.crAdaptiveRenderPosesDevice(d_poses.data_ptr(), 4, 8, o2.data_ptr(), None, None) == 0
        torch.cuda.synchronize()
        again.append(o2.cpu().numpy())
    assert np.array_equal(again[0], again[1])

    # the error budget: one halving moves every entry down one bucket (from
    # the same restarted streams); a fallback entry joins the 1024 bucket
    lv, rs = [], []
    try:
        for h in (0, 1):
            lib.loadGlTFscene(info["gltf"].encode())
            eh.gotoFirstCompoundEye(lib)
            assert lib.crSetAllocatorHalvings(h) == 0 and lib.crGetAllocatorHalvings() == h
            o2 = torch.zeros_like(out)
            l2 = torch.zeros_like(lev)
            r2 = eh.c_double(0.0)
            assert lib.crAdaptiveRenderPosesDevice(d_poses.data_ptr(), 4, 8, o2.data_ptr(), l2.data_ptr(),
                                                   eh.ctypes.byref(r2)) == 0, eh.lastError(lib)
            torch.cuda.synchronize()
            lv.append(l2.cpu().numpy().astype(np.int64))
            rs.append(r2.value)
    finally:
        lib.crSetAllocatorHalvings(0)
    k0 = np.where(lv[0] == 0xFF, 3, np.where(lv[0] == 0x88, 11, (lv[0] & 0x7F) + 2))
    k1 = np.maximum(k0 - 1, 2)
    assert np.array_equal(lv[1], np.where(k1 <= 3, 0xFF, k1 - 2))
    assert rs[1] < rs[0]
    assert lib.crSetAllocatorHalvings(6.5) == -1
    assert "[-4, 6]" in eh.lastError(lib)

    # the allocation exponent: at 1/2 every entry's count exponent is half of
    # its exponent-1 value, rounded up (within the rounding of the prediction)
    try:
        lib.loadGlTFscene(info["gltf"].encode())
        eh.gotoFirstCompoundEye(lib)
        assert lib.crSetAllocatorExponent(0.5) == 0 and lib.crGetAllocatorExponent() == 0.5
        l3 = torch.zeros_like(lev)
        assert lib.crAdaptiveRenderPosesDevice(d_poses.data_ptr(), 4, 8, torch.zeros_like(out).data_ptr(),
                                               l3.data_ptr(), None) == 0, eh.lastError(lib)
        torch.cuda.synchronize()
    finally:
        lib.crSetAllocatorExponent(1.0)
    lv3 = l3.cpu().numpy().astype(np.int64)
    k3 = np.where(lv3 == 0xFF, 3, np.where(lv3 == 0x88, 11, (lv3 & 0x7F) + 2))
    lo = np.maximum(k0 // 2, 2)        # ceil((k0 - 1) / 2)
    hi = np.maximum((k0 + 1) // 2, 2)  # ceil(k0 / 2)
    feature_only = lv3 == 0xFF         # count <= 8 = the feature render's: exponent <= 3
    ok = np.where(feature_only, lo <= 3, (k3 >= lo) & (k3 <= hi))
    assert ok.all(), (k0[~ok][:10], lv3[~ok][:10])
    assert lib.crSetAllocatorExponent(0.1) == -1

    # Entry by entry against the numpy restatement of the allocation, from
    # the last pass's predictions and traversal costs, with every term on.
    rows = 4 * n
    for ex, h, ce in ((1.0, 0.0, 0.0), (0.75, -0.5, 0.5), (0.5, 1.5, 1.0)):
        try:
            assert lib.crSetAllocatorExponent(ex) == 0 and lib.crSetAllocatorHalvings(h) == 0
            assert lib.crSetAllocatorCostExponent(ce) == 0
            l4 = torch.zeros_like(lev)
            assert lib.crAdaptiveRenderPosesDevice(d_poses.data_ptr(), 4, 8, torch.zeros_like(out).data_ptr(),
                                                   l4.data_ptr(), None) == 0, eh.lastError(lib)
            torch.cuda.synchronize()
        finally:
            lib.crSetAllocatorExponent(1.0)
            lib.crSetAllocatorHalvings(0.0)
            lib.crSetAllocatorCostExponent(0.0)
        pred = np.zeros((rows, 3), np.float32)
        cost = np.zeros(rows, np.float32)
        lvl = np.zeros(rows, np.uint8)
        assert lib.crAdaptiveLastPass(pred.ctypes.data, cost.ctypes.data, lvl.ctypes.data, rows) == 0, \
            eh.lastError(lib)
        assert np.array_equal(lvl, l4.cpu().numpy().reshape(-1))
        # traversal cost: mean node visits + triangle tests per ray, every
        # entry of this terrain eye traverses something
        assert np.isfinite(cost).all() and (cost >= 0).all() and cost.mean() > 1.0
        want, near = allocator_ref.allocate_levels(pred, cost, 8, h, ex, ce)
        assert near.mean() < 0.01
        assert np.array_equal(lvl[~near], want[~near]), (ex, h, ce, lvl[~near][:8], want[~near][:8])
    assert lib.crAdaptiveLastPass(None, None, None, rows + 1) == -1
    assert "rows must equal" in eh.lastError(lib)


def test_labels_match_numpy_restatement(lib, tmp_path):
    """The GPU minimum-sample search gives, entry by entry, the labels that
    oracle/allocator_ref.py computes from the same eight renders per sample
    count (each render recorded separately through crAdaptiveRecord with the
    search's seeds 0x5eed0000 + k)."""
    # a panoramic eye: the horizon and the plants give entries of every count
    info = scenes.terrain_scene(str(tmp_path), cells=128, extent=60.0, cones=300, n_omm=1500, poses=2,
                                eye_kind="panoramic", aa_deg=(0.5, 5.0))
    eh.lastError(lib)
    lib.loadGlTFscene(info["gltf"].encode())
    assert eh.lastError(lib) == ""
    eh.gotoFirstCompoundEye(lib)
    n = lib.getCurrentEyeOmmatidialCount()
    rng = np.random.default_rng(13)
    poses = scenes.random_poses(info["height_fn"], 1, rng, 20.0)
    lib.crDenoiserRelease()
    assert lib.crAllocatorInit(3) == 0
    thr, seeds = 1.0 / 512.0, 8
    got = np.zeros((1, n), np.uint16)
    assert lib.crAllocatorAddTrainingPoses(poses, 1, 8, thr, seeds, got.ctypes.data) == 0, eh.lastError(lib)
    renders = {}
    for c in (4, 8, 16, 32, 64, 128, 256, 512, 1024):
        rec = np.zeros((n * c,), eh.RAY_RECORD_DTYPE)
        outs = np.zeros((seeds, n, 3), np.float32)
        for k in range(seeds):
            assert lib.crAdaptiveRecord(poses, 1, c, 0x5EED0000 + k, rec.ctypes.data, outs[k]) == 0, eh.lastError(lib)
        renders[c] = outs
    want = allocator_ref.min_sample_labels(renders, thr)
    assert np.array_equal(got[0], want), np.flatnonzero(got[0] != want)[:20]
    assert len(np.unique(want)) >= 4
