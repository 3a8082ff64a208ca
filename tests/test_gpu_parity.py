"""GPU parity: the sm_103a render path against the CPU oracle on identical rays.

Bars (from the renderer's correctness contract):
  * hit triangle ids, hit distances and barycentrics: bit-exact against the
    oracle's float watertight search on the GPU's own rays;
  * disagreements with the independent double-precision search only for rays
    that pass within 1e-6 (barycentric) of a triangle edge;
  * ray generation from the same draws: within 2e-6 absolute per direction
    component (the GPU uses the fast sin/cos of the reference build);
  * per-ray shaded colour and per-ommatidium RGB: within 1e-5 relative
    (RTOL), with an absolute floor of 1e-7 for near-black channels, widened
    by SKY_ATOL for sky-shaded rays: the GPU computes the miss shader with the
    fast-math normalise/asin of the reference build, the oracle with libm,
    and near the zenith d(asin y)/dy amplifies their last-bit differences;
  * 8-bit frame: within one step of the oracle's make_color of the same sums.
"""
import ctypes
import os

import numpy as np
import pytest

import eyeRendererHelperFunctions as eh
import gltf_ref
import oracle
import scenes

pytestmark = pytest.mark.gpu

from parity_checks import ATOL, DIR_ATOL, RTOL, SKY_ATOL, _check_frame, _load, _oracle  # noqa: F401


def test_small_scene_spp32(lib, small, small_ref):
    ref, sc = small_ref
    omm = ref.cameras[0]["omm"]
    _load(lib, small["gltf"], 32)
    lib.setCameraPose(0.0, 0.5, 0.0, 0.0, 0.0, 0.0)
    rec, sums = _check_frame(lib, sc, omm, 32, small["pose"])
    assert (rec["hitId"] >= 0).any() and (rec["hitId"] < 0).any()  # both boxes/ground and sky seen

    # 8-bit frame through the reference-facing readout.
    n = len(omm)
    name = b"single_dimension_fast"
    lib.setCurrentEyeShaderName(name)
    eh.setRenderSize(lib, n, 1)
    lib.renderFrame()
    frame = eh.getFrame(lib, n, 1)[0]
    sums = eh.getOmmatidialColours(lib)
    want = oracle.make_color(sums)
    assert np.abs(frame.astype(int) - want.astype(int)).max() <= 1
    assert (frame[:, 3] == 255).all()


@pytest.mark.parametrize("spp", [1, 5, 100])
def test_small_scene_other_sample_counts(lib, small, small_ref, spp):
    ref, sc = small_ref
    omm = ref.cameras[0]["omm"]
    _load(lib, small["gltf"], spp)
    lib.setCameraPose(0.3, 0.6, -0.2, 0.1, 0.7, -0.05)
    pos = eh.getCameraPosition(lib)
    ls = np.zeros(9, np.float32)
    lib.crGetCameraLocalSpace(ls)
    pose12 = np.concatenate([pos, ls]).astype(np.float32)
    _check_frame(lib, sc, omm, spp, pose12)


def test_terrain_scene(lib, tmp_path):
    info = scenes.terrain_scene(str(tmp_path), cells=64, extent=40.0, cones=60, n_omm=400, spp=64, poses=3)
    ref, sc, omm = _oracle(info["gltf"])
    _load(lib, info["gltf"], 64)
    for p in info["poses"]:
        lib.setCameraPosition(*[float(v) for v in p[:3]])
        lib.setCameraLocalSpace(*[float(v) for v in p[3:]])
        _check_frame(lib, sc, omm, 64, p)


def test_batched_poses_equal_sequential_frames(lib, small):
    """P poses in one batched launch == P renderFrame calls (bit-exact)."""
    _load(lib, small["gltf"], 48)
    rng = np.random.default_rng(3)
    poses = []
    for k in range(5):
        yaw = rng.uniform(0, 6.28)
        poses.append(scenes.pose_rows(np.array([rng.uniform(-1, 1), 0.5, rng.uniform(-1, 1)]), yaw))
    poses = np.stack(poses)
    seq = []
    for p in poses:
        lib.setCameraPosition(*[float(v) for v in p[:3]])
        lib.setCameraLocalSpace(*[float(v) for v in p[3:]])
        assert lib.renderFrame() >= 0
        seq.append(eh.getOmmatidialColours(lib))
    lib.setCurrentEyeSamplesPerOmmatidium(48)  # resets the random streams
    batch = eh.renderPoses(lib, poses)
    assert np.array_equal(batch, np.stack(seq))


@pytest.mark.parametrize("spp,prior", [(8, 0), (8, 3), (4, 1), (32, 2)])
def test_spread_poses_equal_sequential_frames(lib, small, spp, prior):
    """Small eyes render their poses from random numbers drawn up front and
    spread over many warps: after `prior` frames (an odd count leaves a
    cached Box-Muller normal in every state) a 40-pose launch equals 40
    renderFrame calls, bit for bit, and leaves the same generator states."""
    _load(lib, small["gltf"], spp)
    rng = np.random.default_rng(spp + prior)
    poses = np.stack([scenes.pose_rows(np.array([rng.uniform(-2, 2), rng.uniform(0.3, 1.2), rng.uniform(-2, 2)]),
                                       rng.uniform(0, 6.28)) for _ in range(40)])
    n = lib.getCurrentEyeOmmatidialCount()
    states = np.zeros(8 * n * spp, np.uint32)

    def frames(ps):
        out = []
        for p in ps:
            lib.setCameraPosition(*[float(v) for v in p[:3]])
            lib.setCameraLocalSpace(*[float(v) for v in p[3:]])
            assert lib.renderFrame() >= 0
            out.append(eh.getOmmatidialColours(lib))
        return np.stack(out) if out else None

    frames(poses[:prior])
    seq = frames(poses)
    assert lib.crGetRandomStates(states) == 0
    seq_states = states.copy()
    lib.setCurrentEyeSamplesPerOmmatidium(spp)  # resets the random streams
    frames(poses[:prior])
    batch = eh.renderPoses(lib, poses)
    assert lib.crGetRandomStates(states) == 0
    assert np.array_equal(batch, seq)
    assert np.array_equal(states, seq_states)


def test_random_stream_ids_and_persistence(lib, small):
    """Stream id = sample * N + ommatidium (shaders.cu:669, 684); states
    persist across frames and reset on a sample-count change."""
    _load(lib, small["gltf"], 8)
    lib.setCameraPose(0.0, 0.5, 0.0, 0.0, 0.0, 0.0)
    one = eh.c_ommatidiumPacket(0.0, 0.0, 0.0, 0.3, 0.2, 0.9, 0.05, 0.0)
    # Eye A: one ommatidium, 8 samples -> ids 0..7.
    eh.setOmmatidiaFromPacketList(lib, [one])
    lib.setCurrentEyeSamplesPerOmmatidium(8)
    a1 = eh.renderFrameRecorded(lib)
    a2 = eh.renderFrameRecorded(lib)
    # Eye B: eight ommatidia, one sample -> ids 0..7.
    eh.setOmmatidiaFromPacketList(lib, [one] * 8)
    lib.setCurrentEyeSamplesPerOmmatidium(1)
    b1 = eh.renderFrameRecorded(lib)
    assert np.array_equal(a1["normalDraw"][0], b1["normalDraw"][:, 0])
    assert np.array_equal(a1["uniformDraw"][0], b1["uniformDraw"][:, 0])
    # Later frames continue the streams.
    assert not np.array_equal(a1["normalDraw"], a2["normalDraw"])
    # Same count again: records only; the streams are kept.
    b2 = eh.renderFrameRecorded(lib)
    assert np.array_equal(b2["normalDraw"][:, 0], a2["normalDraw"][0])
    # A sample-count change resets them.
    lib.setCurrentEyeSamplesPerOmmatidium(1)
    b3 = eh.renderFrameRecorded(lib)
    assert np.array_equal(b3["normalDraw"], b1["normalDraw"])


def test_draw_distribution(lib, small):
    _load(lib, small["gltf"], 64)
    rec = eh.renderFrameRecorded(lib)
    n = rec["normalDraw"].ravel().astype(np.float64)
    u = rec["uniformDraw"].ravel().astype(np.float64)
    assert abs(n.mean()) < 0.02 and abs(n.std() - 1.0) < 0.02
    assert u.min() > 0.0 and u.max() <= 1.0 and abs(u.mean() - 0.5) < 0.01


def test_autotune_changes_no_result(lib, small):
    """Every kernel variant renders the same bits, and tuning leaves the
    random streams where they were."""
    import ctypes

    import torch

    _load(lib, small["gltf"], 64)
    poses = np.stack([scenes.pose_rows(np.array([0.1 * k, 0.5, 0.0]), 0.3 * k) for k in range(4)])
    p16 = np.zeros((4, 16), np.float32)
    for k in range(4):
        p16[:, 4 * k:4 * k + 3] = poses[:, 3 * k:3 * k + 3]
    d = torch.from_numpy(p16).cuda()
    torch.cuda.synchronize()
    ms = np.zeros(lib.crGetRenderVariantCount(), np.float32)
    best = ctypes.c_int(-1)
    assert lib.crAutotune(d.data_ptr(), 4, ctypes.byref(best), ms) == 0, eh.lastError(lib)
    assert 0 <= best.value < len(ms) and (ms > 0).all()
    outs = []
    for v in range(len(ms)):
        assert lib.crSetRenderVariant(v) == 0
        lib.setCurrentEyeSamplesPerOmmatidium(64)  # same streams for every variant
        outs.append(eh.renderPoses(lib, poses))
    for o in outs[1:]:
        assert np.array_equal(o, outs[0])
    # tuning did not advance the streams: a fresh eye renders the same frames
    # (with the layout and variant of outs[0]: a smaller warp segment sums
    # the samples in another order)
    bt, spw = ctypes.c_int(0), ctypes.c_int(0)
    assert lib.crGetRenderLayout(ctypes.byref(bt), ctypes.byref(spw)) == 0
    lib.setCurrentEyeSamplesPerOmmatidium(64)
    assert lib.crAutotune(d.data_ptr(), 4, ctypes.byref(best), ms) == 0
    times = np.zeros(20, np.float32)
    assert lib.crGetAutotuneTimes(times, 20) == 0 and (times[:18] > 0).all()
    # the cut refinement ran exactly when the best grid radius was not 0
    if lib.crGetCutRadius() > 0:
        assert (times[18:] > 0).all()
    else:
        assert (times[18:] == 0).all()
    assert lib.crSetRenderLayout(bt.value, spw.value) == 0 and lib.crSetRenderVariant(0) == 0
    assert np.array_equal(eh.renderPoses(lib, poses), outs[0])
    lib.crSetRenderVariant(best.value)
    lib.crSetRenderLayout(0, 32)
    lib.crSetBvhWidth(2)


@pytest.mark.parametrize("spp", [48, 100, 256])
def test_render_layouts(lib, small, spp):
    """Block sizes 128 / 256 / 512 render the same bits, whether the chunk
    partials of an ommatidium are summed in shared memory (blocks holding all
    its chunk warps) or in scratch by a second kernel; warp segments of 8 or
    16 samples give the same frames within float rounding (another summing
    order of the same samples: same streams, same rays)."""
    _load(lib, small["gltf"], spp)
    poses = np.stack([scenes.pose_rows(np.array([0.2 * k, 0.6, -0.1 * k]), 0.5 * k) for k in range(3)])
    outs = {}
    try:
        for block in (128, 256, 512):
            for spw in (8, 16, 32):
                assert lib.crSetRenderLayout(block, spw) == 0, eh.lastError(lib)
                lib.setCurrentEyeSamplesPerOmmatidium(spp + 1)
                lib.setCurrentEyeSamplesPerOmmatidium(spp)  # the same streams for every layout
                # one pose per call: a small eye's multi-pose launches spread
                # their poses over warps and keep the partials in scratch
                outs[block, spw] = np.concatenate([eh.renderPoses(lib, poses[k:k + 1]) for k in range(len(poses))])
                assert eh.lastError(lib) == ""
    finally:
        lib.crSetRenderLayout(0, 32)
    for spw in (8, 16, 32):
        for block in (256, 512):
            assert np.array_equal(outs[block, spw], outs[128, spw]), (block, spw)
    ref = outs[128, 32]
    for spw in (8, 16):
        np.testing.assert_allclose(outs[128, spw], ref, rtol=1e-5, atol=1e-7)


def test_in_block_sums_over_pose_groups(lib, small):
    """A multi-pose launch whose chunk partials are summed in shared memory
    (512-thread blocks holding the 16 chunk warps of an ommatidium at 512
    samples) flushes them every 16 poses; 40 poses (groups of 16, 16 and 8)
    render the same bits as the scratch layout (128-thread blocks)."""
    _load(lib, small["gltf"], 512)
    rng = np.random.default_rng(3)
    poses = scenes.open_poses(small["boxes"], 40, rng)
    outs = {}
    try:
        for block in (128, 512):
            assert lib.crSetRenderLayout(block, 32) == 0, eh.lastError(lib)
            lib.setCurrentEyeSamplesPerOmmatidium(511)
            lib.setCurrentEyeSamplesPerOmmatidium(512)  # the same streams for both layouts
            outs[block] = eh.renderPoses(lib, poses)
            assert eh.lastError(lib) == ""
    finally:
        lib.crSetRenderLayout(0, 32)
    assert np.array_equal(outs[512], outs[128])
    assert np.isfinite(outs[128]).all() and (outs[128] > 0).any()


@pytest.mark.parametrize("size", ["small", "terrain"])
def test_gpu_built_bvh_renders_identical_bits(lib, small, tmp_path, size):
    """The GPU linear BVH and the host SAH BVH give bit-identical renders:
    the closest hit is the (t, id) minimum whatever the tree."""
    if size == "small":
        path, spp, poses = small["gltf"], 32, np.stack([small["pose"]])
    else:
        info = scenes.terrain_scene(str(tmp_path), cells=96, extent=40.0, cones=80, n_omm=300, spp=64, poses=4)
        path, spp, poses = info["gltf"], 64, info["poses"]
    outs = []
    stats = []
    for builder in (0, 1):
        assert lib.crSetBvhBuilder(builder) == 0
        _load(lib, path, spp)
        outs.append(eh.renderPoses(lib, poses))
        inner, leaves, depth = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
        assert lib.crGetBvhStats(ctypes.byref(inner), ctypes.byref(leaves), ctypes.byref(depth)) == 0
        stats.append((inner.value, leaves.value, depth.value))
    lib.crSetBvhBuilder(0)
    assert np.array_equal(outs[0], outs[1])
    assert stats[1][0] > 0 and stats[1][1] > stats[1][0] and 0 < stats[1][2] < 62
    # and the GPU-built tree passes the full per-ray parity check
    assert lib.crSetBvhBuilder(1) == 0
    ref, sc, omm = _oracle(path)
    _load(lib, path, spp)
    lib.setCameraPosition(*[float(v) for v in poses[0][:3]])
    lib.setCameraLocalSpace(*[float(v) for v in poses[0][3:]])
    _check_frame(lib, sc, omm, spp, poses[0])
    lib.crSetBvhBuilder(0)


def _sphere_points(w, h, split=False):
    x = np.arange(w, dtype=np.float32) / np.float32(w)
    y = np.arange(h, dtype=np.float32) / np.float32(h)
    ux, uy = np.meshgrid(x, y)
    if split:
        sx = ux * 2.0
        dx = (sx - (sx > 1.0)) * 2.0 - 1.0
    else:
        dx = 2.0 * ux - 1.0
    dy = 2.0 * uy - 1.0
    ax = dx * -np.pi + np.pi / 2
    ay = dy * (np.pi / 2)
    p = np.stack([np.cos(ax) * np.cos(ay), np.sin(ay), np.sin(ax) * np.cos(ay)], axis=-1)
    return p, ux


@pytest.mark.parametrize("kind", ["spherical_orientationwise_ids", "spherical_positionwise_ids",
                                  "spherical_orientationwise", "spherical_split_orientationwise"])
def test_spherical_projections(lib, small, small_ref, kind):
    """Voronoi projections of shaders.cu:412-640: each pixel shows the
    ommatidium with the smallest angle to its sphere point (first on ties)."""
    ref, sc = small_ref
    omm = ref.cameras[0]["omm"].astype(np.float64)
    _load(lib, small["gltf"], 32)
    w, h = 96, 48
    lib.setCurrentEyeShaderName(kind.encode())
    eh.setRenderSize(lib, w, h)
    assert lib.renderFrame() >= 0, eh.lastError(lib)
    frame = eh.getFrame(lib, w, h).astype(np.int64)
    p, ux = _sphere_points(w, h, split="split" in kind)
    v = omm[:, 0:3] if "positionwise" in kind else omm[:, 3:6]
    cosang = (p.reshape(-1, 3) @ v.T) / np.linalg.norm(v, axis=1)[None, :]
    ang = np.arccos(np.clip(cosang, -1, 1))
    if "split" in kind:
        ok = ((omm[None, :, 0] > 0) & (ux.reshape(-1, 1) > 0.5)) | ((omm[None, :, 0] < 0) & (ux.reshape(-1, 1) < 0.5))
        ok[:, 0] = True  # ommatidium 0 is the starting candidate whatever its side
        ang = np.where(ok, ang, np.inf)
    want = ang.argmin(axis=1)
    srt = np.sort(ang, axis=1)
    clear = (srt[:, 1] - srt[:, 0]) > 1e-4  # pixels not on a Voronoi boundary
    if kind.endswith("_ids"):
        got = (frame[..., 0] << 24) | (frame[..., 1] << 16) | (frame[..., 2] << 8) | frame[..., 3]
        got = got.reshape(-1)
        assert (got[clear] == want[clear]).all()
        assert clear.mean() > 0.9
    else:
        sums = eh.getOmmatidialColours(lib)
        colours = oracle.make_color(sums)[want]
        d = np.abs(frame.reshape(-1, 4) - colours.astype(np.int64))[clear]
        assert d.max() <= 1


def test_raw_samples_projection(lib, small):
    _load(lib, small["gltf"], 8)
    n = lib.getCurrentEyeOmmatidialCount()
    lib.setCurrentEyeShaderName(b"raw_ommatidial_samples")
    eh.setRenderSize(lib, n, 12)
    assert lib.renderFrame() >= 0, eh.lastError(lib)
    frame = eh.getFrame(lib, n, 12)
    assert (frame[:8, :, 3] == 255).all() and (frame[8:] == 0).all()
    assert frame[:8, :, :3].any()


@pytest.mark.parametrize("fraction", [1.0 / 512, 1.0 / 64, 1.0 / 8])
def test_near_field_cut_changes_no_result(lib, small, tmp_path, fraction):
    """Rays that search the pose's near-field cut first give the same closest
    hits, colours and random streams as rays that start at the root, on the
    small scene (eye among boxes) and the terrain (eye just above ground)."""
    info = scenes.terrain_scene(str(tmp_path), cells=128, extent=60.0, cones=300, n_omm=1500, poses=12)
    for path, spp, poses in ((small["gltf"], 32, None), (info["gltf"], 16, info["poses"])):
        if poses is None:
            rng = np.random.default_rng(1)
            poses = np.stack([scenes.pose_rows(np.array([rng.uniform(-6, 6), rng.uniform(0.2, 1.5), rng.uniform(-6, 6)]),
                                               rng.uniform(0, 6.28)) for _ in range(12)])
        outs, recs = [], []
        for f in (0.0, fraction):
            assert lib.crSetCutRadius(f) == 0
            _load(lib, path, spp)
            outs.append(eh.renderPoses(lib, poses))
            lib.setCameraPosition(*[float(v) for v in poses[3][:3]])
            lib.setCameraLocalSpace(*[float(v) for v in poses[3][3:]])
            recs.append(eh.renderFrameRecorded(lib))
        lib.crSetCutRadius(0.0)
        assert np.array_equal(outs[0], outs[1])
        assert np.array_equal(recs[0]["hitId"], recs[1]["hitId"])
        assert np.array_equal(recs[0]["t"], recs[1]["t"])


def test_cut_follows_same_count_ommatidia(lib, small):
    """Replacing an eye's ommatidia with the same count of records whose
    positions lie much farther from the pose position (0.3 m instead of
    1 mm, beyond the cut's radius) keeps the near-field cut exact: the
    guaranteed radius is recomputed from the new records."""
    rng = np.random.default_rng(5)
    poses = np.stack([scenes.pose_rows(np.array([rng.uniform(-6, 6), rng.uniform(0.2, 1.5), rng.uniform(-6, 6)]),
                                       rng.uniform(0, 6.28)) for _ in range(8)])
    outs = []
    for f in (0.0, 1.0 / 64):
        assert lib.crSetCutRadius(f) == 0
        _load(lib, small["gltf"], 16)
        omm = eh.getOmmatidia(lib)
        eh.renderPoses(lib, poses)  # the eye's device state (and its cut bound) from the first records
        wide = omm.copy()
        wide[:, 0:3] *= 300.0  # 1 mm -> 0.3 m from the pose position
        eh.setOmmatidiaFromPacketList(lib, [eh.c_ommatidiumPacket(*[float(x) for x in row]) for row in wide])
        assert eh.lastError(lib) == ""
        assert lib.getCurrentEyeOmmatidialCount() == len(omm)
        outs.append(eh.renderPoses(lib, poses))
    lib.crSetCutRadius(0.0)
    assert np.array_equal(outs[0], outs[1])


def test_hitbox_batch_matches_point_queries(lib, tmp_path):
    """crInsideHitGeometryBatch (GPU) answers as isInsideHitGeometry does,
    point by point, for a rotated, scaled, translated hitbox mesh (whose
    translation the query ignores, as the reference's does)."""
    g = scenes.GltfBuilder()
    v, f = scenes.box_mesh([-1, -1, -1], [1, 1, 1])
    g.mesh("ground", np.array([[-5, 0, -5], [5, 0, -5], [5, 0, 5]], np.float64), np.array([[0, 2, 1]]))
    g.mesh("arena", v, f, extras={"hitbox": True}, translation=[2.0, 0.5, -1.0],
           rotation=[0.0, np.sin(0.35), 0.0, np.cos(0.35)], scale=[1.5, 0.8, 2.0])
    g.perspective_camera("cam")
    eh.lastError(lib)
    lib.loadGlTFscene(g.write(str(tmp_path / "hb.gltf")).encode())
    assert eh.lastError(lib) == ""
    rng = np.random.default_rng(8)
    pts = rng.uniform([-3, -1.5, -3], [3, 1.5, 3], size=(3000, 3)).astype(np.float32)
    out = np.zeros(len(pts), np.uint8)
    assert lib.crInsideHitGeometryBatch(pts, len(pts), b"arena", out) == 0, eh.lastError(lib)
    want = np.array([lib.isInsideHitGeometry(float(x), float(y), float(z), b"arena") for x, y, z in pts], np.uint8)
    assert np.array_equal(out, want)
    assert 200 < want.sum() < 2800
    assert lib.crInsideHitGeometryBatch(pts, len(pts), b"nothing", out) == -1


def test_hitbox_batch_grid_on_a_large_mesh(lib, tmp_path):
    """The batched query searches a (y, z) grid of the hitbox's triangles:
    same answers as the full loop of isInsideHitGeometry on a 9216-triangle
    sphere, for random points and for points whose (y, z) is a vertex's
    (rays through vertices and along edges), untransformed and transformed."""
    eh.lastError(lib)
    lib.loadGlTFscene(scenes.hitbox_scene(str(tmp_path / "ball.gltf")).encode())
    assert eh.lastError(lib) == ""
    pts = scenes.hitbox_points()
    for name in (b"ball", b"egg"):
        out = np.zeros(len(pts), np.uint8)
        assert lib.crInsideHitGeometryBatch(pts, len(pts), name, out) == 0, eh.lastError(lib)
        want = np.array([lib.isInsideHitGeometry(float(x), float(y), float(z), name) for x, y, z in pts], np.uint8)
        assert np.array_equal(out, want), (name, np.flatnonzero(out != want)[:10])
        assert 300 < want.sum() < 2700
        # and as the reference's own code (sutil/hitscanprocessing.cpp,
        # compiled here into tests/golden/reference_hitscan.npz): the same
        # float cast on the same object-space floats
        ref = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_hitscan.npz"))
        assert np.array_equal(ref["points"], pts)
        assert np.array_equal(out, ref[name.decode() + "__inside"]), np.flatnonzero(out != ref[name.decode() + "__inside"])
