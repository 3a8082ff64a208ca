"""The CPU oracle itself: internal consistency, the reference's documented
quirks, and agreement with brute force and double precision."""
import math

import numpy as np

import oracle
import scenes


def _draws(n, seed):
    rng = np.random.default_rng(seed)
    return np.stack([rng.standard_normal(n), 1.0 - rng.random(n)], axis=1).astype(np.float32)


def test_float_search_vs_double_search(small, small_ref):
    ref, sc = small_ref
    omm = ref.cameras[0]["omm"]
    spp = 32
    org, dirs = oracle.gen_rays(omm, spp, small["pose"], _draws(len(omm) * spp, 1))
    hit, t, b1, b2 = sc.trace(org, dirs, 0.0)
    h64, t64, e32, e64 = sc.trace_f64(org, dirs, 0.0, hit32=hit)
    diff = hit != h64
    assert not (diff & ~((e32 < 1e-6) | (e64 < 1e-6))).any()
    m = hit >= 0
    np.testing.assert_allclose(t[m], t64[m], rtol=1e-5)
    assert 0.2 < m.mean() < 0.95  # boxes, ground and sky are all visible


def test_bvh_search_equals_brute_force(tmp_path):
    """The oracle's BVH result equals the exhaustive (t, id) minimum: one
    triangle at a time through a one-triangle scene."""
    info = scenes.small_scene(str(tmp_path), n_omm=50)
    import gltf_ref

    ref = gltf_ref.load(info["gltf"])
    v, c, f = ref.arrays()
    sc = oracle.OracleScene(v, c, f, ref.miss)
    omm = ref.cameras[0]["omm"]
    org, dirs = oracle.gen_rays(omm, 8, info["pose"], _draws(len(omm) * 8, 2))
    hit, t, _, _ = sc.trace(org, dirs, 0.0)
    best_t = np.full(len(org), np.inf, np.float32)
    best_id = np.full(len(org), -1, np.int64)
    for k in range(len(v)):
        one = oracle.OracleScene(v[k:k + 1], c[k:k + 1], f[k:k + 1], ref.miss)
        h, tk, _, _ = one.trace(org, dirs, 0.0)
        better = (h >= 0) & ((tk < best_t) | ((tk == best_t) & (k < best_id)))
        best_t[better] = tk[better]
        best_id[better] = k
    assert np.array_equal(np.where(best_id < 0, -1, best_id), hit)


def test_perpendicular_axis_quirk():
    """generateOffsetRay (shaders.cu:655-657) replaces the perpendicular axis
    by (0,0,1) whenever its components sum to zero, i.e. whenever the
    ommatidial axis has x == z -- not only for a vertical axis."""
    pose = np.array([0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1], np.float32)
    draws = np.array([[1.0, 0.0]], np.float32)  # splay by one sd, no twist
    for axis in ([0.0, 1.0, 0.0], [0.5, 0.7071, 0.5], [0.3, 0.5, 0.3]):
        omm = np.array([[0, 0, 0, *axis, 0.5, 0.0]], np.float32)
        _, d = oracle.gen_rays(omm, 1, pose, draws)
        a = np.asarray(axis, np.float64)
        ang = 0.5 / 2.35482004503094938
        # Rodrigues about (0,0,1)
        k = np.array([0.0, 0.0, 1.0])
        want = a * math.cos(ang) + np.cross(k, a) * math.sin(ang) + k * np.dot(k, a) * (1 - math.cos(ang))
        np.testing.assert_allclose(d[0], want, atol=1e-6)
    # a generic axis uses normalize(cross(up, axis))
    axis = np.array([0.6, 0.0, 0.8])
    omm = np.array([[0, 0, 0, *axis, 0.5, 0.0]], np.float32)
    _, d = oracle.gen_rays(omm, 1, pose, draws)
    k = np.cross([0, 1, 0], axis)
    k /= np.linalg.norm(k)
    ang = 0.5 / 2.35482004503094938
    want = axis * math.cos(ang) + np.cross(k, axis) * math.sin(ang) + k * np.dot(k, axis) * (1 - math.cos(ang))
    np.testing.assert_allclose(d[0], want, atol=1e-6)


def test_ray_generation_properties():
    """Unit axes stay unit directions; the splay angle follows the draw times
    acceptance/2.35482; the twist only rotates about the axis; the origin
    moves back along the axis by the focal offset."""
    d = scenes.fibonacci_sphere(64)
    omm = np.concatenate([d * 0.001, d, np.full((64, 1), 0.1), np.full((64, 1), 0.002)], axis=1).astype(np.float32)
    pose = np.array([1, 2, 3, 1, 0, 0, 0, 1, 0, 0, 0, 1], np.float32)
    dr = _draws(64 * 16, 5)
    org, dirs = oracle.gen_rays(omm, 16, pose, dr)
    np.testing.assert_allclose(np.linalg.norm(dirs, axis=1), 1.0, atol=1e-5)
    ax = np.repeat(d, 16, axis=0)
    dd = dirs.astype(np.float64)
    ang = np.arctan2(np.linalg.norm(np.cross(dd, ax), axis=1), (dd * ax).sum(1))
    np.testing.assert_allclose(ang, np.abs(dr[:, 0]) * 0.1 / 2.35482004503094938, atol=2e-6)
    np.testing.assert_allclose(org, np.repeat(d * 0.001 - d * 0.002, 16, axis=0) + [1, 2, 3], atol=1e-6)


def test_sky_and_make_color():
    import gltf_ref  # noqa: F401

    v = np.zeros((1, 3, 3), np.float32) + 1e6
    sc = oracle.OracleScene(v, np.ones((1, 3, 4), np.float32), np.ones(1, np.uint8), 1)
    dirs = np.array([[0, 1, 0], [0, -1, 0], [1, 0, 0], [0, 0.5, 0.5]], np.float32)
    rgb = sc.shade(dirs, np.full(4, -1, np.int32), np.zeros(4, np.float32), np.zeros(4, np.float32))
    upper = np.array([1, 31, 117]) / 255.0
    lower = np.array([143, 179, 203]) / 255.0 * 0.8
    np.testing.assert_allclose(rgb[0], upper, rtol=1e-6)
    np.testing.assert_allclose(rgb[1], lower, rtol=1e-6)
    np.testing.assert_allclose(rgb[2], lower, rtol=1e-6)
    np.testing.assert_allclose(rgb[3], lower * 0.5 + upper * 0.5, rtol=1e-5)
    # make_color: clamp, x^(1/2.2), *255, truncate, alpha 255
    sums = np.array([[0.0, 1.0, 2.0], [-1.0, 0.5, 0.2176]], np.float32)
    out = oracle.make_color(sums)
    want = [[0, 255, 255, 255], [0, int(0.5 ** (1 / 2.2) * 255), int(np.float32(0.2176) ** (1 / 2.2) * 255), 255]]
    assert out.tolist() == want
    # default background: border lines are black
    sc0 = oracle.OracleScene(v, np.ones((1, 3, 4), np.float32), np.ones(1, np.uint8), 0)
    rgb = sc0.shade(np.array([[0.005, 0.7, 0.7], [0.6, 0.6, 0.52]], np.float32), np.full(2, -1, np.int32),
                    np.zeros(2, np.float32), np.zeros(2, np.float32))
    assert (rgb[0] == 0).all() and rgb[1, 0] > 0 and rgb[1, 2] == 0


def test_vertex_colour_shading_is_linearised_after_interpolation():
    v = np.array([[[0, 0, 5], [1, 0, 5], [0, 1, 5]]], np.float32)
    col = np.array([[[0.2, 0.4, 0.6, 1], [0.8, 0.1, 0.3, 1], [0.5, 0.5, 0.5, 1]]], np.float32)
    sc = oracle.OracleScene(v, col, np.ones(1, np.uint8), 1)
    hit, t, b1, b2 = sc.trace(np.array([[0.25, 0.25, 0]], np.float32), np.array([[0, 0, 1]], np.float32), 0.0)
    assert hit[0] == 0 and t[0] == 5.0
    rgb = sc.shade(np.array([[0, 0, 1]], np.float32), hit, b1, b2)
    w = np.array([1 - b1[0] - b2[0], b1[0], b2[0]])
    want = (w[:, None] * col[0, :, :3]).sum(0) ** 2.2
    np.testing.assert_allclose(rgb[0], want, rtol=1e-5)
    flat = oracle.OracleScene(v, col, np.zeros(1, np.uint8), 1)
    np.testing.assert_array_equal(flat.shade(np.array([[0, 0, 1]], np.float32), hit, b1, b2)[0], col[0, 0, :3])


def test_render_reduction_is_sequential_sum(small, small_ref):
    ref, sc = small_ref
    omm = ref.cameras[0]["omm"][:40]
    spp = 7
    org, dirs = oracle.gen_rays(omm, spp, small["pose"], _draws(40 * spp, 9))
    out = sc.render_rays(omm, spp, org, dirs)[0]
    hit, t, b1, b2 = sc.trace(org, dirs, 0.0)
    rgb = sc.shade(dirs, hit, b1, b2).reshape(40, spp, 3)
    scale = np.float32(1.0) / np.float32(spp)
    acc = np.zeros((40, 3), np.float32)
    for k in range(spp):
        acc = (acc + rgb[:, k] * scale).astype(np.float32)
    assert np.array_equal(out, acc)


def test_adam_restatement_against_float64():
    """oracle/mlp_ref.adam_step follows Adam: within float32 rounding of a
    float64 evaluation of the same update."""
    import mlp_ref

    rng = np.random.default_rng(3)
    w = rng.normal(0, 0.1, 1000).astype(np.float32)
    g = rng.normal(0, 1e-3, 1000).astype(np.float32)
    m = rng.normal(0, 1e-4, 1000).astype(np.float32)
    v = np.abs(rng.normal(0, 1e-6, 1000)).astype(np.float32)
    c1, c2 = 1.0 / (1 - 0.9 ** 3), 1.0 / (1 - 0.999 ** 3)
    w2, m2, v2, bits = mlp_ref.adam_step(w, g, m, v, 1e-3, c1, c2)
    # float64 with the float32 constants: the differences are roundings only,
    # each a few ulp of the terms summed
    b1, b2 = float(np.float32(0.9)), float(np.float32(0.999))
    a1, a2 = float(np.float32(1) - np.float32(0.9)), float(np.float32(1) - np.float32(0.999))
    m64 = b1 * m.astype(np.float64) + a1 * g
    v64 = b2 * v.astype(np.float64) + a2 * g.astype(np.float64) ** 2
    step = 1e-3 * (m64 * c1) / (np.sqrt(v64 * c2) + 1e-8)
    w64 = w - step
    ulp = 2.0 ** -23
    assert (np.abs(m2 - m64) <= 4 * ulp * (np.abs(b1 * m) + np.abs(a1 * g))).all()
    assert (np.abs(v2 - v64) <= 4 * ulp * (np.abs(b2 * v) + a2 * g.astype(np.float64) ** 2)).all()
    assert (np.abs(w2 - w64) <= 4 * ulp * np.abs(w) + 1e-3 * np.abs(step)).all()
    assert np.array_equal(bits, mlp_ref.bf16_bits(w2))


def test_label_restatement_rules():
    """oracle/allocator_ref: the first count whose per-channel deviation
    across the renders is below the threshold in every channel; entries never
    below it keep 0; a planted spread in one channel alone delays the label."""
    import allocator_ref

    rng = np.random.default_rng(4)
    rows, k, thr = 6, 8, 1.0 / 512
    renders = {}
    for i, c in enumerate((4, 8, 16, 32, 64, 128, 256, 512, 1024)):
        spread = np.array([1e-4, 0.05 / np.sqrt(c), 0.2 / np.sqrt(c), 0.5, 1e-4, 1e-4], np.float32)
        r = (0.5 + rng.standard_normal((k, rows, 3)) * spread[None, :, None]).astype(np.float32)
        r[:, 4, 1] = 0.5 + rng.standard_normal(k) * (0.04 / np.sqrt(c))  # one channel only
        renders[c] = r
    lab = allocator_ref.min_sample_labels(renders, thr)
    assert lab[0] == 4 and lab[5] == 4
    assert lab[3] == 0
    assert 4 < lab[1] < lab[2] or lab[2] == 0
    assert lab[4] > 4


def test_allocation_restatement_rules():
    """oracle/allocator_ref.allocate_levels: counts 2^ceil(exponent * log2
    predicted - halvings - cost term), clamped to [4, 2048]; at most the
    feature render's count -> no render; 2048 -> the 1024 fallback; a NaN
    prediction gets the least count; the cost term halves the count of an
    entry 4x costlier at cost exponent 1/2."""
    import allocator_ref

    NR = allocator_ref.NO_RENDER
    # predicted counts 2^(10 l): l = 0.3 -> 8, 0.5 -> 32, 0.8 -> 256, 1.2 -> capped at 2048
    pred = np.repeat(np.array([[0.3], [0.5], [0.8], [1.2], [np.nan]], np.float32), 3, axis=1)
    cost = np.full(5, 16.0, np.float32)
    lv, near = allocator_ref.allocate_levels(pred, cost, 8, 0.0, 1.0, 0.0)
    assert not near[:4].any()
    assert lv.tolist() == [NR, 3, 6, 0x88, NR]  # 8 <= feature spp; 32 = 4 << 3; 256 = 4 << 6; fallback; NaN
    lv, _ = allocator_ref.allocate_levels(pred, cost, 8, 1.0, 1.0, 0.0)
    assert lv.tolist() == [NR, 2, 5, 8, NR]  # one halving: every count halves, the fallback joins 1024
    lv, _ = allocator_ref.allocate_levels(pred, cost, 8, 0.0, 0.5, 0.0)
    assert lv.tolist() == [NR, NR, 2, 4, NR]  # square root: 2^ceil(1.5), 2^ceil(2.5) = 8, 2^4, 2^ceil(5.5)
    lv, _ = allocator_ref.allocate_levels(pred, np.full(5, 64.0, np.float32), 8, 0.0, 1.0, 0.5)
    assert lv.tolist() == [NR, 2, 5, 8, NR]  # cost 4 x 16 at cost exponent 1/2: one halving
    lv, _ = allocator_ref.allocate_levels(pred, np.full(5, 0.25, np.float32), 8, 0.0, 1.0, 0.5)
    assert lv.tolist() == [3, 5, 8, 0x88, NR]  # cost below 1 counts as 1 = 16 / 2^4: 2^(4 x 1/2) times more


def test_net_draws_are_stratified_nets():
    """oracle.net_draws (the adaptive render's draws): the first 2^m samples
    of an entry form a (0, m, 2)-net after the digital shift -- exactly one
    point in each elementary interval of area 2^-m (checked for the
    2^a x 2^(m-a) grids) -- and different entries get different shifts."""
    from statistics import NormalDist

    cdf = NormalDist().cdf
    m = 6
    n = 1 << m
    nd, ud = oracle.net_draws(0xada90000, np.repeat([0, 1, 12345], n), np.tile(np.arange(n), 3))
    for e in range(3):
        u1 = np.array([cdf(x) for x in nd[e * n:(e + 1) * n]])
        u2 = 1.0 - ud[e * n:(e + 1) * n].astype(np.float64)
        for a in range(m + 1):
            cells = np.floor(u1 * (1 << a)).astype(np.int64) * (1 << (m - a)) + \
                np.floor(u2 * (1 << (m - a))).astype(np.int64)
            assert len(set(cells.tolist())) == n, (e, a)
    assert not np.array_equal(nd[:n], nd[n:2 * n])
    assert ud.min() > 0 and ud.max() <= 1
