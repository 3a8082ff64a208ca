"""The learned denoiser: GPU gradients against the numpy reference, training
on renders of this renderer, the gain over the plain low-sample render, and
the checkpoint round trip."""
import numpy as np
import pytest

import eyeRendererHelperFunctions as eh
import mlp_ref
import scenes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kernel", [0, 1])
@pytest.mark.parametrize("rows", [64, 500, 2000])
def test_gradients_match_reference(lib, rows, kernel):
    """kernel 0: the mma.sync GEMMs; 1: the tcgen05 GEMMs (2000 rows also
    take the split-K weight-gradient path)."""
    assert lib.crSetDenoiserKernel(kernel) == 0
    try:
        _gradients_case(lib, rows)
    finally:
        lib.crSetDenoiserKernel(1)


def _gradients_case(lib, rows):
    assert lib.crDenoiserInit(7) == 0, eh.lastError(lib)
    n = lib.crDenoiserParamCount()
    assert n == mlp_ref.N_PARAMS
    rng = np.random.default_rng(rows)
    X = rng.normal(0, 1, size=(rows, mlp_ref.FEAT)).astype(np.float32)
    X[:, 105:] = 0
    base = rng.uniform(0, 1, size=(rows, 3)).astype(np.float32)
    target = (base + rng.normal(0, 0.05, size=(rows, 3))).astype(np.float32)
    grads = np.zeros(n, np.float32)
    params = np.zeros(n, np.float32)
    loss = lib.crDenoiserGradient(mlp_ref.bf16_bits(X), base, target, rows, grads, params)
    assert loss >= 0, eh.lastError(lib)
    ref_loss, ref_g = mlp_ref.forward_backward(params, X, base, target)
    assert abs(loss - ref_loss) <= 1e-4 * ref_loss + 1e-7
    # Per element: the GPU sums in fp32 in its own order, and a bf16 rounding
    # (hidden activations, back-propagated gradients) may land one step
    # (2^-8 relative) apart, so each gradient may differ from the reference
    # by a few bf16 steps of the sum of the absolute values of its terms:
    # 2^-6 of it, elementwise.
    mag = mlp_ref.gradient_magnitudes(params, X, base, target)
    err = np.abs(grads.astype(np.float64) - ref_g)
    tol = 2.0 ** -6 * mag + 1e-9
    for lo, hi, name in [(mlp_ref.OFF_W1, mlp_ref.OFF_B1, "W1"), (mlp_ref.OFF_B1, mlp_ref.OFF_W2, "b1"),
                         (mlp_ref.OFF_W2, mlp_ref.OFF_B2, "W2"), (mlp_ref.OFF_B2, mlp_ref.OFF_W3, "b2"),
                         (mlp_ref.OFF_W3, mlp_ref.OFF_B3, "W3"), (mlp_ref.OFF_B3, mlp_ref.OFF_W4, "b3"),
                         (mlp_ref.OFF_W4, mlp_ref.OFF_B4, "W4"), (mlp_ref.OFF_B4, mlp_ref.N_PARAMS, "b4")]:
        bad = err[lo:hi] > tol[lo:hi]
        assert not bad.any(), "%s: %d elements out of bound, worst %.3g of its bound" % (
            name, bad.sum(), (err[lo:hi] / tol[lo:hi]).max())
        # and in aggregate the gradients agree far more closely
        rel = np.linalg.norm(grads[lo:hi] - ref_g[lo:hi]) / max(np.linalg.norm(ref_g[lo:hi]), 1e-30)
        assert rel < 1e-2, "%s gradient relative error %.3g" % (name, rel)


def test_fused_inference_matches_layer_path(lib, tmp_path):
    """The learned render's fused feature + network kernel against the
    feature rows and the layer-by-layer GEMM path (bit for bit), and against
    the numpy forward pass (float64 accumulation)."""
    info = scenes.terrain_scene(str(tmp_path), cells=64, extent=40.0, cones=50, n_omm=700, poses=4)
    lib.loadGlTFscene(info["gltf"].encode())
    assert eh.lastError(lib) == ""
    eh.gotoFirstCompoundEye(lib)
    n = lib.getCurrentEyeOmmatidialCount()
    rng = np.random.default_rng(2)
    poses = scenes.random_poses(info["height_fn"], 3, rng, 10.0)
    assert lib.crDenoiserInit(4) == 0
    assert lib.crDenoiserAddTrainingPoses(poses, 3, 8, 64) == 0, eh.lastError(lib)
    assert lib.crDenoiserTrain(50, 512, 1e-3, 1, None) == 0, eh.lastError(lib)
    rows = 3 * n
    X = np.zeros((rows, mlp_ref.FEAT), np.uint16)
    base = np.zeros((rows, 3), np.float32)
    # Reload to restart the feature streams before each of the two renders.
    lib.loadGlTFscene(info["gltf"].encode())
    eh.gotoFirstCompoundEye(lib)
    assert lib.crDenoiserFeatureRows(poses, 3, 8, X, base) == 0, eh.lastError(lib)
    lib.loadGlTFscene(info["gltf"].encode())
    eh.gotoFirstCompoundEye(lib)
    fused = np.zeros((3, n, 3), np.float32)
    assert lib.crSetDenoiserKernel(0) == 0  # the mma.sync kernel repeats the training path bit for bit
    assert lib.crDenoiserRenderPoses(poses, 3, 8, fused) == 0, eh.lastError(lib)
    layered = np.zeros((rows, 3), np.float32)
    assert lib.crDenoiserPredictRows(X, base, rows, layered) == 0, eh.lastError(lib)
    assert np.array_equal(fused.reshape(-1, 3).view(np.uint32), layered.view(np.uint32))
    assert (X[:, 105:] == 0).all()
    # the tcgen05 kernel: the same network on the 5th-generation tensor cores
    # (fp32 sums in another order, so bf16 activations may round one step apart)
    assert lib.crSetDenoiserKernel(1) == 0
    try:
        lib.loadGlTFscene(info["gltf"].encode())
        eh.gotoFirstCompoundEye(lib)
        tc = np.zeros((3, n, 3), np.float32)
        assert lib.crDenoiserRenderPoses(poses, 3, 8, tc) == 0, eh.lastError(lib)
    finally:
        lib.crSetDenoiserKernel(1)
    params = np.zeros(mlp_ref.N_PARAMS, np.float32)
    grads = np.zeros(mlp_ref.N_PARAMS, np.float32)
    assert lib.crDenoiserGradient(X[:64].copy(), base[:64].copy(), base[:64].copy(), 64, grads, params) >= 0
    # Bounds in bf16 steps of each output's own pre-activation: a hidden bf16
    # activation that rounds one step (2^-8 relative) apart moves the output
    # by at most that step times its weight, so per row and channel the
    # difference is bounded by 8 bf16 steps of sum_j |H3[j] W4[j, c]| (and the
    # fp32 summation order by far less).
    Xf = mlp_ref.from_bits(X)
    _, (H1, H2, H3), (W1b, W2b, W3b, W4b) = mlp_ref.forward_parts(params, Xf)
    mag = (np.abs(H3) @ np.abs(W4b))[:, :3]
    tol = 2.0 ** -5 * mag + 1e-7
    terr = np.abs(tc.reshape(-1, 3) - layered)
    assert (terr <= tol).all(), ((terr > tol).sum(), (terr / tol).max())
    want = mlp_ref.predict(params, Xf, base)
    err = np.abs(layered - want)  # fp32 sums on the GPU against float64 here
    assert (err <= tol).all(), ((err > tol).sum(), (err / tol).max())


def test_training_beats_the_plain_low_sample_render(lib, tmp_path):
    # A terrain with an eye whose acceptance cones overlap their neighbours'
    # (droplet eye, 1500 ommatidia, 1.5-4 deg), as in the denoiser workload.
    info = scenes.terrain_scene(str(tmp_path), cells=128, extent=60.0, cones=300, n_omm=1500, poses=8)
    lib.loadGlTFscene(info["gltf"].encode())
    assert eh.lastError(lib) == ""
    eh.gotoFirstCompoundEye(lib)
    n = lib.getCurrentEyeOmmatidialCount()
    rng = np.random.default_rng(5)
    train = scenes.random_poses(info["height_fn"], 300, rng, 20.0)
    held = scenes.random_poses(info["height_fn"], 6, rng, 20.0)
    assert lib.crDenoiserInit(1) == 0
    assert lib.crDenoiserAddTrainingPoses(train, len(train), 8, 256) == 0, eh.lastError(lib)
    assert lib.crDenoiserTrainingRows() == len(train) * n
    loss = np.zeros(2000, np.float32)
    assert lib.crDenoiserTrain(2000, 4096, 1e-3, 3, loss.ctypes.data) == 0, eh.lastError(lib)
    assert loss[-50:].mean() < 0.5 * loss[:20].mean()
    learned = np.zeros((6, n, 3), np.float32)
    assert lib.crDenoiserRenderPoses(held, 6, 8, learned) == 0, eh.lastError(lib)
    # plain renders of the held-out poses: 8 samples, and 1024 as the reference
    lib.setCurrentEyeSamplesPerOmmatidium(8)
    plain8 = eh.renderPoses(lib, held)
    lib.setCurrentEyeSamplesPerOmmatidium(1024)
    ref = eh.renderPoses(lib, held)
    rmse_plain = np.sqrt(((plain8 - ref) ** 2).mean())
    rmse_learned = np.sqrt(((learned - ref) ** 2).mean())
    assert rmse_learned < 0.8 * rmse_plain, (rmse_learned, rmse_plain)

    # checkpoint round trip reproduces the learned render bit for bit
    path = str(tmp_path / "den.bin")
    assert lib.crDenoiserSave(path.encode()) == 0, eh.lastError(lib)
    assert lib.crDenoiserInit(99) == 0
    assert lib.crDenoiserLoad(path.encode()) == 0, eh.lastError(lib)
    # Reloading the scene restarts the denoiser's feature streams, so two
    # renders after a reload must agree bit for bit.
    lib.loadGlTFscene(info["gltf"].encode())
    eh.gotoFirstCompoundEye(lib)
    first = np.zeros_like(learned)
    again = np.zeros_like(learned)
    assert lib.crDenoiserRenderPoses(held, 6, 8, first) == 0
    lib.loadGlTFscene(info["gltf"].encode())
    eh.gotoFirstCompoundEye(lib)
    assert lib.crDenoiserRenderPoses(held, 6, 8, again) == 0
    assert np.array_equal(first, again)
    (tmp_path / "bad.bin").write_bytes(b"nope")
    assert lib.crDenoiserLoad(str(tmp_path / "bad.bin").encode()) == -1
    assert "checkpoint" in eh.lastError(lib)


def test_denoiser_gains_on_the_small_scene(lib, small, tmp_path):
    """The denoiser workload of the small scene (ground + 64 boxes, the
    1000-ommatidium eye with 3 deg acceptance, whose cones do not overlap):
    trained on 8-sample features of 200 random poses against 1024-sample
    targets, with the number of steps and the correction strength chosen on
    200 validation poses, it renders 1000 held-out poses with a lower RMSE
    against their 1024-sample render than the plain 8-sample render, in the
    worst channel.  A longer training over-fits these 200k rows, which the
    validation choice guards against."""
    import torch

    rng = np.random.default_rng(scenes.SEED + 11)
    train = scenes.open_poses(small["boxes"], 200, rng)
    held = scenes.open_poses(small["boxes"], 1000, rng)
    val = scenes.open_poses(small["boxes"], 200, rng)
    lib.crSetDenoiserKernel(1)
    lib.loadGlTFscene(small["gltf"].encode())
    assert eh.lastError(lib) == ""
    eh.gotoFirstCompoundEye(lib)
    N = lib.getCurrentEyeOmmatidialCount()
    assert lib.crDenoiserInit(1) == 0 and lib.crDenoiserAddTrainingPoses(train, 200, 8, 1024) == 0, eh.lastError(lib)

    def dev(p12):
        q = np.zeros((len(p12), 16), np.float32)
        for k in range(4):
            q[:, 4 * k:4 * k + 3] = p12[:, 3 * k:3 * k + 3]
        return torch.from_numpy(q).cuda()

    def worst(a, b):
        d = (a.astype(np.float64) - b).reshape(-1, 3)
        return float(np.sqrt((d * d).mean(axis=0)).max())

    def fetch(t):
        # The library renders on its own stream: wait for it before reading.
        assert lib.crSynchronize() == 0, eh.lastError(lib)
        return t.cpu().numpy()

    d_val, d_held = dev(val), dev(held)
    out_val = torch.empty((200, N, 3), dtype=torch.float32, device="cuda")
    out_held = torch.empty((1000, N, 3), dtype=torch.float32, device="cuda")
    lib.setCurrentEyeSamplesPerOmmatidium(1024)
    assert lib.crRenderPosesDevice(d_val.data_ptr(), 200, out_val.data_ptr()) == 0
    val_ref = fetch(out_val)
    assert lib.crRenderPosesDevice(d_held.data_ptr(), 1000, out_held.data_ptr()) == 0
    held_ref = fetch(out_held)
    lib.setCurrentEyeSamplesPerOmmatidium(8)
    assert lib.crRenderPosesDevice(d_held.data_ptr(), 1000, out_held.data_ptr()) == 0
    plain8 = fetch(out_held)

    def val_rmse():
        assert lib.crDenoiserRenderPosesDevice(d_val.data_ptr(), 200, 8, out_val.data_ptr()) == 0, eh.lastError(lib)
        return worst(fetch(out_val), val_ref)

    ck = lambda name: str(tmp_path / name).encode()
    assert lib.crDenoiserSave(ck("init.bin")) == 0
    by_steps = {}
    for st in (500, 1000, 2000):
        assert lib.crDenoiserLoad(ck("init.bin")) == 0
        assert lib.crDenoiserTrain(st, 8192, 1e-3, 3, None) == 0, eh.lastError(lib)
        by_steps[st] = val_rmse()
        assert lib.crDenoiserSave(ck("s%d.bin" % st)) == 0
    best = min(by_steps, key=by_steps.get)
    by_alpha = {}
    for a in (1.0, 0.75, 0.5, 0.25, 0.0):
        assert lib.crDenoiserLoad(ck("s%d.bin" % best)) == 0 and lib.crDenoiserScaleOutput(a) == 0
        by_alpha[a] = val_rmse()
    alpha = min(by_alpha, key=by_alpha.get)
    assert lib.crDenoiserLoad(ck("s%d.bin" % best)) == 0 and lib.crDenoiserScaleOutput(alpha) == 0
    assert lib.crDenoiserRenderPosesDevice(d_held.data_ptr(), 1000, 8, out_held.data_ptr()) == 0
    learned = fetch(out_held)
    r_learned, r_plain = worst(learned, held_ref), worst(plain8, held_ref)
    print("steps", by_steps, "alpha", by_alpha, "held-out", r_learned, r_plain)
    assert r_learned < r_plain, (r_learned, r_plain, by_steps, by_alpha)
    assert lib.crDenoiserScaleOutput(1.5) == -1


def test_adam_step_matches_reference_bit_for_bit(lib):
    """adamKernel, as the training loop calls it (step size and bias
    corrections from the device schedule), against oracle/mlp_ref.adam_step:
    the fp32 master weights, both moments and the bf16 copies, bit for bit,
    over two consecutive steps; gradients span zeros, tiny and large values."""
    rng = np.random.default_rng(21)
    n = 50000
    w = rng.normal(0, 0.1, n).astype(np.float32)
    m = np.zeros(n, np.float32)
    v = np.zeros(n, np.float32)
    gw, gm, gv = w.copy(), m.copy(), v.copy()
    for t, lr in ((1, 1e-3), (2, 7.5e-4)):
        g = (rng.normal(0, 1, n) * 10.0 ** rng.uniform(-12, 2, n)).astype(np.float32)
        g[rng.integers(0, n, 500)] = 0.0
        c1 = np.float32(1.0) / (np.float32(1.0) - np.float32(0.9) ** np.float32(t))
        c2 = np.float32(1.0) / (np.float32(1.0) - np.float32(0.999) ** np.float32(t))
        bits = np.zeros(n, np.uint16)
        assert lib.crDenoiserAdamStep(gw, g, gm, gv, n, lr, float(c1), float(c2), bits) == 0, eh.lastError(lib)
        w, m, v, wb = mlp_ref.adam_step(w, g, m, v, lr, c1, c2)
        for name, a, b in (("w", gw, w), ("m", gm, m), ("v", gv, v)):
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), (name, t, np.flatnonzero(a != b)[:5])
        assert np.array_equal(bits, wb), (t, np.flatnonzero(bits != wb)[:5])
