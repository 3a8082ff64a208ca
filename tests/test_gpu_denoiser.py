"""The learned denoiser: GPU gradients against the numpy reference, training
on renders of this renderer, the gain over the plain low-sample render, and
the checkpoint round trip."""
import numpy as np
import pytest

import eyeRendererHelperFunctions as eh
import mlp_ref
import scenes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("rows", [64, 500])
def test_gradients_match_reference(lib, rows):
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
    for lo, hi, name in [(mlp_ref.OFF_W1, mlp_ref.OFF_B1, "W1"), (mlp_ref.OFF_B1, mlp_ref.OFF_W2, "b1"),
                         (mlp_ref.OFF_W2, mlp_ref.OFF_B2, "W2"), (mlp_ref.OFF_W3, mlp_ref.OFF_B3, "W3"),
                         (mlp_ref.OFF_W4, mlp_ref.OFF_B4, "W4"), (mlp_ref.OFF_B4, mlp_ref.N_PARAMS, "b4")]:
        a, b = grads[lo:hi].astype(np.float64), ref_g[lo:hi]
        rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
        assert rel < 2e-2, "%s gradient relative error %.3g" % (name, rel)


def test_training_beats_the_plain_low_sample_render(lib, tmp_path):
    info = scenes.small_scene(str(tmp_path), n_omm=400)
    lib.loadGlTFscene(info["gltf"].encode())
    assert eh.lastError(lib) == ""
    eh.gotoFirstCompoundEye(lib)
    rng = np.random.default_rng(5)

    def poses(k):
        return np.stack([scenes.pose_rows(np.array([rng.uniform(-6, 6), 0.5, rng.uniform(-6, 6)]),
                                          rng.uniform(0, 2 * np.pi)) for _ in range(k)])

    train, held = poses(40), poses(6)
    assert lib.crDenoiserInit(1) == 0
    assert lib.crDenoiserAddTrainingPoses(train, len(train), 8, 256) == 0, eh.lastError(lib)
    assert lib.crDenoiserTrainingRows() == 40 * 400
    loss = np.zeros(600, np.float32)
    assert lib.crDenoiserTrain(600, 1024, 2e-3, 3, loss.ctypes.data) == 0, eh.lastError(lib)
    assert loss[-50:].mean() < 0.5 * loss[:20].mean()
    learned = np.zeros((6, 400, 3), np.float32)
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
