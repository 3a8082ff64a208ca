"""Batched rendering of uneven eyes in one persistent, graph-captured launch
must give exactly what rendering each eye on its own gives."""
import ctypes

import numpy as np
import pytest

import eyeRendererHelperFunctions as eh
import scenes

pytestmark = pytest.mark.gpu


def _p16(poses12):
    p = np.asarray(poses12, np.float32).reshape(-1, 12)
    out = np.zeros((len(p), 16), np.float32)
    for k in range(4):
        out[:, 4 * k:4 * k + 3] = p[:, 3 * k:3 * k + 3]
    return out


@pytest.mark.parametrize("cut", [0.0, 1.0 / 16])
def test_batch_equals_per_eye_renders(lib, tmp_path, cut):
    """cut: near-field cut radius (fraction of the scene extent) in force when
    the batch is recorded; the per-eye references are rendered without one."""
    try:
        _batch_case(lib, tmp_path, cut)
    finally:
        lib.crSetCutRadius(0.0)


def _batch_case(lib, tmp_path, cut):
    import torch

    lib.crSetCutRadius(0.0)
    info = scenes.batch_scene(str(tmp_path), n_eyes=5, poses_per_eye=3, n_min=100, n_max=700,
                              spp_choices=(8, 32, 48, 100, 5))
    lib.loadGlTFscene(info["gltf"].encode())
    assert eh.lastError(lib) == ""
    first = info["first_batch_camera"]
    cams = np.arange(first, first + 5, dtype=np.int32)
    P = 3
    d_poses = torch.from_numpy(_p16(info["poses"].reshape(-1, 12))).cuda()
    sizes = [n * P * 3 for n in info["n"]]
    refs = [[], []]
    for i, c in enumerate(cams):
        lib.gotoCamera(int(c))
        lib.setCurrentEyeSamplesPerOmmatidium(info["spp"][i])
        assert lib.getCurrentEyeOmmatidialCount() == info["n"][i]
        for k in range(2):
            out = torch.empty(sizes[i], dtype=torch.float32, device="cuda")
            assert lib.crRenderPosesDevice(d_poses[i * P].data_ptr(), P, out.data_ptr()) == 0, eh.lastError(lib)
            assert lib.crSynchronize() == 0
            refs[k].append(out.cpu().numpy())
    # Reset every eye's streams, then render all eyes in one batch.
    for i, c in enumerate(cams):
        lib.gotoCamera(int(c))
        lib.setCurrentEyeSamplesPerOmmatidium(info["spp"][i])
    d_out = torch.zeros(sum(sizes), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    assert lib.crSetCutRadius(cut) == 0
    h = lib.crBatchCreate(cams, len(cams), P, d_poses.data_ptr(), d_out.data_ptr())
    assert h > 0, eh.lastError(lib)
    lat = np.zeros(len(cams), np.float32)
    total = ctypes.c_float(0)
    for k in range(2):
        assert lib.crBatchLaunch(h) == 0, eh.lastError(lib)
        assert lib.crBatchLatencies(h, lat, ctypes.byref(total)) == 0, eh.lastError(lib)
        got = d_out.cpu().numpy()
        for i in range(len(cams)):
            off = lib.crBatchOutputOffset(h, i)
            assert off == sum(sizes[:i])
            assert np.array_equal(got[off:off + sizes[i]], refs[k][i]), "eye %d launch %d" % (i, k)
        assert (lat > 0).all() and (lat <= total.value + 1e-3).all()
    # Changing an eye invalidates the batch.
    lib.gotoCamera(int(cams[0]))
    lib.setCurrentEyeSamplesPerOmmatidium(info["spp"][0] + 16)
    assert lib.crBatchLaunch(h) == -1
    assert "invalidated" in eh.lastError(lib)
    assert lib.crBatchDestroy(h) == 0
    assert lib.crBatchLaunch(h) == -1
    assert "unknown batch handle" in eh.lastError(lib)
    # The one-shot form (create, launch, wait, destroy) gives the same frames.
    for i, c in enumerate(cams):
        lib.gotoCamera(int(c))
        lib.setCurrentEyeSamplesPerOmmatidium(info["spp"][i])
    d_out.zero_()
    assert lib.renderBatch(cams, len(cams), P, d_poses.data_ptr(), d_out.data_ptr()) == 0, eh.lastError(lib)
    got = d_out.cpu().numpy()
    for i in range(len(cams)):
        off = sum(sizes[:i])
        assert np.array_equal(got[off:off + sizes[i]], refs[0][i]), "one-shot batch, eye %d" % i
    assert lib.renderBatch(cams, 0, P, d_poses.data_ptr(), d_out.data_ptr()) == -1
    assert "empty batch" in eh.lastError(lib)
