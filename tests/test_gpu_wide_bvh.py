"""The wide BVH (4 or 8 children, 8-bit quantised child boxes) on the GPU:
every closest hit, and so every render, is the same bits as on the two-wide
BVH, for the plain render (host-built and GPU-built trees), the batched
launch and the adaptive kernel; and the wide trees need fewer node visits.
The reference's equivalent is the OptiX acceleration structure
(libEyeRenderer3/MulticamScene.cpp:1052-1428), which is closed code: the
closest hit, not the tree, is what is compared."""
import ctypes

import numpy as np
import pytest

import eyeRendererHelperFunctions as eh
import scenes

pytestmark = pytest.mark.gpu


def _render_widths(lib, path, spp, poses, builder=0):
    outs = {}
    try:
        assert lib.crSetBvhBuilder(builder) == 0
        for W in (2, 4, 8):
            assert lib.crSetBvhWidth(W) == 0
            eh.lastError(lib)
            lib.loadGlTFscene(path.encode())
            assert eh.lastError(lib) == ""
            eh.gotoFirstCompoundEye(lib)
            lib.setCurrentEyeSamplesPerOmmatidium(spp)
            outs[W] = eh.renderPoses(lib, poses)
            assert eh.lastError(lib) == ""
            if W > 2:
                nodes, depth, kids = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_double()
                assert lib.crGetWideBvhStats(ctypes.byref(nodes), ctypes.byref(depth), ctypes.byref(kids)) == 0
                assert nodes.value > 0 and kids.value > 2.5
    finally:
        lib.crSetBvhWidth(2)
        lib.crSetBvhBuilder(0)
    return outs


@pytest.mark.parametrize("builder", [0, 1])
def test_wide_bvh_renders_identical_bits(lib, small, tmp_path, builder):
    info = scenes.terrain_scene(str(tmp_path), cells=96, extent=50.0, cones=200, n_omm=800, poses=4)
    for path, spp, poses in ((small["gltf"], 32, np.stack([small["pose"]] * 2)), (info["gltf"], 48, info["poses"])):
        outs = _render_widths(lib, path, spp, poses, builder)
        assert np.array_equal(outs[4], outs[2])
        assert np.array_equal(outs[8], outs[2])


def test_wide_bvh_visits_fewer_nodes(lib, tmp_path):
    import torch

    info = scenes.terrain_scene(str(tmp_path), cells=128, extent=60.0, cones=300, n_omm=600, poses=4)
    p16 = np.zeros((4, 16), np.float32)
    for k in range(4):
        p16[:, 4 * k:4 * k + 3] = info["poses"][:, 3 * k:3 * k + 3]
    d = torch.from_numpy(p16).cuda()
    visits = {}
    try:
        for W in (2, 4, 8):
            assert lib.crSetBvhWidth(W) == 0
            lib.loadGlTFscene(info["gltf"].encode())
            eh.gotoFirstCompoundEye(lib)
            lib.setCurrentEyeSamplesPerOmmatidium(16)
            nv, tt = ctypes.c_double(), ctypes.c_double()
            assert lib.crMeasureTraversal(d.data_ptr(), 4, ctypes.byref(nv), ctypes.byref(tt)) == 0, eh.lastError(lib)
            visits[W] = (nv.value, tt.value)
    finally:
        lib.crSetBvhWidth(2)
    assert visits[4][0] < 0.7 * visits[2][0] and visits[8][0] < visits[4][0]
    # the same leaves are reached: triangle tests within a few percent
    assert abs(visits[4][1] - visits[2][1]) < 0.25 * visits[2][1]


def test_wide_bvh_batch_and_adaptive_identical(lib, small):
    """The batched launch and the adaptive kernel search the wide tree too."""
    import torch

    poses = np.stack([small["pose"], scenes.pose_rows(np.array([1.0, 0.7, -2.0]), 0.8)]).astype(np.float32)
    res = {}
    try:
        for W in (2, 4, 8):
            assert lib.crSetBvhWidth(W) == 0
            lib.loadGlTFscene(small["gltf"].encode())
            eh.gotoFirstCompoundEye(lib)
            N = lib.getCurrentEyeOmmatidialCount()
            rec = np.zeros((2 * N * 64,), eh.RAY_RECORD_DTYPE)
            sums = np.zeros((2, N, 3), np.float32)
            assert lib.crAdaptiveRecord(poses, 2, 64, 7, rec.ctypes.data, sums) == 0, eh.lastError(lib)
            cam = np.array([lib.getCurrentCameraIndex()], np.int32)
            lib.setCurrentEyeSamplesPerOmmatidium(48)
            p16 = np.zeros((2, 16), np.float32)
            for k in range(4):
                p16[:, 4 * k:4 * k + 3] = poses[:, 3 * k:3 * k + 3]
            d_p = torch.from_numpy(p16).cuda()
            d_o = torch.zeros(2 * N * 3, dtype=torch.float32, device="cuda")
            assert lib.renderBatch(cam, 1, 2, d_p.data_ptr(), d_o.data_ptr()) == 0, eh.lastError(lib)
            res[W] = (rec["hitId"].copy(), sums, d_o.cpu().numpy())
    finally:
        lib.crSetBvhWidth(2)
    for W in (4, 8):
        for a, b in zip(res[W], res[2]):
            assert np.array_equal(a, b), W
