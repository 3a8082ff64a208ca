"""The allocation-free render entry point (crRenderPosesDeviceNoAlloc).

It serves callers that cannot allocate device memory while they render (a
stream being captured into a graph, a real-time loop, a host whose device
memory belongs to another allocator).  It must give what crRenderPosesDevice
gives: two identical eyes of one scene are rendered, one through each entry
point, and two consecutive no-alloc calls must match the second and third
calls of the allocating one.  Collected last so a failure here leaves every
other test already run.
"""
import ctypes

import numpy as np
import pytest

import eyeRendererHelperFunctions as eh
import scenes

pytestmark = pytest.mark.gpu

def _scene(tmp_path):
    g = scenes.GltfBuilder()
    g.scene_extras = {"background-shader": "simple_sky"}
    rng = np.random.default_rng(11)
    ground = np.array([[-10, 0, -10], [10, 0, -10], [10, 0, 10], [-10, 0, 10]], np.float64)
    g.mesh("ground", ground, np.array([[0, 2, 1], [0, 3, 2]]), colours=np.tile([0.5, 0.5, 0.5, 1.0], (4, 1)))
    verts, faces, cols = [], [], []
    for k in range(24):
        c = rng.uniform(-6, 6, size=2)
        if abs(c[0]) < 1.5 and abs(c[1]) < 1.5:
            c += 3.0
        v, f = scenes.box_mesh([c[0] - 0.5, 0.0, c[1] - 0.5], [c[0] + 0.5, rng.uniform(0.3, 2.0), c[1] + 0.5])
        faces.append(f + 8 * k)
        verts.append(v)
        cols.append(np.concatenate([rng.uniform(0, 1, size=(8, 3)), np.ones((8, 1))], axis=1))
    g.mesh("boxes", np.concatenate(verts), np.concatenate(faces), colours=np.concatenate(cols))
    d = scenes.fibonacci_sphere(300)
    scenes.write_eye(str(tmp_path / "eye.eye"), d * 0.001, d, 0.06, 0.0)
    g.compound_camera("eye-a", "eye.eye")
    g.compound_camera("eye-b", "eye.eye")
    return g.write(str(tmp_path / "noalloc.gltf"))


def _device_poses(P):
    import torch

    rows = np.stack([scenes.pose_rows(np.array([0.2 * k, 0.5, -0.1 * k]), 0.4 * k) for k in range(P)])
    p16 = np.zeros((P, 16), np.float32)
    for k in range(4):
        p16[:, 4 * k:4 * k + 3] = rows[:, 3 * k:3 * k + 3]
    return torch.from_numpy(p16).cuda()


def test_no_alloc_matches_allocating_entry_point(lib, tmp_path):
    import torch

    lib.setVerbosity(False)
    eh.lastError(lib)  # start from a clean error state whatever ran before
    lib.loadGlTFscene(_scene(tmp_path).encode())
    assert eh.lastError(lib) == ""
    spp, P, N = 100, 6, 300  # spp > 32: the render uses chunk scratch
    poses = _device_poses(P)
    outs = [torch.empty((P, N, 3), dtype=torch.float32, device="cuda") for _ in range(6)]
    torch.cuda.synchronize()

    # Eye A through the allocating entry point: three calls in a row.
    assert lib.gotoCameraByName(b"eye-a")
    lib.setCurrentEyeSamplesPerOmmatidium(spp)
    for k in range(3):
        assert lib.crRenderPosesDevice(poses.data_ptr(), P, outs[k].data_ptr()) == 0, eh.lastError(lib)
    assert lib.crSynchronize() == 0, eh.lastError(lib)

    # Eye B: the same eye.  Its first frames come from the allocating entry
    # point (which sets up its device state), the next two from the
    # allocation-free one.
    assert lib.gotoCameraByName(b"eye-b")
    lib.setCurrentEyeSamplesPerOmmatidium(spp)
    assert lib.crRenderPosesDeviceNoAlloc(poses.data_ptr(), P, outs[5].data_ptr()) == -1
    assert "not set up" in eh.lastError(lib)
    assert lib.crRenderPosesDevice(poses.data_ptr(), P, outs[3].data_ptr()) == 0, eh.lastError(lib)
    assert lib.crSynchronize() == 0
    free_before = torch.cuda.mem_get_info()[0]
    assert lib.crRenderPosesDeviceNoAlloc(poses.data_ptr(), P, outs[4].data_ptr()) == 0, eh.lastError(lib)
    assert lib.crRenderPosesDeviceNoAlloc(poses.data_ptr(), P, outs[5].data_ptr()) == 0, eh.lastError(lib)
    assert lib.crSynchronize() == 0, eh.lastError(lib)
    assert torch.cuda.mem_get_info()[0] == free_before

    # Same draws, rays, hits and chunk sums in the same order: the bits agree,
    # although the allocating call pre-draws the random numbers and spreads
    # the poses over more warps while the allocation-free one does not.
    a = [o.cpu().numpy() for o in outs]
    assert np.array_equal(a[3], a[0])
    assert np.array_equal(a[4], a[1])
    assert np.array_equal(a[5], a[2])
    assert not np.array_equal(a[4], a[5])  # the streams advanced between the two calls


def test_no_alloc_rejects_oversized_eyes(lib, tmp_path):
    lib.loadGlTFscene(_scene(tmp_path).encode())
    assert lib.gotoCameraByName(b"eye-a")
    n = 50000
    pk = [eh.c_ommatidiumPacket(0, 0, 0, 0, 1, 0, 0.05, 0.0)] * n
    eh.setOmmatidiaFromPacketList(lib, pk)
    lib.setCurrentEyeSamplesPerOmmatidium(1024)  # 50000 * 32 * 3 floats per pose > 4 Mi
    dummy = ctypes.c_float(0.0)
    assert lib.crRenderPosesDeviceNoAlloc(ctypes.addressof(dummy), 1, ctypes.addressof(dummy)) == -1
    assert "floats of scratch per pose" in eh.lastError(lib)
