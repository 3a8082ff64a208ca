"""GPU parity at the benchmark workloads' real sizes.

The parity tests of test_gpu_parity.py run on scenes of a few thousand
triangles.  These render the benchmark workloads themselves and check them
against the CPU oracle on the GPU's own rays, with the same bars
(parity_checks: hit ids, distances and barycentrics bit-exact, fp64
disagreements only within 1e-6 of an edge, RGB within 1e-5 relative), on
every ray of the rendered frames:

  * the terrain trajectory (588,288 triangles, 6000-ommatidium droplet eye,
    256 samples: eight 32-sample chunks per ommatidium summed in chunk
    order, render variant 2 and the near-field cut at 1/128 of the scene
    extent, the autotuner's choices), two poses; the production render of
    the same frames through crRenderPoses must give the recorded frames'
    sums bit for bit;
  * the sample-allocator scene (9,028,608 triangles) on the GPU-built linear
    BVH (63-bit Morton codes), 100,000-ommatidium panoramic eye, one pose at
    16 samples;
  * one eye of the uneven batch (the eye of at most 4 M rays per pose with
    the most samples) rendered inside the persistent batch launch: its
    first frame must equal a recorded render of the same frame bit for bit,
    and that record passes the oracle checks.

Each renders the reference's path (libEyeRenderer3/shaders.cu:664-731 with
the summing of :341-347) at the workload's N and spp.
"""
import numpy as np
import pytest

import eyeRendererHelperFunctions as eh
import scenes
from parity_checks import _check_frame, _load, _oracle

pytestmark = pytest.mark.gpu


def _set_pose(lib, p12):
    lib.setCameraPosition(*[float(v) for v in p12[:3]])
    lib.setCameraLocalSpace(*[float(v) for v in p12[3:]])


def _restart_streams(lib, spp):
    """A sample-count change re-initialises the generators (as the
    reference's CompoundEye.cpp:98-115): the next frame is frame 0 again."""
    lib.setCurrentEyeSamplesPerOmmatidium(spp + 1)
    lib.setCurrentEyeSamplesPerOmmatidium(spp)


def test_terrain_workload_at_full_size(lib, tmp_path):
    info = scenes.terrain_scene(str(tmp_path), poses=4)
    assert info["triangles"] == 588288 and info["n_omm"] == 6000 and info["spp"] == 256
    ref, sc, omm = _oracle(info["gltf"])
    spp = 256
    assert lib.crSetBvhBuilder(0) == 0
    assert lib.crSetRenderVariant(2) == 0 and lib.crSetCutRadius(1.0 / 128) == 0
    try:
        _load(lib, info["gltf"], spp)
        assert lib.getCurrentEyeOmmatidialCount() == 6000
        poses = info["poses"][:2]
        recorded = []
        for p in poses:
            _set_pose(lib, p)
            rec, sums = _check_frame(lib, sc, omm, spp, p)
            assert (rec["hitId"] >= 0).mean() > 0.5
            recorded.append(sums)
        # The production path: the same two frames through crRenderPoses.
        _restart_streams(lib, spp)
        out = eh.renderPoses(lib, poses)
        assert eh.lastError(lib) == ""
        assert np.array_equal(out, np.stack(recorded)), "production render differs from the recorded frames"
    finally:
        lib.crSetCutRadius(0.0)


def test_large_scene_on_gpu_linear_bvh(lib, tmp_path):
    info = scenes.terrain_scene(str(tmp_path), cells=2048, extent=400.0, cones=20000, n_omm=100000, poses=2,
                                eye_kind="panoramic", aa_deg=(0.5, 5.0))
    assert info["triangles"] == 9028608
    ref, sc, omm = _oracle(info["gltf"])
    spp = 16
    assert lib.crSetBvhBuilder(1) == 0
    try:
        _load(lib, info["gltf"], spp)
        p = info["poses"][0]
        _set_pose(lib, p)
        rec, _ = _check_frame(lib, sc, omm, spp, p)
        assert (rec["hitId"] >= 0).mean() > 0.3
    finally:
        lib.crSetBvhBuilder(0)


def test_uneven_batch_eye(lib, tmp_path):
    import torch

    info = scenes.batch_scene(str(tmp_path))
    n_eyes, P = len(info["n"]), info["poses"].shape[1]
    first = info["first_batch_camera"]
    cams = np.arange(first, first + n_eyes, dtype=np.int32)
    eh.lastError(lib)
    lib.loadGlTFscene(info["gltf"].encode())
    assert eh.lastError(lib) == ""
    for i, c in enumerate(cams):
        lib.gotoCamera(int(c))
        lib.setCurrentEyeSamplesPerOmmatidium(int(info["spp"][i]))
    rays = np.array([n * s for n, s in zip(info["n"], info["spp"])])
    k = int(max(np.flatnonzero(rays <= 4_000_000), key=lambda i: (info["spp"][i], rays[i])))
    p16 = np.zeros((n_eyes * P, 16), np.float32)
    p12 = info["poses"].reshape(-1, 12)
    for j in range(4):
        p16[:, 4 * j:4 * j + 3] = p12[:, 3 * j:3 * j + 3]
    d_poses = torch.from_numpy(p16).cuda()
    d_out = torch.zeros(sum(3 * P * n for n in info["n"]), dtype=torch.float32, device="cuda")
    h = lib.crBatchCreate(cams, n_eyes, P, d_poses.data_ptr(), d_out.data_ptr())
    assert h > 0, eh.lastError(lib)
    assert lib.crBatchLaunch(h) == 0, eh.lastError(lib)
    assert lib.crSynchronize() == 0, eh.lastError(lib)
    off = lib.crBatchOutputOffset(h, k)
    N = int(info["n"][k])
    batch_first = d_out[off:off + 3 * N].cpu().numpy().reshape(N, 3)
    assert lib.crBatchDestroy(h) == 0

    # The same eye's first frame, recorded, against the batch and the oracle.
    ref, sc, _ = _oracle(info["gltf"])
    lib.gotoCamera(int(cams[k]))
    spp = int(info["spp"][k])
    _restart_streams(lib, spp)
    omm = eh.getOmmatidia(lib)
    assert len(omm) == N
    pose = info["poses"][k, 0]
    _set_pose(lib, pose)
    rec, sums = _check_frame(lib, sc, omm, spp, pose)
    assert np.array_equal(sums, batch_first), "batched frame differs from the recorded frame"
