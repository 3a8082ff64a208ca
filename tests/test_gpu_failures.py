"""Failure paths, exercised without faulting the GPU: an allocation refused
by the library's device-memory cap (the allocator's fault injection) and the
tcgen05 kernels' bounded mbarrier wait running out on a barrier that nothing
arrives on.  Either way the call reports an error and the library keeps
working."""
import numpy as np
import pytest

import eyeRendererHelperFunctions as eh

pytestmark = pytest.mark.gpu


def _load(lib, path, spp):
    eh.lastError(lib)
    lib.loadGlTFscene(path.encode())
    assert eh.lastError(lib) == ""
    eh.gotoFirstCompoundEye(lib)
    lib.setCurrentEyeSamplesPerOmmatidium(spp)


def test_device_memory_cap_refuses_and_recovers(lib, small):
    _load(lib, small["gltf"], 32)
    poses = np.stack([small["pose"]] * 3).astype(np.float32)
    want = eh.renderPoses(lib, poses)
    held = lib.crGetDeviceMemoryHeld()
    assert held > 0
    try:
        _load(lib, small["gltf"], 32)  # a fresh scene and eye: everything is allocated again
        assert lib.crSetDeviceMemoryCap(4096) == 0
        out = np.zeros((3, lib.getCurrentEyeOmmatidialCount(), 3), np.float32)
        assert lib.crRenderPoses(poses, 3, out) == -1
        assert "device memory cap reached" in eh.lastError(lib)
    finally:
        lib.crSetDeviceMemoryCap(0)
    _load(lib, small["gltf"], 32)
    got = eh.renderPoses(lib, poses)
    assert np.array_equal(got, want)


def test_bounded_wait_runs_out_and_reports(lib, small):
    _load(lib, small["gltf"], 8)
    assert lib.crSelfTestBoundedWait(1000) == 1, eh.lastError(lib)
    # the context is still usable and the error word is clear
    assert lib.renderFrame() >= 0, eh.lastError(lib)
    assert eh.lastError(lib) == ""
