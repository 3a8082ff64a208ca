import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for sub in ("compound-ray_gb300", "oracle"):
    p = os.path.join(ROOT, sub)
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300 / sm_103a)")


@pytest.fixture(scope="session")
def lib():
    import eyeRendererHelperFunctions as eh

    L = eh.loadRenderer()
    L.setVerbosity(False)
    return L


@pytest.fixture(scope="session")
def small(tmp_path_factory):
    import scenes

    return scenes.small_scene(str(tmp_path_factory.mktemp("small")))


@pytest.fixture(scope="session")
def small_ref(small):
    import gltf_ref
    import oracle

    ref = gltf_ref.load(small["gltf"])
    v, c, f = ref.arrays()
    return ref, oracle.OracleScene(v, c, f, ref.miss)
