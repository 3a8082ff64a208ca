"""The C-ABI library loads and exports every entry point that
include/libEyeRenderer.h declares (symbol lookup only, no calls)."""
import ctypes
import os
import re

import eyeRendererHelperFunctions as eh

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "libEyeRenderer.h")

# The reference's extern "C" block (libEyeRenderer3/libEyeRenderer.h:16-67).
REFERENCE_ENTRY_POINTS = [
    "setVerbosity", "loadGlTFscene", "stop", "setRenderSize", "renderFrame", "displayFrame", "saveFrameAs",
    "getFramePointer", "getCameraCount", "nextCamera", "previousCamera", "getCurrentCameraIndex",
    "getCurrentCameraName", "gotoCamera", "gotoCameraByName", "setCameraPosition", "getCameraPosition",
    "setCameraLocalSpace", "rotateCameraAround", "rotateCameraLocallyAround", "translateCamera",
    "translateCameraLocally", "resetCameraPose", "setCameraPose", "isCompoundEyeActive",
    "setCurrentEyeSamplesPerOmmatidium", "getCurrentEyeSamplesPerOmmatidium",
    "changeCurrentEyeSamplesPerOmmatidiumBy", "getCurrentEyeOmmatidialCount", "setOmmatidia",
    "getCurrentEyeDataPath", "setCurrentEyeShaderName", "isInsideHitGeometry", "getGeometryMaxBounds",
    "getGeometryMinBounds",
]


def declared_c_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    block = text[text.index('extern "C" {') + len('extern "C" {'):]
    depth, end = 1, 0
    for i, ch in enumerate(block):
        depth += ch == "{"
        depth -= ch == "}"
        if depth == 0:
            end = i
            break
    block = block[:end]
    return re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\([^;{]*\)\s*;", block)


def test_header_lists_every_reference_entry_point():
    names = set(declared_c_functions())
    missing = [n for n in REFERENCE_ENTRY_POINTS if n not in names]
    assert not missing, missing


def test_library_exports_every_declared_symbol(lib):
    names = declared_c_functions()
    assert len(names) >= len(REFERENCE_ENTRY_POINTS)
    raw = ctypes.CDLL(eh.LIB_PATH)
    missing = [n for n in names if not hasattr(raw, n)]
    assert not missing, missing
    # getWindowPointer is declared outside the extern "C" block in the
    # reference too (C++ linkage).
    assert hasattr(raw, "_Z16getWindowPointerv")


def test_loading_opens_no_window():
    import subprocess
    import sys

    code = "import ctypes; ctypes.CDLL(%r); print('loaded')" % eh.LIB_PATH
    out = subprocess.run([sys.executable, "-c", code], env={"PATH": os.environ.get("PATH", ""), "DISPLAY": ""},
                         capture_output=True, text=True, timeout=60)
    assert out.returncode == 0 and "loaded" in out.stdout
