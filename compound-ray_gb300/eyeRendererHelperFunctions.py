"""ctypes helpers for libEyeRenderer3.so.

Same helper names and behaviour as the reference's
python-examples/eyeRendererHelperFunctions.py (configureFunctions,
setRenderSize, setOmmatidiaFromPacketList, readEyeFile, ...), so its callers
run unchanged, plus `configureExtras` for the entry points this library adds
and `loadRenderer` which finds (or builds) the in-tree library.  The one
deliberate difference: getCameraPosition is bound with its real signature
(three float pointers); the reference helper declares a double-array return
type that does not match the C function.
"""
import ctypes
import math
import os
from ctypes import (CDLL, POINTER, Structure, c_bool, c_char_p, c_double, c_float, c_int, c_size_t, c_ubyte,
                    c_uint, c_uint32, c_ulonglong, c_void_p)

import numpy as np
from numpy.ctypeslib import ndpointer

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libEyeRenderer3.so")


class c_float3(Structure):
    _fields_ = [("x", c_float), ("y", c_float), ("z", c_float)]

    def toNumpy(self):
        return np.asarray([self.x, self.y, self.z])


class Ommatidium:
    def __init__(self, position, direction, acceptanceAngle, focalpointOffset):
        self.position = position
        self.direction = direction
        self.acceptanceAngle = acceptanceAngle
        self.focalpointOffset = focalpointOffset

    def getSolidAngle(self):
        """Solid angle (steradians) of this ommatidium's cone of vision."""
        return 2.0 * math.pi * (1.0 - math.cos(self.acceptanceAngle / 2.0))

    def copy(self):
        return Ommatidium(self.position.copy(), self.direction.copy(), self.acceptanceAngle, self.focalpointOffset)


class c_ommatidiumPacket(Structure):
    _fields_ = [("posX", c_float), ("posY", c_float), ("posZ", c_float),
                ("dirX", c_float), ("dirY", c_float), ("dirZ", c_float),
                ("acceptanceAngle", c_float), ("focalpointOffset", c_float)]


RAY_RECORD_DTYPE = np.dtype([("normalDraw", "<f4"), ("uniformDraw", "<f4"), ("origin", "<f4", 3),
                             ("direction", "<f4", 3), ("t", "<f4"), ("b1", "<f4"), ("b2", "<f4"),
                             ("hitId", "<i4"), ("rgb", "<f4", 3), ("pad", "<f4")])
assert RAY_RECORD_DTYPE.itemsize == 64


def loadRenderer(path=None, build_if_missing=True):
    """Loads libEyeRenderer3.so (building it in place when absent) and binds
    every entry point.  Raises if the library cannot be built or loaded."""
    path = path or LIB_PATH
    if not os.path.exists(path):
        if not build_if_missing:
            raise FileNotFoundError(path)
        import importlib.util
        spec = importlib.util.spec_from_file_location("cr_build", os.path.join(HERE, "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
    lib = CDLL(path)
    configureFunctions(lib)
    configureExtras(lib)
    return lib


def configureFunctions(eyeRenderer):
    """Configures argument and return types of the reference entry points."""
    eyeRenderer.setVerbosity.argtypes = [c_bool]
    eyeRenderer.loadGlTFscene.argtypes = [c_char_p]
    eyeRenderer.renderFrame.restype = c_double
    eyeRenderer.getCameraCount.restype = c_size_t
    eyeRenderer.getCurrentCameraIndex.restype = c_size_t
    eyeRenderer.getCurrentCameraName.restype = c_char_p
    eyeRenderer.gotoCamera.argtypes = [c_int]
    eyeRenderer.gotoCameraByName.argtypes = [c_char_p]
    eyeRenderer.gotoCameraByName.restype = c_bool
    eyeRenderer.setCameraPosition.argtypes = [c_float] * 3
    eyeRenderer.getCameraPosition.argtypes = [POINTER(c_float)] * 3
    eyeRenderer.getCameraPosition.restype = None
    eyeRenderer.setCameraLocalSpace.argtypes = [c_float] * 9
    eyeRenderer.rotateCameraAround.argtypes = [c_float] * 4
    eyeRenderer.rotateCameraLocallyAround.argtypes = [c_float] * 4
    eyeRenderer.translateCamera.argtypes = [c_float] * 3
    eyeRenderer.translateCameraLocally.argtypes = [c_float] * 3
    eyeRenderer.isCompoundEyeActive.restype = c_bool
    eyeRenderer.setCurrentEyeSamplesPerOmmatidium.argtypes = [c_int]
    eyeRenderer.getCurrentEyeSamplesPerOmmatidium.restype = c_int
    eyeRenderer.changeCurrentEyeSamplesPerOmmatidiumBy.argtypes = [c_int]
    eyeRenderer.getCurrentEyeOmmatidialCount.restype = c_size_t
    eyeRenderer.getCurrentEyeDataPath.restype = c_char_p
    eyeRenderer.setCurrentEyeShaderName.argtypes = [c_char_p]
    eyeRenderer.setCameraPose.argtypes = [c_float] * 6
    eyeRenderer.saveFrameAs.argtypes = [c_char_p]
    eyeRenderer.getGeometryMaxBounds.argtypes = [c_char_p]
    eyeRenderer.getGeometryMaxBounds.restype = c_float3
    eyeRenderer.getGeometryMinBounds.argtypes = [c_char_p]
    eyeRenderer.getGeometryMinBounds.restype = c_float3
    eyeRenderer.isInsideHitGeometry.restype = c_bool
    eyeRenderer.isInsideHitGeometry.argtypes = [c_float, c_float, c_float, c_char_p]
    eyeRenderer.setRenderSize.argtypes = [c_int, c_int]
    eyeRenderer.getFramePointer.restype = c_void_p


def configureExtras(eyeRenderer):
    """Binds the entry points this library adds to the reference ABI."""
    L = eyeRenderer
    L.crGetLastError.argtypes = [ctypes.c_char_p, c_size_t]
    L.crGetLastError.restype = c_int
    L.getOmmatidialColoursF32.argtypes = [ndpointer(np.float32, flags="C_CONTIGUOUS")]
    L.getOmmatidialColoursF32.restype = c_int
    L.crRenderPoses.argtypes = [ndpointer(np.float32, flags="C_CONTIGUOUS"), c_size_t,
                                ndpointer(np.float32, flags="C_CONTIGUOUS")]
    L.crRenderPoses.restype = c_int
    L.crRenderPosesDevice.argtypes = [c_void_p, c_size_t, c_void_p]
    L.crRenderPosesDevice.restype = c_int
    f32 = ndpointer(np.float32, flags="C_CONTIGUOUS")
    L.crDenoiserInit.argtypes = [c_int]
    L.crDenoiserInit.restype = c_int
    L.crDenoiserParamCount.restype = c_size_t
    L.crDenoiserAddTrainingPoses.argtypes = [f32, c_size_t, c_int, c_int]
    L.crDenoiserAddTrainingPoses.restype = c_int
    L.crDenoiserTrainingRows.restype = c_size_t
    L.crDenoiserTrain.argtypes = [c_int, c_int, c_float, c_int, c_void_p]
    L.crDenoiserFeatureRows.argtypes = [ndpointer(np.float32, flags="C_CONTIGUOUS"), c_size_t, c_int,
                                        ndpointer(np.uint16, flags="C_CONTIGUOUS"),
                                        ndpointer(np.float32, flags="C_CONTIGUOUS")]
    L.crDenoiserFeatureRows.restype = c_int
    L.crDenoiserPredictRows.argtypes = [ndpointer(np.uint16, flags="C_CONTIGUOUS"),
                                        ndpointer(np.float32, flags="C_CONTIGUOUS"), c_size_t,
                                        ndpointer(np.float32, flags="C_CONTIGUOUS")]
    L.crDenoiserPredictRows.restype = c_int
    L.crDenoiserRelease.restype = None
    L.crSetDenoiserKernel.argtypes = [c_int]
    L.crSetDenoiserKernel.restype = c_int
    L.crGetDenoiserKernel.restype = c_int
    L.crAllocatorInit.argtypes = [c_int]
    L.crAllocatorInit.restype = c_int
    L.crAllocatorAddTrainingPoses.argtypes = [ndpointer(np.float32, flags="C_CONTIGUOUS"), c_size_t, c_int, c_float,
                                              c_int, c_void_p]
    L.crAllocatorAddTrainingPoses.restype = c_int
    L.crAllocatorTrain.argtypes = [c_int, c_int, c_float, c_int, c_void_p]
    L.crAllocatorTrain.restype = c_int
    L.crAllocatorTrainingRows.restype = c_size_t
    L.crAllocatorSave.argtypes = [c_char_p]
    L.crAllocatorSave.restype = c_int
    L.crAllocatorLoad.argtypes = [c_char_p]
    L.crAllocatorLoad.restype = c_int
    L.crSetAllocatorHalvings.argtypes = [c_float]
    L.crSetAllocatorHalvings.restype = c_int
    L.crGetAllocatorHalvings.restype = c_float
    L.crSetAllocatorExponent.argtypes = [c_float]
    L.crSetAllocatorExponent.restype = c_int
    L.crGetAllocatorExponent.restype = c_float
    L.crSetAllocatorCostExponent.argtypes = [c_float]
    L.crSetAllocatorCostExponent.restype = c_int
    L.crGetAllocatorCostExponent.restype = c_float
    L.crAdaptiveLastPass.argtypes = [c_void_p, c_void_p, c_void_p, c_size_t]
    L.crAdaptiveLastPass.restype = c_int
    L.crAdaptiveRenderPosesDevice.argtypes = [c_void_p, c_size_t, c_int, c_void_p, c_void_p, c_void_p]
    L.crAdaptiveRenderPosesDevice.restype = c_int
    L.crAdaptiveRecord.argtypes = [ndpointer(np.float32, flags="C_CONTIGUOUS"), c_size_t, c_int, c_ulonglong,
                                   c_void_p, ndpointer(np.float32, flags="C_CONTIGUOUS")]
    L.crAdaptiveRecord.restype = c_int
    L.crDenoiserTrain.restype = c_int
    L.crDenoiserRenderPosesDevice.argtypes = [c_void_p, c_size_t, c_int, c_void_p]
    L.crDenoiserRenderPosesDevice.restype = c_int
    L.crDenoiserRenderPoses.argtypes = [f32, c_size_t, c_int, f32]
    L.crDenoiserRenderPoses.restype = c_int
    L.crDenoiserGradient.argtypes = [ndpointer(np.uint16, flags="C_CONTIGUOUS"), f32, f32, c_int, f32, f32]
    L.crDenoiserGradient.restype = c_float
    L.crDenoiserScaleOutput.argtypes = [c_float]
    L.crSetBvhWidth.argtypes = [c_int]
    L.crGetWideBvhHost.argtypes = [c_int, ctypes.c_void_p, c_size_t, ctypes.POINTER(ctypes.c_uint32),
                                   ctypes.c_void_p]
    L.crGetWideBvhStats.argtypes = [ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint32),
                                    ctypes.POINTER(c_double)]
    L.crSetRenderLayout.argtypes = [c_int, c_int]
    L.crGetRenderLayout.argtypes = [ctypes.POINTER(c_int), ctypes.POINTER(c_int)]
    L.crGetAutotuneTimes.argtypes = [f32, c_size_t]
    L.crSetAdaptiveSchedule.argtypes = [c_int, c_int]
    L.crSetAdaptiveOccupancy.argtypes = [c_int]
    L.crGetAdaptiveSchedule.argtypes = [ctypes.POINTER(c_int), ctypes.POINTER(c_int)]
    L.crDenoiserAdamStep.argtypes = [f32, f32, f32, f32, c_size_t, c_float, c_float, c_float,
                                     ndpointer(np.uint16, flags="C_CONTIGUOUS")]
    L.crDenoiserSave.argtypes = [c_char_p]
    L.crDenoiserSave.restype = c_int
    L.crDenoiserLoad.argtypes = [c_char_p]
    L.crDenoiserLoad.restype = c_int
    L.crSetBvhBuilder.argtypes = [c_int]
    L.crSetBvhBuilder.restype = c_int
    L.crGetBvhBuilder.restype = c_int
    L.crBatchCreate.argtypes = [ndpointer(np.int32, flags="C_CONTIGUOUS"), c_size_t, c_size_t, c_void_p, c_void_p]
    L.crBatchCreate.restype = c_int
    L.crBatchLaunch.argtypes = [c_int]
    L.crBatchLaunch.restype = c_int
    L.crBatchLatencies.argtypes = [c_int, ndpointer(np.float32, flags="C_CONTIGUOUS"), POINTER(c_float)]
    L.crBatchLatencies.restype = c_int
    L.crBatchOutputOffset.argtypes = [c_int, c_size_t]
    L.crBatchOutputOffset.restype = c_size_t
    L.crBatchDestroy.argtypes = [c_int]
    L.crBatchDestroy.restype = c_int
    L.renderBatch.argtypes = [ndpointer(np.int32, flags="C_CONTIGUOUS"), c_size_t, c_size_t, c_void_p, c_void_p]
    L.renderBatch.restype = c_int
    L.crRenderPosesDeviceNoAlloc.argtypes = [c_void_p, c_size_t, c_void_p]
    L.crRenderPosesDeviceNoAlloc.restype = c_int
    L.crMeasureTraversal.argtypes = [c_void_p, c_size_t, POINTER(c_double), POINTER(c_double)]
    L.crMeasureTraversal.restype = c_int
    L.crAutotune.argtypes = [c_void_p, c_size_t, POINTER(c_int), ndpointer(np.float32, flags="C_CONTIGUOUS")]
    L.crAutotune.restype = c_int
    L.crSetLighting.argtypes = [c_int]
    L.crSetLighting.restype = c_int
    L.crGetLighting.restype = c_int
    L.crInsideHitGeometryBatch.argtypes = [ndpointer(np.float32, flags="C_CONTIGUOUS"), c_size_t, c_char_p,
                                           ndpointer(np.uint8, flags="C_CONTIGUOUS")]
    L.crInsideHitGeometryBatch.restype = c_int
    L.crGetSceneLighting.argtypes = [c_void_p, c_void_p, c_void_p]
    L.crGetSceneLighting.restype = c_int
    L.crSetCutRadius.argtypes = [c_float]
    L.crSetCutRadius.restype = c_int
    L.crGetCutRadius.restype = c_float
    L.crSetRenderVariant.argtypes = [c_int]
    L.crSetRenderVariant.restype = c_int
    L.crSetDeviceMemoryCap.argtypes = [c_size_t]
    L.crSetDeviceMemoryCap.restype = c_int
    L.crGetDeviceMemoryHeld.restype = c_size_t
    L.crSelfTestBoundedWait.argtypes = [c_uint]
    L.crSelfTestBoundedWait.restype = c_int
    L.crSetProjectionSearch.argtypes = [c_int]
    L.crSetProjectionSearch.restype = c_int
    L.crGetProjectionSearch.restype = c_int
    L.crGetRenderVariant.restype = c_int
    L.crGetRenderVariantCount.restype = c_int
    L.crSetStream.argtypes = [c_void_p]
    L.crSetStream.restype = c_int
    L.crSynchronize.restype = c_int
    L.crRenderFrameRecorded.argtypes = [c_void_p]
    L.crRenderFrameRecorded.restype = c_int
    L.crGetTriangleCount.restype = c_size_t
    L.crGetSceneTriangles.argtypes = [c_void_p, c_void_p, c_void_p]
    L.crGetSceneTriangles.restype = c_int
    L.crGetTextureCount.restype = c_size_t
    L.crGetTexelCount.restype = c_size_t
    L.crGetSceneTextures.argtypes = [c_void_p, c_void_p]
    L.crGetSceneTextures.restype = c_int
    L.crCompareTextureSampling.argtypes = [ndpointer(np.uint32, flags="C_CONTIGUOUS"), c_int, c_int,
                                           ndpointer(np.float32, flags="C_CONTIGUOUS"), c_int,
                                           ndpointer(np.float32, flags="C_CONTIGUOUS"),
                                           ndpointer(np.float32, flags="C_CONTIGUOUS")]
    L.crCompareTextureSampling.restype = c_int
    L.crGetOmmatidia.argtypes = [ndpointer(np.float32, flags="C_CONTIGUOUS")]
    L.crGetOmmatidia.restype = c_int
    L.crGetCameraLocalSpace.argtypes = [ndpointer(np.float32, flags="C_CONTIGUOUS")]
    L.crGetCameraLocalSpace.restype = c_int
    L.crGetRandomStates.argtypes = [ndpointer(np.uint32, flags="C_CONTIGUOUS")]
    L.crGetRandomStates.restype = c_int
    L.crGetBvhStats.argtypes = [POINTER(c_uint32)] * 3
    L.crGetBvhStats.restype = c_int


def lastError(eyeRenderer):
    buf = ctypes.create_string_buffer(4096)
    n = eyeRenderer.crGetLastError(buf, 4096)
    return buf.value.decode() if n else ""


def getCameraPosition(eyeRenderer):
    x, y, z = c_float(), c_float(), c_float()
    eyeRenderer.getCameraPosition(ctypes.byref(x), ctypes.byref(y), ctypes.byref(z))
    return np.array([x.value, y.value, z.value], np.float32)


def getFrame(eyeRenderer, width, height):
    """Copy of the current frame as an (height, width, 4) uint8 array."""
    ptr = eyeRenderer.getFramePointer()
    if isinstance(ptr, np.ndarray):  # restype set by setRenderSize
        return ptr.reshape(height, width, 4).copy()
    if not ptr:
        raise RuntimeError(lastError(eyeRenderer) or "getFramePointer returned null")
    return np.ctypeslib.as_array((c_ubyte * (width * height * 4)).from_address(ptr)).reshape(height, width, 4).copy()


def getOmmatidialColours(eyeRenderer):
    n = eyeRenderer.getCurrentEyeOmmatidialCount()
    out = np.zeros((n, 3), np.float32)
    if eyeRenderer.getOmmatidialColoursF32(out) != 0:
        raise RuntimeError(lastError(eyeRenderer))
    return out


def renderPoses(eyeRenderer, poses):
    """Renders (P, 12) poses of the current eye; returns (P, N, 3) float32."""
    poses = np.ascontiguousarray(poses, np.float32).reshape(-1, 12)
    n = eyeRenderer.getCurrentEyeOmmatidialCount()
    out = np.zeros((len(poses), n, 3), np.float32)
    if eyeRenderer.crRenderPoses(poses, len(poses), out) != 0:
        raise RuntimeError(lastError(eyeRenderer))
    return out


def renderFrameRecorded(eyeRenderer):
    """Renders one frame and returns its per-ray records (N, spp)."""
    n = eyeRenderer.getCurrentEyeOmmatidialCount()
    spp = eyeRenderer.getCurrentEyeSamplesPerOmmatidium()
    rec = np.zeros((n, spp), RAY_RECORD_DTYPE)
    if eyeRenderer.crRenderFrameRecorded(rec.ctypes.data) != 0:
        raise RuntimeError(lastError(eyeRenderer))
    return rec


def getSceneTriangles(eyeRenderer):
    t = eyeRenderer.crGetTriangleCount()
    verts = np.zeros((t, 3, 3), np.float32)
    cols = np.zeros((t, 3, 4), np.float32)
    flags = np.zeros(t, np.uint8)
    if eyeRenderer.crGetSceneTriangles(verts.ctypes.data, cols.ctypes.data, flags.ctypes.data) != 0:
        raise RuntimeError(lastError(eyeRenderer))
    return verts, cols, flags


def getSceneTextures(eyeRenderer):
    """Decoded textures: (K, 3) int32 table of (first texel, width, height)
    and the RGBA8 texels as uint32 (red in the low byte)."""
    k, n = eyeRenderer.crGetTextureCount(), eyeRenderer.crGetTexelCount()
    table = np.zeros((k, 3), np.int32)
    texels = np.zeros(n, np.uint32)
    if eyeRenderer.crGetSceneTextures(table.ctypes.data, texels.ctypes.data) != 0:
        raise RuntimeError(lastError(eyeRenderer))
    return table, texels


def compareTextureSampling(eyeRenderer, texels, width, height, uv):
    """(renderer filter, hardware texture unit) lookups, each (n, 4)."""
    texels = np.ascontiguousarray(texels, np.uint32).reshape(-1)
    uv = np.ascontiguousarray(uv, np.float32).reshape(-1, 2)
    soft = np.zeros((len(uv), 4), np.float32)
    hard = np.zeros((len(uv), 4), np.float32)
    if eyeRenderer.crCompareTextureSampling(texels, int(width), int(height), uv.reshape(-1), len(uv), soft, hard) != 0:
        raise RuntimeError(lastError(eyeRenderer))
    return soft, hard


def getSceneLighting(eyeRenderer):
    """(T, 20) lighting-on records, (4, 4) light positions + intensities, (4, 3) colours."""
    light = np.zeros((eyeRenderer.crGetTriangleCount(), 20), np.float32)
    pos = np.zeros((4, 4), np.float32)
    col = np.zeros((4, 3), np.float32)
    if eyeRenderer.crGetSceneLighting(light.ctypes.data, pos.ctypes.data, col.ctypes.data) != 0:
        raise RuntimeError(lastError(eyeRenderer))
    return light, pos, col


def getOmmatidia(eyeRenderer):
    """Current eye's ommatidium records as an (N, 8) float32 array."""
    out = np.zeros((eyeRenderer.getCurrentEyeOmmatidialCount(), 8), np.float32)
    if eyeRenderer.crGetOmmatidia(out) != 0:
        raise RuntimeError(lastError(eyeRenderer))
    return out


def setCameraLocalSpace(eyeRenderer, npMatrix):
    newX, newY, newZ = npMatrix[:, 0], npMatrix[:, 1], npMatrix[:, 2]
    eyeRenderer.setCameraLocalSpace(*newX, *newY, *newZ)


def setRenderSize(eyeRenderer, width, height):
    """Updates the render size and the return type of getFramePointer."""
    eyeRenderer.setRenderSize(width, height)
    eyeRenderer.getFramePointer.restype = ndpointer(dtype=c_ubyte, shape=(height, width, 4))


def setOmmatidiaFromPacketList(eyeRenderer, packetList):
    ommCount = len(packetList)
    c_omm_array_type = c_ommatidiumPacket * ommCount
    eyeRenderer.setOmmatidia.argtypes = [c_omm_array_type, c_size_t]
    c_ommArray = c_omm_array_type(*packetList)
    eyeRenderer.setOmmatidia(c_ommArray, c_size_t(ommCount))


def setOmmatidiaFromOmmatidiumList(eyeRenderer, ommList):
    packetList = [c_ommatidiumPacket(*[float(n) for n in o.position], *[float(n) for n in o.direction],
                                     o.acceptanceAngle, o.focalpointOffset) for o in ommList]
    setOmmatidiaFromPacketList(eyeRenderer, packetList)


def gotoFirstCompoundEye(eyeRenderer):
    """Goes to the first compound eye of the scene; raises when there is none."""
    for i in range(eyeRenderer.getCameraCount()):
        eyeRenderer.gotoCamera(int(i))
        if eyeRenderer.isCompoundEyeActive():
            return
    raise Exception("Error: Could not find compound eye in provided GlTF scene.")


def readEyeFile(path):
    """Reads an .eye file into a list of Ommatidium objects."""
    output = []
    with open(path) as eyeFile:
        for line in eyeFile:
            data = [float(n) for n in line.split(" ")]
            output.append(Ommatidium(np.asarray(data[:3]), np.asarray(data[3:6]), data[6], data[7]))
    return output


def saveEyeFile(path, omms):
    """Saves a list of Ommatidium objects as an .eye file."""
    with open(path, "w") as eyeFile:
        for omm in omms:
            eyeFile.write("{:0.10f} {:0.10f} {:0.10f} {:0.10f} {:0.10f} {:0.10f} {:0.10f} {:0.10f}\n".format(
                omm.position[0], omm.position[1], omm.position[2], omm.direction[0], omm.direction[1],
                omm.direction[2], omm.acceptanceAngle, omm.focalpointOffset))
