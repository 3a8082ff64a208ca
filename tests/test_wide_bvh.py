"""The wide BVH (4 or 8 children per node, 8-bit quantised child boxes),
collapsed on the host from the two-wide BVH: decoded in numpy, every child's
box contains the exact box of everything below it, every triangle sits in
exactly one leaf, and every node has between 2 and W children.  No GPU."""
import ctypes

import numpy as np
import pytest

import eyeRendererHelperFunctions as eh
import scenes


def _decode(nodes, W):
    """Per node: origin, scales, count, (lo, hi) byte planes, refs."""
    F = 16 if W == 4 else 24
    n = nodes.reshape(-1, F)
    u = n.view(np.uint32)
    p = n[:, 0:3].astype(np.float64)
    meta = u[:, 3]
    exps = np.stack([(meta >> (8 * a)) & 0xFF for a in range(3)], axis=1).astype(np.int64)
    scale = np.ldexp(1.0, exps - 127)
    count = (meta >> 24).astype(np.int64)
    words = u[:, 4:4 + (8 if W == 4 else 12)]
    if W == 4:
        lo = [words[:, 0], words[:, 1], words[:, 2]]
        hi = [words[:, 3], words[:, 4], words[:, 5]]
        qlo = np.stack([np.stack([(lo[a] >> (8 * k)) & 0xFF for k in range(4)], 1) for a in range(3)], 1)
        qhi = np.stack([np.stack([(hi[a] >> (8 * k)) & 0xFF for k in range(4)], 1) for a in range(3)], 1)
        refs = n[:, 12:16].view(np.int32)
    else:
        def unpack(w0, w1):
            return np.stack([(w0 >> (8 * k)) & 0xFF for k in range(4)] + [(w1 >> (8 * k)) & 0xFF for k in range(4)], 1)
        qlo = np.stack([unpack(words[:, 2 * a], words[:, 2 * a + 1]) for a in range(3)], 1)
        qhi = np.stack([unpack(words[:, 6 + 2 * a], words[:, 6 + 2 * a + 1]) for a in range(3)], 1)
        refs = n[:, 16:24].view(np.int32)
    return p, scale, count, qlo.astype(np.float64), qhi.astype(np.float64), refs


@pytest.mark.parametrize("W", [4, 8])
@pytest.mark.parametrize("scene", ["small", "terrain"])
def test_wide_bvh_boxes_contain_their_subtrees(lib, small, tmp_path, scene, W):
    lib.crSetBvhBuilder(0)
    path = small["gltf"] if scene == "small" else scenes.terrain_scene(
        str(tmp_path), cells=64, extent=40.0, cones=60, n_omm=50, spp=16, poses=2)["gltf"]
    eh.lastError(lib)
    lib.loadGlTFscene(path.encode())
    assert eh.lastError(lib) == ""
    cnt = ctypes.c_uint32(0)
    assert lib.crGetWideBvhHost(W, None, 0, ctypes.byref(cnt), None) == 0, eh.lastError(lib)
    T = len(eh.getSceneTriangles(lib)[0])
    nodes = np.zeros(cnt.value * (16 if W == 4 else 24), np.float32)
    tris = np.zeros((T, 3, 3), np.float32)
    assert lib.crGetWideBvhHost(W, nodes.ctypes.data, nodes.size, ctypes.byref(cnt), tris.ctypes.data) == 0
    p, scale, count, qlo, qhi, refs = _decode(nodes, W)
    assert ((count >= 2) & (count <= W)).all()
    seen = np.zeros(T, np.int64)

    def box(ref):  # exact box of a subtree, and its triangles counted
        if ref < 0:
            code = (~np.int64(ref)) & 0xFFFFFFFF
            first, c = int(code >> 3), int(code & 7) + 1
            seen[first:first + c] += 1
            v = tris[first:first + c].reshape(-1, 3).astype(np.float64)
            return v.min(0), v.max(0)
        los, his = [], []
        for k in range(count[ref]):
            lo_k, hi_k = box(int(refs[ref, k]))
            # the quantised box holds the exact child box
            qlo_k = p[ref] + qlo[ref, :, k] * scale[ref]
            qhi_k = p[ref] + qhi[ref, :, k] * scale[ref]
            assert (qlo_k <= lo_k).all() and (qhi_k >= hi_k).all(), (ref, k, qlo_k, lo_k, qhi_k, hi_k)
            los.append(lo_k)
            his.append(hi_k)
        return np.min(los, 0), np.max(his, 0)

    import sys
    sys.setrecursionlimit(10000)
    box(0)
    assert (seen == 1).all()
    # the tree is wider than the two-wide one: about W children per inner node
    assert count.mean() > (2.9 if W == 4 else 4.5)
