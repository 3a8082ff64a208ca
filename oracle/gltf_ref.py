"""Independent numpy restatement of the reference's glTF scene rules.
TEST INFRASTRUCTURE ONLY (the oracle's scene loader; never used by the
product).

Restates libEyeRenderer3/MulticamScene.cpp:
  * root nodes = nodes that are nobody's child, in index order (:723-735);
  * node transform = parent * matrix * T * R * S (:173-205);
  * camera nodes add a camera and stop; compound eyes from the camera extras
    (:207-327); .eye parsing (:289-299);
  * mesh nodes add their triangle primitives and stop, hitbox meshes are
    kept apart (:329-518); only other nodes recurse (:519-525);
  * COLOR_0 shaded from vertices only when VEC4 float / u16 / u8
    (:415-516, cuda/LocalGeometry.h:105-156), else the material
    baseColorFactor (default white, cuda/MaterialData.h:42);
  * background shader from the scene extras (:555-565).
Transforms are composed and applied in float64 with the same operation order
as the library's loader and rounded once to float32 (the reference composes
in float32); the parity tests compare the two loaders bit for bit.
"""
import base64
import ctypes
import ctypes.util
import json
import os

import numpy as np

_libc = ctypes.CDLL(ctypes.util.find_library("c"))
_libc.strtof.restype = ctypes.c_float
_libc.strtof.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_char_p)]

COMP = {5120: np.int8, 5121: np.uint8, 5122: np.int16, 5123: np.uint16, 5125: np.uint32, 5126: np.float32}
NCOMP = {"SCALAR": 1, "VEC2": 2, "VEC3": 3, "VEC4": 4, "MAT4": 16}


def _strtof(tok):
    return _libc.strtof(tok.encode(), None)


def parse_eye(path):
    """.eye records as an (N, 8) float32 array, parsed with the C library's
    strtof like the reference's std::stof."""
    rows = []
    with open(path) as f:
        for lineno, line in enumerate(f, 1):
            line = line.rstrip("\n")
            toks = [t for t in line.split(" ") if t != ""]
            if len(toks) < 8:
                raise ValueError("%s line %d: expected 8 values" % (path, lineno))
            rows.append([_strtof(t) for t in toks[:8]])
    return np.asarray(rows, np.float32).reshape(-1, 8)


def _ident():
    return [1.0 if i % 5 == 0 else 0.0 for i in range(16)]


def _mul(a, b):
    r = [0.0] * 16
    for i in range(4):
        for j in range(4):
            s = a[i * 4 + 0] * b[0 * 4 + j]
            s = s + a[i * 4 + 1] * b[1 * 4 + j]
            s = s + a[i * 4 + 2] * b[2 * 4 + j]
            s = s + a[i * 4 + 3] * b[3 * 4 + j]
            r[i * 4 + j] = s
    return r


def _quat(x, y, z, w):
    m = _ident()
    xx, yy, zz = x * x, y * y, z * z
    xy, xz, yz = x * y, x * z, y * z
    wx, wy, wz = w * x, w * y, w * z
    m[0] = 1.0 - 2.0 * (yy + zz)
    m[1] = 2.0 * (xy - wz)
    m[2] = 2.0 * (xz + wy)
    m[4] = 2.0 * (xy + wz)
    m[5] = 1.0 - 2.0 * (xx + zz)
    m[6] = 2.0 * (yz - wx)
    m[8] = 2.0 * (xz - wy)
    m[9] = 2.0 * (yz + wx)
    m[10] = 1.0 - 2.0 * (xx + yy)
    return m


def _apply(m, x, y, z, w):
    """M * (x, y, z, w) rows summed left to right; works on arrays."""
    out = []
    for i in range(3):
        s = m[i * 4 + 0] * x
        s = s + m[i * 4 + 1] * y
        s = s + m[i * 4 + 2] * z
        s = s + m[i * 4 + 3] * w
        out.append(s)
    return out


def _extra_true(extras, key):
    v = (extras or {}).get(key)
    if isinstance(v, bool):
        return v
    if isinstance(v, str):
        return v.lower() == "true"
    return False


class RefScene:
    def __init__(self):
        self.verts = []
        self.colours = []
        self.flags = []
        self.meshes = []  # (name, tri offset, tri count)
        self.cameras = []
        self.hitboxes = []
        self.miss_name = "default_background"

    @property
    def miss(self):
        return 1 if self.miss_name == "simple_sky" else 0

    def arrays(self):
        if self.verts:
            v = np.concatenate(self.verts).astype(np.float32)
            c = np.concatenate(self.colours).astype(np.float32)
            f = np.concatenate(self.flags).astype(np.uint8)
        else:
            v, c, f = np.zeros((0, 3, 3), np.float32), np.zeros((0, 3, 4), np.float32), np.zeros(0, np.uint8)
        return v, c, f


def load(path):
    with open(path) as f:
        doc = json.load(f)
    gdir = os.path.dirname(path)
    gdir = gdir + "/" if gdir else ""
    buffers = []
    for b in doc.get("buffers", []):
        uri = b["uri"]
        if uri.startswith("data:"):
            buffers.append(base64.b64decode(uri.split(",", 1)[1]))
        else:
            with open(gdir + uri, "rb") as fh:
                buffers.append(fh.read())

    def accessor(i):
        a = doc["accessors"][i]
        bv = doc["bufferViews"][a["bufferView"]]
        dt = np.dtype(COMP[a["componentType"]])
        nc = NCOMP[a["type"]]
        off = bv.get("byteOffset", 0) + a.get("byteOffset", 0)
        stride = bv.get("byteStride", 0) or dt.itemsize * nc
        count = a["count"]
        raw = np.frombuffer(buffers[bv["buffer"]], np.uint8)
        rows = np.stack([raw[off + k * stride: off + k * stride + dt.itemsize * nc] for k in range(count)]) \
            if stride != dt.itemsize * nc else raw[off: off + count * stride].reshape(count, stride)
        return np.ascontiguousarray(rows).view(dt).reshape(count, nc), a

    sc = RefScene()
    for s in doc.get("scenes", []):
        bg = (s.get("extras") or {}).get("background-shader", "")
        if isinstance(bg, str) and bg:
            sc.miss_name = bg

    nodes = doc.get("nodes", [])
    is_root = [True] * len(nodes)
    for n in nodes:
        for c in n.get("children", []):
            is_root[c] = False

    def node_xf(n, parent):
        t, r, s, mx = _ident(), _ident(), _ident(), _ident()
        if "translation" in n:
            t[3], t[7], t[11] = (float(v) for v in n["translation"])
        if "rotation" in n:
            r = _quat(*(float(v) for v in n["rotation"]))
        if "scale" in n:
            s[0], s[5], s[10] = (float(v) for v in n["scale"])
        if "matrix" in n:
            m = [float(v) for v in n["matrix"]]
            mx = [m[j * 4 + i] for i in range(4) for j in range(4)]
        return _mul(_mul(_mul(_mul(parent, mx), t), r), s)

    def f3(m, x, y, z, w):
        return np.array([np.float32(v) for v in _apply(m, x, y, z, w)], np.float32)

    def visit(i, parent):
        n = nodes[i]
        xf = node_xf(n, parent)
        if n.get("camera", -1) >= 0:
            cam = doc["cameras"][n["camera"]]
            c = {"name": cam.get("name", ""), "position": f3(xf, 0.0, 0.0, 0.0, 1.0),
                 "ls": np.stack([f3(xf, 1.0, 0.0, 0.0, 0.0), f3(xf, 0.0, 1.0, 0.0, 0.0), f3(xf, 0.0, 0.0, -1.0, 0.0)])}
            ex = cam.get("extras") or {}
            if cam.get("type") == "orthographic":
                c["kind"] = "orthographic"
            elif _extra_true(ex, "panoramic"):
                c["kind"] = "panoramic"
            elif _extra_true(ex, "compound-eye"):
                eye = ex.get("compound-structure", "")
                proj = ex.get("compound-projection", "")
                if not eye or not proj:
                    return
                p = eye if os.path.exists(eye) else gdir + eye
                if not os.path.exists(p):
                    return
                omm = parse_eye(p)
                if len(omm) == 0:
                    return
                c.update(kind="compound", eye=p, projection=proj, omm=omm)
            else:
                c["kind"] = "perspective"
            sc.cameras.append(c)
        elif n.get("mesh", -1) >= 0 and _extra_true(doc["meshes"][n["mesh"]].get("extras"), "hitbox"):
            sc.hitboxes.append(doc["meshes"][n["mesh"]].get("name", ""))
        elif n.get("mesh", -1) >= 0:
            mesh = doc["meshes"][n["mesh"]]
            for prim in mesh["primitives"]:
                if prim.get("mode", 4) != 4:
                    continue
                pos, _ = accessor(prim["attributes"]["POSITION"])
                off = sum(len(v) for v in sc.verts)
                if "indices" not in prim:
                    sc.meshes.append((mesh.get("name", ""), off, 0))
                    continue
                idx, _ = accessor(prim["indices"])
                idx = idx.reshape(-1).astype(np.int64)
                tri = idx[: len(idx) // 3 * 3].reshape(-1, 3)
                p64 = pos.astype(np.float64)
                wx, wy, wz = _apply(xf, p64[:, 0], p64[:, 1], p64[:, 2], 1.0)
                world = np.stack([wx, wy, wz], axis=1).astype(np.float32)
                base = np.ones(4, np.float32)
                mat = prim.get("material", -1)
                if mat is not None and mat >= 0:
                    bcf = doc["materials"][mat].get("pbrMetallicRoughness", {}).get("baseColorFactor")
                    if bcf is not None:
                        base = np.array([np.float32(v) for v in bcf], np.float32)
                flag = 0
                vcol = np.tile(base, (len(pos), 1))
                if "COLOR_0" in prim["attributes"]:
                    col, acc = accessor(prim["attributes"]["COLOR_0"])
                    if acc["type"] == "VEC4" and acc["componentType"] in (5126, 5123, 5121):
                        flag = 1
                        if acc["componentType"] == 5126:
                            vcol = col.astype(np.float32)
                        elif acc["componentType"] == 5123:
                            vcol = col.astype(np.float32) / np.float32(65535.0)
                        else:
                            vcol = col.astype(np.float32) / np.float32(255.0)
                sc.verts.append(world[tri])
                sc.colours.append(vcol[tri])
                sc.flags.append(np.full(len(tri), flag, np.uint8))
                sc.meshes.append((mesh.get("name", ""), off, len(tri)))
        else:
            for c in n.get("children", []):
                visit(c, xf)

    for i in range(len(nodes)):
        if is_root[i]:
            visit(i, _ident())
    if not sc.cameras:
        sc.cameras.append({"name": "Default Camera", "kind": "perspective", "position": np.zeros(3, np.float32),
                           "ls": np.eye(3, dtype=np.float32)})
    return sc
