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
  * without vertex colours a material baseColorTexture gives texture
    shading at TEXCOORD_0 (float VEC2) or at the barycentrics
    (shaders.cu:801-805, cuda/LocalGeometry.h:88-103); records (u, v,
    texture, 0) per vertex with the default coordinates (0,0) (1,0) (0,1);
  * every image decoded to RGBA8 as a forced 4-component load would
    (tiny_gltf.h:2305-2389), here with Python's zlib and the PNG
    specification's unfiltering and Adam7 passes; 16-bit images refused;
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
import struct
import zlib

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


def _unfilter(data, pos, h, stride, bpp):
    out = np.zeros((h, stride), np.int32)
    prev = np.zeros(stride, np.int32)
    for y in range(h):
        f = data[pos]
        line = np.frombuffer(data, np.uint8, stride, pos + 1).astype(np.int32)
        pos += stride + 1
        cur = np.zeros(stride, np.int32)
        for i in range(stride):
            a = cur[i - bpp] if i >= bpp else 0
            b = prev[i]
            c = prev[i - bpp] if i >= bpp else 0
            if f == 0:
                p = 0
            elif f == 1:
                p = a
            elif f == 2:
                p = b
            elif f == 3:
                p = (a + b) >> 1
            elif f == 4:
                pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                p = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
            else:
                raise ValueError("bad PNG filter")
            cur[i] = (line[i] + p) & 0xFF
        out[y] = cur
        prev = cur
    return out, pos


def decode_png(data):
    """PNG -> (h, w, 4) uint8 with a forced four-channel expansion."""
    assert data[:8] == b"\x89PNG\r\n\x1a\n", "not a PNG image"
    pos, idat, palette, trns = 8, b"", None, b""
    while pos + 8 <= len(data):
        n, kind = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8: pos + 8 + n]
        if kind == b"IHDR":
            w, h, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", body[:13])
        elif kind == b"PLTE":
            palette = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif kind == b"tRNS":
            trns = body
        elif kind == b"IDAT":
            idat += body
        elif kind == b"IEND":
            break
        pos += 12 + n
    if depth == 16:
        raise ValueError("16-bit images are not supported")
    raw = zlib.decompress(idat)
    ch = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    img = np.zeros((h, w, 4), np.uint8)
    img[:, :, 3] = 255
    passes = [(0, 0, 1, 1)] if not interlace else [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4),
                                                    (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]
    at = 0
    for x0, y0, dx, dy in passes:
        pw, ph = (w - x0 + dx - 1) // dx if x0 < w else 0, (h - y0 + dy - 1) // dy if y0 < h else 0
        if pw == 0 or ph == 0:
            continue
        stride = (pw * ch * depth + 7) // 8
        rows, at = _unfilter(raw, at, ph, stride, max(1, ch * depth // 8))
        if depth == 8:
            s = rows[:, : pw * ch].reshape(ph, pw, ch)
        else:
            bits = np.unpackbits(rows.astype(np.uint8), axis=1)[:, : pw * depth].reshape(ph, pw, depth)
            s = (bits * (1 << np.arange(depth - 1, -1, -1))).sum(axis=2)[:, :, None]
            if ctype == 0:
                s = s * (255 // ((1 << depth) - 1))
        sub_img = np.zeros((ph, pw, 4), np.uint8)
        sub_img[:, :, 3] = 255
        if ctype == 3:
            sub_img[:, :, :3] = palette[s[:, :, 0]]
            alpha = np.full(len(palette), 255, np.uint8)
            alpha[: len(trns)] = np.frombuffer(trns, np.uint8)[: len(palette)]
            sub_img[:, :, 3] = alpha[s[:, :, 0]]
        elif ctype in (0, 4):
            sub_img[:, :, :3] = s[:, :, :1]
            if ctype == 4:
                sub_img[:, :, 3] = s[:, :, 1]
        else:
            sub_img[:, :, :ch] = s
        img[y0::dy, x0::dx] = sub_img
    return img


class RefScene:
    def __init__(self):
        self.verts = []
        self.colours = []
        self.flags = []
        self.light = []  # (T, 20) lighting-on records per primitive
        self.world_boxes = []  # (lo, hi) float32 per primitive
        self.images = []  # (h, w, 4) uint8 per image
        self.meshes = []  # (name, tri offset, tri count)
        self.cameras = []
        self.hitboxes = []
        self.hitbox_meshes = []  # {"name", "xform" (4x4 double), "tris" (T, 9) float32 object space}
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

    def lighting(self):
        """Lighting-on data: (T, 20) records, light positions + intensities
        (4, 4) and colours (4, 3) around the scene box (libEyeRenderer.cpp:100-118)."""
        light = np.concatenate(self.light).astype(np.float32) if self.light else np.zeros((0, 20), np.float32)
        lo = np.min([b[0] for b in self.world_boxes], axis=0).astype(np.float32)
        hi = np.max([b[1] for b in self.world_boxes], axis=0).astype(np.float32)
        c = ((lo + hi) * np.float32(0.5)).astype(np.float32)
        e = np.float32((hi - lo).max())
        f = np.float32
        pos = np.array([[c[0] + e, c[1] + e, c[2] + e, 5.0],
                        [c[0] - e, c[1] + f(0.5) * e, c[2] - f(0.5) * e, 3.0],
                        [c[0] + f(0.0), c[1] + f(4.0), c[2] - f(5.0), 5.0],
                        [c[0] + f(1.0), c[1] - f(6.0), c[2] + f(0.0), 0.5]], np.float32)
        col = np.array([[1.0, 1.0, 0.8], [0.8, 0.8, 1.0], [1.0, 1.0, 0.8], [1.0, 1.0, 0.8]], np.float32)
        return light, pos, col

    def textures(self):
        """(table (K,3) of first texel / width / height, uint32 texels)."""
        table, words, off = [], [], 0
        for im in self.images:
            h, w = im.shape[:2]
            table.append((off, w, h))
            q = im.reshape(-1, 4).astype(np.uint32)
            words.append(q[:, 0] | (q[:, 1] << 8) | (q[:, 2] << 16) | (q[:, 3] << 24))
            off += w * h
        t = np.array(table, np.int32).reshape(-1, 3)
        return t, (np.concatenate(words) if words else np.zeros(0, np.uint32))


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
    for im in doc.get("images", []):
        uri = im.get("uri", "")
        if uri.startswith("data:"):
            data = base64.b64decode(uri.split(",", 1)[1])
        elif uri:
            with open(gdir + uri, "rb") as fh:
                data = fh.read()
        else:
            bv = doc["bufferViews"][im["bufferView"]]
            o = bv.get("byteOffset", 0)
            data = bytes(buffers[bv["buffer"]][o: o + bv["byteLength"]])
        sc.images.append(decode_png(data))
    tex_image = [t["source"] for t in doc.get("textures", [])]
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
            mesh = doc["meshes"][n["mesh"]]
            sc.hitboxes.append(mesh.get("name", ""))
            # object-space triangles and the node transform, as the reference
            # keeps them per hitbox (MulticamScene.cpp:329-344)
            tris = []
            for prim in mesh["primitives"]:
                if prim.get("mode", 4) != 4 or "indices" not in prim:
                    continue
                pos, _ = accessor(prim["attributes"]["POSITION"])
                idx, _ = accessor(prim["indices"])
                idx = idx.reshape(-1).astype(np.int64)
                tris.append(pos.astype(np.float32)[idx[: len(idx) // 3 * 3].reshape(-1, 3)].reshape(-1, 9))
            sc.hitbox_meshes.append({"name": mesh.get("name", ""), "xform": np.array(xf, np.float64).reshape(4, 4),
                                     "tris": np.concatenate(tris) if tris else np.zeros((0, 9), np.float32)})
        elif n.get("mesh", -1) >= 0:
            mesh = doc["meshes"][n["mesh"]]
            for prim in mesh["primitives"]:
                if prim.get("mode", 4) != 4:
                    continue
                pos, pacc = accessor(prim["attributes"]["POSITION"])
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
                tex = -1
                if mat is not None and mat >= 0:
                    pbr = doc["materials"][mat].get("pbrMetallicRoughness", {})
                    bcf = pbr.get("baseColorFactor")
                    if bcf is not None:
                        base = np.array([np.float32(v) for v in bcf], np.float32)
                    if "baseColorTexture" in pbr:
                        tex = tex_image[pbr["baseColorTexture"]["index"]]
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
                if flag == 0 and tex >= 0:
                    flag = 2
                    if "TEXCOORD_0" in prim["attributes"]:
                        uv, _ = accessor(prim["attributes"]["TEXCOORD_0"])
                        rec = np.zeros((len(tri), 3, 4), np.float32)
                        rec[:, :, :2] = uv.astype(np.float32)[tri]
                    else:
                        rec = np.zeros((len(tri), 3, 4), np.float32)
                        rec[:, 1, 0] = 1.0
                        rec[:, 2, 1] = 1.0
                    rec[:, :, 2] = tex
                    sc.colours.append(rec)
                else:
                    sc.colours.append(vcol[tri])
                sc.verts.append(world[tri])
                sc.flags.append(np.full(len(tri), flag, np.uint8))
                # lighting-on records
                lo = np.array(pacc["min"], np.float32) if "min" in pacc else pos.min(axis=0)
                hi = np.array(pacc["max"], np.float32) if "max" in pacc else pos.max(axis=0)
                corners = np.array([[hi[0] if c & 1 else lo[0], hi[1] if c & 2 else lo[1], hi[2] if c & 4 else lo[2]]
                                    for c in range(8)], np.float64)
                cx, cy, cz = _apply(xf, corners[:, 0], corners[:, 1], corners[:, 2], 1.0)
                cw = np.stack([cx, cy, cz], axis=1)
                sc.world_boxes.append((cw.min(axis=0).astype(np.float32), cw.max(axis=0).astype(np.float32)))
                a, b_, c_, d, e, f, g, h, i = xf[0], xf[1], xf[2], xf[4], xf[5], xf[6], xf[8], xf[9], xf[10]
                det = a * (e * i - f * h) - b_ * (d * i - f * g) + c_ * (d * h - e * g)
                idt = 1.0 / det if det != 0.0 else 0.0
                nm = [(e * i - f * h) * idt, -(d * i - f * g) * idt, (d * h - e * g) * idt,
                      -(b_ * i - c_ * h) * idt, (a * i - c_ * g) * idt, -(a * h - b_ * g) * idt,
                      (b_ * f - c_ * e) * idt, -(a * f - c_ * d) * idt, (a * e - b_ * d) * idt]
                rec = np.zeros((len(tri), 20), np.float32)
                lflags = 0
                if "NORMAL" in prim["attributes"]:
                    nrm, nacc = accessor(prim["attributes"]["NORMAL"])
                    if nacc["componentType"] == 5126 and nacc["type"] == "VEC3":
                        lflags |= 1
                        n64 = nrm.astype(np.float64)
                        wn = np.stack([nm[3 * q] * n64[:, 0] + nm[3 * q + 1] * n64[:, 1] + nm[3 * q + 2] * n64[:, 2]
                                       for q in range(3)], axis=1).astype(np.float32)
                        rec[:, 0:9] = wn[tri].reshape(len(tri), 9)
                uvs = np.tile(np.array([0, 0, 0, 1, 1, 0], np.float32), (len(tri), 1))
                if "TEXCOORD_0" in prim["attributes"]:
                    uv, uacc = accessor(prim["attributes"]["TEXCOORD_0"])
                    if uacc["componentType"] == 5126 and uacc["type"] == "VEC2":
                        lflags |= 2
                        uvs = uv.astype(np.float32)[tri].reshape(len(tri), 6)
                rec[:, 9:15] = uvs
                met, rough, mrt, nt = 1.0, 1.0, -1, -1
                if mat is not None and mat >= 0:
                    m_ = doc["materials"][mat]
                    pb = m_.get("pbrMetallicRoughness", {})
                    met = pb.get("metallicFactor", 1.0)
                    rough = pb.get("roughnessFactor", 1.0)
                    if "metallicRoughnessTexture" in pb:
                        mrt = tex_image[pb["metallicRoughnessTexture"]["index"]]
                    if "normalTexture" in m_:
                        nt = tex_image[m_["normalTexture"]["index"]]
                rec[:, 15] = np.float32(met)
                rec[:, 16] = np.float32(rough)
                rec[:, 17] = mrt
                rec[:, 18] = nt
                rec[:, 19] = lflags
                sc.light.append(rec)
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
