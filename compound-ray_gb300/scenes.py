"""Seeded synthetic scenes, eyes and pose trajectories for the renderer.

Everything is written as real glTF 2.0 + .eye files so the same inputs feed
the C ABI (loadGlTFscene) and the CPU oracle.  Vertex colours are VEC4 float
COLOR_0, the only colour form the reference shades from vertices besides
u8/u16 VEC4 (libEyeRenderer3/MulticamScene.cpp:415-516).

Workloads (all seeded from SEED with numpy's PCG64):
  * small scene: 2-triangle grey ground (20 m square) + 64 axis-aligned boxes,
    simple_sky; 1000-ommatidium Fibonacci-sphere eye of radius 1 mm,
    acceptance 3 deg, 32 samples, one pose 0.5 m above the origin.
  * terrain scene: 512 x 512-cell value-noise heightfield over 200 m
    (2 m amplitude, 6 octaves) + 2000 cones of 32 triangles; 6000-ommatidium
    sinewave-droplet eye (eyeGenerator/SinewaveDropletCoordinate.cpp:33-60),
    acceptance 1.5-4 deg, 256 samples; 1024-pose random walk
    (0.1 m steps, yaw noise 10 deg).
"""
import base64
import json
import math
import os
import struct
import zlib

import numpy as np

SEED = 20261203
DEG = math.pi / 180.0


# ---------------------------------------------------------------------------
# File writers
# ---------------------------------------------------------------------------
def write_eye(path, pos, dirs, aa, fpo):
    """Writes a .eye file: 8 space-separated floats per line
    (data/eyes/eye-specification.txt), printed with 9 significant digits so
    every float32 round-trips exactly."""
    pos = np.asarray(pos, np.float32)
    dirs = np.asarray(dirs, np.float32)
    aa = np.broadcast_to(np.asarray(aa, np.float32), (len(pos),))
    fpo = np.broadcast_to(np.asarray(fpo, np.float32), (len(pos),))
    with open(path, "w") as f:
        for i in range(len(pos)):
            vals = [pos[i, 0], pos[i, 1], pos[i, 2], dirs[i, 0], dirs[i, 1], dirs[i, 2], aa[i], fpo[i]]
            f.write(" ".join("%.9g" % float(v) for v in vals) + "\n")


def read_eye(path):
    """Reads a .eye file into an (N, 8) float32 array."""
    rows = []
    with open(path) as f:
        for line in f:
            toks = [t for t in line.split(" ") if t != ""]
            rows.append([float(t) for t in toks[:8]])
    return np.asarray(rows, np.float32).reshape(-1, 8)


def _png_chunk(kind, body):
    return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = np.abs(p - a), np.abs(p - b), np.abs(p - c)
    return np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c))


def _filter_rows(rows, bpp, filters):
    """PNG scanline filtering (ISO/IEC 15948 section 9): row y uses filter
    filters[y % len(filters)]."""
    out = bytearray()
    prev = np.zeros(rows.shape[1], np.int32)
    for y in range(rows.shape[0]):
        cur = rows[y].astype(np.int32)
        a = np.concatenate([np.zeros(bpp, np.int32), cur[:-bpp]]) if bpp < len(cur) else np.zeros_like(cur)
        c = np.concatenate([np.zeros(bpp, np.int32), prev[:-bpp]]) if bpp < len(cur) else np.zeros_like(cur)
        f = filters[y % len(filters)]
        pred = [np.zeros_like(cur), a, prev, (a + prev) >> 1, _paeth(a, prev, c)][f]
        out.append(f)
        out += ((cur - pred) & 0xFF).astype(np.uint8).tobytes()
        prev = cur
    return bytes(out)


def _pack_rows(samples, depth):
    """(h, w*channels) integer samples -> (h, stride) bytes at `depth` bits."""
    samples = np.asarray(samples)
    if depth == 8:
        return samples.astype(np.uint8)
    if depth == 16:
        return samples.astype(">u2").view(np.uint8).reshape(samples.shape[0], -1)
    per = 8 // depth
    h, n = samples.shape
    padded = np.zeros((h, -(-n // per) * per), np.uint8)
    padded[:, :n] = samples
    out = np.zeros((h, padded.shape[1] // per), np.uint8)
    for k in range(per):
        out |= (padded[:, k::per] << (8 - depth * (k + 1))).astype(np.uint8)
    return out


def png_bytes(samples, colour_type=6, depth=8, palette=None, trns=None, filters=(0, 1, 2, 3, 4), interlace=False,
              level=6):
    """Encodes an (h, w, channels) integer array as a PNG file (colour type
    0 grey, 2 RGB, 3 palette index, 4 grey+alpha, 6 RGBA) at the given bit
    depth, cycling the scanline filters, optionally Adam7-interlaced."""
    samples = np.asarray(samples)
    if samples.ndim == 2:
        samples = samples[:, :, None]
    h, w, ch = samples.shape
    bpp = max(1, ch * depth // 8)
    raw = bytearray()
    if interlace:
        for x0, y0, dx, dy in ((0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2),
                               (0, 1, 1, 2)):
            sub_img = samples[y0::dy, x0::dx]
            if sub_img.size == 0:
                continue
            raw += _filter_rows(_pack_rows(sub_img.reshape(sub_img.shape[0], -1), depth), bpp, filters)
    else:
        raw += _filter_rows(_pack_rows(samples.reshape(h, -1), depth), bpp, filters)
    out = b"\x89PNG\r\n\x1a\n"
    out += _png_chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, colour_type, 0, 0, 1 if interlace else 0))
    if palette is not None:
        out += _png_chunk(b"PLTE", np.asarray(palette, np.uint8).tobytes())
    if trns is not None:
        out += _png_chunk(b"tRNS", bytes(trns))
    comp = zlib.compress(bytes(raw), level)
    # Split the image data over two IDAT chunks (decoders must join them).
    half = len(comp) // 2
    out += _png_chunk(b"IDAT", comp[:half]) + _png_chunk(b"IDAT", comp[half:])
    out += _png_chunk(b"IEND", b"")
    return out


def rgba_words(rgba):
    """(h, w, 4) uint8 -> (h*w,) uint32 with red in the low byte."""
    rgba = np.asarray(rgba, np.uint8).reshape(-1, 4).astype(np.uint32)
    return rgba[:, 0] | (rgba[:, 1] << 8) | (rgba[:, 2] << 16) | (rgba[:, 3] << 24)


class GltfBuilder:
    """Accumulates meshes/cameras into one glTF document with one buffer."""

    def __init__(self):
        self.blob = bytearray()
        self.accessors = []
        self.views = []
        self.meshes = []
        self.nodes = []
        self.cameras = []
        self.materials = []
        self.images = []
        self.image_files = {}
        self.textures = []
        self.samplers = []
        self.scene_extras = {}

    def image(self, data, how="data", name="img"):
        """Adds an image from encoded bytes: as a data URI, a bufferView or
        an external file written next to the glTF."""
        if how == "data":
            self.images.append({"name": name, "uri": "data:image/png;base64," + base64.b64encode(data).decode()})
        elif how == "bufferView":
            self.images.append({"name": name, "bufferView": self._view(data), "mimeType": "image/png"})
        else:
            fname = "%s_%d.png" % (name, len(self.images))
            self.image_files[fname] = data
            self.images.append({"name": name, "uri": fname})
        return len(self.images) - 1

    def texture(self, image, wrap=None, nearest=False):
        """A texture of an image; `wrap` / `nearest` add a sampler (which
        the reference ends up ignoring)."""
        tex = {"source": image}
        if wrap is not None or nearest:
            smp = {}
            if wrap is not None:
                smp["wrapS"] = smp["wrapT"] = wrap
            if nearest:
                smp["minFilter"] = smp["magFilter"] = 9728
            self.samplers.append(smp)
            tex["sampler"] = len(self.samplers) - 1
        self.textures.append(tex)
        return len(self.textures) - 1

    def textured_material(self, texture, rgba=(1, 1, 1, 1), name="texmat"):
        self.materials.append({"name": name, "pbrMetallicRoughness": {
            "baseColorFactor": [float(c) for c in rgba], "baseColorTexture": {"index": int(texture)}}})
        return len(self.materials) - 1

    def _view(self, data):
        while len(self.blob) % 16:
            self.blob.append(0)
        off = len(self.blob)
        self.blob += data
        self.views.append({"buffer": 0, "byteOffset": off, "byteLength": len(data)})
        return len(self.views) - 1

    def accessor(self, arr, comp_type, typ, minmax=False):
        arr = np.ascontiguousarray(arr)
        view = self._view(arr.tobytes())
        count = arr.shape[0] if typ != "SCALAR" else arr.size
        acc = {"bufferView": view, "componentType": comp_type, "count": int(count), "type": typ}
        if minmax:
            acc["min"] = [float(v) for v in arr.min(axis=0)]
            acc["max"] = [float(v) for v in arr.max(axis=0)]
        self.accessors.append(acc)
        return len(self.accessors) - 1

    def material(self, rgba, name="mat", metallic=None, roughness=None, mr_texture=None, normal_texture=None,
                 base_texture=None):
        pbr = {"baseColorFactor": [float(c) for c in rgba]}
        if metallic is not None:
            pbr["metallicFactor"] = float(metallic)
        if roughness is not None:
            pbr["roughnessFactor"] = float(roughness)
        if mr_texture is not None:
            pbr["metallicRoughnessTexture"] = {"index": int(mr_texture)}
        if base_texture is not None:
            pbr["baseColorTexture"] = {"index": int(base_texture)}
        mat = {"name": name, "pbrMetallicRoughness": pbr}
        if normal_texture is not None:
            mat["normalTexture"] = {"index": int(normal_texture)}
        self.materials.append(mat)
        return len(self.materials) - 1

    def mesh(self, name, positions, indices, colours=None, material=None, translation=None, rotation=None,
             scale=None, matrix=None, index_type=None, colour_type=5126, extras=None, texcoords=None,
             normals=None):
        positions = np.asarray(positions, np.float32).reshape(-1, 3)
        attrs = {"POSITION": self.accessor(positions, 5126, "VEC3", minmax=True)}
        if normals is not None:
            attrs["NORMAL"] = self.accessor(np.asarray(normals, np.float32).reshape(-1, 3), 5126, "VEC3")
        if texcoords is not None:
            attrs["TEXCOORD_0"] = self.accessor(np.asarray(texcoords, np.float32).reshape(-1, 2), 5126, "VEC2")
        if colours is not None:
            colours = np.asarray(colours)
            if colour_type == 5126:
                attrs["COLOR_0"] = self.accessor(colours.astype(np.float32), 5126, "VEC4" if colours.shape[1] == 4 else "VEC3")
            elif colour_type == 5123:
                attrs["COLOR_0"] = self.accessor(colours.astype(np.uint16), 5123, "VEC4")
            else:
                attrs["COLOR_0"] = self.accessor(colours.astype(np.uint8), 5121, "VEC4")
        indices = np.asarray(indices).reshape(-1)
        if index_type is None:
            index_type = 5123 if positions.shape[0] <= 65535 else 5125
        idx_dtype = {5121: np.uint8, 5123: np.uint16, 5125: np.uint32}[index_type]
        prim = {"attributes": attrs, "indices": self.accessor(indices.astype(idx_dtype), index_type, "SCALAR")}
        if material is not None:
            prim["material"] = material
        mesh = {"name": name, "primitives": [prim]}
        if extras:
            mesh["extras"] = extras
        self.meshes.append(mesh)
        node = {"name": name, "mesh": len(self.meshes) - 1}
        for key, val in (("translation", translation), ("rotation", rotation), ("scale", scale), ("matrix", matrix)):
            if val is not None:
                node[key] = [float(v) for v in val]
        self.nodes.append(node)
        return len(self.nodes) - 1

    def compound_camera(self, name, eye_file, projection="single_dimension_fast", translation=None, rotation=None):
        self.cameras.append({"name": name, "type": "perspective",
                             "perspective": {"yfov": 0.4, "znear": 0.1, "zfar": 100.0},
                             "extras": {"compound-eye": "true", "compound-structure": eye_file,
                                        "compound-projection": projection}})
        node = {"name": name, "camera": len(self.cameras) - 1}
        if translation is not None:
            node["translation"] = [float(v) for v in translation]
        if rotation is not None:
            node["rotation"] = [float(v) for v in rotation]
        self.nodes.append(node)
        return len(self.nodes) - 1

    def perspective_camera(self, name, translation=None):
        self.cameras.append({"name": name, "type": "perspective",
                             "perspective": {"yfov": 0.4, "znear": 0.1, "zfar": 100.0}})
        node = {"name": name, "camera": len(self.cameras) - 1}
        if translation is not None:
            node["translation"] = [float(v) for v in translation]
        self.nodes.append(node)
        return len(self.nodes) - 1

    def write(self, path, embed=True):
        doc = {"asset": {"version": "2.0", "generator": "compound-ray_gb300 scenes.py"},
               "scene": 0,
               "scenes": [{"name": "Scene", "nodes": list(range(len(self.nodes))), "extras": self.scene_extras}],
               "nodes": self.nodes, "meshes": self.meshes, "accessors": self.accessors,
               "bufferViews": self.views}
        if self.cameras:
            doc["cameras"] = self.cameras
        if self.materials:
            doc["materials"] = self.materials
        for key in ("images", "textures", "samplers"):
            if getattr(self, key):
                doc[key] = getattr(self, key)
        for fname, data in self.image_files.items():
            with open(os.path.join(os.path.dirname(path) or ".", fname), "wb") as f:
                f.write(data)
        if embed:
            uri = "data:application/octet-stream;base64," + base64.b64encode(bytes(self.blob)).decode()
        else:
            binname = os.path.splitext(os.path.basename(path))[0] + ".bin"
            with open(os.path.join(os.path.dirname(path) or ".", binname), "wb") as f:
                f.write(bytes(self.blob))
            uri = binname
        doc["buffers"] = [{"byteLength": len(self.blob), "uri": uri}]
        with open(path, "w") as f:
            json.dump(doc, f)
        return path


# ---------------------------------------------------------------------------
# Geometry helpers
# ---------------------------------------------------------------------------
def fibonacci_sphere(n):
    """n unit vectors on a Fibonacci (golden-angle) spiral."""
    i = np.arange(n, dtype=np.float64) + 0.5
    y = 1.0 - 2.0 * i / n
    r = np.sqrt(np.maximum(0.0, 1.0 - y * y))
    phi = i * math.pi * (3.0 - math.sqrt(5.0))
    return np.stack([r * np.cos(phi), y, r * np.sin(phi)], axis=1)


def box_mesh(lo, hi):
    """8 corners and 12 triangles of an axis-aligned box."""
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    v = np.array([[x0, y0, z0], [x1, y0, z0], [x1, y1, z0], [x0, y1, z0],
                  [x0, y0, z1], [x1, y0, z1], [x1, y1, z1], [x0, y1, z1]], np.float64)
    f = np.array([[0, 2, 1], [0, 3, 2], [4, 5, 6], [4, 6, 7], [0, 1, 5], [0, 5, 4],
                  [3, 7, 6], [3, 6, 2], [0, 4, 7], [0, 7, 3], [1, 2, 6], [1, 6, 5]], np.int64)
    return v, f


def uv_sphere(nu, nv):
    """Unit sphere of nu latitude bands x nv longitude steps: (nu + 1) * nv
    vertices (the poles repeated per step) and 2 * nu * nv triangles."""
    th = np.pi * np.arange(nu + 1) / nu
    ph = 2 * np.pi * np.arange(nv) / nv
    v = np.stack([np.outer(np.sin(th), np.cos(ph)), np.outer(np.cos(th), np.ones(nv)),
                  np.outer(np.sin(th), np.sin(ph))], axis=-1).reshape(-1, 3)
    f = []
    for i in range(nu):
        for j in range(nv):
            a, b = i * nv + j, i * nv + (j + 1) % nv
            c, d = a + nv, b + nv
            f += [[a, c, b], [b, c, d]]
    return v, np.array(f)


# Hitbox fixture of the point-in-mesh tests: a 9216-triangle sphere as
# "ball" (untransformed) and as "egg" (translated, rotated, scaled).
HITBOX_EGG = {"translation": [0.3, -0.2, 0.1], "rotation": [0.2, float(np.sin(0.5)), 0.1, float(np.cos(0.5))],
              "scale": [1.2, 0.7, 1.6]}


def hitbox_scene(path):
    """Writes the hitbox fixture scene (a ground triangle, the two hitboxes,
    a perspective camera) to `path`; returns the path."""
    v, f = uv_sphere(48, 96)
    g = GltfBuilder()
    g.mesh("ground", np.array([[-5, 0, -5], [5, 0, -5], [5, 0, 5]], np.float64), np.array([[0, 2, 1]]))
    g.mesh("ball", v, f, extras={"hitbox": True})
    g.mesh("egg", v, f, extras={"hitbox": True}, **HITBOX_EGG)
    g.perspective_camera("cam")
    return g.write(path)


def hitbox_points(seed=12, n_random=2400, n_vertex=600):
    """Query points of the hitbox tests: uniform points around the sphere,
    then points whose (y, z) is a vertex's (rays along x through vertices
    and edges), the first half with both y and z from one vertex."""
    rng = np.random.default_rng(seed)
    vf = uv_sphere(48, 96)[0].astype(np.float32)
    on_vertex = np.stack([rng.uniform(-1.1, 1.1, n_vertex).astype(np.float32),
                          vf[rng.integers(0, len(vf), n_vertex), 1], vf[rng.integers(0, len(vf), n_vertex), 2]], axis=1)
    on_vertex[:n_vertex // 2, 1:] = vf[rng.integers(0, len(vf), n_vertex // 2)][:, 1:]
    return np.concatenate([rng.uniform(-1.4, 1.4, size=(n_random, 3)).astype(np.float32), on_vertex])


def value_noise(nx, nz, octaves, rng):
    """Sum of `octaves` bilinearly interpolated lattice-noise layers on an
    (nx, nz) vertex grid, frequency doubling and amplitude halving per octave;
    normalised to [-1, 1]."""
    h = np.zeros((nx, nz))
    amp = 1.0
    for o in range(octaves):
        cells = 4 * (2 ** o)
        lat = rng.uniform(-1.0, 1.0, size=(cells + 1, cells + 1))
        u = np.linspace(0.0, cells, nx)
        w = np.linspace(0.0, cells, nz)
        i0 = np.minimum(np.floor(u).astype(int), cells - 1)
        j0 = np.minimum(np.floor(w).astype(int), cells - 1)
        fu = (u - i0)[:, None]
        fw = (w - j0)[None, :]
        fu = fu * fu * (3 - 2 * fu)
        fw = fw * fw * (3 - 2 * fw)
        a = lat[i0][:, j0]
        b = lat[i0 + 1][:, j0]
        c = lat[i0][:, j0 + 1]
        d = lat[i0 + 1][:, j0 + 1]
        h += amp * ((a * (1 - fu) + b * fu) * (1 - fw) + (c * (1 - fu) + d * fu) * fw)
        amp *= 0.5
    h -= h.min()
    h /= max(h.max(), 1e-12)
    return 2.0 * h - 1.0


def cone_mesh(cx, cy, cz, radius, height, segments=16):
    """Cone with `segments` side and `segments` base triangles."""
    ang = np.arange(segments) * (2 * math.pi / segments)
    ring = np.stack([cx + radius * np.cos(ang), np.full(segments, cy), cz + radius * np.sin(ang)], axis=1)
    apex = np.array([[cx, cy + height, cz]])
    centre = np.array([[cx, cy, cz]])
    verts = np.concatenate([ring, apex, centre])
    a, c = segments, segments + 1
    tris = []
    for k in range(segments):
        k1 = (k + 1) % segments
        tris.append([k, a, k1])
        tris.append([k, k1, c])
    return verts, np.array(tris, np.int64)


def droplet_eye(n, rng, wavelength=1.0, size=0.002):
    """Ommatidia on the sinewave-droplet surface y = sin(wavelength * r)
    over the square [-0.5, 0.5]^2, with the surface normal construction of
    eyeGenerator/SinewaveDropletCoordinate.cpp:33-60 (a point pulled 1% towards
    the centre gives the radial tangent; crossing with the vertical twice
    gives the normal).  Points are a jittered grid; the whole eye is scaled to
    `size` metres."""
    side = int(math.ceil(math.sqrt(n)))
    gx, gz = np.meshgrid((np.arange(side) + 0.5) / side - 0.5, (np.arange(side) + 0.5) / side - 0.5, indexing="ij")
    pts = np.stack([gx.ravel(), gz.ravel()], axis=1)
    pts = pts[rng.permutation(len(pts))[:n]]
    pts += rng.uniform(-0.4 / side, 0.4 / side, size=pts.shape)
    r = np.linalg.norm(pts, axis=1)
    pos = np.stack([pts[:, 0], np.sin(wavelength * r), pts[:, 1]], axis=1)
    inner = pts * 0.99
    ri = np.linalg.norm(inner, axis=1)
    inner3 = np.stack([inner[:, 0], np.sin(wavelength * ri), inner[:, 1]], axis=1)
    diff = inner3 - pos
    diff /= np.linalg.norm(diff, axis=1, keepdims=True)
    up = np.array([0.0, 1.0, 0.0])
    temp = np.cross(up, diff)
    temp /= np.linalg.norm(temp, axis=1, keepdims=True)
    normal = np.cross(temp, diff)
    normal /= np.linalg.norm(normal, axis=1, keepdims=True)
    return pos * size, normal


def rotation_about(axis, angle):
    """3x3 rotation (row-major) about a unit axis (Rodrigues)."""
    a = np.asarray(axis, np.float64)
    a = a / np.linalg.norm(a)
    c, s = math.cos(angle), math.sin(angle)
    k = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    return c * np.eye(3) + s * k + (1 - c) * np.outer(a, a)


def pose_rows(position, yaw):
    """12-float pose (position, local x, y, z axes) for a yaw about world Y,
    the frame setCameraPose(p, 0, yaw, 0) produces."""
    r = rotation_about([0, 1, 0], yaw)
    x, y, z = r[:, 0], r[:, 1], r[:, 2]
    return np.concatenate([position, x, y, z]).astype(np.float32)


# ---------------------------------------------------------------------------
# Workloads
# ---------------------------------------------------------------------------
def small_scene(outdir, seed=SEED, n_omm=1000, spp=32):
    """Ground + 64 boxes + simple_sky and a Fibonacci-sphere eye.  Returns a
    dict with the glTF path, eye path, pose (12 floats) and spp."""
    os.makedirs(outdir, exist_ok=True)
    rng = np.random.default_rng(seed)
    g = GltfBuilder()
    g.scene_extras = {"background-shader": "simple_sky"}
    ground = np.array([[-10, 0, -10], [10, 0, -10], [10, 0, 10], [-10, 0, 10]], np.float64)
    g.mesh("ground", ground, np.array([[0, 2, 1], [0, 3, 2]]), colours=np.tile([0.5, 0.5, 0.5, 1.0], (4, 1)))
    verts, faces, cols, boxes = [], [], [], []
    placed = 0
    while placed < 64:
        c = rng.uniform(-8.0, 8.0, size=2)
        e = rng.uniform(0.2, 2.0, size=3)
        col = np.concatenate([rng.uniform(0.0, 1.0, size=(8, 3)), np.ones((8, 1))], axis=1)
        # Keep the eye (0, 0.5, 0) outside every box.
        if abs(c[0]) < e[0] / 2 + 0.3 and abs(c[1]) < e[2] / 2 + 0.3:
            continue
        lo, hi = [c[0] - e[0] / 2, 0.0, c[1] - e[2] / 2], [c[0] + e[0] / 2, e[1], c[1] + e[2] / 2]
        v, f = box_mesh(lo, hi)
        faces.append(f + 8 * placed)
        verts.append(v)
        cols.append(col)
        boxes.append((lo, hi))
        placed += 1
    g.mesh("boxes", np.concatenate(verts), np.concatenate(faces), colours=np.concatenate(cols))
    d = fibonacci_sphere(n_omm)
    eye_path = os.path.join(outdir, "small.eye")
    write_eye(eye_path, d * 0.001, d, 3.0 * DEG, 0.0)
    g.compound_camera("insect-eye", "small.eye", translation=[0.0, 0.5, 0.0])
    path = g.write(os.path.join(outdir, "small.gltf"), embed=True)
    pose = pose_rows(np.array([0.0, 0.5, 0.0]), 0.0)
    return {"gltf": path, "eye": eye_path, "pose": pose, "spp": spp, "n_omm": n_omm,
            "boxes": np.asarray(boxes, np.float64)}


def open_poses(boxes, count, rng, half_width=8.0, eye_height=0.5, margin=0.05):
    """(count, 12) random poses of the small scene: x, z uniform in
    +-half_width, `eye_height` above the ground, uniform yaw, outside every
    box (boxes: (n, 2, 3) min/max corners) by at least `margin`."""
    out = np.zeros((count, 12), np.float32)
    i = 0
    while i < count:
        x, z = rng.uniform(-half_width, half_width, size=2)
        yaw = rng.uniform(0, 2 * math.pi)
        p = np.array([x, eye_height, z])
        inside = ((boxes[:, 0] - margin <= p) & (p <= boxes[:, 1] + margin)).all(axis=1)
        if inside.any():
            continue
        out[i] = pose_rows(p, yaw)
        i += 1
    return out


def textured_scene(outdir, seed=SEED, n_omm=1000, spp=32):
    """Textured variant of the small scene: a ground quad with an RGB noise
    texture repeated through wrapped coordinates in [-3.3, 4.7], 24 boxes
    with textures of the other PNG forms (palette, 4-bit grey, grey+alpha,
    RGBA, Adam7-interlaced; no TEXCOORD_0, so they sample at the hit's
    barycentrics), 4 boxes with vertex colours under a textured material
    (vertex colours win) and 4 plain boxes; simple_sky.  Images are stored
    as data URIs, bufferViews and external files.  Returns the small-scene
    dict plus the decoded RGBA arrays of the images in order."""
    os.makedirs(outdir, exist_ok=True)
    rng = np.random.default_rng(seed + 7)
    g = GltfBuilder()
    g.scene_extras = {"background-shader": "simple_sky"}
    images = []

    def add_image(rgba_expected, data, how):
        images.append(np.asarray(rgba_expected, np.uint8))
        return g.texture(g.image(data, how=how, name="tex%d" % len(images)))

    # 64 x 48 RGB noise, every filter type, data URI
    rgb = rng.integers(0, 256, size=(48, 64, 3), dtype=np.uint8)
    t_ground = add_image(np.concatenate([rgb, np.full((48, 64, 1), 255, np.uint8)], axis=2),
                         png_bytes(rgb, colour_type=2), "data")
    # 16 x 16 palette of 12 colours with tRNS, bufferView
    pal = rng.integers(0, 256, size=(12, 3), dtype=np.uint8)
    idx = rng.integers(0, 12, size=(16, 16), dtype=np.uint8)
    trns = rng.integers(0, 256, size=5, dtype=np.uint8)
    alpha = np.full(12, 255, np.uint8)
    alpha[:5] = trns
    t_pal = add_image(np.concatenate([pal[idx], alpha[idx][:, :, None]], axis=2),
                      png_bytes(idx, colour_type=3, palette=pal, trns=trns.tobytes()), "bufferView")
    # 20 x 12 4-bit grey, external file
    grey4 = rng.integers(0, 16, size=(12, 20), dtype=np.uint8)
    g8 = (grey4.astype(np.int32) * 17).astype(np.uint8)
    t_grey = add_image(np.stack([g8, g8, g8, np.full_like(g8, 255)], axis=2),
                       png_bytes(grey4, colour_type=0, depth=4), "file")
    # 9 x 7 grey + alpha
    ga = rng.integers(0, 256, size=(7, 9, 2), dtype=np.uint8)
    t_ga = add_image(np.stack([ga[:, :, 0]] * 3 + [ga[:, :, 1]], axis=2), png_bytes(ga, colour_type=4), "data")
    # 33 x 17 RGBA, Adam7 interlaced, with a sampler (ignored: wrap + linear)
    rgba = rng.integers(0, 256, size=(17, 33, 4), dtype=np.uint8)
    t_rgba = add_image(rgba, png_bytes(rgba, colour_type=6, interlace=True), "data")
    g.samplers.append({"wrapS": 33071, "wrapT": 33648, "magFilter": 9728, "minFilter": 9728})
    g.textures[t_rgba]["sampler"] = len(g.samplers) - 1

    ground = np.array([[-10, 0, -10], [10, 0, -10], [10, 0, 10], [-10, 0, 10]], np.float64)
    uv = np.array([[-3.3, -3.3], [4.7, -3.3], [4.7, 4.7], [-3.3, 4.7]], np.float32)
    g.mesh("ground", ground, np.array([[0, 2, 1], [0, 3, 2]]), material=g.textured_material(t_ground),
           texcoords=uv)
    box_tex = [t_pal, t_grey, t_ga, t_rgba]
    mats = [g.textured_material(t) for t in box_tex]
    plain = g.material([0.8, 0.3, 0.2, 1.0])
    placed = 0
    while placed < 32:
        c = rng.uniform(-8.0, 8.0, size=2)
        e = rng.uniform(0.2, 2.0, size=3)
        if abs(c[0]) < e[0] / 2 + 0.3 and abs(c[1]) < e[2] / 2 + 0.3:
            continue
        v, f = box_mesh([c[0] - e[0] / 2, 0.0, c[1] - e[2] / 2], [c[0] + e[0] / 2, e[1], c[1] + e[2] / 2])
        if placed < 24:
            g.mesh("tbox%d" % placed, v, f, material=mats[placed % 4])
        elif placed < 28:
            col = np.concatenate([rng.uniform(0.0, 1.0, size=(8, 3)), np.ones((8, 1))], axis=1)
            g.mesh("cbox%d" % placed, v, f, colours=col, material=mats[placed % 4])
        else:
            g.mesh("pbox%d" % placed, v, f, material=plain)
        placed += 1
    d = fibonacci_sphere(n_omm)
    eye_path = os.path.join(outdir, "textured.eye")
    write_eye(eye_path, d * 0.001, d, 3.0 * DEG, 0.0)
    g.compound_camera("insect-eye", "textured.eye", translation=[0.0, 0.5, 0.0])
    path = g.write(os.path.join(outdir, "textured.gltf"), embed=True)
    pose = pose_rows(np.array([0.0, 0.5, 0.0]), 0.0)
    return {"gltf": path, "eye": eye_path, "pose": pose, "spp": spp, "n_omm": n_omm, "images": images}


def fixture_scene(npz, variant, outdir):
    """Rebuilds a flattened fixture scene (tests/golden/reference_test_scene.npz
    layout) as glTF + .eye files: one mesh per material colour (shading kind
    0) and one vertex-coloured mesh (kind 1), world-space vertices, and each
    compound camera at its stored pose through a node matrix whose columns
    are the local x, y and -z axes.  Returns the glTF path."""
    os.makedirs(outdir, exist_ok=True)
    z = np.load(npz) if isinstance(npz, str) else npz
    v = z[variant + "__verts"]
    c = z[variant + "__colours"]
    f = z[variant + "__flags"]
    g = GltfBuilder()
    g.scene_extras = {"background-shader": "simple_sky" if int(z[variant + "__miss"]) == 1 else "default_background"}
    flat = f == 0
    if flat.any():
        keys = c[flat][:, 0, :]
        uniq, inv = np.unique(keys, axis=0, return_inverse=True)
        tri_idx = np.where(flat)[0]
        for m, col in enumerate(uniq):
            sel = tri_idx[inv.reshape(-1) == m]
            pos = v[sel].reshape(-1, 3).astype(np.float64)
            g.mesh("flat%d" % m, pos, np.arange(len(pos)).reshape(-1, 3), material=g.material(col), index_type=5125)
    if (f == 1).any():
        sel = np.where(f == 1)[0]
        pos = v[sel].reshape(-1, 3).astype(np.float64)
        g.mesh("coloured", pos, np.arange(len(pos)).reshape(-1, 3), colours=c[sel].reshape(-1, 4), index_type=5125)
    for k, name in enumerate(z[variant + "__cams"]):
        key = "%s__cam%d" % (variant, k)
        pose = z[key + "__pose"].astype(np.float64)
        omm = z[key + "__omm"]
        eye = os.path.join(outdir, "%s_cam%d.eye" % (variant, k))
        write_eye(eye, omm[:, :3], omm[:, 3:6], omm[:, 6], omm[:, 7])
        ls = pose[3:].reshape(3, 3)
        cols = [ls[0], ls[1], -ls[2], pose[:3]]
        matrix = [float(cols[j][i]) if i < 3 else (1.0 if j == 3 else 0.0) for j in range(4) for i in range(4)]
        g.cameras.append({"name": str(name), "type": "perspective",
                          "perspective": {"yfov": 0.4, "znear": 0.1, "zfar": 100.0},
                          "extras": {"compound-eye": "true", "compound-structure": os.path.basename(eye),
                                     "compound-projection": str(z[key + "__projection"])}})
        g.nodes.append({"name": str(name), "camera": len(g.cameras) - 1, "matrix": matrix})
    return g.write(os.path.join(outdir, variant + ".gltf"), embed=True)


def lit_scene(outdir, seed=SEED, n_omm=600, spp=16):
    """A scene for the lighting-on path: a ground quad with vertex normals,
    a base-colour texture and a normal texture; 24 boxes, half with smooth
    vertex normals (corner directions) and half with flat normals, on
    materials of random metallic / roughness factors, some with a
    metallic-roughness texture and some with a normal texture, a few under a
    rotated and uniformly scaled node; simple_sky.  Returns the small-scene
    dict."""
    os.makedirs(outdir, exist_ok=True)
    rng = np.random.default_rng(seed + 13)
    g = GltfBuilder()
    g.scene_extras = {"background-shader": "simple_sky"}
    rgb = rng.integers(0, 256, size=(16, 16, 3), dtype=np.uint8)
    t_base = g.texture(g.image(png_bytes(rgb, colour_type=2)))
    nrm = np.clip(np.stack([rng.normal(0.5, 0.08, (8, 8)), rng.normal(0.5, 0.08, (8, 8)),
                            rng.uniform(0.85, 1.0, (8, 8))], axis=2) * 255, 0, 255).astype(np.uint8)
    t_norm = g.texture(g.image(png_bytes(nrm, colour_type=2)))
    mr = np.stack([np.full((8, 8), 255), rng.integers(60, 256, (8, 8)), rng.integers(0, 256, (8, 8))],
                  axis=2).astype(np.uint8)
    t_mr = g.texture(g.image(png_bytes(mr, colour_type=2)))
    ground = np.array([[-10, 0, -10], [10, 0, -10], [10, 0, 10], [-10, 0, 10]], np.float64)
    g.mesh("ground", ground, np.array([[0, 2, 1], [0, 3, 2]]),
           material=g.material([1, 1, 1, 1], metallic=0.0, roughness=0.7, base_texture=t_base, normal_texture=t_norm),
           texcoords=np.array([[0, 0], [4, 0], [4, 4], [0, 4]], np.float32), normals=np.tile([0, 1, 0], (4, 1)))
    placed = 0
    while placed < 24:
        c = rng.uniform(-7.0, 7.0, size=2)
        e = rng.uniform(0.3, 1.6, size=3)
        if abs(c[0]) < e[0] / 2 + 0.4 and abs(c[1]) < e[2] / 2 + 0.4:
            continue
        v, f = box_mesh([c[0] - e[0] / 2, 0.0, c[1] - e[2] / 2], [c[0] + e[0] / 2, e[1], c[1] + e[2] / 2])
        kw = {}
        if placed % 2 == 0:
            centre = v.mean(axis=0)
            n = v - centre
            kw["normals"] = n / np.linalg.norm(n, axis=1, keepdims=True)
        if placed % 3 == 0:
            kw["texcoords"] = rng.uniform(-1, 2, size=(8, 2)).astype(np.float32)
        mat = g.material(np.concatenate([rng.uniform(0.1, 1.0, 3), [1.0]]), metallic=rng.uniform(0, 1),
                         roughness=rng.uniform(0.2, 1.0), mr_texture=t_mr if placed % 4 == 1 else None,
                         normal_texture=t_norm if placed % 4 == 2 else None)
        if placed >= 20:  # rotated and uniformly scaled about the origin
            g.mesh("rbox%d" % placed, v * 0.5, f, material=mat, rotation=[0.0, math.sin(0.3), 0.0, math.cos(0.3)],
                   scale=[1.5, 1.5, 1.5], **kw)
        else:
            g.mesh("box%d" % placed, v, f, material=mat, **kw)
        placed += 1
    d = fibonacci_sphere(n_omm)
    eye_path = os.path.join(outdir, "lit.eye")
    write_eye(eye_path, d * 0.001, d, 3.0 * DEG, 0.0)
    g.compound_camera("insect-eye", "lit.eye", translation=[0.0, 0.5, 0.0])
    path = g.write(os.path.join(outdir, "lit.gltf"), embed=True)
    pose = pose_rows(np.array([0.0, 0.5, 0.0]), 0.0)
    return {"gltf": path, "eye": eye_path, "pose": pose, "spp": spp, "n_omm": n_omm}


def terrain_height_fn(heights, extent):
    """Bilinear lookup in the heightfield vertex grid (heights[i, j] at
    x = -extent/2 + i*dx, z = -extent/2 + j*dz)."""
    n = heights.shape[0] - 1
    cell = extent / n

    def h(x, z):
        u = np.clip((x + extent / 2) / cell, 0, n - 1e-9)
        w = np.clip((z + extent / 2) / cell, 0, n - 1e-9)
        i, j = int(u), int(w)
        fu, fw = u - i, w - j
        return ((heights[i, j] * (1 - fu) + heights[i + 1, j] * fu) * (1 - fw)
                + (heights[i, j + 1] * (1 - fu) + heights[i + 1, j + 1] * fu) * fw)
    return h


def terrain_scene(outdir, seed=SEED, cells=512, extent=200.0, cones=2000, n_omm=6000, spp=256, poses=1024,
                  eye_height=0.5, eye_kind="droplet", aa_deg=(1.5, 4.0)):
    """Heightfield + cones and an eye with a random-walk trajectory: the
    sinewave-droplet eye, or (eye_kind "panoramic") a Fibonacci sphere of
    radius 1 mm looking in every direction.  Acceptance angles U(aa_deg).
    Returns a dict with paths, the (poses, 12) trajectory and spp."""
    os.makedirs(outdir, exist_ok=True)
    rng = np.random.default_rng(seed)
    g = GltfBuilder()
    g.scene_extras = {"background-shader": "simple_sky"}
    n = cells + 1
    heights = 2.0 * value_noise(n, n, 6, rng)
    xs = np.linspace(-extent / 2, extent / 2, n)
    X, Z = np.meshgrid(xs, xs, indexing="ij")
    pos = np.stack([X.ravel(), heights.ravel(), Z.ravel()], axis=1)
    t = (heights.ravel() + 2.0) / 4.0
    low, mid, high = np.array([0.20, 0.35, 0.10]), np.array([0.45, 0.35, 0.20]), np.array([0.85, 0.85, 0.80])
    col = np.where(t[:, None] < 0.5, low + (mid - low) * (t[:, None] / 0.5), mid + (high - mid) * ((t[:, None] - 0.5) / 0.5))
    col = np.concatenate([col, np.ones((len(col), 1))], axis=1)
    ii, jj = np.meshgrid(np.arange(cells), np.arange(cells), indexing="ij")
    v00 = (ii * n + jj).ravel()
    v10 = ((ii + 1) * n + jj).ravel()
    v01 = (ii * n + jj + 1).ravel()
    v11 = ((ii + 1) * n + jj + 1).ravel()
    faces = np.stack([np.stack([v00, v01, v10], 1), np.stack([v10, v01, v11], 1)], axis=1).reshape(-1, 3)
    g.mesh("terrain", pos, faces, colours=col, index_type=5125)
    hfn = terrain_height_fn(heights, extent)
    cv, cf, cc = [], [], []
    nv = 0
    for k in range(cones):
        x, z = rng.uniform(-extent / 2 + 5, extent / 2 - 5, size=2)
        hgt = math.exp(rng.uniform(math.log(0.3), math.log(3.0)))
        rad = hgt * rng.uniform(0.1, 0.3)
        v, f = cone_mesh(x, hfn(x, z) - 0.05, z, rad, hgt)
        tt = (v[:, 1] - v[:, 1].min()) / max(hgt, 1e-6)
        c = np.stack([0.05 + 0.2 * tt, 0.3 + 0.5 * tt, 0.05 + 0.1 * tt, np.ones_like(tt)], axis=1)
        cf.append(f + nv)
        nv += len(v)
        cv.append(v)
        cc.append(c)
    g.mesh("plants", np.concatenate(cv), np.concatenate(cf), colours=np.concatenate(cc), index_type=5125)
    if eye_kind == "droplet":
        epos, edir = droplet_eye(n_omm, rng)
    else:
        edir = fibonacci_sphere(n_omm)
        epos = edir * 0.001
    aa = rng.uniform(aa_deg[0] * DEG, aa_deg[1] * DEG, size=n_omm)
    eye_name = "droplet" if eye_kind == "droplet" else "panoramic"
    eye_path = os.path.join(outdir, eye_name + ".eye")
    write_eye(eye_path, epos, edir, aa, 0.0)
    g.compound_camera(eye_name + "-eye", eye_name + ".eye", translation=[0.0, hfn(0.0, 0.0) + eye_height, 0.0])
    path = g.write(os.path.join(outdir, "terrain.gltf"), embed=False)
    traj = random_walk(hfn, poses, rng, eye_height=eye_height)
    return {"gltf": path, "eye": eye_path, "poses": traj, "spp": spp, "n_omm": n_omm,
            "triangles": int(len(faces) + 32 * cones), "height_fn": hfn, "extent": extent, "eye_height": eye_height}


def random_poses(hfn, count, rng, half_width, eye_height=0.5):
    """(count, 12) independent poses: x, z uniform in +-half_width, height
    terrain + eye_height, uniform yaw."""
    out = np.zeros((count, 12), np.float32)
    for i in range(count):
        x, z = rng.uniform(-half_width, half_width, size=2)
        out[i] = pose_rows(np.array([x, hfn(x, z) + eye_height, z]), rng.uniform(0, 2 * math.pi))
    return out


def random_walk(hfn, count, rng, step=0.1, yaw_sd=10.0 * DEG, eye_height=0.5):
    """(count, 12) poses: 0.1 m steps along the heading, heading noise N(0, 10 deg),
    height = terrain + eye_height."""
    out = np.zeros((count, 12), np.float32)
    x = z = 0.0
    yaw = rng.uniform(0, 2 * math.pi)
    for i in range(count):
        out[i] = pose_rows(np.array([x, hfn(x, z) + eye_height, z]), yaw)
        yaw += rng.normal(0.0, yaw_sd)
        x += step * math.sin(yaw)
        z += step * math.cos(yaw)
    return out


def batch_scene(outdir, seed=SEED, n_eyes=64, poses_per_eye=16, n_min=500, n_max=30000,
                spp_choices=tuple(range(16, 513, 16)), aa_deg=(1.0, 6.0)):
    """The small scene (ground + 64 boxes, simple_sky) with `n_eyes` compound
    cameras of uneven size: ommatidium counts log-uniform in [n_min, n_max]
    on Fibonacci spheres of radius 1 mm, acceptance angles uniform in aa_deg,
    per-eye sample counts drawn from spp_choices, and `poses_per_eye` random
    poses per eye (0.5 m above the ground, random yaw, within +-8 m).
    Returns a dict with the glTF path, per-eye N and spp, and the poses
    (n_eyes, poses_per_eye, 12)."""
    base = small_scene(outdir, seed=seed)
    rng = np.random.default_rng(seed + 3)
    with open(base["gltf"]) as f:
        doc = json.load(f)
    ns, spps = [], []
    cams = doc.setdefault("cameras", [])
    for e in range(n_eyes):
        n = int(round(math.exp(rng.uniform(math.log(n_min), math.log(n_max)))))
        aa = rng.uniform(aa_deg[0] * DEG, aa_deg[1] * DEG)
        d = fibonacci_sphere(n)
        name = "batch-eye-%02d.eye" % e
        write_eye(os.path.join(outdir, name), d * 0.001, d, aa, 0.0)
        cams.append({"name": "batch-eye-%02d" % e, "type": "perspective",
                     "perspective": {"yfov": 0.4, "znear": 0.1, "zfar": 100.0},
                     "extras": {"compound-eye": "true", "compound-structure": name,
                                "compound-projection": "single_dimension_fast"}})
        doc["nodes"].append({"name": "batch-eye-%02d" % e, "camera": len(cams) - 1, "translation": [0.0, 0.5, 0.0]})
        doc["scenes"][0]["nodes"].append(len(doc["nodes"]) - 1)
        ns.append(n)
        spps.append(int(rng.choice(spp_choices)))
    poses = np.zeros((n_eyes, poses_per_eye, 12), np.float32)
    for e in range(n_eyes):
        for k in range(poses_per_eye):
            poses[e, k] = pose_rows(np.array([rng.uniform(-8, 8), 0.5, rng.uniform(-8, 8)]), rng.uniform(0, 2 * math.pi))
    path = os.path.join(outdir, "batch.gltf")
    with open(path, "w") as f:
        json.dump(doc, f)
    return {"gltf": path, "n": ns, "spp": spps, "poses": poses, "first_batch_camera": 1}
