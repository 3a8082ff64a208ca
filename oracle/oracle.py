"""Python side of the CPU oracle.  TEST INFRASTRUCTURE ONLY: imported by
tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
checker, never by the product.

Parity status: unpinned against the reference's own outputs (the reference
needs OptiX and a window and ships no golden renders); the oracle restates
the reference's shader and scene arithmetic, see oracle.cpp and gltf_ref.py.
"""
import ctypes
import os
import subprocess
from ctypes import c_double, c_float, c_int, c_size_t, c_uint32, c_void_p

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SRC = os.path.join(HERE, "oracle.cpp")


def build(force=False):
    """Compiles oracle.cpp with OpenMP (no contraction of float operations)."""
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    tmp = LIB + ".tmp"
    cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
           SRC, "-o", tmp]
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + proc.stdout)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(build())
        f32 = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
        i32 = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
        f64 = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
        u8 = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
        L.orc_scene_create.argtypes = [f32, f32, u8, c_uint32]
        L.orc_scene_create.restype = c_void_p
        L.orc_scene_destroy.argtypes = [c_void_p]
        L.orc_trace.argtypes = [c_void_p, f32, f32, f32, c_float, c_size_t, i32, f32, f32, f32, c_int]
        L.orc_trace_f64.argtypes = [c_void_p, f32, f32, f32, c_double, c_size_t, c_void_p, i32, f64, f64, f64, c_int]
        L.orc_shade.argtypes = [c_void_p, c_int, f32, i32, f32, f32, c_size_t, f32]
        L.orc_gen_rays.argtypes = [f32, c_uint32, c_uint32, f32, f32, f32, f32]
        L.orc_render_rays.argtypes = [c_void_p, c_int, f32, c_uint32, c_uint32, c_uint32, f32, f32, f32, c_int]
        L.orc_render_draws.argtypes = [c_void_p, c_int, f32, c_uint32, c_uint32, c_uint32, f32, f32, f32, c_int]
        L.orc_render_draws.restype = c_size_t
        L.orc_make_color.argtypes = [f32, c_size_t, u8]
        u32 = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
        L.orc_scene_set_textures.argtypes = [c_void_p, u32, c_size_t, i32, c_uint32]
        L.orc_scene_set_lighting.argtypes = [c_void_p, f32, f32, f32, c_int]
        L.orc_sample_texture.argtypes = [u32, c_int, c_int, f32, c_size_t, f32]
        L.orc_max_threads.restype = c_int
        _lib = L
    return _lib


def _f32(a):
    return np.ascontiguousarray(a, np.float32)


class OracleScene:
    """World-space triangles (T,3,3), colour records (T,3,4), shading kinds
    (T,) (0 base colour, 1 vertex colours, 2 texture with (u, v, texture, 0)
    records), the miss shader id (0 = default_background, 1 = simple_sky) and
    optionally the textures: (table (K,3) of first texel / width / height,
    RGBA8 texels as uint32)."""

    def __init__(self, verts, colours, flags, miss, textures=None):
        self.verts = _f32(verts).reshape(-1, 9)
        self.colours = _f32(colours).reshape(-1, 12)
        self.flags = np.ascontiguousarray(flags, np.uint8).reshape(-1)
        self.miss = int(miss)
        self.T = len(self.flags)
        self._h = lib().orc_scene_create(self.verts, self.colours, self.flags, self.T)
        if textures is not None:
            table = np.ascontiguousarray(textures[0], np.int32).reshape(-1)
            texels = np.ascontiguousarray(textures[1], np.uint32).reshape(-1)
            self._tex = (table, texels)
            lib().orc_scene_set_textures(self._h, texels, texels.size, table, table.size // 3)

    def set_lighting(self, light, light_pos, light_col, on=True):
        """Lighting-on shading: (T, 20) per-triangle data, (4, 4) light
        positions + intensities, (4, 3) colours."""
        self._light = _f32(light).reshape(-1)
        assert self._light.size == 20 * self.T
        lib().orc_scene_set_lighting(self._h, self._light, _f32(light_pos).reshape(-1), _f32(light_col).reshape(-1),
                                     1 if on else 0)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_scene_destroy(self._h)
            self._h = None

    def trace(self, org, dirs, tmin, tmax=1e16, threads=0):
        org, dirs = _f32(org).reshape(-1, 3), _f32(dirs).reshape(-1, 3)
        n = len(org)
        tmin = _f32(np.broadcast_to(np.asarray(tmin, np.float32), (n,)))
        hit = np.zeros(n, np.int32)
        t = np.zeros(n, np.float32)
        b1 = np.zeros(n, np.float32)
        b2 = np.zeros(n, np.float32)
        lib().orc_trace(self._h, org, dirs, tmin, tmax, n, hit, t, b1, b2, threads)
        return hit, t, b1, b2

    def trace_f64(self, org, dirs, tmin, hit32=None, tmax=1e16, threads=0):
        org, dirs = _f32(org).reshape(-1, 3), _f32(dirs).reshape(-1, 3)
        n = len(org)
        tmin = _f32(np.broadcast_to(np.asarray(tmin, np.float32), (n,)))
        hit = np.zeros(n, np.int32)
        t = np.zeros(n, np.float64)
        e32 = np.zeros(n, np.float64)
        e64 = np.zeros(n, np.float64)
        h32 = None
        if hit32 is not None:
            hit32 = np.ascontiguousarray(hit32, np.int32)
            h32 = hit32.ctypes.data
        lib().orc_trace_f64(self._h, org, dirs, tmin, tmax, n, h32, hit, t, e32, e64, threads)
        return hit, t, e32, e64

    def shade(self, dirs, hit, b1, b2):
        dirs = _f32(dirs).reshape(-1, 3)
        n = len(dirs)
        out = np.zeros((n, 3), np.float32)
        lib().orc_shade(self._h, self.miss, dirs, np.ascontiguousarray(hit, np.int32), _f32(b1), _f32(b2), n, out)
        return out

    def render_rays(self, omm, spp, org, dirs, poses=1, threads=0):
        omm = _f32(omm).reshape(-1, 8)
        N = len(omm)
        out = np.zeros((poses, N, 3), np.float32)
        lib().orc_render_rays(self._h, self.miss, omm, N, spp, poses, _f32(org).reshape(-1),
                              _f32(dirs).reshape(-1), out, threads)
        return out

    def render_draws(self, omm, spp, poses12, draws, threads=0):
        omm = _f32(omm).reshape(-1, 8)
        poses12 = _f32(poses12).reshape(-1, 12)
        N, P = len(omm), len(poses12)
        draws = _f32(draws).reshape(-1)
        assert draws.size == 2 * P * N * spp
        out = np.zeros((P, N, 3), np.float32)
        lib().orc_render_draws(self._h, self.miss, omm, N, spp, P, poses12, draws, out, threads)
        return out


def gen_rays(omm, spp, pose12, draws):
    omm = _f32(omm).reshape(-1, 8)
    N = len(omm)
    org = np.zeros((N * spp, 3), np.float32)
    dirs = np.zeros((N * spp, 3), np.float32)
    lib().orc_gen_rays(omm, N, spp, _f32(pose12).reshape(-1), _f32(draws).reshape(-1), org, dirs)
    return org, dirs


def sample_texture(texels, width, height, uv):
    """Bilinear lookups of one RGBA8 texture (uint32 texels, red in the low
    byte) at (n, 2) coordinates: (n, 4) float32."""
    texels = np.ascontiguousarray(texels, np.uint32).reshape(-1)
    assert texels.size == width * height
    uv = _f32(uv).reshape(-1, 2)
    out = np.zeros((len(uv), 4), np.float32)
    lib().orc_sample_texture(texels, int(width), int(height), uv.reshape(-1), len(uv), out)
    return out


def make_color(sums):
    sums = _f32(sums).reshape(-1, 3)
    out = np.zeros((len(sums), 4), np.uint8)
    lib().orc_make_color(sums, len(sums), out)
    return out


def max_threads():
    return lib().orc_max_threads()


# ---------------------------------------------------------------------------
# The reference's own code where it compiles here (oracle/build_ref.py).
# ---------------------------------------------------------------------------
REF_DIR = os.path.join(HERE, "_ref")


def reference_root():
    """The reference checkout used to build oracle/_ref ($CR_REFERENCE_ROOT,
    else the path the build recorded), or None."""
    root = os.environ.get("CR_REFERENCE_ROOT")
    if not root:
        try:
            with open(os.path.join(REF_DIR, "reference_root.txt")) as f:
                root = f.read().strip()
        except OSError:
            return None
    return root if root and os.path.isdir(root) else None


_ref_hitscan = None


def ref_hitscan():
    """ctypes handle of oracle/_ref/libref_hitscan.so (the reference's
    sutil::hitscan::isPointWithinMesh), or None when it is not built."""
    global _ref_hitscan
    if _ref_hitscan is None:
        path = os.path.join(REF_DIR, "libref_hitscan.so")
        if not os.path.exists(path):
            return None
        try:
            L = ctypes.CDLL(path)
        except OSError:  # a library built for another machine
            return None
        f32 = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
        u8 = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
        L.ref_points_in_mesh.argtypes = [f32, c_size_t, f32, f32, c_size_t, u8]
        L.ref_points_in_mesh.restype = c_int
        _ref_hitscan = L
    return _ref_hitscan


def ref_points_in_mesh(tris, xform, pts):
    """The reference's isPointWithinMesh for every point: tris (T, 9) object
    space, xform a 4x4 node transform (rounded to float, as the reference
    stores it), pts (n, 3) world points.  Returns n uint8 (1 = inside)."""
    L = ref_hitscan()
    if L is None:
        raise RuntimeError("oracle/_ref/libref_hitscan.so is not built (oracle/build_ref.py)")
    pts = _f32(pts).reshape(-1, 3)
    out = np.zeros(len(pts), np.uint8)
    if L.ref_points_in_mesh(_f32(tris).reshape(-1), len(tris), _f32(xform).reshape(-1), pts, len(pts), out) != 0:
        raise RuntimeError("empty hitbox mesh")
    return out


_MASK64 = (1 << 64) - 1


def _mix64(z):
    """SplitMix64's output function on Python ints (mod 2^64)."""
    z &= _MASK64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _MASK64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _MASK64
    return z ^ (z >> 31)


def net_draws(seed, entries, samples):
    """Draws (normal, uniform) of the adaptive render's sample `samples[i]`
    of entry `entries[i]`, restating netDraw (compound-ray_gb300/csrc/
    render.cu): point k of the two-dimensional Sobol' sequence (k
    bit-reversed; and the generator matrix with columns 2^31, v ^ (v >> 1),
    ...) XORed with a per-entry shift from SplitMix64's mix of seed +
    (entry + 1) * 0x9E3779B97F4A7C15; the first coordinate's top 23 bits
    through the inverse normal distribution at the middle of their cell
    (float64 here), the second's as 1 - x / 2^24.  The uniform draw is exact;
    the normal draw is the float64 value of what the GPU computes with
    normcdfinvf."""
    from statistics import NormalDist

    inv = NormalDist().inv_cdf
    entries = np.asarray(entries, np.int64).reshape(-1)
    samples = np.asarray(samples, np.int64).reshape(-1)
    nd = np.empty(len(entries), np.float64)
    ud = np.empty(len(entries), np.float32)
    shifts = {}
    for i, (e, k) in enumerate(zip(entries.tolist(), samples.tolist())):
        h = shifts.get(e)
        if h is None:
            h = shifts[e] = _mix64(seed + (e + 1) * 0x9E3779B97F4A7C15)
        x2, v, b = 0, 0x80000000, k
        while b:
            if b & 1:
                x2 ^= v
            b >>= 1
            v ^= v >> 1
        x1 = int("{:032b}".format(k)[::-1], 2) ^ (h & 0xFFFFFFFF)
        x2 ^= h >> 32
        nd[i] = inv(((x1 >> 9) + 0.5) / 8388608.0)
        ud[i] = np.float32(1.0) - np.float32((x2 >> 8) * (1.0 / 16777216.0))
    return nd, ud
