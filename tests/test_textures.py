"""Base colour textures on the host: PNG decoding of every colour type, bit
depth, filter, interlace and storage form against the arrays that were
encoded and against the oracle's independent decoder (Python zlib); the
texture shading records of the loaded scene against the oracle's loader;
refusals; and the oracle's bilinear filter against a numpy restatement."""
import os

import numpy as np
import pytest

import eyeRendererHelperFunctions as eh
import gltf_ref
import oracle
import scenes


def _load(lib, path):
    eh.lastError(lib)
    lib.loadGlTFscene(path.encode())
    return eh.lastError(lib)


def _one_texture_scene(tmp_path, png, how="data", texcoords=True, name="one"):
    g = scenes.GltfBuilder()
    t = g.texture(g.image(png, how=how))
    quad = np.array([[-1, 0, -1], [1, 0, -1], [1, 0, 1], [-1, 0, 1]], np.float64)
    uv = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32) if texcoords else None
    g.mesh("quad", quad, np.array([[0, 2, 1], [0, 3, 2]]), material=g.textured_material(t), texcoords=uv)
    g.perspective_camera("cam", translation=[0, 1, 0])
    return g.write(str(tmp_path / (name + ".gltf")), embed=True)


def test_textured_scene_loads_like_the_oracle_loader(lib, tmp_path):
    info = scenes.textured_scene(str(tmp_path))
    assert _load(lib, info["gltf"]) == ""
    v, c, f = eh.getSceneTriangles(lib)
    ref = gltf_ref.load(info["gltf"])
    rv, rc, rf = ref.arrays()
    assert np.array_equal(v.view(np.uint32), rv.view(np.uint32))
    assert np.array_equal(c.view(np.uint32), rc.view(np.uint32))
    assert np.array_equal(f, rf)
    # 2 ground + 24 textured boxes, 4 vertex-coloured (over a textured
    # material), 4 plain
    assert np.bincount(f, minlength=3).tolist() == [48, 48, 2 + 24 * 12]
    table, texels = eh.getSceneTextures(lib)
    rt, rtx = ref.textures()
    assert np.array_equal(table, rt) and np.array_equal(texels, rtx)
    assert len(table) == len(info["images"])
    for (off, w, h), want in zip(table, info["images"]):
        assert want.shape == (h, w, 4)
        assert np.array_equal(texels[off:off + w * h], scenes.rgba_words(want))
    # textured boxes without TEXCOORD_0 carry the (0,0) (1,0) (0,1) records
    box = f == 2
    uv = c[box][:, :, :2]
    assert (uv[2:] == np.array([[0, 0], [1, 0], [0, 1]], np.float32)).all()


@pytest.mark.parametrize("form", ["rgb8", "rgba8", "grey1", "grey2", "grey4", "grey8", "greyalpha", "pal1", "pal2",
                                  "pal4", "pal8", "interlaced", "interlaced_tiny", "stored", "onepixel"])
def test_png_forms(lib, tmp_path, form):
    rng = np.random.default_rng(abs(hash(form)) % 1000)
    h, w = 13, 29
    pal = rng.integers(0, 256, size=(256, 3), dtype=np.uint8)
    kw = {}
    if form in ("rgb8", "stored"):
        s = rng.integers(0, 256, size=(h, w, 3), dtype=np.uint8)
        want = np.concatenate([s, np.full((h, w, 1), 255, np.uint8)], axis=2)
        kw = dict(colour_type=2, level=0 if form == "stored" else 9)
    elif form in ("rgba8", "interlaced", "interlaced_tiny", "onepixel"):
        if form == "interlaced_tiny":
            h, w = 3, 5
        if form == "onepixel":
            h, w = 1, 1
        s = rng.integers(0, 256, size=(h, w, 4), dtype=np.uint8)
        want = s
        kw = dict(colour_type=6, interlace=form.startswith("interlaced"))
    elif form.startswith("grey") and form != "greyalpha":
        depth = int(form[4:])
        s = rng.integers(0, 1 << depth, size=(h, w), dtype=np.uint8)
        g8 = (s.astype(np.int32) * (255 // ((1 << depth) - 1))).astype(np.uint8)
        want = np.stack([g8, g8, g8, np.full_like(g8, 255)], axis=2)
        kw = dict(colour_type=0, depth=depth)
    elif form == "greyalpha":
        s = rng.integers(0, 256, size=(h, w, 2), dtype=np.uint8)
        want = np.stack([s[:, :, 0]] * 3 + [s[:, :, 1]], axis=2)
        kw = dict(colour_type=4)
    else:
        depth = int(form[3:])
        n = 1 << depth
        s = rng.integers(0, n, size=(h, w), dtype=np.uint8)
        trns = rng.integers(0, 256, size=min(n, 3), dtype=np.uint8)
        alpha = np.full(n, 255, np.uint8)
        alpha[:len(trns)] = trns
        want = np.concatenate([pal[:n][s], alpha[s][:, :, None]], axis=2)
        kw = dict(colour_type=3, depth=depth, palette=pal[:n], trns=trns.tobytes())
    png = scenes.png_bytes(s, **kw)
    path = _one_texture_scene(tmp_path, png, how=["data", "bufferView", "file"][len(form) % 3], name=form)
    assert _load(lib, path) == ""
    table, texels = eh.getSceneTextures(lib)
    assert table.tolist() == [[0, w, h]]
    assert np.array_equal(texels, scenes.rgba_words(want))
    assert np.array_equal(gltf_ref.decode_png(png), want)


def test_refusals(lib, tmp_path):
    s = np.arange(4 * 5 * 3, dtype=np.uint16).reshape(4, 5, 3) * 1000
    assert "16-bit" in _load(lib, _one_texture_scene(tmp_path, scenes.png_bytes(s, colour_type=2, depth=16), name="d16"))
    jpeg_like = b"\xff\xd8\xff\xe0" + bytes(64)
    assert "only PNG" in _load(lib, _one_texture_scene(tmp_path, jpeg_like, name="jpg"))
    png = bytearray(scenes.png_bytes(np.zeros((4, 4, 3), np.uint8), colour_type=2))
    assert "image 0" in _load(lib, _one_texture_scene(tmp_path, bytes(png[:40]), name="trunc"))
    # a material naming a texture that does not exist
    g = scenes.GltfBuilder()
    quad = np.array([[-1, 0, -1], [1, 0, -1], [1, 0, 1]], np.float64)
    g.mesh("tri", quad, np.array([[0, 2, 1]]), material=g.textured_material(3))
    g.perspective_camera("cam")
    assert "texture index out of range" in _load(lib, g.write(str(tmp_path / "badtex.gltf")))
    # the library stays usable
    assert _load(lib, _one_texture_scene(tmp_path, scenes.png_bytes(np.zeros((2, 2, 3), np.uint8), colour_type=2),
                                         name="ok")) == ""


def _numpy_sample(words, w, h, uv):
    """The bilinear rule restated in numpy (axis weights in 1/256 steps
    rounded half up, corner weights rounded to 1/256 ties-to-even, integer
    accumulation) as a check on the oracle's C version."""
    words = words.astype(np.int64)
    out = np.zeros((len(uv), 4), np.float32)
    for n, (u, v) in enumerate(uv.astype(np.float32)):
        idx, wts = [], []
        for c, size in ((u, w), (v, h)):
            f = np.float32(c - np.floor(c))
            xb = np.float32(f * np.float32(size)) - np.float32(0.5)
            fl = np.floor(xb)
            idx.append(int(fl))
            wts.append(int(np.floor(np.float32(np.float32(xb - fl) * np.float32(256)) + np.float32(0.5))))
        (i, j), (a, b) = idx, wts
        corner = [words[(jj % h) * w + (ii % w)] for jj, ii in ((j, i), (j, i + 1), (j + 1, i), (j + 1, i + 1))]
        ws = [int(np.rint(x / 256.0)) for x in ((256 - a) * (256 - b), a * (256 - b), (256 - a) * b, a * b)]
        for k in range(4):
            acc = sum(wk * ((int(t) >> (8 * k)) & 255) for wk, t in zip(ws, corner))
            out[n, k] = np.float32(acc) / np.float32(65280)
    return out


def test_oracle_filter_matches_numpy():
    rng = np.random.default_rng(3)
    w, h = 7, 5
    words = scenes.rgba_words(rng.integers(0, 256, size=(h, w, 4), dtype=np.uint8))
    uv = np.concatenate([rng.uniform(-3, 3, size=(300, 2)),
                         [[0, 0], [1, 1], [0.5 / w, 0.5 / h], [-1e-9, 1 - 1e-9], [2.5, -7.25]]]).astype(np.float32)
    got = oracle.sample_texture(words, w, h, uv)
    want = _numpy_sample(words, w, h, uv)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
