"""Textures on the CPU: PNG decoding/encoding, the loaders' texture
coordinates and images, the node texture API, and the oracle's texture
convention pinned by a known-answer render (bilinear filtering with texel
centres at (i + 0.5) / w, repeat wrap, v = 0 at the bottom row of the image,
perspective-correct coordinates)."""
import json
import struct
import zlib

import numpy as np
import pytest
import torch

import pybatchrender_gb300 as pbr
from pybatchrender_gb300.renderer import meshes, textures


def _png_with_filters(img: np.ndarray, ctype: int, filters) -> bytes:
    """Reference PNG writer applying the given per-row filter types (PNG
    specification, section 9), used to exercise every decoder path."""
    h, w = img.shape[:2]
    ch = {0: 1, 2: 3, 4: 2, 6: 4}[ctype]
    bpp = ch
    rows = img.reshape(h, w * ch).astype(np.int32)
    out = bytearray()
    prev = np.zeros(w * ch, np.int32)
    for y in range(h):
        f = filters[y % len(filters)]
        cur = rows[y]
        a = np.concatenate([np.zeros(bpp, np.int32), cur[:-bpp]])
        c = np.concatenate([np.zeros(bpp, np.int32), prev[:-bpp]])
        if f == 0:
            line = cur
        elif f == 1:
            line = cur - a
        elif f == 2:
            line = cur - prev
        elif f == 3:
            line = cur - ((a + prev) >> 1)
        else:
            p = a + prev - c
            pa, pb, pc = np.abs(p - a), np.abs(p - prev), np.abs(p - c)
            line = cur - np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, prev, c))
        out.append(f)
        out += (line & 255).astype(np.uint8).tobytes()
        prev = cur

    def chunk(tag, body):
        return struct.pack(">I", len(body)) + tag + body + struct.pack(">I", zlib.crc32(tag + body) & 0xFFFFFFFF)

    return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, ctype, 0, 0, 0))
            + chunk(b"IDAT", zlib.compress(bytes(out))) + chunk(b"IEND", b""))


@pytest.mark.parametrize("ctype", [0, 2, 4, 6])
def test_png_decoder_all_filters(ctype):
    rng = np.random.default_rng(ctype)
    ch = {0: 1, 2: 3, 4: 2, 6: 4}[ctype]
    img = rng.integers(0, 256, size=(7, 5, ch), dtype=np.uint8)
    data = _png_with_filters(img, ctype, [0, 1, 2, 3, 4])
    rgba = textures.decode_png(data)
    assert rgba.shape == (7, 5, 4)
    if ch in (1, 2):
        assert np.array_equal(rgba[..., 0], img[..., 0]) and np.array_equal(rgba[..., 2], img[..., 0])
        assert np.array_equal(rgba[..., 3], img[..., 1] if ch == 2 else np.full((7, 5), 255))
    else:
        assert np.array_equal(rgba[..., :3], img[..., :3])
        assert np.array_equal(rgba[..., 3], img[..., 3] if ch == 4 else np.full((7, 5), 255))


def test_png_roundtrip_and_palette():
    rng = np.random.default_rng(3)
    for c in (1, 2, 3, 4):
        img = rng.integers(0, 256, size=(9, 11, c), dtype=np.uint8)
        back = textures.decode_png(textures.encode_png(img))
        ref = textures.as_rgba8(img) if c != 2 else np.concatenate([np.repeat(img[..., :1], 3, 2), img[..., 1:]], 2)
        assert np.array_equal(back, ref)
    # 2-bit palette image with transparency
    plte = np.array([[255, 0, 0], [0, 255, 0], [0, 0, 255], [9, 9, 9]], np.uint8)
    idx = np.array([[0, 1, 2, 3, 0], [3, 2, 1, 0, 3]], np.uint8)
    packed = []
    for row in idx:
        bits = 0
        b = bytearray()
        for i, v in enumerate(row):
            bits = (bits << 2) | int(v)
            if i % 4 == 3:
                b.append(bits)
                bits = 0
        if len(row) % 4:
            b.append(bits << (2 * (4 - len(row) % 4)))
        packed.append(b"\x00" + bytes(b))

    def chunk(tag, body):
        return struct.pack(">I", len(body)) + tag + body + struct.pack(">I", zlib.crc32(tag + body) & 0xFFFFFFFF)

    data = (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", 5, 2, 2, 3, 0, 0, 0))
            + chunk(b"PLTE", plte.tobytes()) + chunk(b"tRNS", bytes([255, 128]))
            + chunk(b"IDAT", zlib.compress(b"".join(packed))) + chunk(b"IEND", b""))
    rgba = textures.decode_png(data)
    assert np.array_equal(rgba[..., :3], plte[idx])
    assert rgba[0, 1, 3] == 128 and rgba[0, 2, 3] == 255
    with pytest.raises(ValueError):
        textures.decode_png(b"not a png")


def test_node_texture_api(tmp_path):
    r = pbr.PBRRenderer(num_scenes=2, device="cpu")
    img = np.zeros((2, 3, 3), np.uint8)
    img[0] = (255, 0, 0)  # top row red
    img[1] = (0, 0, 255)  # bottom row blue
    n = r.add_node("models/box", 1, texture=img)
    assert n.texture.shape == (2, 3, 4)
    assert tuple(n.texture[0, 0]) == (0, 0, 255, 255)  # row 0 of the kernels' layout is the image's bottom row
    n.set_texture(None)
    assert n.texture is None
    n.set_texture(True)  # the box brings no texture: white
    assert np.array_equal(n.texture, np.full((1, 1, 4), 255, np.uint8))
    n.set_texture(torch.full((4, 4), 0.5))
    assert np.all(n.texture[..., :3] == 128) and np.all(n.texture[..., 3] == 255)
    path = tmp_path / "t.png"
    path.write_bytes(textures.encode_png(img))
    n.set_texture(str(path))
    assert tuple(n.texture[1, 2]) == (255, 0, 0, 255)
    with pytest.raises(ValueError):
        n.set_texture(np.zeros((2, 2, 2, 2), np.uint8))
    # the soft mode rejects textured nodes (checked before any CUDA work)
    r.cfg.raster_mode = "soft"
    with pytest.raises(NotImplementedError):
        r.render_soft()


def test_egg_and_gltf_texture_coordinates(tmp_path):
    img = np.arange(2 * 2 * 3, dtype=np.uint8).reshape(2, 2, 3) * 20
    (tmp_path / "tex.png").write_bytes(textures.encode_png(img))
    egg = """<CoordinateSystem> { Z-Up }
<Texture> tex1 {
  "tex.png"
}
<VertexPool> quad {
  <Vertex> 0 { 0 0 0 <UV> { 0 0 } }
  <Vertex> 1 { 1 0 0 <UV> { 1 0 } }
  <Vertex> 2 { 1 0 1 <UV> { 1 1 } }
  <Vertex> 3 { 0 0 1 <UV> { 0 1 } }
}
<Polygon> {
  <TRef> { tex1 }
  <VertexRef> { 0 1 2 3 <Ref> { quad } }
}
"""
    (tmp_path / "quad.egg").write_text(egg)
    m = meshes.resolve_model(str(tmp_path / "quad.egg"))
    assert m.num_triangles == 2
    assert np.allclose(m.uvs, [[0, 0], [1, 0], [1, 1], [0, 1]])
    assert m.texture.shape == (2, 2, 4) and np.array_equal(m.texture[..., :3], img)
    # glTF: TEXCOORD_0 with v = 0 at the top of the image becomes 1 - v
    pos = np.array([[0, 0, 0], [1, 0, 0], [0, 0, 1]], np.float32)
    uv = np.array([[0.0, 0.0], [1.0, 0.25], [0.5, 1.0]], np.float32)
    idx = np.array([0, 1, 2], np.uint16)
    blob = pos.tobytes() + uv.tobytes() + idx.tobytes() + b"\x00\x00"
    (tmp_path / "tri.bin").write_bytes(blob)
    doc = {
        "buffers": [{"uri": "tri.bin", "byteLength": len(blob)}],
        "bufferViews": [{"buffer": 0, "byteOffset": 0, "byteLength": 36},
                        {"buffer": 0, "byteOffset": 36, "byteLength": 24},
                        {"buffer": 0, "byteOffset": 60, "byteLength": 6}],
        "accessors": [{"bufferView": 0, "componentType": 5126, "count": 3, "type": "VEC3"},
                      {"bufferView": 1, "componentType": 5126, "count": 3, "type": "VEC2"},
                      {"bufferView": 2, "componentType": 5123, "count": 3, "type": "SCALAR"}],
        "images": [{"uri": "tex.png"}], "textures": [{"source": 0}],
        "materials": [{"pbrMetallicRoughness": {"baseColorTexture": {"index": 0}}}],
        "meshes": [{"primitives": [{"attributes": {"POSITION": 0, "TEXCOORD_0": 1}, "indices": 2, "material": 0}]}],
    }
    (tmp_path / "tri.gltf").write_text(json.dumps(doc))
    g = meshes.resolve_model(str(tmp_path / "tri.gltf"))
    assert np.allclose(g.uvs, [[0.0, 1.0], [1.0, 0.75], [0.5, 0.0]])
    assert g.texture is not None
    # baking keeps the coordinates
    b = meshes.bake(g, 2.0, (30.0, 0.0, 0.0), (0.5, 0.5, 0.5))
    assert np.array_equal(b.uvs, g.uvs)


def _bilinear_repeat(tex_gl: np.ndarray, u: np.ndarray, v: np.ndarray) -> np.ndarray:
    """GL bilinear filtering with repeat wrap; tex_gl row 0 at v = 0."""
    h, w = tex_gl.shape[:2]
    t = tex_gl[..., :3].astype(np.float64) / 255.0
    x = (u - np.floor(u)) * w - 0.5
    y = (v - np.floor(v)) * h - 0.5
    x0, y0 = np.floor(x), np.floor(y)
    ax, ay = (x - x0)[..., None], (y - y0)[..., None]
    x0 = x0.astype(np.int64) % w
    y0 = y0.astype(np.int64) % h
    x1, y1 = (x0 + 1) % w, (y0 + 1) % h
    top = (1 - ax) * t[y0, x0] + ax * t[y0, x1]
    bot = (1 - ax) * t[y1, x0] + ax * t[y1, x1]
    return (1 - ay) * top + ay * bot


def test_oracle_texture_known_answer(oracle):
    """A textured unit-cube face seen straight on: every covered pixel centre
    is intersected with the face plane analytically, its (u, v) mapped through
    an independent bilinear formula, and the oracle's pixels must equal it."""
    rng = np.random.default_rng(11)
    img = rng.integers(0, 256, size=(5, 7, 3), dtype=np.uint8)
    r = pbr.PBRRenderer(num_scenes=1, tile_resolution=(64, 48), device="cpu")
    s = 1.6
    node = r.add_node("models/box", 1, model_pivot_relative_point=(0.5, 0.5, 0.5), texture=img)
    node.set_scales(s)
    node.set_colors(torch.tensor([[1.0, 0.75, 0.5, 1.0]]))
    r.add_camera(fov_y_deg=45.0)
    eye = np.array([0.0, -4.0, 0.0])
    r._pbr_cam.set_positions_and_lookat(torch.tensor(eye, dtype=torch.float32), torch.tensor([0.0, 0.0, 0.0]))
    r.add_light(strength=0.0)  # l = mix(1, light, 0) = 1: pixel = texel * colour
    sc, me, no = r.export_scene()
    ref = oracle.render_hard(sc, me, no, want_winner=True, want_ambiguous=True)
    W, H = 64, 48
    VP = sc["vp"].reshape(4, 4).astype(np.float64)
    inv = np.linalg.inv(VP)
    ys, xs = np.mgrid[0:H, 0:W]
    ndc_x = (xs + 0.5) / W * 2 - 1
    ndc_y = 1 - (ys + 0.5) / H * 2
    near = inv @ np.stack([ndc_x, ndc_y, -np.ones_like(ndc_x), np.ones_like(ndc_x)]).reshape(4, -1)
    far = inv @ np.stack([ndc_x, ndc_y, np.ones_like(ndc_x), np.ones_like(ndc_x)]).reshape(4, -1)
    p0, p1 = near[:3] / near[3], far[:3] / far[3]
    t = (-s / 2 - p0[1]) / (p1[1] - p0[1])  # the front face lies in the plane y = -s/2
    hit = p0 + t * (p1 - p0)
    u = ((hit[0] + s / 2) / s).reshape(H, W)  # unit-cube front face: u along +x, v along +z
    v = ((hit[2] + s / 2) / s).reshape(H, W)
    inside = (u > 0) & (u < 1) & (v > 0) & (v < 1)
    keep = inside & (ref["winner"][0] >= 0) & ~ref["ambiguous"][0]
    assert keep.sum() > 500
    expect = _bilinear_repeat(textures.gl_rows(textures.as_rgba8(img)), u, v) * np.array([1.0, 0.75, 0.5])
    expect8 = np.floor(np.clip(expect, 0, 1) * 255 + 0.5)
    got = ref["pixels"][0].transpose(1, 2, 0).astype(np.float64)
    diff = np.abs(got - expect8)[keep]
    assert diff.max() <= 1 and (diff == 0).mean() > 0.99
    # image orientation: the top image row shows the top of the picture
    top_row = int(np.argmax(keep.any(axis=1)))
    col = int(np.argmax(keep[top_row]))
    assert np.abs(got[top_row, col] - expect8[top_row, col]).max() <= 1


def test_one_row_texture_has_positive_strides():
    """A one-row image flipped to the texel layout must still be a fresh
    array with positive strides: numpy calls a one-row view with a negative
    row stride contiguous, and torch.from_numpy rejects it."""
    import torch
    import pybatchrender_gb300 as pbr
    r = pbr.PBRRenderer(num_scenes=2, device="cpu")
    node = r.add_node("models/box", 1)
    for img in (np.zeros((1, 2, 4), np.uint8), np.zeros((1, 1, 3), np.uint8), np.zeros((3, 1), np.uint8)):
        node.set_texture(img)
        assert all(s > 0 for s in node.texture.strides)
        assert torch.from_numpy(node.texture).shape[2] == 4
