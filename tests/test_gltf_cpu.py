"""Model loading (CPU). glTF: scene traversal with node transforms (matrix and
translation/rotation/scale), several primitives and meshes flattened into one
mesh, the Y-up to Z-up axis change, embedded (data: URI) buffers and the binary
.glb container, all giving the same mesh."""
import base64
import json
import math
import struct

import numpy as np
import pytest

from pybatchrender_gb300.renderer import meshes

TRI = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)  # in the z = 0 plane, normal +z (glTF frame)
IDX = np.array([0, 1, 2], np.uint16)


def _doc(uri):
    blob = TRI.tobytes() + IDX.tobytes() + b"\x00\x00"
    q = (math.sin(math.pi / 4), 0.0, 0.0, math.cos(math.pi / 4))  # +90 degrees about x
    doc = {
        "asset": {"version": "2.0"},
        "buffers": [{"byteLength": len(blob)} if uri is None else {"uri": uri, "byteLength": len(blob)}],
        "bufferViews": [{"buffer": 0, "byteOffset": 0, "byteLength": 36}, {"buffer": 0, "byteOffset": 36, "byteLength": 6}],
        "accessors": [{"bufferView": 0, "componentType": 5126, "count": 3, "type": "VEC3"},
                      {"bufferView": 1, "componentType": 5123, "count": 3, "type": "SCALAR"}],
        "meshes": [{"primitives": [{"attributes": {"POSITION": 0}, "indices": 1},
                                   {"attributes": {"POSITION": 0}, "indices": 1}]}],
        "nodes": [
            {"children": [1], "translation": [10.0, 0.0, 0.0]},
            {"mesh": 0, "rotation": list(q), "scale": [2.0, 2.0, 2.0]},
            {"mesh": 0, "matrix": [1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 5, 0, 1]},  # column-major, +5 in y
        ],
        "scenes": [{"nodes": [0, 2]}], "scene": 0,
    }
    return doc, blob


def _expected():
    # node 0 -> 1: scale 2, rotate +90 deg about x ((x, y, z) -> (x, -z, y)), translate +10 x; twice (2 primitives)
    a = TRI * 2.0
    a = np.stack([a[:, 0], -a[:, 2], a[:, 1]], 1) + np.array([10.0, 0.0, 0.0])
    b = TRI + np.array([0.0, 5.0, 0.0])
    glb = np.concatenate([a, a, b, b])
    return np.stack([glb[:, 0], -glb[:, 2], glb[:, 1]], 1)  # Y-up -> Z-up


def test_gltf_scene_traversal_and_axes(tmp_path):
    doc, blob = _doc("tri.bin")
    (tmp_path / "tri.bin").write_bytes(blob)
    (tmp_path / "s.gltf").write_text(json.dumps(doc))
    m = meshes.resolve_model(str(tmp_path / "s.gltf"))
    assert m.num_triangles == 4 and m.num_vertices == 12
    assert np.allclose(m.positions, _expected(), atol=1e-6)
    # flat face normals: the glTF +z normal of the plain copy becomes -y in Z-up
    assert np.allclose(m.normals[6:], [[0.0, -1.0, 0.0]] * 6, atol=1e-6)
    assert np.array_equal(m.indices, [[0, 1, 2], [3, 4, 5], [6, 7, 8], [9, 10, 11]])


def test_gltf_embedded_and_glb_match(tmp_path):
    doc, blob = _doc("tri.bin")
    (tmp_path / "tri.bin").write_bytes(blob)
    (tmp_path / "s.gltf").write_text(json.dumps(doc))
    ref = meshes.resolve_model(str(tmp_path / "s.gltf"))
    d2, _ = _doc("data:application/octet-stream;base64," + base64.b64encode(blob).decode())
    (tmp_path / "e.gltf").write_text(json.dumps(d2))
    e = meshes.resolve_model(str(tmp_path / "e.gltf"))
    d3, _ = _doc(None)
    js = json.dumps(d3).encode()
    js += b" " * ((4 - len(js) % 4) % 4)
    bn = blob + b"\x00" * ((4 - len(blob) % 4) % 4)
    glb = (b"glTF" + struct.pack("<II", 2, 12 + 8 + len(js) + 8 + len(bn)) + struct.pack("<II", len(js), 0x4E4F534A) + js
           + struct.pack("<II", len(bn), 0x004E4942) + bn)
    (tmp_path / "s.glb").write_bytes(glb)
    g = meshes.resolve_model(str(tmp_path / "s.glb"))
    for m in (e, g):
        assert np.array_equal(m.positions, ref.positions) and np.array_equal(m.indices, ref.indices)


EGG = """<CoordinateSystem> { %s }
<Comment> { "two pools, nested groups, a polygon normal" }
<Group> root {
  <Transform> { <Translate> { 5 0 0 } }
  <VertexPool> a {
    <Vertex> 0 { 0 0 0 }
    <Vertex> 1 { 1 0 0 }
    <Vertex> 2 { 1 1 0 <UV> { 0.5 0.25 } }
  }
  <Group> inner {
    <VertexPool> b {
      <Vertex> 7 { 0 0 1 <Normal> { 0 0 1 } }
      <Vertex> 8 { 1 0 1 <Normal> { 0 0 1 } }
      <Vertex> 9 { 1 1 1 <Normal> { 0 0 1 } }
      <Vertex> 10 { 0 1 1 <Normal> { 0 0 1 } }
    }
    <Polygon> { <Normal> { 0 0 -1 } <VertexRef> { 0 1 2 <Ref> { a } } }
    <Polygon> { <VertexRef> { 7 8 9 10 <Ref> { b } } }
  }
}
"""


def test_egg_pools_groups_and_axes(tmp_path):
    (tmp_path / "z.egg").write_text(EGG % "Z-Up")
    m = meshes.resolve_model(str(tmp_path / "z.egg"))
    assert m.num_triangles == 3 and m.num_vertices == 7
    # vertex positions are in model space: the group transform does not move them
    assert np.allclose(m.positions[:3], [[0, 0, 0], [1, 0, 0], [1, 1, 0]])
    assert np.allclose(m.normals[:3], [[0, 0, -1]] * 3)       # the polygon's own normal
    assert np.allclose(m.normals[3:], [[0, 0, 1]] * 4)        # the vertices' normals
    assert np.allclose(m.uvs[2], [0.5, 0.25]) and np.allclose(m.uvs[0], [0.0, 0.0])
    (tmp_path / "y.egg").write_text(EGG % "Y-Up")
    y = meshes.resolve_model(str(tmp_path / "y.egg"))
    assert np.allclose(y.positions, np.stack([m.positions[:, 0], -m.positions[:, 2], m.positions[:, 1]], 1))
    (tmp_path / "bad.egg").write_text((EGG % "Z-Up").replace("<Ref> { b }", "<Ref> { nope }"))
    with pytest.raises(ValueError):
        meshes.resolve_model(str(tmp_path / "bad.egg"))


def test_egg_pz_and_paths_without_extension(tmp_path):
    """Panda3D's compressed ``.egg.pz`` (one zlib stream) loads like the
    plain file, and a path without an extension finds the file with one."""
    import zlib
    (tmp_path / "plain.egg").write_text(EGG % "Z-Up")
    (tmp_path / "packed.egg.pz").write_bytes(zlib.compress((EGG % "Z-Up").encode()))
    a = meshes.resolve_model(str(tmp_path / "plain.egg"))
    b = meshes.resolve_model(str(tmp_path / "packed.egg.pz"))
    c = meshes.resolve_model(str(tmp_path / "plain"))
    d = meshes.resolve_model(str(tmp_path / "packed"))
    for m in (b, c, d):
        assert np.array_equal(m.positions, a.positions) and np.array_equal(m.indices, a.indices)
    with pytest.raises(FileNotFoundError):
        meshes.resolve_model(str(tmp_path / "missing"))


def test_gltf_normalized_texcoords(tmp_path):
    doc, blob = _doc("tri.bin")
    uv16 = np.array([[0, 0], [65535, 0], [0, 32768]], np.uint16)
    blob2 = blob + uv16.tobytes()
    doc["buffers"][0]["byteLength"] = len(blob2)
    doc["bufferViews"].append({"buffer": 0, "byteOffset": len(blob), "byteLength": 12})
    doc["accessors"].append({"bufferView": 2, "componentType": 5123, "count": 3, "type": "VEC2", "normalized": True})
    doc["meshes"][0]["primitives"] = [{"attributes": {"POSITION": 0, "TEXCOORD_0": 2}, "indices": 1}]
    doc["scenes"][0]["nodes"] = [2]
    (tmp_path / "tri.bin").write_bytes(blob2)
    (tmp_path / "u.gltf").write_text(json.dumps(doc))
    m = meshes.resolve_model(str(tmp_path / "u.gltf"))
    assert np.allclose(m.uvs, [[0.0, 1.0], [1.0, 1.0], [0.0, 1.0 - 32768 / 65535]], atol=1e-6)
