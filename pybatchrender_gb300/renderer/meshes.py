"""Triangle meshes for the batch renderer: procedural shapes, file loaders and
model baking.

The reference loads models through Panda3D's loader (``renderer/node.py:61-71``)
and bakes ``model_scale`` / ``model_hpr`` / the pivot into the vertices with
``flattenStrong`` (``renderer/node.py:214-268,313-341``).  Panda3D's bundled
``models/box`` is a unit cube spanning ``[0,1]^3`` with one quad per face; it is
not shipped with the reference, so it is restated here procedurally (24
vertices, 12 triangles, per-face normals, counter-clockwise outward winding).

A :class:`Mesh` is plain host data (float32 positions/normals, int32 indices).
The renderer uploads it once to device memory at ``setup_environment``.
"""
from __future__ import annotations

import json
import math
import os
import struct
import zlib
from collections.abc import Sequence
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Mesh:
    """Indexed triangle mesh.

    positions: ``[nv,3]`` float32, normals: ``[nv,3]`` float32 (unit length),
    indices: ``[nt,3]`` int32, counter-clockwise when seen from the outside.
    ``smooth`` is False when every triangle's three vertex normals are
    identical (flat shading: a triangle is lit with its first vertex's normal).
    ``uvs``: ``[nv,2]`` float32 texture coordinates (GL convention, ``v = 0`` at
    the bottom of the image) or None; ``texture``: the model's own texture,
    ``[h,w,4]`` uint8 RGBA in image order, or None.
    """

    positions: np.ndarray
    normals: np.ndarray
    indices: np.ndarray
    name: str = "mesh"
    smooth: bool = field(default=False)
    uvs: np.ndarray | None = None
    texture: np.ndarray | None = None

    def __post_init__(self) -> None:
        # fresh C-ordered copies: a view that numpy calls contiguous may still carry a negative stride on a
        # length-1 axis, which torch.from_numpy rejects
        self.positions = np.array(self.positions, dtype=np.float32, order="C").reshape(-1, 3)
        self.normals = np.array(self.normals, dtype=np.float32, order="C").reshape(-1, 3)
        self.indices = np.array(self.indices, dtype=np.int32, order="C").reshape(-1, 3)
        if self.positions.shape != self.normals.shape:
            raise ValueError("positions and normals must have the same shape")
        if self.indices.size and (self.indices.min() < 0 or self.indices.max() >= len(self.positions)):
            raise ValueError("mesh indices out of range")
        if self.uvs is not None:
            self.uvs = np.array(self.uvs, dtype=np.float32, order="C").reshape(-1, 2)
            if self.uvs.shape[0] != self.positions.shape[0]:
                raise ValueError("uvs must have one row per vertex")
        tri_n = self.normals[self.indices]  # [nt,3,3]
        self.smooth = bool(np.any(tri_n != tri_n[:, :1, :]))

    @property
    def num_vertices(self) -> int:
        return int(self.positions.shape[0])

    @property
    def num_triangles(self) -> int:
        return int(self.indices.shape[0])

    def tight_bounds(self) -> tuple[np.ndarray, np.ndarray]:
        return self.positions.min(axis=0), self.positions.max(axis=0)

    def bounding_sphere(self) -> tuple[tuple[float, float, float], float]:
        """(centre, radius) containing every vertex: the bounds-box centre and
        the largest distance to it, widened by a relative 1e-5."""
        if self.positions.size == 0:
            return (0.0, 0.0, 0.0), 0.0
        p = self.positions.astype(np.float64)
        c = (p.min(axis=0) + p.max(axis=0)) * 0.5
        r = float(np.sqrt(((p - c) ** 2).sum(axis=1)).max())
        return (float(c[0]), float(c[1]), float(c[2])), r * (1.0 + 1e-5) + 1e-7

    CLUSTER_TRIANGLES = 32

    def clusters(self) -> np.ndarray:
        """Per group of 32 consecutive triangles (the last one may hold fewer),
        8 float32: the group's bounding sphere (centre, radius) and the cone of
        its triangles' geometric normals (unit axis, cosine of the half-angle;
        -1 when the normals span a half-space or more).  Both are widened
        slightly (radius by a relative 1e-5, the half-angle by 1e-4 in its
        cosine), so that the float32 values still bound the float64 ones."""
        ct = self.CLUSTER_TRIANGLES
        nt = self.num_triangles
        ncl = (nt + ct - 1) // ct
        out = np.zeros((ncl, 8), np.float32)
        p = self.positions.astype(np.float64)
        f = self.indices.astype(np.int64)
        fn = np.cross(p[f[:, 1]] - p[f[:, 0]], p[f[:, 2]] - p[f[:, 0]])
        fl = np.linalg.norm(fn, axis=1)
        valid = fl > 0
        n = np.zeros_like(fn)
        n[valid] = fn[valid] / fl[valid, None]
        for c in range(ncl):
            sl = slice(c * ct, min((c + 1) * ct, nt))
            pts = p[np.unique(f[sl].ravel())]
            ctr = (pts.min(axis=0) + pts.max(axis=0)) * 0.5
            r = float(np.sqrt(((pts - ctr) ** 2).sum(axis=1)).max()) * (1.0 + 1e-5) + 1e-7
            ns = n[sl][valid[sl]]
            axis, cos_t = np.array([0.0, 0.0, 1.0]), -1.0
            if len(ns):
                a = ns.sum(axis=0)
                al = float(np.linalg.norm(a))
                if al > 1e-9:
                    axis = a / al
                    cos_t = float((ns @ axis).min()) - 1e-4
            out[c] = (*ctr, r, *axis, cos_t if cos_t > 0.0 else -1.0)
        return out

    def copy(self) -> "Mesh":
        return Mesh(self.positions.copy(), self.normals.copy(), self.indices.copy(), self.name,
                    uvs=None if self.uvs is None else self.uvs.copy(), texture=self.texture)


# ---------------------------------------------------------------------------
# Procedural meshes
# ---------------------------------------------------------------------------

def unit_cube() -> Mesh:
    """Unit cube on ``[0,1]^3``: 6 faces x 4 vertices, 12 triangles, face
    normals; each face maps the whole texture, (0,0) at its origin corner."""
    # (normal, origin corner, edge u, edge v) with u x v == normal so that
    # (o, o+u, o+u+v) and (o, o+u+v, o+v) wind counter-clockwise seen from outside.
    faces = [
        ((1, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1)),
        ((-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1)),
        ((0, 1, 0), (1, 1, 0), (-1, 0, 0), (0, 0, 1)),
        ((0, -1, 0), (0, 0, 0), (1, 0, 0), (0, 0, 1)),
        ((0, 0, 1), (0, 0, 1), (1, 0, 0), (0, 1, 0)),
        ((0, 0, -1), (0, 1, 0), (1, 0, 0), (0, -1, 0)),
    ]
    pos, nrm, idx, uvs = [], [], [], []
    for n, o, u, v in faces:
        o, u, v = np.array(o, float), np.array(u, float), np.array(v, float)
        assert np.allclose(np.cross(u, v), n)
        base = len(pos)
        for corner, uv in ((o, (0, 0)), (o + u, (1, 0)), (o + u + v, (1, 1)), (o + v, (0, 1))):
            pos.append(corner)
            nrm.append(n)
            uvs.append(uv)
        idx += [(base, base + 1, base + 2), (base, base + 2, base + 3)]
    return Mesh(np.array(pos), np.array(nrm), np.array(idx), name="box", uvs=np.array(uvs))


def cylinder(segments: int = 64, radius: float = 0.5, height: float = 1.0) -> Mesh:
    """Closed cylinder along +z centred at the origin.

    Side: two rings of ``segments`` vertices with radial (smooth) normals,
    ``2*segments`` triangles.  Caps: a centre vertex plus a ring each with flat
    normals, ``segments`` triangles per cap.  Total ``4*segments`` triangles
    (256 for 64 segments).
    """
    s = int(segments)
    if s < 3:
        raise ValueError("cylinder needs at least 3 segments")
    ang = 2.0 * math.pi * np.arange(s) / s
    ca, sa = np.cos(ang), np.sin(ang)
    z0, z1 = -0.5 * height, 0.5 * height
    pos, nrm, idx = [], [], []
    # side rings
    for z in (z0, z1):
        for i in range(s):
            pos.append((radius * ca[i], radius * sa[i], z))
            nrm.append((ca[i], sa[i], 0.0))
    for i in range(s):
        j = (i + 1) % s
        a0, a1, b0, b1 = i, j, s + i, s + j
        idx += [(a0, a1, b1), (a0, b1, b0)]
    # caps
    for z, nz in ((z1, 1.0), (z0, -1.0)):
        c = len(pos)
        pos.append((0.0, 0.0, z))
        nrm.append((0.0, 0.0, nz))
        for i in range(s):
            pos.append((radius * ca[i], radius * sa[i], z))
            nrm.append((0.0, 0.0, nz))
        for i in range(s):
            j = (i + 1) % s
            if nz > 0:
                idx.append((c, c + 1 + i, c + 1 + j))
            else:
                idx.append((c, c + 1 + j, c + 1 + i))
    return Mesh(np.array(pos), np.array(nrm), np.array(idx), name=f"cylinder{s}")


def icosphere(subdivisions: int = 2, radius: float = 0.5) -> Mesh:
    """Geodesic sphere from a subdivided icosahedron with smooth normals.

    20 * 4**subdivisions triangles: 320 at level 2, 1280 at level 3.
    """
    t = (1.0 + math.sqrt(5.0)) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0),
             (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = [np.array(v, float) / np.linalg.norm(v) for v in verts]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11),
             (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6), (7, 1, 8),
             (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9),
             (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(int(subdivisions)):
        cache: dict[tuple[int, int], int] = {}

        def mid(a: int, b: int) -> int:
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca_ = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca_), (b, bc, ab), (c, ca_, bc), (ab, bc, ca_)]
        faces = nf
    v = np.array(verts)
    f = np.array(faces)
    # make every face wind counter-clockwise seen from outside
    p0, p1, p2 = v[f[:, 0]], v[f[:, 1]], v[f[:, 2]]
    flip = np.einsum("ij,ij->i", np.cross(p1 - p0, p2 - p0), p0 + p1 + p2) < 0
    f[flip] = f[flip][:, [0, 2, 1]]
    return Mesh(v * radius, v, f, name=f"icosphere{int(subdivisions)}")


# ---------------------------------------------------------------------------
# File loaders (Panda3D .egg text with polygons, glTF 2.0 with an external .bin)
# ---------------------------------------------------------------------------

def _triangulate_fan(poly: Sequence[int]) -> list[tuple[int, int, int]]:
    return [(poly[0], poly[i], poly[i + 1]) for i in range(1, len(poly) - 1)]


def _egg_tokens(text: str) -> list[str]:
    import re
    return re.findall(r'"(?:[^"\\]|\\.)*"|<[^>]*>|[{}]|[^\s{}<"]+', text)


def _egg_parse(tokens: list[str], i: int = 0, depth: int = 0) -> tuple[list, int]:
    """Egg syntax tree: entries ``(tag, name, children)`` and loose value tokens."""
    if depth > 256:
        raise ValueError("egg nesting too deep")
    items: list = []
    while i < len(tokens):
        t = tokens[i]
        if t == "}":
            return items, i + 1
        if t.startswith("<") and t.endswith(">"):
            tag, name = t[1:-1], None
            i += 1
            if i < len(tokens) and tokens[i] != "{":
                name = tokens[i].strip('"')
                i += 1
            if i >= len(tokens) or tokens[i] != "{":
                raise ValueError(f"egg: expected '{{' after <{tag}>")
            children, i = _egg_parse(tokens, i + 1, depth + 1)
            items.append((tag, name, children))
        else:
            items.append(t.strip('"'))
            i += 1
    if depth:
        raise ValueError("egg: unbalanced braces")
    return items, i


def _egg_values(items) -> list[str]:
    return [x for x in items if isinstance(x, str)]


def _egg_entries(items, tag: str):
    return [x for x in items if isinstance(x, tuple) and x[0].lower() == tag.lower()]


def load_egg(path: str) -> Mesh:
    """Panda3D ``.egg`` reader for static geometry: every ``<VertexPool>``
    (vertices with an optional ``<Normal>`` and ``<UV>``), every ``<Polygon>``
    at any ``<Group>`` depth with ``<VertexRef>`` into a named pool, flattened
    into one mesh as ``flattenStrong`` does.  Egg vertices are written in the
    model's coordinate space, so group ``<Transform>`` entries do not move
    them.  Polygons are fan-triangulated; a vertex without a normal takes the
    polygon's ``<Normal>`` or its face normal.  ``<CoordinateSystem> { Y-Up }``
    files are turned to Panda3D's Z-up ((x, y, z) -> (x, -z, y)).  The first
    referenced ``<Texture>`` whose image is a PNG becomes the mesh's own
    texture."""
    from .textures import load_image

    with open(path, "rb") as f:
        raw = f.read()
    if path.lower().endswith(".pz"):
        raw = zlib.decompress(raw)  # Panda3D's pzip: one zlib stream
    items, _ = _egg_parse(_egg_tokens(raw.decode("utf-8")))
    cs = "z-up"
    for e in _egg_entries(items, "CoordinateSystem"):
        cs = " ".join(_egg_values(e[2])).lower()
    if cs not in ("z-up", "z-up-right", "y-up", "y-up-right"):
        raise ValueError(f"unsupported egg coordinate system '{cs}'")
    yup = cs.startswith("y-up")
    textures: dict[str, str] = {}
    pools: dict[str, dict[int, tuple]] = {}
    polys: list[tuple[str, list[int], tuple | None, list[str]]] = []

    def walk(entries, depth=0):
        for e in entries:
            if not isinstance(e, tuple):
                continue
            tag, name, children = e[0].lower(), e[1], e[2]
            if tag == "texture":
                vals = _egg_values(children)
                if vals:
                    textures[name or ""] = vals[0]
            elif tag == "vertexpool":
                pool = pools.setdefault(name or "", {})
                for v in _egg_entries(children, "Vertex"):
                    coords = [float(x) for x in _egg_values(v[2])]
                    if len(coords) < 3:
                        raise ValueError("egg vertex without three coordinates")
                    if len(coords) == 4 and coords[3] not in (0.0, 1.0):
                        coords = [c / coords[3] for c in coords[:3]]
                    nrm = _egg_entries(v[2], "Normal")
                    uv = _egg_entries(v[2], "UV")
                    pool[int(v[1])] = (tuple(coords[:3]),
                                       tuple(float(x) for x in _egg_values(nrm[0][2])[:3]) if nrm else None,
                                       tuple(float(x) for x in _egg_values(uv[0][2])[:2]) if uv else None)
            elif tag == "polygon":
                refs = _egg_entries(children, "VertexRef")
                if not refs:
                    continue
                ids = [int(x) for x in _egg_values(refs[0][2])]
                pool_ref = _egg_entries(refs[0][2], "Ref")
                pool_name = _egg_values(pool_ref[0][2])[0] if pool_ref else ""
                pn = _egg_entries(children, "Normal")
                tref = [t for r in _egg_entries(children, "TRef") for t in _egg_values(r[2])]
                polys.append((pool_name, ids, tuple(float(x) for x in _egg_values(pn[0][2])[:3]) if pn else None, tref))
            elif tag in ("group", "instance") and depth < 256:
                walk(children, depth + 1)

    walk(items)
    out_p, out_n, out_i, out_uv = [], [], [], []
    any_uv = False
    used_tex: list[str] = []
    for pool_name, ids, pnorm, tref in polys:
        pool = pools.get(pool_name) if pool_name in pools else (next(iter(pools.values())) if len(pools) == 1 else None)
        if pool is None:
            raise ValueError(f"egg polygon refers to unknown vertex pool '{pool_name}'")
        if len(ids) < 3:
            continue
        pts = np.array([pool[r][0] for r in ids], float)
        fn = np.cross(pts[1] - pts[0], pts[2] - pts[0])
        ln = np.linalg.norm(fn)
        fn = fn / ln if ln > 0 else np.array([0.0, 0.0, 1.0])
        base = len(out_p)
        for r in ids:
            p, nrm, uv = pool[r]
            out_p.append(p)
            out_n.append(nrm if nrm is not None else (pnorm if pnorm is not None else tuple(fn)))
            out_uv.append(uv if uv is not None else (0.0, 0.0))
            any_uv = any_uv or uv is not None
        out_i += _triangulate_fan(list(range(base, base + len(ids))))
        used_tex += [t for t in tref if t not in used_tex]
    if not out_p:
        raise ValueError(f"no polygons in {os.path.basename(path)}")
    texture = None
    for t in used_tex + [k for k in textures if k not in used_tex]:
        rel = textures.get(t)
        if rel:
            tex_path = os.path.join(os.path.dirname(path), rel)
            if os.path.isfile(tex_path) and tex_path.lower().endswith(".png"):
                texture = load_image(tex_path)
                break
    p = np.array(out_p, float)
    n = np.array(out_n, float)
    if yup:
        p = np.stack([p[:, 0], -p[:, 2], p[:, 1]], 1)
        n = np.stack([n[:, 0], -n[:, 2], n[:, 1]], 1)
    n /= np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-12)
    return Mesh(p, n, np.array(out_i), name=os.path.basename(path),
                uvs=np.array(out_uv) if any_uv else None, texture=texture)


def _quat_matrix(q) -> np.ndarray:
    x, y, z, w = (float(v) for v in q)
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def _gltf_node_matrix(node: dict) -> np.ndarray:
    """Local 4x4 transform of a glTF node: ``matrix`` (column-major) or T * R * S."""
    if "matrix" in node:
        return np.array(node["matrix"], dtype=np.float64).reshape(4, 4).T
    m = np.eye(4)
    m[:3, :3] = _quat_matrix(node.get("rotation", (0.0, 0.0, 0.0, 1.0))) @ np.diag(node.get("scale", (1.0, 1.0, 1.0)))
    m[:3, 3] = node.get("translation", (0.0, 0.0, 0.0))
    return m


# glTF is Y-up, Panda3D Z-up: (x, y, z) -> (x, -z, y), a rotation about +x
_YUP_TO_ZUP = np.array([[1.0, 0.0, 0.0, 0.0], [0.0, 0.0, -1.0, 0.0], [0.0, 1.0, 0.0, 0.0], [0.0, 0.0, 0.0, 1.0]])


def _read_gltf(path: str) -> tuple[dict, list[bytes], str]:
    """(document, buffers, base directory) of a ``.gltf`` (external or base64
    ``data:`` buffers) or a binary ``.glb`` container."""
    import base64

    base = os.path.dirname(path)
    raw = open(path, "rb").read()
    bin_chunk = None
    if raw[:4] == b"glTF":
        version, length = struct.unpack("<II", raw[4:12])
        if version != 2:
            raise ValueError(f"unsupported glb version {version}")
        pos, doc = 12, None
        while pos + 8 <= min(length, len(raw)):
            clen, ctype = struct.unpack("<II", raw[pos:pos + 8])
            body = raw[pos + 8:pos + 8 + clen]
            if ctype == 0x4E4F534A:  # JSON
                doc = json.loads(body.decode("utf-8"))
            elif ctype == 0x004E4942:  # BIN
                bin_chunk = body
            pos += 8 + clen
        if doc is None:
            raise ValueError("glb without a JSON chunk")
    else:
        doc = json.loads(raw.decode("utf-8"))
    buffers = []
    for b in doc.get("buffers", []):
        uri = b.get("uri")
        if uri is None:
            if bin_chunk is None:
                raise ValueError("glTF buffer without a uri outside a glb container")
            buffers.append(bin_chunk)
        elif uri.startswith("data:"):
            buffers.append(base64.b64decode(uri.split(",", 1)[1]))
        else:
            buffers.append(open(os.path.join(base, uri), "rb").read())
    return doc, buffers, base


def load_gltf(path: str) -> Mesh:
    """glTF 2.0 reader (``.gltf`` with external or embedded buffers, ``.glb``):
    every triangle primitive of every mesh reached from the default scene, with
    its node transforms applied, flattened into one mesh as Panda3D's loader +
    ``flattenStrong`` do; the file's Y-up axes become Panda3D's Z-up ones
    ((x, y, z) -> (x, -z, y)).  POSITION / NORMAL / TEXCOORD_0 accessors;
    missing normals are the area-weighted face normals.  glTF puts ``v = 0`` at
    the top of the image; the coordinates are flipped (``v -> 1 - v``) to the GL
    convention.  The first PNG ``baseColorTexture`` becomes the mesh's own
    texture."""
    import base64

    from .textures import decode_png, load_image

    doc, buffers, base = _read_gltf(path)

    def accessor(i: int) -> np.ndarray:
        acc = doc["accessors"][i]
        bv = doc["bufferViews"][acc["bufferView"]]
        comp = {5126: np.float32, 5125: np.uint32, 5123: np.uint16, 5121: np.uint8}[acc["componentType"]]
        ncomp = {"SCALAR": 1, "VEC2": 2, "VEC3": 3, "VEC4": 4}[acc["type"]]
        off = bv.get("byteOffset", 0) + acc.get("byteOffset", 0)
        itemsize = np.dtype(comp).itemsize * ncomp
        stride = bv.get("byteStride", itemsize)
        raw = buffers[bv["buffer"]]
        if "sparse" in acc:
            raise ValueError("sparse glTF accessors are not supported")
        if stride == itemsize:
            arr = np.frombuffer(raw, dtype=comp, count=acc["count"] * ncomp, offset=off)
        else:
            arr = np.stack([np.frombuffer(raw, dtype=comp, count=ncomp, offset=off + k * stride)
                            for k in range(acc["count"])])
        arr = arr.reshape(acc["count"], ncomp)
        if acc.get("normalized") and comp is not np.float32:
            arr = arr.astype(np.float64) / float(np.iinfo(comp).max)  # unsigned normalised integers
        return arr

    def texture_of(prim) -> np.ndarray | None:
        try:
            mat = doc["materials"][prim["material"]]
            tex = doc["textures"][mat["pbrMetallicRoughness"]["baseColorTexture"]["index"]]
            img = doc["images"][tex["source"]]
        except (KeyError, IndexError, TypeError):
            return None
        if "uri" in img:
            if img["uri"].startswith("data:image/png;base64,"):
                return decode_png(base64.b64decode(img["uri"].split(",", 1)[1]))
            tex_path = os.path.join(base, img["uri"])
            if os.path.isfile(tex_path) and tex_path.lower().endswith(".png"):
                return load_image(tex_path)
            return None
        if img.get("mimeType") == "image/png" and "bufferView" in img:
            bv = doc["bufferViews"][img["bufferView"]]
            data = buffers[bv["buffer"]][bv.get("byteOffset", 0):bv.get("byteOffset", 0) + bv["byteLength"]]
            return decode_png(data)
        return None

    parts_p, parts_n, parts_i, parts_uv = [], [], [], []
    any_uv, texture, count = False, None, 0

    def emit(mesh_index: int, world: np.ndarray) -> None:
        nonlocal any_uv, texture, count
        lin = world[:3, :3]
        nmat = np.linalg.inv(lin).T if abs(np.linalg.det(lin)) > 0 else lin
        flip = np.linalg.det(lin) < 0
        for prim in doc["meshes"][mesh_index].get("primitives", []):
            if prim.get("mode", 4) != 4:
                raise ValueError("only triangle-list glTF primitives are supported")
            p = accessor(prim["attributes"]["POSITION"]).astype(np.float64)
            idx = accessor(prim["indices"]).reshape(-1, 3).astype(np.int64) if "indices" in prim else \
                np.arange(len(p)).reshape(-1, 3)
            if "NORMAL" in prim["attributes"]:
                n = accessor(prim["attributes"]["NORMAL"]).astype(np.float64)
            else:
                n = np.zeros_like(p)
            if not np.any(n):
                tri = p[idx]
                fn = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
                for k in range(3):
                    np.add.at(n, idx[:, k], fn)
            uv = None
            if "TEXCOORD_0" in prim["attributes"]:
                t = accessor(prim["attributes"]["TEXCOORD_0"]).astype(np.float64)
                uv = np.stack([t[:, 0], 1.0 - t[:, 1]], axis=1)
                any_uv = True
            parts_p.append(p @ world[:3, :3].T + world[:3, 3])
            parts_n.append(n @ nmat.T)
            parts_i.append((idx[:, [0, 2, 1]] if flip else idx) + count)
            parts_uv.append(uv if uv is not None else np.zeros((len(p), 2)))
            count += len(p)
            if texture is None:
                texture = texture_of(prim)

    def walk(node_index: int, parent: np.ndarray, depth: int = 0) -> None:
        if depth > 64:
            raise ValueError("glTF node hierarchy too deep (a cycle?)")
        node = doc["nodes"][node_index]
        world = parent @ _gltf_node_matrix(node)
        if "mesh" in node:
            emit(node["mesh"], world)
        for c in node.get("children", []):
            walk(c, world, depth + 1)

    scenes = doc.get("scenes")
    if scenes:
        for r in scenes[doc.get("scene", 0)].get("nodes", []):
            walk(r, _YUP_TO_ZUP)
    else:
        for m in range(len(doc.get("meshes", []))):
            emit(m, _YUP_TO_ZUP)
    if not parts_p:
        raise ValueError(f"no triangle geometry in {os.path.basename(path)}")
    p = np.concatenate(parts_p)
    n = np.concatenate(parts_n)
    n /= np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-12)
    return Mesh(p.astype(np.float32), n.astype(np.float32), np.concatenate(parts_i).astype(np.int32),
                name=os.path.basename(path), uvs=np.concatenate(parts_uv) if any_uv else None, texture=texture)


_BUILTIN = {
    "box": unit_cube,
    "cube": unit_cube,
    "cylinder": lambda: cylinder(64),
    "sphere": lambda: icosphere(2),
    "icosphere": lambda: icosphere(2),
    # Panda3D's bundled smiley (a textured sphere) is not available: an untextured sphere stands in
    "smiley": lambda: icosphere(2),
    # the reference's rail model (pybatchrender/models/cylinder/scene.gltf) when its file is not on the
    # model search path: a procedural cylinder along the same (z) axis
    "cylinder/scene.gltf": lambda: cylinder(64),
}


_MODEL_EXTENSIONS = (".egg", ".egg.pz", ".gltf", ".glb")

MODEL_PATH_ENV = "PBR_MODEL_PATH"


def model_search_path() -> list[str]:
    """Directories searched for model files given by a relative path: the
    entries of the ``PBR_MODEL_PATH`` environment variable (separated by
    ``os.pathsep``), Panda3D's ``model-path`` in the reference.  A path
    ``"models/<rel>"`` is looked up as ``<dir>/models/<rel>`` and as
    ``<dir>/<rel>``, so both a directory holding ``models/`` (such as the
    reference's package directory) and the models directory itself work --
    the lookup of the reference's Steering renderer
    (``envs/steering/renderer.py:89-108``)."""
    return [d for d in os.environ.get(MODEL_PATH_ENV, "").split(os.pathsep) if d]


def _find_model_file(model: str) -> str | None:
    """The file a model path names: the path itself, then the model search
    path; like Panda3D's loader, a path without an extension finds the file
    with one."""
    cands = [model]
    if not os.path.isabs(model):
        rel = model[len("models/"):] if model.startswith("models/") else None
        for d in model_search_path():
            cands.append(os.path.join(d, model))
            if rel:
                cands.append(os.path.join(d, rel))
    for c in cands:
        if os.path.isfile(c):
            return c
        for ext in _MODEL_EXTENSIONS:
            if os.path.isfile(c + ext):
                return c + ext
    return None


def resolve_model(model: "str | Mesh") -> Mesh:
    """Map a reference-style model path to a mesh.

    An existing ``.egg`` / ``.egg.pz`` / ``.gltf`` / ``.glb`` file, given
    directly or found on the model search path (:func:`model_search_path`;
    the extension may be left out, as with Panda3D's loader) -> the loaders
    above.  Otherwise built-in meshes: ``"models/box"`` / ``"box"`` ->
    :func:`unit_cube` (Panda3D's bundled box); ``"cylinder"``,
    ``"cylinder:<segments>"``, ``"icosphere:<level>"`` -> procedural shapes;
    ``"models/smiley"`` and the reference's rail model
    ``"models/cylinder/scene.gltf"`` -> procedural stand-ins when their files
    are not found.  A :class:`Mesh` is returned as a copy.
    """
    if isinstance(model, Mesh):
        return model.copy()
    if not isinstance(model, str):
        raise TypeError(f"model_path must be a str or Mesh, got {type(model).__name__}")
    found = _find_model_file(model)
    if found is not None:
        model = found
        low = model.lower()
        if low.endswith(".egg") or low.endswith(".egg.pz"):
            return load_egg(model)
        if low.endswith(".gltf") or low.endswith(".glb"):
            return load_gltf(model)
        raise ValueError(f"unsupported model file type: {model}")
    name = model
    if name.startswith("models/"):
        name = name[len("models/"):]
    for suffix in (".egg", ".bam", ".egg.pz"):
        if name.endswith(suffix):
            name = name[: -len(suffix)]
    if ":" in name:
        kind, arg = name.split(":", 1)
        if kind == "cylinder":
            return cylinder(int(arg))
        if kind in ("icosphere", "sphere"):
            return icosphere(int(arg))
    if name in _BUILTIN:
        return _BUILTIN[name]()
    raise FileNotFoundError(f"unknown model '{model}' (no such file and no built-in mesh of that name)")


# ---------------------------------------------------------------------------
# Baking (Panda3D setScale / setHpr / flattenStrong / pivot_to_rel)
# ---------------------------------------------------------------------------

def panda_hpr_matrix(h_deg: float, p_deg: float, r_deg: float) -> np.ndarray:
    """Rotation of Panda3D's ``NodePath.setHpr`` (degrees) for column vectors:
    roll about +y, then pitch about +x, then heading about +z
    (``R = Rz(h) @ Rx(p) @ Ry(r)``).  Only ``model_hpr`` baking uses it; the
    per-instance rotations use the shader convention of
    ``renderer/shader_context.py:47-84`` instead."""
    h, p, r = (math.radians(float(a)) for a in (h_deg, p_deg, r_deg))
    ch, sh, cp, sp, cr, sr = math.cos(h), math.sin(h), math.cos(p), math.sin(p), math.cos(r), math.sin(r)
    rz = np.array([[ch, -sh, 0], [sh, ch, 0], [0, 0, 1]])
    rx = np.array([[1, 0, 0], [0, cp, -sp], [0, sp, cp]])
    ry = np.array([[cr, 0, sr], [0, 1, 0], [-sr, 0, cr]])
    return rz @ rx @ ry


def _coerce_scale(model_scale) -> tuple[tuple[float, float, float], bool] | None:
    """Follows ``PBRNode._coerce_model_scale`` (``renderer/node.py:180-201``)."""
    if model_scale is None:
        return None
    if isinstance(model_scale, (int, float)):
        v = float(model_scale)
        return (v, v, v), True
    if isinstance(model_scale, Sequence) or isinstance(model_scale, np.ndarray):
        seq = tuple(float(v) for v in model_scale)
        if len(seq) == 0:
            raise ValueError("model_scale sequence cannot be empty")
        if len(seq) == 1:
            return (seq[0],) * 3, True
        if len(seq) != 3:
            raise ValueError("model_scale sequence must have length 1 or 3")
        return seq, False
    raise TypeError("model_scale must be a number, a sequence of length 1 or 3, or None")


def _coerce_hpr(model_hpr) -> tuple[float, float, float] | None:
    """Follows ``PBRNode._coerce_model_hpr`` (``renderer/node.py:203-212``)."""
    if model_hpr is None:
        return None
    if not (isinstance(model_hpr, Sequence) or isinstance(model_hpr, np.ndarray)):
        raise TypeError("model_hpr must be a sequence of length 3 or None")
    hpr = tuple(float(v) for v in model_hpr)
    if len(hpr) != 3:
        raise ValueError("model_hpr sequence must have length 3")
    return hpr


def bake(mesh: Mesh, model_scale=None, model_hpr=None, pivot_relative_point=None,
         model_scale_units: str = "relative") -> Mesh:
    """Bake model scale, model HPR and pivot into the vertices.

    Mirrors ``renderer/node.py:61-67``: ``_apply_model_scale`` (``:214-260``;
    "absolute" divides the target size by the tight-bounds extent, uniform
    targets by the longest side), ``_apply_model_hpr`` (``:262-268``), the
    ``flattenStrong`` bake, then ``pivot_to_rel`` (``:313-341``) which moves the
    bounds-relative point to the origin.  Normals are transformed by the
    inverse transpose and renormalised, as Panda3D's flatten does.
    """
    out = mesh.copy()
    p = out.positions.astype(np.float64)
    n = out.normals.astype(np.float64)
    lin = np.eye(3)
    coerced = _coerce_scale(model_scale)
    if coerced is not None:
        vals, uniform = coerced
        if model_scale_units == "relative":
            svec = np.array(vals)
        elif model_scale_units == "absolute":
            lo, hi = p.min(axis=0), p.max(axis=0)
            dims = hi - lo
            longest = max(float(dims.max()), 1e-8)
            if uniform:
                svec = np.full(3, vals[0] / longest)
            else:
                comps = []
                for target, src in zip(vals, dims):
                    denom = src if abs(src) >= 1e-8 else longest
                    if abs(denom) < 1e-8:
                        denom = 1.0
                    comps.append(target / denom)
                svec = np.array(comps)
        else:
            raise ValueError(f"Unknown model_scale_units '{model_scale_units}'")
        lin = np.diag(svec) @ lin
    hpr = _coerce_hpr(model_hpr)
    if hpr is not None:
        lin = panda_hpr_matrix(*hpr) @ lin
    p = p @ lin.T
    if coerced is not None or hpr is not None:
        det = np.linalg.det(lin)
        if abs(det) > 0:
            n = n @ np.linalg.inv(lin)
            n /= np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-12)
        if det < 0:  # mirrored transform: keep counter-clockwise outward winding
            out.indices = out.indices[:, [0, 2, 1]].copy()
    if pivot_relative_point is not None:
        lo, hi = p.min(axis=0), p.max(axis=0)
        rel = np.array([float(v) for v in pivot_relative_point])
        p = p - (lo + (hi - lo) * rel)
    out.positions = p.astype(np.float32)
    out.normals = n.astype(np.float32)
    return Mesh(out.positions, out.normals, out.indices, mesh.name, uvs=out.uvs, texture=out.texture)
