"""Known-answer raster scenes with analytic results, shared by the oracle's
CPU tests and the CUDA kernels' GPU tests.

Every scene uses an orthographic view-projection (clip = world, w = 1), so a
vertex at screen position (sx, sy) of a W x H image has world x = 2 sx / W - 1,
y = 1 - 2 sy / H exactly when those are dyadic rationals.  The answers follow
from the GL rules the renderer restates: pixel centres at +0.5, top-left fill
rule, counter-clockwise front faces (in GL's y-up window coordinates), window
depth = 0.5 z + 0.5, UNORM8 = floor(clamp(c) * 255 + 0.5).
"""
from __future__ import annotations

import numpy as np

W = H = 32


def ndc(sx: float, sy: float) -> tuple[float, float]:
    return 2.0 * sx / W - 1.0, 1.0 - 2.0 * sy / H


class KMesh:
    def __init__(self, pts, tris, normal=(0.0, 0.0, 1.0)):
        self.positions = np.asarray(pts, np.float32).reshape(-1, 3)
        self.normals = np.tile(np.asarray(normal, np.float32), (len(self.positions), 1))
        self.indices = np.asarray(tris, np.int32).reshape(-1, 3)
        self.uvs = None


def screen_mesh(corners_screen, tris, z=0.25) -> KMesh:
    pts = [(*ndc(sx, sy), z) for sx, sy in corners_screen]
    return KMesh(pts, tris)


# axis-aligned square with its edges through pixel centres: x in [8.5, 16.5], y in [4.5, 12.5]
SQUARE = [(8.5, 12.5), (16.5, 12.5), (16.5, 4.5), (8.5, 4.5)]  # BL, BR, TR, TL (counter-clockwise, y up)
SQUARE_TRIS = [(0, 1, 2), (0, 2, 3)]  # sharing the diagonal BL-TR


def square_expected() -> np.ndarray:
    """Top-left rule: centres on the left and top edges are inside, on the
    right and bottom edges outside -> columns 8..15, rows 4..11."""
    m = np.zeros((H, W), bool)
    m[4:12, 8:16] = True
    return m


def scene(n_scenes: int = 1, strength: float = 0.0, ambient=(0.0, 0.0, 0.0), ldir=(0.0, 0.0, 1.0),
          lcol=(0.0, 0.0, 0.0), vp=None) -> dict:
    vp = np.eye(4, dtype=np.float32) if vp is None else np.asarray(vp, np.float32)
    return {"N": n_scenes, "W": W, "H": H, "C": 3, "vp": np.tile(vp.reshape(1, 16), (n_scenes, 1)),
            "ambient": ambient, "ldir": ldir, "lcol": lcol, "strength": strength, "bg": (0.0, 0.0, 0.0, 1.0),
            "cull": 1}


def node(mesh_index: int, color=(0.8, 0.4, 0.2, 1.0), n_scenes: int = 1) -> dict:
    return {"mesh": mesh_index, "I": 1, "shared": True, "mode": 0, "counts": None,
            "pos": np.zeros((1, 3), np.float32), "rot": np.zeros((1, 3), np.float32),
            "scale": np.ones(1, np.float32), "color": np.asarray([color], np.float32)}


def unorm8(v: float) -> int:
    return int(np.floor(min(max(v, 0.0), 1.0) * 255.0 + 0.5))


# flat-lit face seen head-on: colour * (ambient + ndl * light colour), ndl = 1
FACE_COLOR = (0.4, 0.6, 0.8, 1.0)
FACE_AMBIENT = (0.2, 0.2, 0.2)
FACE_EXPECT = tuple(unorm8(np.float32(c) * (np.float32(0.2) + np.float32(1.0))) for c in FACE_COLOR[:3])


def textured_square(uvs, z=0.25) -> KMesh:
    """The square with per-corner texture coordinates (BL, BR, TR, TL)."""
    m = screen_mesh(SQUARE, SQUARE_TRIS, z=z)
    m.uvs = np.asarray(uvs, np.float32).reshape(4, 2)
    return m


def texture(rgb_rows) -> np.ndarray:
    """[h][w] lists of (r, g, b) -> an RGBA8 texture [h, w, 4], row 0 at v = 0."""
    t = np.asarray(rgb_rows, np.uint8)
    return np.concatenate([t, np.full(t.shape[:2] + (1,), 255, np.uint8)], axis=2)


# A plane seen in perspective: clip = (x, y, z - 2, z), so NDC x = x / z.
# The quad's left edge lies at NDC x = -0.5 and depth z0, its right edge at
# NDC x = +0.5 and depth z1 (two vertical segments, so the quad is planar).
PERSP_Z0, PERSP_Z1 = 1.5, 3.0
PERSP_VP = np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, -2], [0, 0, 1, 0]], np.float32)  # ndc z = 1 - 2 / z


def perspective_quad() -> KMesh:
    z0, z1 = PERSP_Z0, PERSP_Z1
    pts = [(-0.5 * z0, -0.5 * z0, z0), (0.5 * z1, -0.5 * z1, z1), (0.5 * z1, 0.5 * z1, z1), (-0.5 * z0, 0.5 * z0, z0)]
    m = KMesh(pts, SQUARE_TRIS)
    m.uvs = np.array([(0, 0), (1, 0), (1, 1), (0, 1)], np.float32)
    return m


def perspective_u(ndc_x):
    """u at NDC x on the quad: u = (z - z0) / (z1 - z0) is affine in world
    space, and the point of the plane seen at NDC x solves
    ndc_x * z(u) = x(u), which gives u = z0 (0.5 + ndc_x) / (0.5 (z0 + z1) - ndc_x (z1 - z0))."""
    z0, z1 = PERSP_Z0, PERSP_Z1
    return z0 * (0.5 + ndc_x) / (0.5 * (z0 + z1) - ndc_x * (z1 - z0))
