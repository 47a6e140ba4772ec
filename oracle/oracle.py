"""Python side of the oracle: ctypes bindings to ``liboracle.so`` (built from
``raster_ref.c``) plus helpers to build, render and compare.

TEST INFRASTRUCTURE ONLY.  The oracle is the parity reference for the CUDA renderer
and the timed CPU baseline; the product package never imports this module.
Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py`` (its
``cpu_baseline`` leg and ``--impl reference`` arm) may use it.

Pixel parity against the reference's own (Panda3D/OpenGL) renders is
unpinned: that path cannot run here.  The stages before rasterisation are
pinned by fixtures recorded from the reference (``tests/golden/``) and the
raster rules by analytic known-answer tests.

Scene format (the same fp32 arrays the CUDA kernels read; produced by
``PBRRenderer.export_scene()``):

* ``scene``: dict with ``N, W, H, C``, ``vp`` ``[N,4,4]`` row-major view-projection,
  ``ambient``/``ldir``/``lcol`` (3 floats), ``strength``, ``bg`` (4 floats),
  ``cull``, and for the soft mode ``znear, zfar, sigma, gamma``.
* ``meshes``: list of objects with ``positions [nv,3]``, ``normals [nv,3]``,
  ``indices [nt,3]``.
* ``nodes``: list of dicts with ``mesh`` (index), ``I`` (instances per scene),
  ``shared``, ``mode`` (0 = HPR, 1 = 3x3 rotation, 2 = 4x4 matrix), ``counts``
  (``[N]`` int32 or None), ``pos [B,3]``, ``rot`` (``[B,3]`` / ``[B,9]`` / ``[B,16]``),
  ``scale [B]``, ``color [B,4]``, optional ``texture`` ``[h,w,4]`` uint8 RGBA (row 0
  at v = 0, i.e. the bottom row of the image) sampled at the mesh's ``uvs [nv,2]``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

MODE_HPR, MODE_ROT, MODE_MAT = 0, 1, 2


class OrcMesh(ctypes.Structure):
    _fields_ = [("nv", ctypes.c_int32), ("nt", ctypes.c_int32),
                ("pos", ctypes.c_void_p), ("nrm", ctypes.c_void_p), ("idx", ctypes.c_void_p),
                ("uv", ctypes.c_void_p)]


class OrcNode(ctypes.Structure):
    _fields_ = [("mesh", ctypes.c_int32), ("inst_per_scene", ctypes.c_int32),
                ("shared", ctypes.c_int32), ("mode", ctypes.c_int32),
                ("counts", ctypes.c_void_p), ("pos", ctypes.c_void_p), ("rot", ctypes.c_void_p),
                ("scale", ctypes.c_void_p), ("color", ctypes.c_void_p),
                ("tex", ctypes.c_void_p), ("tex_w", ctypes.c_int32), ("tex_h", ctypes.c_int32)]


class OrcScene(ctypes.Structure):
    _fields_ = [("N", ctypes.c_int32), ("W", ctypes.c_int32), ("H", ctypes.c_int32), ("C", ctypes.c_int32),
                ("vp", ctypes.c_void_p),
                ("ambient", ctypes.c_float * 3), ("ldir", ctypes.c_float * 3), ("lcol", ctypes.c_float * 3),
                ("strength", ctypes.c_float), ("bg", ctypes.c_float * 4), ("cull", ctypes.c_int32),
                ("znear", ctypes.c_float), ("zfar", ctypes.c_float), ("sigma", ctypes.c_float),
                ("gamma", ctypes.c_float), ("soft_dense", ctypes.c_int32)]


def build(force: bool = False) -> str:
    """Compile ``liboracle.so`` with the committed Makefile (gcc only)."""
    src = os.path.join(HERE, "raster_ref.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE, "clean"], check=True)
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(LIB_PATH)
        for prec in ("f32", "f64"):
            f = getattr(_lib, f"orc_render_hard_{prec}")
            f.restype = ctypes.c_int
            f.argtypes = [ctypes.POINTER(OrcScene), ctypes.c_int, ctypes.POINTER(OrcMesh), ctypes.c_int,
                          ctypes.POINTER(OrcNode), ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_float,
                          ctypes.c_float, ctypes.c_int]
            g = getattr(_lib, f"orc_render_soft_{prec}")
            g.restype = ctypes.c_int
            g.argtypes = [ctypes.POINTER(OrcScene), ctypes.c_int, ctypes.POINTER(OrcMesh), ctypes.c_int,
                          ctypes.POINTER(OrcNode), ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
            h = getattr(_lib, f"orc_instance_matrices_{prec}")
            h.restype = ctypes.c_int
            h.argtypes = [ctypes.POINTER(OrcNode), ctypes.c_int64, ctypes.c_void_p]
    return _lib


def _ptr(a: np.ndarray | None) -> int | None:
    return None if a is None else a.ctypes.data


class _Packed:
    """Keeps the contiguous arrays alive while C reads them."""

    def __init__(self, scene: dict, meshes: list, nodes: list):
        self.keep = []

        def f32(a, shape=None):
            arr = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
            if shape is not None:
                arr = arr.reshape(shape)
            self.keep.append(arr)
            return arr

        def i32(a):
            arr = np.ascontiguousarray(np.asarray(a, dtype=np.int32))
            self.keep.append(arr)
            return arr

        sc = OrcScene()
        sc.N, sc.W, sc.H = int(scene["N"]), int(scene["W"]), int(scene["H"])
        sc.C = int(scene.get("C", 3))
        sc.vp = _ptr(f32(scene["vp"], (-1, 16)))
        for name in ("ambient", "ldir", "lcol"):
            getattr(sc, name)[:] = [float(v) for v in scene[name]]
        sc.strength = float(scene["strength"])
        sc.bg[:] = [float(v) for v in scene.get("bg", (0, 0, 0, 1))]
        sc.cull = int(scene.get("cull", 1))
        sc.znear = float(scene.get("znear", 0.05))
        sc.zfar = float(scene.get("zfar", 100.0))
        sc.sigma = float(scene.get("sigma", 0.5 / (2 * np.log(9.0))))
        sc.gamma = float(scene.get("gamma", 1e-3))
        sc.soft_dense = int(scene.get("soft_dense", 0))
        self.scene = sc
        self.meshes = (OrcMesh * max(1, len(meshes)))()
        for i, m in enumerate(meshes):
            pos, nrm, idx = (m["positions"], m["normals"], m["indices"]) if isinstance(m, dict) else \
                (m.positions, m.normals, m.indices)
            uv = m.get("uvs") if isinstance(m, dict) else getattr(m, "uvs", None)
            p, n, ix = f32(pos, (-1, 3)), f32(nrm, (-1, 3)), i32(np.asarray(idx).reshape(-1, 3))
            self.meshes[i].nv, self.meshes[i].nt = p.shape[0], ix.shape[0]
            self.meshes[i].pos, self.meshes[i].nrm, self.meshes[i].idx = _ptr(p), _ptr(n), _ptr(ix)
            self.meshes[i].uv = _ptr(f32(uv, (-1, 2))) if uv is not None else None
        self.nodes = (OrcNode * max(1, len(nodes)))()
        for i, nd in enumerate(nodes):
            o = self.nodes[i]
            o.mesh, o.inst_per_scene, o.shared = int(nd["mesh"]), int(nd["I"]), int(bool(nd["shared"]))
            o.mode = int(nd["mode"])
            o.counts = _ptr(i32(nd["counts"])) if nd.get("counts") is not None else None
            o.pos = _ptr(f32(nd["pos"], (-1, 3)))
            o.rot = _ptr(f32(nd["rot"]).reshape(-1))
            o.scale = _ptr(f32(nd["scale"]).reshape(-1))
            o.color = _ptr(f32(nd["color"], (-1, 4)))
            tex = nd.get("texture")
            if tex is not None:
                t = np.ascontiguousarray(np.asarray(tex, dtype=np.uint8))
                if t.ndim != 3 or t.shape[2] != 4:
                    raise ValueError("node texture must be [h, w, 4] uint8")
                self.keep.append(t)
                o.tex, o.tex_h, o.tex_w = _ptr(t), t.shape[0], t.shape[1]
        self.nmeshes, self.nnodes = len(meshes), len(nodes)


def render_hard(scene: dict, meshes: list, nodes: list, k0: int = 0, k1: int | None = None, *,
                want_depth: bool = False, want_winner: bool = False, want_ambiguous: bool = False,
                tol_px: float = 1e-4, tol_z: float = 2e-6, precision: str = "f64",
                nthreads: int = 1) -> dict:
    """Hard-raster scenes [k0, k1).  Returns a dict of numpy arrays holding
    those scenes: ``pixels [n,C,H,W] u8`` and optionally ``depth [n,H,W] f32``,
    ``winner [n,H,W] i32`` and ``ambiguous [n,H,W] bool``."""
    pk = _Packed(scene, meshes, nodes)
    N, W, H, C = pk.scene.N, pk.scene.W, pk.scene.H, pk.scene.C
    k1 = N if k1 is None else k1
    out = np.zeros((N, C, H, W), np.uint8)
    depth = np.zeros((N, H, W), np.float32) if want_depth else None
    winner = np.zeros((N, H, W), np.int32) if want_winner else None
    amb = np.zeros((N, H, W), np.uint8) if want_ambiguous else None
    fn = getattr(lib(), f"orc_render_hard_{precision}")
    rc = fn(ctypes.byref(pk.scene), pk.nmeshes, pk.meshes, pk.nnodes, pk.nodes, k0, k1, _ptr(out),
            _ptr(depth), _ptr(winner), _ptr(amb), tol_px, tol_z, nthreads)
    if rc != 0:
        raise RuntimeError(f"oracle hard raster failed with status {rc}")
    res = {"pixels": out[k0:k1]}
    if want_depth:
        res["depth"] = depth[k0:k1]
    if want_winner:
        res["winner"] = winner[k0:k1]
    if want_ambiguous:
        res["ambiguous"] = amb[k0:k1].astype(bool)
    return res


def render_soft(scene: dict, meshes: list, nodes: list, k0: int = 0, k1: int | None = None, *,
                precision: str = "f64", out_dtype=np.float32) -> np.ndarray:
    """Soft-coverage render of scenes [k0, k1) -> [n,3,H,W] (float32, or
    float64 with ``out_dtype=np.float64`` for finite differences)."""
    pk = _Packed(scene, meshes, nodes)
    N, W, H = pk.scene.N, pk.scene.W, pk.scene.H
    k1 = N if k1 is None else k1
    out = np.zeros((N, 3, H, W), out_dtype)
    fn = getattr(lib(), f"orc_render_soft_{precision}")
    rc = fn(ctypes.byref(pk.scene), pk.nmeshes, pk.meshes, pk.nnodes, pk.nodes, k0, k1, _ptr(out),
            int(out.dtype == np.float64))
    if rc != 0:
        raise RuntimeError(f"oracle soft raster failed with status {rc}")
    return out[k0:k1]


def instance_matrices(node: dict, precision: str = "f64") -> np.ndarray:
    """Per-instance 4x4 model matrices ``[B,4,4]`` (row-major) of one node."""
    pk = _Packed({"N": 1, "W": 1, "H": 1, "vp": np.eye(4), "ambient": (0, 0, 0), "ldir": (0, 0, 1),
                  "lcol": (0, 0, 0), "strength": 0}, [], [node])
    B = np.asarray(node["pos"]).reshape(-1, 3).shape[0]
    out = np.zeros((B, 16), np.float32)
    fn = getattr(lib(), f"orc_instance_matrices_{precision}")
    fn(pk.nodes, B, _ptr(out))
    return out.reshape(B, 4, 4)


def compare_hard(gpu: dict, ref: dict) -> dict:
    """Parity summary between a CUDA render and an oracle render of the same
    scenes.  Pixels flagged ambiguous by the oracle (centre within tol_px of an
    edge, or a depth tie within tol_z) are excluded from the exact winner
    check; colour is compared on every pixel."""
    amb = ref["ambiguous"]
    keep = ~amb
    res = {"pixels": int(amb.size), "ambiguous": int(amb.sum())}
    if "winner" in gpu:
        res["winner_mismatch"] = int(((gpu["winner"] != ref["winner"]) & keep).sum())
    d = np.abs(gpu["pixels"].astype(np.int16) - ref["pixels"].astype(np.int16))
    per_px = d.max(axis=1)
    res["color_max_diff_unambiguous"] = int(per_px[keep].max()) if keep.any() else 0
    res["color_within_1"] = float((per_px <= 1).mean())
    res["color_exact"] = float((per_px == 0).mean())
    if "depth" in gpu and "depth" in ref:
        dz = np.abs(gpu["depth"] - ref["depth"])
        res["depth_max_diff_unambiguous"] = float(dz[keep].max()) if keep.any() else 0.0
    return res
