"""Instanced node (``renderer/node.py``).

A node is one mesh drawn ``instances_per_scene`` times in every scene.  Its
per-instance state lives in device tensors that the CUDA kernels read
directly; the setters write those tensors in place (their addresses never
change, which is what CUDA-graph replay needs).  The kernels build each model
matrix ``M = [R(hpr) * s | t]`` themselves, so unlike the reference
(``node.py:110-126``) no 4x4 matrices are packed or uploaded per step.

Buffer rows: ``B = instances_per_scene`` when ``shared_across_scenes`` (row i is
instance i of every scene), else ``B = num_scenes * instances_per_scene`` (row
``k*I + i`` is instance i of scene k) -- ``node.py:43-46`` and
``shaders/basic.vert:25-28``.

Differences from the reference, all deliberate:

* ``lazy=True`` is accepted but every setter takes effect at the next render
  (the reference defers the texture upload, so a lazy update that is never
  followed by a non-lazy one is not drawn there).
* A shared node with ``1 < I < num_scenes`` draws instance i of every scene from
  row i.  The reference sets ``instancesPerScene = max(1, B // N)`` (``node.py:90``),
  which is 1 in that case and makes every instance decode as its own scene.
* ``texture`` also accepts an image array or tensor, and ``True`` falls back to
  a white texture when the model brings none (the reference leaves that case to
  whatever Panda3D binds).  Textured nodes are drawn in the hard raster modes;
  the soft (differentiable) mode rejects them.
"""
from __future__ import annotations

import warnings
from collections.abc import Sequence
from typing import Literal

import numpy as np
import torch

from .meshes import Mesh, bake, resolve_model
from .shader_context import PBRShaderContext
from .textures import WHITE, as_rgba8, gl_rows, load_image

MODE_HPR, MODE_ROT, MODE_MAT = 0, 1, 2


class PBRNode(PBRShaderContext):
    def __init__(self,
                 showbase,
                 model_path: "str | Mesh | None",
                 num_scenes: int = 1,
                 instances_per_scene: int = 1,
                 texture=None,
                 model_pivot_relative_point: tuple[float, float, float] | None = None,
                 model_scale: float | Sequence[float] | None = None,
                 model_hpr: tuple[float, float, float] | Sequence[float] | None = None,
                 model_scale_units: Literal["relative", "absolute"] = "relative",
                 positions: torch.Tensor | None = None,
                 hprs: torch.Tensor | None = None,
                 scales: torch.Tensor | None = None,
                 colors: torch.Tensor | None = None,
                 backend: Literal["loop", "instanced"] = "instanced",
                 shared_across_scenes: bool = False,
                 parent: "PBRNode | None" = None,
                 name: str | None = None) -> None:
        if positions is not None or colors is not None or scales is not None or hprs is not None:
            warnings.warn("initializing positions, colors, scales are not implemented yet, they will be ignored")
        super().__init__(showbase, backend=backend)
        self.num_scenes = int(num_scenes)
        self.instances_per_scene = int(instances_per_scene)
        if self.instances_per_scene < 0:
            raise ValueError("instances_per_scene must be >= 0")
        self.shared_across = bool(shared_across_scenes)
        self.total_instances = self.num_scenes * self.instances_per_scene
        self.buf_instances = self.instances_per_scene if self.shared_across else self.total_instances
        self.model_pivot_relative_point = model_pivot_relative_point
        self.model_scale = model_scale
        self.model_hpr = model_hpr
        self.model_scale_units = model_scale_units
        self.name = name
        self.device = getattr(showbase, "state_device", torch.device("cpu"))
        self.texture: np.ndarray | None = None  # [h,w,4] uint8 RGBA, row 0 at v = 0

        if model_path:
            self.mesh: Mesh | None = bake(resolve_model(model_path), model_scale, model_hpr,
                                          model_pivot_relative_point, model_scale_units)
            self.has_geometry = True
        else:
            self.mesh = None
            self.has_geometry = False
        self.set_texture(texture)

        B = self.buf_instances
        dev = self.device
        self.mode = MODE_HPR
        self.pos = torch.zeros((B, 3), dtype=torch.float32, device=dev)
        self.hpr = torch.zeros((B, 3), dtype=torch.float32, device=dev)
        self.rot3 = None  # [B,3,3], allocated by set_transforms
        self.scale = torch.ones((B,), dtype=torch.float32, device=dev)
        self.color = torch.ones((B, 4), dtype=torch.float32, device=dev)
        self.counts = None  # [N] int32 active instances per scene (uneven batching)
        self._register_self()

    def remove(self) -> None:
        """Remove this node from its renderer (``NodePath.removeNode``)."""
        remove = getattr(self.base, "remove_node", None)
        if remove is not None:
            remove(self)

    # ------------------------------------------------------------------ state
    def _as(self, x, cols: int | None) -> torch.Tensor:
        t = torch.as_tensor(x, dtype=torch.float32)
        if t.device != self.device:
            t = t.to(self.device, non_blocking=True)
        return t.reshape(-1, cols) if cols else t.reshape(-1)

    def set_positions(self, pos_si3, lazy: bool = False) -> None:
        """Instance positions, any shape reshaping to (-1,3); the first
        ``buf_instances`` rows are used, a single row broadcasts
        (``node.py:128-134``)."""
        if not self.has_geometry:
            return
        with torch.no_grad():
            self.pos.copy_(self._as(pos_si3, 3)[:self.buf_instances])

    def set_hprs(self, hpr_si3, lazy: bool = False) -> None:
        """Instance heading/pitch/roll in radians, ``R = Rz(H) Ry(P) Rx(R)``
        (``node.py:136-143``)."""
        if not self.has_geometry:
            return
        with torch.no_grad():
            self.hpr.copy_(self._as(hpr_si3, 3)[:self.buf_instances])
        if self.mode != MODE_HPR:
            self.mode = MODE_HPR
            self._rebind()

    def set_scales(self, scale_si1, lazy: bool = False) -> None:
        """Uniform per-instance scale: a number or (-1,) values
        (``node.py:145-154``)."""
        if not self.has_geometry:
            return
        if isinstance(scale_si1, (float, int)):
            with torch.no_grad():
                self.scale.fill_(float(scale_si1))
        else:
            with torch.no_grad():
                self.scale.copy_(self._as(scale_si1, None)[:self.buf_instances])

    def set_colors(self, col_si4) -> None:
        """Per-instance RGBA (``node.py:156-161``)."""
        if not self.has_geometry:
            return
        with torch.no_grad():
            self.color.copy_(self._as(col_si4, 4)[:self.buf_instances])

    def set_transforms(self, mats_b44) -> None:
        """Full per-instance matrices (B,4,4).  As in ``node.py:163-178`` the
        matrix is split into rotation, uniform scale (mean of the 3x3 row
        norms, clamped to 1e-8) and translation, so later ``set_positions`` /
        ``set_scales`` calls modify it the same way."""
        if not self.has_geometry:
            return
        mats = self._as(mats_b44, None).reshape(-1, 4, 4)
        rot3 = mats[:, 0:3, 0:3].clone()
        s = (torch.linalg.norm(rot3[:, 0, :], dim=1) + torch.linalg.norm(rot3[:, 1, :], dim=1)
             + torch.linalg.norm(rot3[:, 2, :], dim=1)) / 3.0
        s = torch.clamp(s, min=1e-8)
        B = self.buf_instances
        if self.rot3 is None:
            self.rot3 = torch.zeros((B, 3, 3), dtype=torch.float32, device=self.device)
        with torch.no_grad():
            self.rot3.copy_((rot3 / s.reshape(-1, 1, 1))[:B])
            self.scale.copy_(s[:B])
            self.pos.copy_(mats[:, 0:3, 3][:B])
        if self.mode != MODE_ROT:
            self.mode = MODE_ROT
            self._rebind()

    def set_active_counts(self, counts_n) -> None:
        """Uneven batching (no reference counterpart): scene k draws only the
        first ``counts[k]`` instances of this node.  ``None`` draws all."""
        if counts_n is None:
            if self.counts is not None:
                self.counts = None
                self._rebind()
            return
        c = torch.as_tensor(counts_n).to(device=self.device, dtype=torch.int32).reshape(-1)
        if c.numel() != self.num_scenes:
            raise ValueError(f"counts must have num_scenes={self.num_scenes} entries, got {c.numel()}")
        if self.counts is None:
            self.counts = c.clone()
            self._rebind()
        else:
            self.counts.copy_(c)

    # --------------------------------------------------------------- getters
    def rotation_matrices(self) -> torch.Tensor:
        """(B,3,3) rotations of the current mode (host-side helper)."""
        if self.mode == MODE_ROT and self.rot3 is not None:
            return self.rot3.clone()
        return PBRShaderContext._rotation_mats_from_hpr(self.hpr)

    def get_transforms(self) -> torch.Tensor:
        """(B,4,4) model matrices ``[R*s | t]`` -- what the reference uploads to
        ``matbuf`` (before column packing).  Host-side helper; the kernels build
        the same matrices on the fly."""
        B = self.buf_instances
        M = torch.zeros((B, 4, 4), dtype=torch.float32, device=self.device)
        M[:, 0:3, 0:3] = self.rotation_matrices() * self.scale.reshape(-1, 1, 1)
        M[:, 0:3, 3] = self.pos
        M[:, 3, 3] = 1.0
        return M

    @property
    def transforms_b44(self) -> torch.Tensor:
        return self.get_transforms()

    @property
    def rot3_b33(self) -> torch.Tensor:
        return self.rotation_matrices()

    @property
    def scale_b11(self) -> torch.Tensor:
        return self.scale.reshape(-1, 1, 1)

    # ----------------------------------------------------------------- misc
    def set_texture(self, texture=None) -> None:
        """``useTexture`` and ``p3d_Texture0`` (``renderer/node.py:277-287``).

        ``texture``: a PNG path (or ``.npy``), an image array / tensor
        ``[h,w]`` or ``[h,w,1|3|4]`` (uint8, or float in [0,1]; row 0 = top),
        ``True`` for the model's own texture (white if it has none), or
        None / False for no texture."""
        if texture is None or texture is False:
            self.texture = None
            self._set_shader_input('useTexture', 0.0)
        else:
            if texture is True:
                own = self.mesh.texture if self.mesh is not None else None
                img = own if own is not None else WHITE
            elif isinstance(texture, str):
                img = load_image(texture)
            else:
                img = as_rgba8(texture)
            self.texture = gl_rows(img)
            self._set_shader_input('useTexture', 1.0)
        changed = getattr(self.base, "_texture_changed", None)
        if changed is not None:
            changed(self)

    def reparent_to(self, parent) -> None:
        raise NotImplementedError("PBRNode.reparent_to is not implemented yet")

    def pivot_to_rel(self, relative_point=None) -> None:
        """Re-centre the mesh so the bounds-relative point becomes the origin
        (``node.py:313-341``).  Only valid before ``setup_environment``."""
        if relative_point is None or self.mesh is None:
            return
        if getattr(self.base, "_ctx", None) is not None:
            raise RuntimeError("pivot_to_rel must be called before setup_environment()")
        self.mesh = bake(self.mesh, None, None, relative_point)

    def _register_self(self) -> None:
        nodes = getattr(self.base, "_pbr_nodes", None)
        if nodes is None:
            self.base._pbr_nodes = nodes = []
        if self not in nodes:
            nodes.append(self)

    def _rebind(self) -> None:
        rebind = getattr(self.base, "_rebind_node", None)
        if rebind is not None:
            rebind(self)

    # kernel-facing view
    def kernel_buffers(self) -> tuple[int, torch.Tensor, torch.Tensor, torch.Tensor, torch.Tensor]:
        """(mode, pos, rot, scale, color) tensors as the C ABI binds them."""
        if self.mode == MODE_ROT:
            return MODE_ROT, self.pos, self.rot3.reshape(-1, 9), self.scale, self.color
        return MODE_HPR, self.pos, self.hpr, self.scale, self.color

    def export(self) -> dict:
        """Host copy of the node in the oracle's scene format."""
        mode, pos, rot, scale, color = self.kernel_buffers()
        return {
            "I": self.instances_per_scene, "shared": self.shared_across, "mode": mode,
            "counts": None if self.counts is None else self.counts.detach().cpu().numpy(),
            "pos": pos.detach().cpu().numpy(), "rot": rot.detach().cpu().numpy(),
            "scale": scale.detach().cpu().numpy(), "color": color.detach().cpu().numpy(),
            "texture": self.texture,
        }


def mesh_key(mesh: Mesh) -> bytes:
    """Content key used to share identical baked meshes between nodes."""
    return (mesh.positions.tobytes() + b"|" + mesh.normals.tobytes() + b"|" + mesh.indices.tobytes()
            + b"|" + (mesh.uvs.tobytes() if mesh.uvs is not None else b"-")
            + np.int64(mesh.num_vertices).tobytes())
