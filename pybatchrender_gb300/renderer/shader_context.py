"""Base class of nodes, camera and light (``renderer/shader_context.py``).

In the reference this class wraps Panda3D shader inputs.  Here the "shader
inputs" are kernel arguments owned by the renderer's C context, so the
helpers that matter are the tensor math ones: the HPR rotation convention and
column packing.
"""
from __future__ import annotations

from abc import ABC, abstractmethod
from typing import Literal

import torch


class PBRShaderContext(ABC):
    def __init__(self, showbase, backend: Literal["instanced", "loop"] = "instanced") -> None:
        self.base = showbase
        if backend == "loop":
            raise NotImplementedError("Loop backend is not implemented yet. Use instanced backend instead.")
        self.backend = backend

    @staticmethod
    def _pack_columns(mat_batch: torch.Tensor) -> torch.Tensor:
        """(B,4,4) -> (B,4,4) column-packed, as uploaded for GLSL
        (``renderer/shader_context.py:42-45``)."""
        return mat_batch.transpose(1, 2).to(torch.float32)

    @staticmethod
    def _rotation_mats_from_hpr(hpr_b3: torch.Tensor) -> torch.Tensor:
        """Rotation matrices from (H, P, R) radians: ``R = Rz(H) @ Ry(P) @ Rx(R)``
        (``renderer/shader_context.py:47-84``).  Returns (B,3,3) float32 on the
        input's device."""
        hpr_b3 = torch.as_tensor(hpr_b3).to(torch.float32)
        h, p, r = hpr_b3[:, 0], hpr_b3[:, 1], hpr_b3[:, 2]
        ch, sh = torch.cos(h), torch.sin(h)
        cp, sp = torch.cos(p), torch.sin(p)
        cr, sr = torch.cos(r), torch.sin(r)
        B = hpr_b3.shape[0]
        dev = hpr_b3.device
        Rz = torch.zeros((B, 3, 3), dtype=torch.float32, device=dev)
        Rz[:, 0, 0] = ch; Rz[:, 0, 1] = -sh
        Rz[:, 1, 0] = sh; Rz[:, 1, 1] = ch
        Rz[:, 2, 2] = 1.0
        Ry = torch.zeros((B, 3, 3), dtype=torch.float32, device=dev)
        Ry[:, 0, 0] = cp; Ry[:, 0, 2] = sp
        Ry[:, 1, 1] = 1.0
        Ry[:, 2, 0] = -sp; Ry[:, 2, 2] = cp
        Rx = torch.zeros((B, 3, 3), dtype=torch.float32, device=dev)
        Rx[:, 0, 0] = 1.0
        Rx[:, 1, 1] = cr; Rx[:, 1, 2] = -sr
        Rx[:, 2, 1] = sr; Rx[:, 2, 2] = cr
        return torch.einsum('bij,bjk->bik', torch.einsum('bij,bjk->bik', Rz, Ry), Rx).to(torch.float32)

    @staticmethod
    def _normalize(v: torch.Tensor) -> torch.Tensor:
        n = torch.linalg.norm(v, dim=-1, keepdim=True)
        return v / n.clamp_min(1e-8)

    def _set_shader_input(self, input_name: str, value) -> None:
        """Kept for subclasses written against the reference: records the
        value; kernel arguments come from the renderer's own state."""
        inputs = self.__dict__.setdefault("_shader_inputs", {})
        inputs[input_name] = value

    def _auto_screen_size_input(self) -> None:
        cfg = getattr(self.base, "cfg", None)
        if cfg is not None:
            self._set_shader_input('screenSize', (float(cfg.window_resolution[0]), float(cfg.window_resolution[1])))

    @abstractmethod
    def _register_self(self) -> None:
        raise NotImplementedError
