"""Per-scene cameras (``renderer/camera.py``).

The view and projection math follows the reference line by line, in float32
torch on the renderer's device:

* view (``camera.py:201-240``): rows ``s, u, -f`` with
  ``s = normalize(f x up)``, ``u = s x f``, translation ``(-s.e, -u.e, f.e)``;
* projection (``camera.py:150-166``): GL perspective with
  ``f = 1/tan(fov/2)``, aspect = **window** width / height, i.e. the whole
  atlas of ``tiles x tile_resolution`` (``camera.py:154``) -- kept so that
  each scene's image matches the reference's tile pixel for pixel;
* ``VP = P @ V`` per scene (``camera.py:252-262``).

``VP_k44`` is written in place into a device tensor that the renderer binds
once, so camera updates need no rebinding.  On a CUDA device each update is
one launch of ``pbr_camera_update`` (the same formulas in float32, view and
view-projection together) instead of a dozen tensor operations; on the CPU
the tensor operations run.  One deliberate difference:
``set_projection`` takes effect (the reference only clears a cache that
``_update_vp`` never reads again, so there it has no effect).
"""
from __future__ import annotations

import ctypes
import math
from typing import Literal

import torch

from .shader_context import PBRShaderContext


class PBRCam(PBRShaderContext):
    def __init__(self, showbase,
                 num_scenes: int,
                 cols: int | None = None,
                 rows: int | None = None,
                 backend: Literal["loop", "instanced"] = "instanced",
                 fov_y_deg: float = 55.0,
                 z_near: float = 0.05,
                 z_far: float = 100.0,
                 auto_tiles: bool = True,
                 fixed_projection: bool = True) -> None:
        super().__init__(showbase, backend=backend)
        self.num_scenes = int(num_scenes)
        self.fov_y_deg = float(fov_y_deg)
        self.z_near = float(z_near)
        self.z_far = float(z_far)
        self.fixed_projection = fixed_projection
        self.device = getattr(showbase, "device", torch.device("cpu"))
        self.cols = cols
        self.rows = rows
        self._set_tiles()

        dev, K = self.device, self.num_scenes
        self.eye_k3 = torch.zeros((K, 3), dtype=torch.float32, device=dev)
        self.forward_k3 = torch.zeros((K, 3), dtype=torch.float32, device=dev)
        self.up_k3 = torch.zeros((K, 3), dtype=torch.float32, device=dev)
        self.hpr_k3 = torch.zeros((K, 3), dtype=torch.float32, device=dev)
        self.target_k3 = torch.zeros((K, 3), dtype=torch.float32, device=dev)
        self.V_k44 = torch.eye(4, dtype=torch.float32, device=dev)[None].repeat(K, 1, 1)
        # device buffer bound by the renderer; updated in place
        self.VP_k44 = torch.zeros((K, 4, 4), dtype=torch.float32, device=dev)

        self._proj_cache_key = None
        self._proj_cache = None
        self.P_k44 = self._get_projection()
        self._update_view(eye_k3=torch.tensor([0., -12., 0.], dtype=torch.float32),
                          forward_k3=torch.tensor([0.0, 1., 0.], dtype=torch.float32),
                          up_k3=torch.tensor([0.0, 0.0, 1.], dtype=torch.float32))
        self._update_vp()
        self.sync_from_base_cam = False
        self._register_self()

    # --------------------------------------------------------------- tiling
    def _set_tiles(self) -> None:
        """Atlas tile rectangles (``camera.py:110-135``).  The renderer draws
        each scene into its own image, so these are informational only."""
        if self.num_scenes is None and (self.cols is None or self.rows is None):
            raise ValueError("num_scenes or (cols and rows) must be provided")
        if self.cols is None and self.rows is None:
            self.cols = math.ceil(math.sqrt(self.num_scenes))
        if self.rows is None:
            self.rows = math.ceil(self.num_scenes / self.cols)
        if self.num_scenes is None:
            self.num_scenes = self.cols * self.rows
        K = int(self.num_scenes)
        idx = torch.arange(K, dtype=torch.float32)
        cols, rows = float(self.cols), float(self.rows)
        col = torch.remainder(idx, cols)
        row = torch.floor(idx / cols)
        self.tiles_k4 = torch.stack([col / cols, (col + 1.0) / cols,
                                     1.0 - (row + 1.0) / rows, 1.0 - row / rows], dim=1).to(torch.float32)

    # ----------------------------------------------------------- projection
    def _window_size(self) -> tuple[float, float]:
        cfg = getattr(self.base, "cfg", None)
        if cfg is not None and cfg.window_resolution is not None:
            return float(cfg.window_resolution[0]), float(cfg.window_resolution[1])
        return float(self.cols or 1), float(self.rows or 1)

    def _get_projection(self) -> torch.Tensor:
        if self.fixed_projection and self._proj_cache is not None:
            return self._proj_cache
        wx, wy = self._window_size()
        aspect = max(1e-6, wx / max(1, wy))
        key = (float(self.fov_y_deg), float(self.z_near), float(self.z_far), float(aspect))
        if self._proj_cache_key != key or self._proj_cache is None:
            f = 1.0 / math.tan(math.radians(self.fov_y_deg) * 0.5)
            P = torch.zeros((4, 4), dtype=torch.float32)
            P[0, 0] = torch.tensor(f / aspect, dtype=torch.float32)
            P[1, 1] = torch.tensor(f, dtype=torch.float32)
            P[2, 2] = torch.tensor((self.z_far + self.z_near) / (self.z_near - self.z_far), dtype=torch.float32)
            P[2, 3] = torch.tensor((2.0 * self.z_far * self.z_near) / (self.z_near - self.z_far), dtype=torch.float32)
            P[3, 2] = torch.tensor(-1.0, dtype=torch.float32)
            self._proj_cache_key = key
            self._P_host = (ctypes.c_float * 16)(*P.reshape(-1).tolist())
            self._proj_cache = P.to(self.device)
        return self._proj_cache

    def set_projection(self, fov_y_deg: float | None = None, z_near: float | None = None,
                       z_far: float | None = None) -> None:
        if fov_y_deg is not None:
            self.fov_y_deg = float(fov_y_deg)
        if z_near is not None:
            self.z_near = float(z_near)
        if z_far is not None:
            self.z_far = float(z_far)
        self._proj_cache_key = None
        self._proj_cache = None
        self.P_k44 = self._get_projection()
        self._update_vp()
        notify = getattr(self.base, "_camera_changed", None)
        if notify is not None:
            notify(self)

    # ----------------------------------------------------------------- view
    def _ensure_kx3(self, arr, name: str) -> torch.Tensor:
        a = torch.as_tensor(arr, dtype=torch.float32)
        if a.device != self.device:
            a = a.to(self.device)
        if a.ndim == 1:
            a = a.unsqueeze(0)
        if a.shape[-1] != 3:
            raise ValueError(f"{name} must have shape (K,3) or (3,), got {tuple(a.shape)}")
        if a.shape[0] == 1 and self.num_scenes > 1:
            a = a.repeat(self.num_scenes, 1)
        if a.shape[0] != self.num_scenes:
            raise ValueError(f"{name} first dim must be K={self.num_scenes}, got {a.shape[0]}")
        return a

    def _camera_kernel(self, eye=None, fwd=None, up=None, vp: bool = False) -> None:
        """One ``pbr_camera_update`` launch on the current stream: the view's
        basis from ``fwd`` / ``up`` (when given), its translation from ``eye``
        (when given), and ``VP_k44`` when ``vp``."""
        from .. import _capi
        lib = _capi.load()
        stream = torch.cuda.current_stream(self.device).cuda_stream
        rc = lib.pbr_camera_update(_capi.ptr(eye), _capi.ptr(fwd), _capi.ptr(up), _capi.ptr(self.V_k44),
                                   self._P_host, _capi.ptr(self.VP_k44) if vp else None, int(self.num_scenes),
                                   stream)
        if rc != _capi.PBR_OK:
            raise _capi.PBRError("pbr_camera_update", rc, "invalid arguments or launch failure")

    def _update_view(self, eye_k3=None, forward_k3=None, up_k3=None, vp: bool = False) -> None:
        """Update the view from a new eye, forward and/or up (rows s, u, -f,
        translation from the eye); with ``vp`` also the view-projection."""
        basis_changed = (forward_k3 is not None) or (up_k3 is not None)
        eye_changed = eye_k3 is not None
        if not basis_changed and not eye_changed:
            if vp:
                self._update_vp()
            return
        if self.device.type == "cuda":
            f = self._ensure_kx3(forward_k3, 'forward_k3').contiguous() if forward_k3 is not None else None
            u = self._ensure_kx3(up_k3, 'up_k3').contiguous() if up_k3 is not None else None
            if eye_changed:
                self.eye_k3 = self._ensure_kx3(eye_k3, 'eye_k3').contiguous()
            self._camera_kernel(eye=self.eye_k3, fwd=f, up=u, vp=vp)
            return
        if basis_changed:
            if forward_k3 is not None:
                f = type(self)._normalize(self._ensure_kx3(forward_k3, 'forward_k3'))
            else:
                f = -self.V_k44[:, 2, 0:3]
            if up_k3 is not None:
                up_in = type(self)._normalize(self._ensure_kx3(up_k3, 'up_k3'))
            else:
                up_in = self.V_k44[:, 1, 0:3]
            s = type(self)._normalize(torch.cross(f, up_in, dim=-1))
            u = torch.cross(s, f, dim=-1)
            self.V_k44[:, 0, 0:3] = s
            self.V_k44[:, 1, 0:3] = u
            self.V_k44[:, 2, 0:3] = -f
        else:
            s = self.V_k44[:, 0, 0:3]
            u = self.V_k44[:, 1, 0:3]
            f = -self.V_k44[:, 2, 0:3]
        if eye_changed:
            self.eye_k3 = self._ensure_kx3(eye_k3, 'eye_k3')
        self.V_k44[:, 0, 3] = -torch.einsum('ij,ij->i', s, self.eye_k3)
        self.V_k44[:, 1, 3] = -torch.einsum('ij,ij->i', u, self.eye_k3)
        self.V_k44[:, 2, 3] = torch.einsum('ij,ij->i', f, self.eye_k3)
        if vp:
            self._update_vp()

    @staticmethod
    def _fwd_up_from_hpr(hpr_k3: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor]:
        R = PBRShaderContext._rotation_mats_from_hpr(hpr_k3)
        unit_fwd = torch.tensor([0.0, 1.0, 0.0], dtype=torch.float32, device=R.device)
        unit_up = torch.tensor([0.0, 0.0, 1.0], dtype=torch.float32, device=R.device)
        return torch.einsum('bij,j->bi', R, unit_fwd), torch.einsum('bij,j->bi', R, unit_up)

    def _update_vp(self) -> None:
        if self.device.type == "cuda":
            self._camera_kernel(vp=True)
            return
        VP = torch.einsum('ij,bjk->bik', self.P_k44, self.V_k44).reshape(-1, 4, 4)
        self.VP_k44.copy_(VP.to(torch.float32))

    def get_vp(self) -> torch.Tensor:
        return self.VP_k44.clone()

    # --- public API (camera.py:268-344) ---
    def look_at(self, target_k3, lazy: bool = False) -> None:
        fwd = self._fwd_from_lookat(target_k3)
        self._update_view(forward_k3=fwd, vp=not lazy)

    def set_positions(self, eye_k3, keep_lookat: bool = False, lazy: bool = False) -> None:
        if keep_lookat:
            raise NotImplementedError("Target can't be reconsturcted from eye and forward, needs to be stored in memory then")
        self.set_eye(eye_k3, lazy=lazy)

    def set_positions_and_lookat(self, eye_k3, target_k3, lazy: bool = False) -> None:
        eye_k3 = self._ensure_kx3(eye_k3, 'eye_k3')
        target_k3 = self._ensure_kx3(target_k3, 'target_k3')
        fwd = self._fwd_from_lookat(target_k3, eye_k3)
        self._update_view(eye_k3=eye_k3, forward_k3=fwd, vp=not lazy)

    def _fwd_from_lookat(self, target_k3, eye_k3=None) -> torch.Tensor:
        eye = eye_k3 if eye_k3 is not None else self.eye_k3
        target = self._ensure_kx3(target_k3, 'target_k3')
        eye = self._ensure_kx3(eye, 'eye_k3')
        return target - eye

    def set_hprs(self, hpr_k3, lazy: bool = False) -> None:
        hpr = self._ensure_kx3(hpr_k3, 'hpr_k3')
        fwd, up = self._fwd_up_from_hpr(hpr)
        self._update_view(forward_k3=fwd, up_k3=up, vp=not lazy)

    def set_eye(self, eye_k3, lazy: bool = False) -> None:
        self._update_view(eye_k3=eye_k3, vp=not lazy)

    def set_forward(self, forward_k3, lazy: bool = False) -> None:
        self._update_view(forward_k3=forward_k3, vp=not lazy)

    def set_up(self, up_k3, lazy: bool = False) -> None:
        self._update_view(up_k3=up_k3, vp=not lazy)

    def set_right(self, right_k3, lazy: bool = False) -> None:
        right_k3 = type(self)._normalize(torch.as_tensor(right_k3, dtype=torch.float32).to(self.device))
        f = -self.V_k44[:, 2, 0:3]
        u = torch.cross(right_k3.expand_as(f), f, dim=-1)
        self._update_view(forward_k3=f, up_k3=u, vp=not lazy)

    def start_tasks(self, taskMgr=None, name: str = "pbr_cam_update") -> None:
        """``camera.py:404-420`` registers a per-frame task that re-uploads the
        view-projection and the screen size.  Here every setter writes
        ``VP_k44`` in place, which the kernels read at each launch, and there is
        no Panda3D base camera to follow: nothing to schedule."""
        return None

    def get_eye(self) -> torch.Tensor:
        return self.eye_k3.clone()

    def get_forward(self) -> torch.Tensor:
        return (-self.V_k44[:, 2, 0:3]).clone()

    def get_up(self) -> torch.Tensor:
        return self.V_k44[:, 1, 0:3].clone()

    def get_right(self) -> torch.Tensor:
        return self.V_k44[:, 0, 0:3].clone()

    # compatibility no-ops (the reference's shader-input broadcast)
    def attach(self, node) -> None:
        return None

    def attach_many(self, nodes) -> None:
        return None

    def attach_all(self) -> None:
        return None

    def enable_base_cam_sync(self) -> None:
        raise NotImplementedError("there is no Panda3D base camera to follow")

    def disable_base_cam_sync(self) -> None:
        self.sync_from_base_cam = False

    def _register_self(self) -> None:
        self.base._pbr_cam = self
