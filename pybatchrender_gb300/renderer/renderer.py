"""``PBRRenderer``: the reference's renderer API (``renderer/renderer.py``)
on top of the sm_103a kernels in ``libpbr.so``.

The reference subclasses Panda3D's ShowBase, draws one instanced GL call per
node into a ``cols x rows`` atlas and reads it back into ``[N,C,H,W]``
(``renderer.py:326-363``).  Here the scene state is device tensors, and
``step()`` runs the subclass hook ``_step`` then one kernel launch that writes
the final ``[N,C,H,W]`` uint8 pixels.  Two raster methods:

* ``raster_method='batched'`` (default): one fused launch for all nodes,
  matrices built on the device, optionally captured with ``_step`` into a
  CUDA graph (``cuda_graph=True``).
* ``raster_method='plain'``: the reference's per-step flow -- per node, host
  (CPU torch) matrix building, a host-to-device copy and one launch into a
  depth/colour buffer, then a resolve launch and a synchronisation.

There is no CPU fallback: on a machine without a CUDA device the scene API
works (it is plain tensor bookkeeping) but rendering raises
:class:`RendererUnavailable`.
"""
from __future__ import annotations

import ctypes
import math
from collections.abc import Sequence
from typing import Literal

import numpy as np
import torch

from .. import _capi
from .._capi import RendererUnavailable
from ..config import PBRConfig
from .camera import PBRCam
from .light import PBRLight
from .node import MODE_MAT, PBRNode, mesh_key


KERNELS = {"auto": 0, "warp": 1, "tile": 2, "binned": 3}


class PBRRenderer:
    """Batch renderer for ``num_scenes`` independent scenes."""

    def __init__(self, cfg: PBRConfig | dict | None = None, **cfg_overrides):
        self.cfg = PBRConfig.from_config(cfg, **cfg_overrides)
        self.num_scenes = int(self.cfg.num_scenes)
        self.device = torch.device(self.cfg.device)
        if self.device.type == "cuda" and self.device.index is None:
            self.device = torch.device("cuda", torch.cuda.current_device())
        # the plain method keeps per-instance state on the host like the reference
        self.state_device = torch.device("cpu") if self.cfg.raster_method == "plain" else self.device
        self._pbr_nodes: list[PBRNode] = []
        self._pbr_cam: PBRCam | None = None
        self._pbr_light: PBRLight | None = None
        self._background_color = (0.0, 0.0, 0.0, 1.0)
        self._fps_text = None
        self._ctx = None
        self._lib = None
        self._unavailable: str | None = None
        self._graph = None
        self._static_out = None
        self._static_depth = None
        self._plain_staging: dict = {}
        self.autotune_result = None
        self._state_bindings: list[tuple[PBRNode, int, int]] = []
        # keyboard state of the manual camera control (renderer.py:162-222); no window here, so the keys are
        # set through set_key and update_camera applies them
        self.keys = {"w": False, "s": False, "a": False, "d": False, "z": False, "x": False}
        self._camera_speed = 25.0
        self._last_camera_update: float | None = None

    # ------------------------------------------------------------- scene API
    def set_background_color(self, r: float, g: float, b: float, a: float = 1.0) -> None:
        self._background_color = (float(r), float(g), float(b), float(a))
        if self._ctx is not None:
            _capi.call(self._lib, self._ctx, "pbr_background_set", (ctypes.c_float * 4)(*self._background_color))
            self._graph = None

    def add_node(self,
                 model_path,
                 instances_per_scene: int,
                 texture=None,
                 model_pivot_relative_point: tuple[float, float, float] | None = None,
                 model_scale: float | Sequence[float] | None = None,
                 model_hpr: tuple[float, float, float] | None = None,
                 model_scale_units: Literal["relative", "absolute"] = "relative",
                 positions: "torch.Tensor | None" = None,
                 hprs: "torch.Tensor | None" = None,
                 scales: "torch.Tensor | None" = None,
                 colors: "torch.Tensor | None" = None,
                 backend: Literal["loop", "instanced"] = "instanced",
                 shared_across_scenes: bool = False,
                 parent: "PBRNode | None" = None,
                 name: str | None = None) -> PBRNode:
        node = PBRNode(self, model_path=model_path, num_scenes=self.num_scenes,
                       instances_per_scene=int(instances_per_scene), texture=texture,
                       model_pivot_relative_point=model_pivot_relative_point, model_scale=model_scale,
                       model_hpr=model_hpr, model_scale_units=model_scale_units, positions=positions,
                       hprs=hprs, scales=scales, colors=colors, backend=backend,
                       shared_across_scenes=shared_across_scenes, parent=parent, name=name)
        if self._ctx is not None:
            self._build_context()
        return node

    def remove_node(self, node: PBRNode) -> None:
        """Remove a node from the scene (Panda3D's ``NodePath.removeNode`` in
        the reference, e.g. ``envs/steering/renderer.py:171-179`` when the
        obstacles are rebuilt).  Its state bindings go with it."""
        if node in self._pbr_nodes:
            self._pbr_nodes.remove(node)
        self._state_bindings = [b for b in self._state_bindings if b[0] is not node]
        self._graph = None
        if self._ctx is not None:
            self._build_context()

    # ------------------------------------------------------ manual camera control
    def set_key(self, key, value) -> None:
        """``renderer.py:162-163``."""
        self.keys[key] = value

    def enable_camera_control(self) -> None:
        """``renderer.py:165-197``: there is no window to take keyboard and mouse
        input from, which is the reference's offscreen case: warn and switch
        the option off."""
        print('WARNING: Manual camera control is not possible in offscreen mode, disabling.')
        self.cfg.manual_camera_control = False

    def update_camera(self, task=None, dt: float | None = None):
        """Keyboard part of ``renderer.py:199-222``: move every scene's eye by
        ``25 * dt`` along +y (w), -y (s), -x (a), +x (d), +z (z), -z (x).  ``dt``
        defaults to the time since the previous call.  There is no mouse."""
        import time
        now = time.perf_counter()
        if dt is None:
            dt = 0.0 if self._last_camera_update is None else now - self._last_camera_update
        self._last_camera_update = now
        if self._pbr_cam is not None:
            eye = self._pbr_cam.get_eye().reshape(-1, 3).clone()
            step = self._camera_speed * float(dt)
            for key, axis, sign in (("w", 1, 1.0), ("s", 1, -1.0), ("a", 0, -1.0), ("d", 0, 1.0), ("z", 2, 1.0),
                                    ("x", 2, -1.0)):
                if self.keys.get(key):
                    eye[:, axis] += sign * step
            self._pbr_cam.set_eye(eye)
        return getattr(task, "cont", None)

    def add_camera(self, fov_y_deg: float = 55.0, z_near: float = 0.05, z_far: float = 100.0,
                   fixed_projection: bool = True) -> PBRCam:
        self._pbr_cam = PBRCam(self, num_scenes=self.cfg.num_scenes, cols=self.cfg.tiles[0], rows=self.cfg.tiles[1],
                               fov_y_deg=fov_y_deg, z_near=z_near, z_far=z_far, fixed_projection=fixed_projection)
        if self._ctx is not None:
            self._camera_changed(self._pbr_cam)
        return self._pbr_cam

    def _set_tiles_auto(self) -> None:
        if self._pbr_cam is None:
            self.add_camera()
        self._pbr_cam._set_tiles()

    def add_light(self, ambient: tuple[float, float, float] = (0.2, 0.2, 0.25),
                  dir_dir: tuple[float, float, float] = (0.4, -0.6, -0.7),
                  dir_col: tuple[float, float, float] = (1.0, 1.0, 1.0),
                  strength: float = 1.0) -> PBRLight:
        self._pbr_light = PBRLight(self, ambient=ambient, dir_dir=dir_dir, dir_col=dir_col, strength=strength)
        return self._pbr_light

    def setup_environment(self) -> None:
        """Finish scene construction (``renderer.py:400-406``): add a default
        camera if none, create the CUDA context, bind every buffer and, with
        ``cfg.autotune``, pick the fastest launch configuration."""
        if self._pbr_cam is None:
            self.add_camera()
        if self.device.type != "cuda":
            self._unavailable = f"the renderer needs a CUDA device (cfg.device={self.cfg.device!r})"
            return
        self._build_context()
        if self.cfg.autotune and self.cfg.raster_method == "batched" and self.cfg.raster_mode == "hard":
            self.autotune()

    # ----------------------------------------------------------- state binding
    POSE_COMPONENTS = {"x": 0, "y": 1, "z": 2, "h": 3, "p": 4, "r": 5}

    def bind_state(self, node: PBRNode, component, column: int) -> None:
        """Declare that pose ``component`` of ``node`` (``"x"``, ``"y"``,
        ``"z"`` position or ``"h"``, ``"p"``, ``"r"`` HPR angle in radians;
        or 0..5) equals column ``column`` of the state passed to ``step``.

        When every argument of ``step`` is a single CUDA float32 ``[N, S]``
        state (one row per scene; row ``k * instances_per_scene + i`` for
        nodes with several instances), the bound components are read by the
        raster launch itself and written back into the node's tensors, and
        ``_step`` is not called: the env step is one kernel launch.  Any other
        argument falls back to ``_step`` + render, so ``_step`` must still
        perform the same copies."""
        comp = self.POSE_COMPONENTS[component] if isinstance(component, str) else int(component)
        if not 0 <= comp <= 5:
            raise ValueError("component must be x, y, z, h, p, r or 0..5")
        if column < 0:
            raise ValueError("column must be >= 0")
        if comp >= 3 and node.mode != _capi.MODE_HPR:
            raise ValueError("angle bindings need a node in HPR mode")
        self._state_bindings = [b for b in self._state_bindings if not (b[0] is node and b[1] == comp)]
        self._state_bindings.append((node, comp, int(column)))
        self._graph = None
        if self._ctx is not None and node in self._node_ids:
            _capi.call(self._lib, self._ctx, "pbr_node_bind_state", self._node_ids[node], comp, int(column))

    def _bound_state(self, args, kwargs):
        """The state tensor of a step that can take the fused path, else None."""
        if not self._state_bindings or kwargs or len(args) != 1 or self._ctx is None:
            return None
        s = args[0]
        if not (torch.is_tensor(s) and s.device == self.device and s.dtype == torch.float32 and s.dim() == 2
                and s.stride(1) == 1 and s.shape[0] == self.num_scenes and not s.requires_grad):
            return None
        if max(col for _, _, col in self._state_bindings) >= s.shape[1]:
            return None
        for node, comp, _ in self._state_bindings:
            if node.shared_across or node.instances_per_scene != 1 or node.mode == _capi.MODE_MAT \
                    or (comp >= 3 and node.mode != _capi.MODE_HPR):
                return None
        return s

    def _render_state(self, state: torch.Tensor):
        N, C, H, W = self._out_shape()
        want_depth = self.cfg.return_depth
        if self.cfg.reuse_output or self.cfg.cuda_graph:
            if self._static_out is None:
                self._static_out = torch.empty((N, C, H, W), dtype=torch.uint8, device=self.device)
            if want_depth and self._static_depth is None:
                self._static_depth = torch.empty((N, H, W), dtype=torch.float32, device=self.device)
            out, depth = self._static_out, (self._static_depth if want_depth else None)
        else:
            out = torch.empty((N, C, H, W), dtype=torch.uint8, device=self.device)
            depth = torch.empty((N, H, W), dtype=torch.float32, device=self.device) if want_depth else None
        _capi.call(self._lib, self._ctx, "pbr_render_state", _capi.ptr(state), int(state.shape[0]),
                   int(state.shape[1]), int(state.stride(0)), _capi.ptr(out), _capi.ptr(depth), None, self._stream())
        return (out, depth) if want_depth else out

    # ---------------------------------------------------------------- stepping
    def _step(self, *args, **kwargs):
        """Subclass hook: write the scene state for this step (default no-op)."""
        return None

    def _interactive_step(self):
        return None

    def step(self, *args, return_pixels: bool = True, **kwargs):
        """Run ``_step(*args, **kwargs)`` then render; returns uint8
        ``[N,C,H,W]`` on the CUDA device (plus float32 ``[N,H,W]`` depth when
        ``cfg.return_depth``), ``None`` when ``return_pixels`` is False
        (``renderer.py:377-390``)."""
        if self.cfg.report_fps:
            self.report_fps()
        fused = return_pixels and not self.cfg.interactive and self.cfg.raster_method == "batched" \
            and self.cfg.raster_mode == "hard"
        if fused:
            state = self._bound_state(args, kwargs)
            if state is not None:
                return self._render_state(state)
        if self.cfg.cuda_graph and fused:
            return self._graph_step(args, kwargs)
        if not getattr(self.cfg, "interactive", False):
            self._step(*args, **kwargs)
        if return_pixels:
            if self.cfg.raster_mode == "soft":
                return self.render_soft()
            return self.render()
        return None

    def __call__(self, *args, return_pixels: bool = True, **kwargs):
        return self.step(*args, return_pixels=return_pixels, **kwargs)

    # --------------------------------------------------------------- rendering
    def _require_ready(self) -> None:
        if self._ctx is None:
            if self._unavailable:
                raise RendererUnavailable(self._unavailable)
            raise RuntimeError("setup_environment() must be called before rendering")

    def _stream(self) -> int:
        return torch.cuda.current_stream(self.device).cuda_stream

    def _out_shape(self) -> tuple[int, int, int, int]:
        W, H = self.cfg.tile_resolution
        return (self.num_scenes, int(self.cfg.num_channels), int(H), int(W))

    def render(self, return_depth: bool | None = None, return_winner: bool = False):
        """Render the current scene state (no ``_step``)."""
        self._require_ready()
        want_depth = self.cfg.return_depth if return_depth is None else bool(return_depth)
        if self.cfg.raster_method == "plain":
            out, depth = self._render_plain(want_depth)
            return (out, depth) if want_depth else out
        N, C, H, W = self._out_shape()
        if self.cfg.reuse_output:
            if self._static_out is None:
                self._static_out = torch.empty((N, C, H, W), dtype=torch.uint8, device=self.device)
            out = self._static_out
            if want_depth and self._static_depth is None:
                self._static_depth = torch.empty((N, H, W), dtype=torch.float32, device=self.device)
            depth = self._static_depth if want_depth else None
        else:
            out = torch.empty((N, C, H, W), dtype=torch.uint8, device=self.device)
            depth = torch.empty((N, H, W), dtype=torch.float32, device=self.device) if want_depth else None
        winner = torch.empty((N, H, W), dtype=torch.int32, device=self.device) if return_winner else None
        _capi.call(self._lib, self._ctx, "pbr_render", _capi.ptr(out), _capi.ptr(depth), _capi.ptr(winner),
                   self._stream())
        res = [out]
        if want_depth:
            res.append(depth)
        if return_winner:
            res.append(winner)
        return res[0] if len(res) == 1 else tuple(res)

    # ------------------------------------------------------------ soft mode
    def render_soft(self, light_dir: torch.Tensor | None = None) -> torch.Tensor:
        """Soft-coverage render, float32 ``[N,3,H,W]``.  Differentiable when
        autograd is enabled and a node tensor (``pos``, ``hpr``, ``scale``,
        ``color``) or ``light_dir`` requires grad."""
        from .soft import soft_params, soft_render
        if any(n.texture is not None for n in self.geometry_nodes()):
            raise NotImplementedError("textured nodes are drawn by the hard raster modes only (soft mode: untextured)")
        self._require_ready()
        params = soft_params(self)
        if torch.is_grad_enabled() and (any(p.requires_grad for p in params)
                                        or (light_dir is not None and light_dir.requires_grad)):
            return soft_render(self, light_dir)
        out, _ = self._soft_forward(light_dir, want_stats=False)
        return out

    def _soft_forward(self, light_dir: torch.Tensor | None, want_stats: bool = True):
        if light_dir is not None:
            self._set_light_direction(light_dir)
        N, C, H, W = self._out_shape()
        out = torch.empty((N, 3, H, W), dtype=torch.float32, device=self.device)
        # per pixel: float4 (m, softmax sum, coverage code, dl0) for all pixels, then float2 (dl1, dl2)
        stats = torch.empty((6 * N * H * W,), dtype=torch.float32, device=self.device) if want_stats else None
        _capi.call(self._lib, self._ctx, "pbr_render_soft", _capi.ptr(out), _capi.ptr(stats), self._stream())
        return out, stats

    def _soft_backward(self, out: torch.Tensor, stats: torch.Tensor, gout: torch.Tensor):
        """Run the adjoint kernel; returns ([(gpos, ghpr, gscale, gcol) per
        node], dL/d normalised light direction)."""
        grads = []
        for node, nid in self._node_ids.items():
            B = node.buf_instances
            g = (torch.zeros((B, 3), dtype=torch.float32, device=self.device),
                 torch.zeros((B, 3), dtype=torch.float32, device=self.device),
                 torch.zeros((B,), dtype=torch.float32, device=self.device),
                 torch.zeros((B, 4), dtype=torch.float32, device=self.device))
            _capi.call(self._lib, self._ctx, "pbr_node_set_grads", nid, *[_capi.ptr(t) for t in g])
            grads.append(g)
        g_light = torch.zeros(3, dtype=torch.float32, device=self.device)
        try:
            _capi.call(self._lib, self._ctx, "pbr_backward_soft", _capi.ptr(out), _capi.ptr(stats), _capi.ptr(gout),
                       _capi.ptr(g_light), self._stream())
        finally:
            for nid in self._node_ids.values():
                _capi.call(self._lib, self._ctx, "pbr_node_set_grads", nid, None, None, None, None)
        return grads, g_light

    def _set_light_direction(self, light_dir: torch.Tensor) -> None:
        d = [float(v) for v in torch.as_tensor(light_dir).detach().cpu().reshape(3).tolist()]
        if self._pbr_light is None:
            self.add_light()
        light = self._pbr_light
        if tuple(d) != tuple(light.dir_dir):
            light.set_directional(d, light.dir_col)

    def _render_plain(self, want_depth: bool):
        """The reference's per-step flow on the GPU: per node, host matrices
        (``node.py:116-126``) -> host-to-device copy -> one draw launch; then
        a resolve launch and a blocking synchronisation (the readback of
        ``renderer.py:326-350``)."""
        N, C, H, W = self._out_shape()
        stream = self._stream()
        out = torch.empty((N, C, H, W), dtype=torch.uint8, device=self.device)
        depth = torch.empty((N, H, W), dtype=torch.float32, device=self.device) if want_depth else None
        _capi.call(self._lib, self._ctx, "pbr_plain_clear", stream)
        for node, nid in self._node_ids.items():
            mats_d, col_d = self._plain_staging[nid]
            mats_d.copy_(node.get_transforms().reshape(-1, 16))
            col_d.copy_(node.color)
            _capi.call(self._lib, self._ctx, "pbr_plain_draw", nid, stream)
        _capi.call(self._lib, self._ctx, "pbr_plain_resolve", _capi.ptr(out), _capi.ptr(depth), stream)
        torch.cuda.synchronize(self.device)
        return out, depth

    def _graph_step(self, args, kwargs):
        sig = tuple((tuple(a.shape), a.dtype) if torch.is_tensor(a) else ("v", a) for a in args)
        if self._graph is None or self._graph_sig != sig:
            self._graph = None
            static = [a.detach().to(self.device).clone() if torch.is_tensor(a) else a for a in args]
            N, C, H, W = self._out_shape()
            self._static_out = torch.empty((N, C, H, W), dtype=torch.uint8, device=self.device)
            self._static_depth = torch.empty((N, H, W), dtype=torch.float32, device=self.device) \
                if self.cfg.return_depth else None
            side = torch.cuda.Stream(self.device)
            side.wait_stream(torch.cuda.current_stream(self.device))
            with torch.cuda.stream(side):
                for _ in range(2):
                    self._step(*static, **kwargs)
                    self._launch_static()
            torch.cuda.current_stream(self.device).wait_stream(side)
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                self._step(*static, **kwargs)
                self._launch_static()
            self._graph, self._graph_sig, self._graph_static = g, sig, static
        else:
            for dst, src in zip(self._graph_static, args):
                if torch.is_tensor(dst):
                    dst.copy_(src, non_blocking=True)
        self._graph.replay()
        return (self._static_out, self._static_depth) if self.cfg.return_depth else self._static_out

    def _launch_static(self) -> None:
        _capi.call(self._lib, self._ctx, "pbr_render", _capi.ptr(self._static_out), _capi.ptr(self._static_depth),
                   None, self._stream())

    def autotune(self) -> dict:
        """Time the launch configurations (threads, bin size, chunk size,
        persistent schedule) on the current scene and keep the fastest."""
        self._require_ready()
        N, C, H, W = self._out_shape()
        scratch = torch.empty((N, C, H, W), dtype=torch.uint8, device=self.device)
        vals = [ctypes.c_int() for _ in range(5)]
        ms = ctypes.c_float()
        _capi.call(self._lib, self._ctx, "pbr_autotune", _capi.ptr(scratch), self._stream(),
                   *[ctypes.byref(v) for v in vals], ctypes.byref(ms))
        names = {v: k for k, v in KERNELS.items()}
        self.autotune_result = {"kernel": names[vals[0].value], "threads": vals[1].value, "bin_px": vals[2].value,
                                "tri_cap": vals[3].value, "persistent": vals[4].value, "ms": ms.value}
        c = self.cfg
        c.raster_kernel, c.raster_threads, c.bin_size = names[vals[0].value], vals[1].value, vals[2].value
        c.tri_cap, c.persistent = vals[3].value, bool(vals[4].value)
        self._graph = None
        return self.autotune_result

    def debug_transforms(self, node: PBRNode) -> torch.Tensor:
        """(B,4,4) model matrices as the kernels build them (for tests)."""
        self._require_ready()
        nid = self._node_ids[node]
        out = torch.empty((node.buf_instances, 16), dtype=torch.float32, device=self.device)
        _capi.call(self._lib, self._ctx, "pbr_debug_transforms", nid, _capi.ptr(out), self._stream())
        return out.reshape(-1, 4, 4)

    # ----------------------------------------------------------- atlas views
    def to_atlas(self, pixels: torch.Tensor) -> torch.Tensor:
        """Arrange ``[N,C,H,W]`` images into the reference's atlas
        ``[rows*H, cols*W, C]`` (row 0 at the top): the inverse of
        ``_rearrange_img``."""
        cols, rows = self.cfg.tiles
        N, C, H, W = pixels.shape
        full = torch.zeros((rows * cols, C, H, W), dtype=pixels.dtype, device=pixels.device)
        full[:N] = pixels
        return full.view(rows, cols, C, H, W).permute(0, 3, 1, 4, 2).reshape(rows * H, cols * W, C)

    def grab_pixels(self) -> torch.Tensor:
        """Atlas image of the current state, ``[H_win, W_win, C]`` uint8."""
        return self.to_atlas(self.render(return_depth=False))

    def _rearrange_img(self, img: torch.Tensor) -> torch.Tensor:
        """Atlas ``[H_win, W_win, C]`` -> ``[N,C,H,W]`` (``renderer.py:352-363``)."""
        img = img.permute(2, 0, 1)
        img = img.reshape(self.cfg.num_channels, self.cfg.tiles[1], self.cfg.tile_resolution[1],
                          self.cfg.tiles[0], self.cfg.tile_resolution[0])
        img = img.permute(1, 3, 0, 2, 4)
        img = img.reshape(-1, self.cfg.num_channels, self.cfg.tile_resolution[1], self.cfg.tile_resolution[0])
        return img[:self.cfg.num_scenes]

    # ------------------------------------------------------------ export
    def geometry_nodes(self) -> list[PBRNode]:
        return [n for n in self._pbr_nodes if n.has_geometry and n.instances_per_scene > 0]

    def export_scene(self) -> tuple[dict, list, list]:
        """Host copy of the whole scene in the oracle's format:
        ``(scene, meshes, nodes)``."""
        if self._pbr_cam is None:
            self.add_camera()
        cam = self._pbr_cam
        W, H = self.cfg.tile_resolution
        light = self._pbr_light
        scene = {
            "N": self.num_scenes, "W": int(W), "H": int(H), "C": int(self.cfg.num_channels),
            "vp": cam.VP_k44.detach().cpu().numpy().reshape(-1, 16),
            "ambient": light.ambient if light else (0.0, 0.0, 0.0),
            "ldir": light.dir_dir if light else (0.0, 0.0, 1.0),
            "lcol": light.dir_col if light else (0.0, 0.0, 0.0),
            "strength": min(max(light.strength, 0.0), 1.0) if light else 0.0,
            "bg": self._background_color, "cull": 1,
            "znear": cam.z_near, "zfar": cam.z_far,
            "sigma": self.cfg.soft_sigma, "gamma": self.cfg.soft_gamma,
        }
        meshes, keys, nodes = [], {}, []
        for node in self.geometry_nodes():
            key = mesh_key(node.mesh)
            if key not in keys:
                keys[key] = len(meshes)
                meshes.append(node.mesh)
            d = node.export()
            d["mesh"] = keys[key]
            nodes.append(d)
        return scene, meshes, nodes

    # -------------------------------------------------------- context plumbing
    def _build_context(self) -> None:
        self.close()
        lib = _capi.load()
        ctx = ctypes.c_void_p()
        W, H = self.cfg.tile_resolution
        with torch.cuda.device(self.device):
            rc = lib.pbr_create(ctypes.byref(ctx), self.num_scenes, int(W), int(H), int(self.cfg.num_channels), 0)
            if rc != 0:
                raise _capi.PBRError("pbr_create", rc, lib.pbr_last_error(None).decode())
            self._lib, self._ctx = lib, ctx
            self._mesh_tensors = []
            self._node_ids: dict[PBRNode, int] = {}
            mesh_ids: dict[bytes, int] = {}
            for node in self.geometry_nodes():
                key = mesh_key(node.mesh)
                if key not in mesh_ids:
                    m = node.mesh
                    pos = torch.from_numpy(m.positions).to(self.device)
                    nrm = torch.from_numpy(m.normals).to(self.device)
                    idx = torch.from_numpy(m.indices).to(self.device)
                    self._mesh_tensors.append((pos, nrm, idx))
                    mid = ctypes.c_int()
                    _capi.call(lib, ctx, "pbr_mesh_register", _capi.ptr(pos), _capi.ptr(nrm), _capi.ptr(idx),
                               m.num_vertices, m.num_triangles, int(m.smooth), ctypes.byref(mid))
                    c, rad = m.bounding_sphere()
                    _capi.call(lib, ctx, "pbr_mesh_set_bounds", mid.value, *c, rad)
                    if self.cfg.cluster_cull and m.num_triangles >= 128:
                        cl = torch.from_numpy(m.clusters()).to(self.device)
                        self._mesh_tensors.append((cl,))
                        _capi.call(lib, ctx, "pbr_mesh_set_clusters", mid.value, _capi.ptr(cl), int(cl.shape[0]),
                                   m.CLUSTER_TRIANGLES)
                    if m.uvs is not None:
                        uv = torch.from_numpy(m.uvs).to(self.device)
                        self._mesh_tensors.append((uv,))
                        _capi.call(lib, ctx, "pbr_mesh_set_uv", mid.value, _capi.ptr(uv))
                    mesh_ids[key] = mid.value
                nid = ctypes.c_int()
                _capi.call(lib, ctx, "pbr_node_add", mesh_ids[key], node.instances_per_scene,
                           int(node.shared_across), ctypes.byref(nid))
                self._node_ids[node] = nid.value
                self._bind_node_buffers(node)
                self._bind_node_texture(node)
            for node, comp, col in self._state_bindings:
                if node in self._node_ids:
                    _capi.call(lib, ctx, "pbr_node_bind_state", self._node_ids[node], comp, col)
            self._camera_changed(self._pbr_cam)
            self._light_changed(self._pbr_light)
            _capi.call(lib, ctx, "pbr_background_set", (ctypes.c_float * 4)(*self._background_color))
            _capi.call(lib, ctx, "pbr_raster_config", KERNELS[self.cfg.raster_kernel], int(self.cfg.raster_threads),
                       int(self.cfg.bin_size), int(self.cfg.tri_cap), int(bool(self.cfg.persistent)))
            _capi.call(lib, ctx, "pbr_tile_pretest", {"auto": -1, "off": 0, "on": 1}[self.cfg.tile_pretest])
            _capi.call(lib, ctx, "pbr_soft_config", float(self.cfg.soft_sigma), float(self.cfg.soft_gamma),
                       128 if int(self.cfg.raster_threads) == 128 else 256)

    def _bind_node_buffers(self, node: PBRNode) -> None:
        nid = self._node_ids[node]
        counts = node.counts
        if counts is not None and counts.device != self.device:
            counts = counts.to(self.device)
            self._counts_dev = getattr(self, "_counts_dev", {})
            self._counts_dev[nid] = counts
        if self.cfg.raster_method == "plain":
            mats = torch.empty((node.buf_instances, 16), dtype=torch.float32, device=self.device)
            col = torch.empty((node.buf_instances, 4), dtype=torch.float32, device=self.device)
            self._plain_staging[nid] = (mats, col)
            _capi.call(self._lib, self._ctx, "pbr_node_set_buffers", nid, MODE_MAT, None, _capi.ptr(mats), None,
                       _capi.ptr(col), _capi.ptr(counts))
            return
        mode, pos, rot, scale, color = node.kernel_buffers()
        _capi.call(self._lib, self._ctx, "pbr_node_set_buffers", nid, mode, _capi.ptr(pos), _capi.ptr(rot),
                   _capi.ptr(scale), _capi.ptr(color), _capi.ptr(counts))

    def _bind_node_texture(self, node: PBRNode) -> None:
        nid = self._node_ids[node]
        self._tex_tensors = getattr(self, "_tex_tensors", {})
        if node.texture is None:
            self._tex_tensors.pop(nid, None)
            _capi.call(self._lib, self._ctx, "pbr_node_set_texture", nid, None, 0, 0)
            return
        tex = torch.from_numpy(node.texture).to(self.device)
        self._tex_tensors[nid] = tex
        _capi.call(self._lib, self._ctx, "pbr_node_set_texture", nid, _capi.ptr(tex), int(tex.shape[1]),
                   int(tex.shape[0]))

    def _texture_changed(self, node: PBRNode) -> None:
        if self._ctx is not None and node in getattr(self, "_node_ids", {}):
            self._bind_node_texture(node)
            self._graph = None

    def _rebind_node(self, node: PBRNode) -> None:
        if self._ctx is not None and node in getattr(self, "_node_ids", {}):
            self._bind_node_buffers(node)
            self._graph = None

    def _camera_changed(self, cam: PBRCam) -> None:
        if self._ctx is not None and cam is not None:
            _capi.call(self._lib, self._ctx, "pbr_camera_bind", _capi.ptr(cam.VP_k44), float(cam.z_near),
                       float(cam.z_far))
            self._graph = None

    def _light_changed(self, light: PBRLight | None) -> None:
        if self._ctx is None:
            return
        f3 = ctypes.c_float * 3
        if light is None:
            _capi.call(self._lib, self._ctx, "pbr_light_set", f3(0, 0, 0), f3(0, 0, 1), f3(0, 0, 0), 0.0)
        else:
            _capi.call(self._lib, self._ctx, "pbr_light_set", f3(*light.ambient), f3(*light.dir_dir),
                       f3(*light.dir_col), float(light.strength))
        self._graph = None

    def close(self) -> None:
        if self._ctx is not None:
            if torch.cuda.is_available():
                torch.cuda.synchronize(self.device)
            self._lib.pbr_destroy(self._ctx)
            self._ctx = None
            self._graph = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def report_fps(self, task=None):
        """``renderer.py:242-251``: count frames and, every
        ``cfg.report_fps_interval`` seconds, print the scene frames per second
        (steps per second times ``num_scenes``) since the previous report.
        Called by ``step`` when ``cfg.report_fps`` is set; host time, so a
        queue of launches that have not run yet counts as done."""
        import time
        now = time.perf_counter()
        if getattr(self, "_fps_t0", None) is None:
            self._fps_t0, self._fps_frames = now, 0
            return getattr(task, "cont", None)
        self._fps_frames += 1
        if now - self._fps_t0 >= float(self.cfg.report_fps_interval):
            fps = self._fps_frames * self.num_scenes / (now - self._fps_t0)
            print(f"FPS: {fps:.1f}")
            self._fps_t0, self._fps_frames = now, 0
        return getattr(task, "cont", None)
