"""Steering renderer (``envs/steering/renderer.py:20-271``): a player box,
two lane rails and a row of obstacle spheres per scene; the camera follows
the player.  The per-step state is device-resident (no host round trip)."""
from __future__ import annotations

import torch

from ...renderer.renderer import PBRRenderer
from .config import SteeringConfig


class SteeringRenderer(PBRRenderer):
    """Nodes: player (box), left / right rail (cylinder), obstacle spheres
    (built per reset by :meth:`build_obstacles`, which also runs
    ``setup_environment`` the first time, ``renderer.py:146-220``)."""

    def __init__(self, cfg: SteeringConfig | dict | None = None):
        super().__init__(cfg)
        c = self.cfg
        N = int(c.num_scenes)
        dev = self.state_device
        self._color_player = torch.tensor(c.player_color, dtype=torch.float32, device=dev)
        self._color_red = torch.tensor(c.red_obstacle_color, dtype=torch.float32, device=dev)
        self._color_gold = torch.tensor(c.gold_obstacle_color, dtype=torch.float32, device=dev)
        self._color_border = torch.tensor(c.edge_color, dtype=torch.float32, device=dev)
        self._color_crash = torch.tensor(getattr(c, "crash_player_color", c.player_color), dtype=torch.float32,
                                         device=dev)
        bg = c.background_color
        self.set_background_color(float(bg[0]), float(bg[1]), float(bg[2]), float(bg[3]))
        self.sphere_node = None
        self.cone_node = None
        self._setup_called = False
        self._camera_eye_offset = torch.tensor(c.camera_eye_offset, dtype=torch.float32).reshape(1, 3)

        self.player_node = self.add_node(c.player_model, instances_per_scene=1, model_scale=c.player_dimensions,
                                         model_hpr=c.player_model_hpr, model_scale_units="absolute",
                                         model_pivot_relative_point=c.player_pivot_relative_point,
                                         shared_across_scenes=False)
        self.player_node.set_colors(self._color_player.reshape(1, 4).expand(N, 4))

        self.left_border = self.add_node(c.border_model, instances_per_scene=1, model_scale=c.rail_dimensions,
                                         model_hpr=c.border_model_hpr, model_scale_units="absolute",
                                         shared_across_scenes=False)
        self.right_border = self.add_node(c.border_model, instances_per_scene=1, model_scale=c.rail_dimensions,
                                          model_hpr=c.border_model_hpr, model_scale_units="absolute",
                                          shared_across_scenes=False)
        half = float(c.lane_width) * 0.5
        z_off = float(c.rail_offset[2])
        for node, x in ((self.left_border, -half), (self.right_border, half)):
            node.set_positions(torch.tensor([x, 0.0, z_off]).reshape(1, 3).expand(N, 3))
            node.set_colors(self._color_border.reshape(1, 4).expand(N, 4))

        self.add_camera(z_far=float(c.z_far), z_near=float(c.z_near), fov_y_deg=float(c.fov_y_deg))
        self.add_light(ambient=c.ambient_light, dir_dir=c.directional_light_dir)
        # setup_environment() runs in build_obstacles(), after the obstacle nodes exist

    def build_obstacles(self, obstacles: torch.Tensor | None) -> None:
        """``obstacles [B, n, 4]`` (x, y, gold flag, cone flag): replace the
        obstacle spheres (red, gold where flagged) at (x, y, 0)."""
        for attr in ("sphere_node", "cone_node"):
            node = getattr(self, attr)
            if node is not None:
                self.remove_node(node)
            setattr(self, attr, None)
        if obstacles is not None and obstacles.numel() > 0:
            c = self.cfg
            B, n = int(obstacles.shape[0]), int(obstacles.shape[1])
            ob = obstacles.detach().to(self.state_device)
            pos = torch.zeros((B, n, 3), dtype=torch.float32, device=self.state_device)
            pos[:, :, 0] = ob[:, :, 0]
            pos[:, :, 1] = ob[:, :, 1]
            gold = (ob[:, :, 2] >= 0.5).unsqueeze(-1)
            colors = torch.where(gold, self._color_gold, self._color_red)
            self.sphere_node = self.add_node(c.obstacle_sphere_model, instances_per_scene=n,
                                             model_scale=c.obstacle_dimensions, model_hpr=c.obstacle_model_hpr,
                                             model_scale_units="absolute",
                                             model_pivot_relative_point=c.obstacle_pivot_relative_point,
                                             shared_across_scenes=False)
            self.sphere_node.set_positions(pos)
            self.sphere_node.set_colors(colors)
        if not self._setup_called:
            self.setup_environment()
            self._setup_called = True

    def _step(self, state_batch: torch.Tensor | None = None) -> None:
        """``state [B, obs]``: player x, y, speed, grace flag, ...; pads or
        truncates to N scenes (``renderer.py:222-271``)."""
        if state_batch is None:
            return
        N = int(self.cfg.num_scenes)
        s = torch.as_tensor(state_batch, dtype=torch.float32).detach()
        if s.device != self.state_device:
            s = s.to(self.state_device, non_blocking=True)
        B = int(s.shape[0])
        if B != N:
            s = torch.cat([s, s[-1:].expand(N - B, -1)], dim=0) if B < N else s[:N]
        x, y = s[:, 0], s[:, 1]
        grace = s[:, 3] if s.shape[1] > 3 else torch.zeros_like(x)
        self.player_node.pos[:, 0].copy_(x)
        self.player_node.pos[:, 1].copy_(y)
        self.player_node.color.copy_(torch.where((grace > 0.5).unsqueeze(-1), self._color_crash, self._color_player))
        self.left_border.pos[:, 1].copy_(y)
        self.right_border.pos[:, 1].copy_(y)
        if self._pbr_cam is not None:
            eye = self.player_node.pos + self._camera_eye_offset.to(self.player_node.pos.device)
            self._pbr_cam.set_positions(eye)
