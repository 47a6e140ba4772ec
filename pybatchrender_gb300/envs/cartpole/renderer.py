"""CartPole renderer (``envs/cartpole/renderer.py``): the same scene -- a
shared rail, a cart and a pole built from ``models/box`` with the reference's
sizes, pivots and colours, camera at (5,5,2) looking at the origin, default
light.  ``_step`` maps state ``[B,4]`` to cart x, pole x and pole pitch on the
device (no ``.cpu()`` round trip as in ``renderer.py:112`` of the reference),
padding with the last row or truncating to ``num_scenes``."""
import math

import torch

from ...config import PBRConfig
from ...renderer.renderer import PBRRenderer


class CartPoleRenderer(PBRRenderer):
    def __init__(self, cfg: PBRConfig | dict | None = None):
        super().__init__(cfg)
        instances_per_scene = 1
        self.rail_size = (6.0, 0.05, 0.05)
        self.cart_size = (1.2, 0.8, 0.5)
        self.pole_size = (0.1, 0.1, 2.0)
        self.rail_pos_color = (0.2, 0.2, 0.2, 1.0)
        self.cart_pos_color_range = ((0.6, 0.8, 1.0, 1.0), (1.0, 0.6, 0.8, 1.0))
        self.pole_pos_color = (1.0, 0.7, 0.2, 1.0)

        self.rail = self.add_node("models/box", model_pivot_relative_point=(0.5, 0.5, 0.5),
                                  model_scale=self.rail_size, instances_per_scene=instances_per_scene,
                                  shared_across_scenes=True)
        self.cart = self.add_node("models/box", model_pivot_relative_point=(0.5, 0.5, 0.5),
                                  model_scale=self.cart_size, instances_per_scene=instances_per_scene,
                                  shared_across_scenes=False)
        self.pole = self.add_node("models/box", model_pivot_relative_point=(0.5, 0.5, 0.05),
                                  model_scale=self.pole_size, instances_per_scene=instances_per_scene,
                                  shared_across_scenes=False)

        N = int(self.cfg.num_scenes)
        self.rail.set_positions(torch.zeros((1, instances_per_scene, 3)))
        self.cart.set_positions(torch.zeros((N, instances_per_scene, 3)))
        self.pole_offset_y = (self.cart_size[1] + self.pole_size[1]) * 0.5
        self.pole.set_positions(torch.tensor([0.0, self.pole_offset_y, 0.0]).repeat(N, 1))

        self.rail.set_colors(torch.tensor(self.rail_pos_color).reshape(1, 4))
        start_col = torch.tensor(self.cart_pos_color_range[0], dtype=torch.float32)
        end_col = torch.tensor(self.cart_pos_color_range[1], dtype=torch.float32)
        t = torch.linspace(0.0, 1.0, steps=N, dtype=torch.float32)
        self.cart.set_colors(start_col.unsqueeze(0) + (end_col - start_col).unsqueeze(0) * t.unsqueeze(1))
        self.pole.set_colors(torch.tensor(self.pole_pos_color).repeat(N, 1))

        pole_hpr = torch.zeros((N, 3), dtype=torch.float32)
        pole_hpr[:, 1] = math.pi * 0.5
        self.pole.set_hprs(pole_hpr)

        self.add_camera()
        self._pbr_cam.set_positions(torch.tensor([5, 5, 2], dtype=torch.float32))
        self._pbr_cam.look_at(torch.tensor([0, 0, 0], dtype=torch.float32))
        self.add_light()
        # the copies of _step, done inside the raster launch when step() gets a CUDA state
        self.bind_state(self.cart, "x", 0)
        self.bind_state(self.pole, "x", 0)
        self.bind_state(self.pole, "p", 2)
        self.setup_environment()

    def _step(self, state_batch: torch.Tensor | None = None):
        """state[:, 0] = cart x, state[:, 2] = pole angle (rad)."""
        if state_batch is None:
            return
        s = torch.as_tensor(state_batch, dtype=torch.float32)
        if s.device != self.cart.pos.device:
            s = s.to(self.cart.pos.device, non_blocking=True)
        N = int(self.cfg.num_scenes)
        B = int(s.shape[0])
        if B != N:
            s = torch.cat([s, s[-1:].expand(N - B, -1)], dim=0) if B < N else s[:N]
        x = s[:, 0]
        self.cart.pos[:, 0].copy_(x)
        self.pole.pos[:, 0].copy_(x)
        self.pole.hpr[:, 1].copy_(s[:, 2])
