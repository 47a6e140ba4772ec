"""Seeded synthetic scenes used by the benchmark and the parity tests.

Each builder returns a ready ``PBRRenderer`` (``setup_environment`` done) plus
a ``state(step)`` function that produces that step's inputs.  They are built
only through the public renderer API, exactly as a user's env would.

* :func:`cartpole_bench` -- the headline CartPole render: two unit cubes per
  scene (cart scaled (0.5,0.3,0.2) at x ~ U(-2.4,2.4), pole scaled
  (0.05,0.05,1.0) hinged at the cart top with pitch ~ U(-0.21,0.21)), fov 40
  camera at (0,-8,1.5) looking at the origin, directional light
  (0.3,-1,-0.5) plus ambient 0.2, seeded flat per-instance colours.
* :func:`many_cubes` -- 64 cubes per scene, positions U[-5,5]^3, HPR U[0,2pi)^3,
  scale U(0.2,1.0), colour U[0,1]^3, camera at distance 12 (fov 45).
* :func:`uneven` -- per-scene instance count log-uniform in [1, I_max], each
  instance's mesh uniform over {cube, 64-segment cylinder, icosphere level 3},
  random pose/scale/colour, per-scene camera on a sphere of radius 10-15.
"""
from __future__ import annotations

import math

import torch

from .config import PBRConfig
from .renderer.renderer import PBRRenderer


def _gen(seed: int) -> torch.Generator:
    g = torch.Generator()
    g.manual_seed(int(seed))
    return g


class CartPoleBenchRenderer(PBRRenderer):
    """Two-cube CartPole scene of the benchmark (cart + pole per scene)."""

    CART_SCALE = (0.5, 0.3, 0.2)
    POLE_SCALE = (0.05, 0.05, 1.0)

    def __init__(self, cfg: PBRConfig | dict | None = None, seed: int = 0, **overrides):
        super().__init__(cfg, **overrides)
        N = self.num_scenes
        g = _gen(seed)
        self.cart = self.add_node("models/box", 1, model_pivot_relative_point=(0.5, 0.5, 0.5),
                                  model_scale=self.CART_SCALE)
        self.pole = self.add_node("models/box", 1, model_pivot_relative_point=(0.5, 0.5, 0.0),
                                  model_scale=self.POLE_SCALE)
        self.cart_top = self.CART_SCALE[2] * 0.5
        cart_col = torch.cat([torch.rand((N, 3), generator=g) * 0.8 + 0.2, torch.ones((N, 1))], dim=1)
        pole_col = torch.cat([torch.rand((N, 3), generator=g) * 0.8 + 0.2, torch.ones((N, 1))], dim=1)
        self.cart.set_colors(cart_col)
        self.pole.set_colors(pole_col)
        self.pole.set_positions(torch.tensor([0.0, 0.0, self.cart_top]))
        self.add_camera(fov_y_deg=40.0)
        self._pbr_cam.set_positions_and_lookat(torch.tensor([0.0, -8.0, 1.5]), torch.tensor([0.0, 0.0, 0.0]))
        self.add_light(ambient=(0.2, 0.2, 0.2), dir_dir=(0.3, -1.0, -0.5))
        # the copies of _step, done inside the raster launch when step() gets a CUDA state
        self.bind_state(self.cart, "x", 0)
        self.bind_state(self.pole, "x", 0)
        self.bind_state(self.pole, "p", 2)
        self.setup_environment()

    def _step(self, state: torch.Tensor | None = None):
        """state [N,4]: x, x_dot, theta, theta_dot (CartPole observation layout)."""
        if state is None:
            return
        self.cart.pos[:, 0].copy_(state[:, 0])
        self.pole.pos[:, 0].copy_(state[:, 0])
        self.pole.hpr[:, 1].copy_(state[:, 2])


def cartpole_states(num_scenes: int, seed: int, device="cpu") -> torch.Tensor:
    """[N,4] states with x ~ U(-2.4,2.4) and theta ~ U(-0.21,0.21)."""
    g = _gen(seed)
    s = torch.zeros((num_scenes, 4))
    s[:, 0] = torch.rand(num_scenes, generator=g) * 4.8 - 2.4
    s[:, 1] = torch.randn(num_scenes, generator=g)
    s[:, 2] = torch.rand(num_scenes, generator=g) * 0.42 - 0.21
    s[:, 3] = torch.randn(num_scenes, generator=g)
    return s.to(device)


def cartpole_bench(num_scenes: int = 4096, res: int = 64, seed: int = 0, **cfg) -> CartPoleBenchRenderer:
    return CartPoleBenchRenderer(PBRConfig(num_scenes=num_scenes, tile_resolution=(res, res), report_fps=False,
                                           **cfg), seed=seed)


def _random_poses(B: int, g: torch.Generator):
    pos = torch.rand((B, 3), generator=g) * 10.0 - 5.0
    hpr = torch.rand((B, 3), generator=g) * (2 * math.pi)
    scale = torch.rand((B,), generator=g) * 0.8 + 0.2
    col = torch.cat([torch.rand((B, 3), generator=g), torch.ones((B, 1))], dim=1)
    return pos, hpr, scale, col


def many_cubes(num_scenes: int = 1024, res: int = 128, instances: int = 64, seed: int = 0, **cfg) -> PBRRenderer:
    r = PBRRenderer(PBRConfig(num_scenes=num_scenes, tile_resolution=(res, res), report_fps=False, **cfg))
    g = _gen(seed)
    node = r.add_node("models/box", instances, model_pivot_relative_point=(0.5, 0.5, 0.5))
    pos, hpr, scale, col = _random_poses(node.buf_instances, g)
    node.set_positions(pos)
    node.set_hprs(hpr)
    node.set_scales(scale)
    node.set_colors(col)
    r.add_camera(fov_y_deg=45.0)
    r._pbr_cam.set_positions_and_lookat(torch.tensor([0.0, -12.0, 0.0]), torch.tensor([0.0, 0.0, 0.0]))
    r.add_light()
    r.cubes = node
    r.setup_environment()
    return r


def uneven_counts(num_scenes: int, max_instances: int, g: torch.Generator) -> torch.Tensor:
    """round(exp(U(0, ln max))) clipped to [1, max]."""
    c = torch.exp(torch.rand(num_scenes, generator=g) * math.log(max_instances)).round()
    return c.clamp(1, max_instances).to(torch.int32)


def uneven(num_scenes: int = 4096, res: int = 84, max_instances: int = 512, seed: int = 0,
           meshes=("models/box", "cylinder:64", "icosphere:3"), **cfg) -> PBRRenderer:
    """Uneven instance counts and mixed meshes: one node per mesh kind, each
    with per-scene active counts from a multinomial split of the scene's
    log-uniform count."""
    r = PBRRenderer(PBRConfig(num_scenes=num_scenes, tile_resolution=(res, res), report_fps=False, **cfg))
    g = _gen(seed)
    total = uneven_counts(num_scenes, max_instances, g)
    kinds = torch.randint(0, len(meshes), (num_scenes, max_instances), generator=g)
    active = torch.arange(max_instances)[None, :] < total[:, None]
    r.uneven_nodes = []
    for mi, m in enumerate(meshes):
        counts = ((kinds == mi) & active).sum(dim=1).to(torch.int32)
        node = r.add_node(m, max_instances, model_pivot_relative_point=(0.5, 0.5, 0.5))
        pos, hpr, scale, col = _random_poses(node.buf_instances, g)
        node.set_positions(pos)
        node.set_hprs(hpr)
        node.set_scales(scale)
        node.set_colors(col)
        node.set_active_counts(counts)
        r.uneven_nodes.append(node)
    r.total_counts = total
    r.add_camera(fov_y_deg=45.0)
    theta = torch.rand(num_scenes, generator=g) * 2 * math.pi
    z = torch.rand(num_scenes, generator=g) * 2 - 1
    rad = torch.rand(num_scenes, generator=g) * 5 + 10
    xy = torch.sqrt(1 - z * z)
    eye = torch.stack([xy * torch.cos(theta), xy * torch.sin(theta), z], dim=1) * rad[:, None]
    r._pbr_cam.set_positions_and_lookat(eye, torch.zeros((num_scenes, 3)))
    r.add_light()
    r.setup_environment()
    return r


def soft_large(num_scenes: int = 16384, res: int = 128, instances: int = 128, seed: int = 0, **cfg) -> PBRRenderer:
    """Large soft-coverage workload: per scene ``instances`` non-shared
    instances, half icosphere-s2 (320 triangles, smooth) and half unit cubes
    (12 triangles, flat), random poses as in :func:`many_cubes`."""
    r = PBRRenderer(PBRConfig(num_scenes=num_scenes, tile_resolution=(res, res), report_fps=False,
                              raster_mode="soft", **cfg))
    g = _gen(seed)
    r.soft_nodes = []
    for m in ("icosphere:2", "models/box"):
        node = r.add_node(m, instances // 2, model_pivot_relative_point=(0.5, 0.5, 0.5))
        pos, hpr, scale, col = _random_poses(node.buf_instances, g)
        node.set_positions(pos)
        node.set_hprs(hpr)
        node.set_scales(scale)
        node.set_colors(col)
        r.soft_nodes.append(node)
    r.add_camera(fov_y_deg=45.0)
    r._pbr_cam.set_positions_and_lookat(torch.tensor([0.0, -12.0, 0.0]), torch.tensor([0.0, 0.0, 0.0]))
    r.add_light()
    r.setup_environment()
    return r
