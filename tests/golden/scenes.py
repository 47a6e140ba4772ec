"""Scene scripts written against the public renderer API only, so the same
code drives the reference (under the stubs of ``stub_panda3d.py``) and this
package.  Each returns the renderer and a list of (label, VP) camera snapshots.
"""
from __future__ import annotations

import math

import torch


def random_transforms(n: int, g: torch.Generator) -> torch.Tensor:
    """[n,4,4] rotation * uniform scale + translation."""
    a = torch.rand((n, 3), generator=g) * 6.0
    ch, sh, cp, sp, cr, sr = a[:, 0].cos(), a[:, 0].sin(), a[:, 1].cos(), a[:, 1].sin(), a[:, 2].cos(), a[:, 2].sin()
    R = torch.stack([ch * cp, ch * sp * sr - sh * cr, ch * sp * cr + sh * sr,
                     sh * cp, sh * sp * sr + ch * cr, sh * sp * cr - ch * sr,
                     -sp, cp * sr, cp * cr], 1).reshape(n, 3, 3)
    s = torch.rand((n, 1, 1), generator=g) + 0.5
    M = torch.zeros((n, 4, 4))
    M[:, :3, :3] = R * s
    M[:, :3, 3] = torch.rand((n, 3), generator=g) * 2 - 1
    M[:, 3, 3] = 1.0
    return M


def api_scene(pbr, num_scenes: int = 6, **cfg):
    """Three nodes exercising every node setter, then camera and light."""
    g = torch.Generator().manual_seed(11)
    N = num_scenes

    class Scene(pbr.PBRRenderer):
        def __init__(self):
            super().__init__(num_scenes=N, tile_resolution=(48, 32), **cfg)
            a = self.add_node("models/box", 1, model_pivot_relative_point=(0.5, 0.5, 0.5),
                              model_scale=(2.0, 0.5, 0.25), shared_across_scenes=True)
            b = self.add_node("models/box", 2, model_pivot_relative_point=(0.25, 0.5, 0.0), model_scale=1.5)
            c = self.add_node("models/box", 1, model_scale=0.3, model_scale_units="absolute")
            a.set_positions(torch.tensor([0.5, -1.0, 0.25]))
            a.set_colors(torch.tensor([0.9, 0.1, 0.2, 1.0]))
            b.set_positions(torch.rand((N * 2, 3), generator=g) * 4 - 2)
            b.set_hprs(torch.rand((N * 2, 3), generator=g) * 6.28)
            b.set_scales(torch.rand((N * 2,), generator=g) + 0.5)
            b.set_colors(torch.rand((N * 2, 4), generator=g))
            c.set_transforms(random_transforms(N, g))
            c.set_positions(torch.rand((N, 3), generator=g), lazy=True)
            c.set_scales(0.7)
            c.set_colors(torch.rand((N, 4), generator=g))
            self.add_camera(fov_y_deg=40.0, z_near=0.1, z_far=50.0)
            self.add_light(ambient=(0.1, 0.2, 0.3), dir_dir=(0.2, -0.5, -1.0), dir_col=(0.9, 0.8, 0.7), strength=0.75)
            self.setup_environment()
            self.nodes_abc = (a, b, c)

    r = Scene()
    cam = r._pbr_cam
    snaps = [("initial", cam.get_vp())]
    cam.set_hprs(torch.rand((N, 3), generator=g) * 2 - 1)
    snaps.append(("set_hprs", cam.get_vp()))
    eye = torch.rand((N, 3), generator=g) * 6 - 3 + torch.tensor([0.0, -9.0, 2.0])
    cam.set_positions_and_lookat(eye, torch.tensor([0.0, 0.0, 0.5]))
    snaps.append(("set_positions_and_lookat", cam.get_vp()))
    cam.set_eye(torch.tensor([1.0, -7.0, 3.0]))
    snaps.append(("set_eye", cam.get_vp()))
    cam.look_at(torch.rand((N, 3), generator=g) - 0.5)
    snaps.append(("look_at", cam.get_vp()))
    cam.set_up(torch.tensor([0.1, 0.2, 1.0]))
    snaps.append(("set_up", cam.get_vp()))
    cam.set_forward(torch.tensor([0.2, 1.0, -0.1]))
    snaps.append(("set_forward", cam.get_vp()))
    cam.set_right(torch.tensor([1.0, 0.1, 0.0]).repeat(N, 1))
    snaps.append(("set_right", cam.get_vp()))
    cam.set_positions(torch.tensor([0.0, -8.0, 1.5]))
    snaps.append(("set_positions", cam.get_vp()))
    return r, snaps


def defaults_scene(pbr, num_scenes: int = 3, **cfg):
    """add_node / add_camera / add_light with every argument left at its
    default (the box at the origin, the default eye and light)."""

    class Scene(pbr.PBRRenderer):
        def __init__(self):
            super().__init__(num_scenes=num_scenes, tile_resolution=(40, 24), **cfg)
            self.box = self.add_node("models/box", 1)
            self.add_camera()
            self.light = self.add_light()
            self.setup_environment()

    return Scene()


def cartpole_states(n: int, seed: int) -> torch.Tensor:
    g = torch.Generator().manual_seed(seed)
    st = torch.zeros((n, 4))
    st[:, 0] = torch.rand(n, generator=g) * 4 - 2
    st[:, 1] = torch.randn(n, generator=g)
    st[:, 2] = torch.rand(n, generator=g) * 1.0 - 0.5
    st[:, 3] = torch.randn(n, generator=g)
    return st


CONFIG_CASES = [
    {"num_scenes": 1}, {"num_scenes": 5}, {"num_scenes": 256}, {"num_scenes": 512}, {"num_scenes": 4098},
    {"num_scenes": 16384}, {"tiles": 7}, {"tiles": (3, 2)}, {"tile_resolution": (84, 84)},
    {"window_resolution": (640, 480)}, {"tiles": (4, 4), "tile_resolution": (32, 16)},
    {"tiles": (4, 2), "window_resolution": (256, 64)}, {"tile_resolution": (10, 20), "window_resolution": (100, 40)},
    {"num_scenes": 10, "tiles": (3, 3)}, {"tiles": (2, 2), "tile_resolution": (8, 8), "window_resolution": (16, 17)},
    {"num_scenes": 6, "batch_inner_dim": 9}, {"num_scenes": 6, "batch_inner_dim": 5},
    {"num_scenes": 9, "tile_resolution": (64, 48)},
]
