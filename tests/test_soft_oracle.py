"""Soft-coverage reference consistency (CPU): the FP64 C oracle, the dense
float64 PyTorch reference and FP64 finite differences describe one model."""
import numpy as np
import torch

from oracle import oracle, soft_torch
from pybatchrender_gb300 import PBRRenderer, workloads
from tests.soft_util import fd_light, fd_param, rel_err


def cartpole_scene(n=3, res=32, seed=1):
    r = workloads.cartpole_bench(num_scenes=n, res=res, seed=seed, device="cpu")
    r._step(workloads.cartpole_states(n, seed=seed + 1))
    return r.export_scene()


def sphere_scene():
    r = PBRRenderer(num_scenes=2, tile_resolution=(24, 20), device="cpu")
    node = r.add_node("icosphere:1", 2, model_pivot_relative_point=(0.5, 0.5, 0.5))
    g = torch.Generator().manual_seed(3)
    node.set_positions(torch.rand((4, 3), generator=g) * 2 - 1)
    node.set_hprs(torch.rand((4, 3), generator=g) * 3)
    node.set_scales(torch.rand(4, generator=g) + 1.5)
    node.set_colors(torch.rand((4, 4), generator=g))
    r.add_camera(fov_y_deg=50)
    r._pbr_cam.set_positions_and_lookat([0.0, -7.0, 1.0], [0.0, 0.0, 0.0])
    r.add_light()
    r.set_background_color(0.1, 0.2, 0.3)
    return r.export_scene()


def test_torch_reference_matches_oracle_forward():
    for sc, me, no in (cartpole_scene(), sphere_scene()):
        a = oracle.render_soft(sc, me, no, out_dtype=np.float64)
        img = soft_torch.render(sc, me, no, soft_torch.params_from_nodes(no, False),
                                torch.tensor(np.asarray(sc["ldir"], np.float32), dtype=torch.float64))
        assert np.abs(img.numpy() - a).max() < 1e-9
        assert a.max() > 0.05  # something is drawn


def test_finite_differences_match_autograd():
    for sc, me, no in (cartpole_scene(), sphere_scene()):
        a = oracle.render_soft(sc, me, no, out_dtype=np.float64)
        target = a * 0.8 + 0.05
        prm = soft_torch.params_from_nodes(no)
        L = torch.tensor(np.asarray(sc["ldir"], np.float32), dtype=torch.float64, requires_grad=True)
        loss = ((soft_torch.render(sc, me, no, prm, L) - torch.tensor(target)) ** 2).mean()
        loss.backward()
        got, want = [], []
        rng = np.random.default_rng(0)
        for ni, nd in enumerate(no):
            for key in ("pos", "hpr", "color", "scale"):
                g = prm[ni][key].grad.numpy().reshape(-1)
                for idx in rng.choice(g.size, size=min(4, g.size), replace=False):
                    if key == "color" and idx % 4 == 3:
                        continue
                    got.append(g[idx])
                    want.append(fd_param(sc, me, no, target, ni, key, int(idx)))
        for i in range(3):
            got.append(L.grad.numpy()[i])
            want.append(fd_light(sc, me, no, target, i))
        assert rel_err(got, want) < 1e-5, rel_err(got, want)
