"""The reference's own model files rendered on the GPU against the FP64 oracle:
``models/cone.egg`` (62 smooth triangles) and the Steering rails'
``models/cylinder/scene.gltf`` (320 triangles), loaded by this package's
loaders from the recorded bytes through the model search path.  Bar: the
parity bar of test_gpu_render.py (window depth within 1e-4: the glTF
cylinder is 100 units long before scaling, and its thin, long side triangles
seen at a grazing angle have steep depth planes)."""
import math

import numpy as np
import pytest
import torch

import pybatchrender_gb300 as pbr
from pybatchrender_gb300.renderer import meshes
from tests import model_assets
from tests.test_gpu_render import check_parity

pytestmark = pytest.mark.gpu


@pytest.fixture
def model_dir(tmp_path, monkeypatch):
    d = model_assets.unpack(str(tmp_path))
    monkeypatch.setenv(meshes.MODEL_PATH_ENV, d)
    return d


def _asset_scene(n, kernel, seed=3):
    r = pbr.PBRRenderer(num_scenes=n, tile_resolution=(96, 80), raster_kernel=kernel, report_fps=False,
                        device="cuda")
    cone = r.add_node("models/cone.egg", instances_per_scene=3)
    cyl = r.add_node("models/cylinder/scene.gltf", instances_per_scene=2, model_scale=(0.6, 0.6, 1.8),
                     model_scale_units="absolute", model_pivot_relative_point=(0.5, 0.5, 0.5))
    assert cone.mesh.num_triangles == 62 and cyl.mesh.num_triangles == 320
    g = torch.Generator().manual_seed(seed)
    for node in (cone, cyl):
        B = node.buf_instances
        node.set_positions(torch.rand((B, 3), generator=g) * 5 - 2.5)
        node.set_hprs(torch.rand((B, 3), generator=g) * (2 * math.pi))
        node.set_scales(torch.rand(B, generator=g) * 0.5 + 0.6)
        node.set_colors(torch.cat([torch.rand((B, 3), generator=g) * 0.8 + 0.2, torch.ones((B, 1))], dim=1))
    r.add_camera(fov_y_deg=45.0)
    r._pbr_cam.set_positions_and_lookat(torch.tensor([0.0, -9.0, 3.0]), torch.tensor([0.0, 0.0, 0.0]))
    r.add_light(ambient=(0.2, 0.2, 0.25), dir_dir=(0.4, -0.6, -0.7))
    r.setup_environment()
    return r


@pytest.mark.parametrize("kernel", ["auto", "tile"])
def test_reference_models_parity(cuda, oracle, model_dir, kernel):
    r = _asset_scene(24, kernel)
    cmp, gpu, ref = check_parity(r, oracle, depth_tol=1e-4)
    win = ref["winner"]
    max_tris = max(nd.mesh.num_triangles for nd in r.geometry_nodes())
    rank = np.where(win >= 0, win // max_tris, -1)
    # both meshes are on screen: cone instances have ranks 0..2, cylinder instances 3..4
    assert ((rank >= 0) & (rank < 3)).sum() > 500 and (rank >= 3).sum() > 500, cmp


def test_steering_with_the_reference_rail_model(cuda, oracle, model_dir):
    """Steering-v0 with its default rail model found on the model search path:
    the rails are the reference's 320-triangle glTF cylinder; coverage and
    colour pass the exact bar, rail depths the near-plane-clipping bar of
    test_gpu_render.py's Steering test (5e-3), every other node 1e-5."""
    env = pbr.envs.make("Steering-v0", num_scenes=16, number_of_obstacles=20)
    r = env._renderer
    assert r.left_border.mesh.num_triangles == 320
    td = env.reset()
    td["action"] = env.action_spec.rand()
    env.step(td)
    cmp, gpu, ref = check_parity(r, oracle, depth_tol=1.0)
    max_tris = max(n.mesh.num_triangles for n in r.geometry_nodes())
    rank = ref["winner"] // max_tris
    covered = (ref["winner"] >= 0) & ~ref["ambiguous"]
    rail = covered & ((rank == 1) | (rank == 2))
    other = covered & ~rail
    derr = np.abs(gpu["depth"] - ref["depth"])
    assert other.any() and rail.any()
    assert derr[other].max() <= 1e-5, derr[other].max()
    assert derr[rail].max() <= 5e-3, derr[rail].max()
