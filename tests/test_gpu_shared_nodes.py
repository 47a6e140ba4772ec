"""Shared nodes with several instances per scene (1 < I < N) on the GPU.

The pattern is the reference's many-cubes demo (``demo_many_cubes.py:28``):
one node with ``shared_across_scenes=True`` and one without, both with I
instances per scene, positions U(-15, 15), transforms set through
``set_transforms`` (the shared node gets the first I matrices) and per-instance
colours.  Here instance i of every scene draws buffer row i of a shared node;
the reference's ``instancesPerScene = max(1, B // N)`` (``renderer/node.py:90``)
decodes each instance of such a node as its own scene instead, a divergence
this package documents.  Both raster kernels and the plain per-node method
are held to the FP64 oracle with the bar of test_gpu_render.py, and a scene
made of the shared node alone must render the same image in every scene."""
import math

import numpy as np
import pytest
import torch

import pybatchrender_gb300 as pbr
from pybatchrender_gb300.renderer.shader_context import PBRShaderContext
from tests.test_gpu_render import check_parity

pytestmark = pytest.mark.gpu


def _demo_scene(n, ips, model, raster_kernel="auto", raster_method="batched", with_unshared=True, seed=123):
    r = pbr.PBRRenderer(num_scenes=n, tile_resolution=(64, 64), raster_kernel=raster_kernel,
                        raster_method=raster_method, report_fps=False, device="cuda")
    shared = r.add_node(model, instances_per_scene=ips, shared_across_scenes=True,
                        model_pivot_relative_point=(0.5, 0.5, 0.5))
    own = r.add_node(model, instances_per_scene=ips, shared_across_scenes=False,
                     model_pivot_relative_point=(0.5, 0.5, 0.5)) if with_unshared else None
    rng = np.random.default_rng(seed)
    B = n * ips
    pos = rng.uniform(-15, 15, size=(B, 3)).astype(np.float32)
    hpr = rng.uniform(-math.pi, math.pi, size=(B, 3)).astype(np.float32)
    s = rng.uniform(1.5, 4.0, size=(B,)).astype(np.float32)
    R = PBRShaderContext._rotation_mats_from_hpr(torch.from_numpy(hpr)).numpy()
    mats = np.zeros((B, 4, 4), np.float32)
    mats[:, 3, 3] = 1.0
    mats[:, :3, :3] = R * s[:, None, None]
    mats[:, :3, 3] = pos
    col = np.concatenate([rng.uniform(0.2, 1.0, size=(B, 3)), np.ones((B, 1))], axis=1).astype(np.float32)
    shared.set_transforms(mats[:ips])
    shared.set_colors(col[:ips])
    if own is not None:
        own.set_transforms(mats)
        own.set_colors(col)
    r.add_camera()
    r._pbr_cam.set_positions_and_lookat(torch.tensor([0.0, -50.0, 10.0]), torch.tensor([0.0, 0.0, 0.0]))
    r.add_light(ambient=(0.2, 0.2, 0.25), dir_dir=(0.4, -0.6, -0.7), dir_col=(1, 1, 1), strength=1.0)
    r.setup_environment()
    return r, shared, own


@pytest.mark.parametrize("model,ips,kernel", [("models/box", 2, "warp"), ("models/box", 3, "tile"),
                                              ("models/smiley", 3, "tile"), ("models/smiley", 3, "auto")])
def test_shared_node_several_instances_parity(cuda, oracle, model, ips, kernel):
    n = 48
    r, shared, own = _demo_scene(n, ips, model, raster_kernel=kernel)
    assert shared.buf_instances == ips and own.buf_instances == n * ips
    cmp, gpu, ref = check_parity(r, oracle)
    assert (ref["winner"] >= 0).mean() > 0.005, cmp
    # winner ids are (instance rank * triangles per mesh + triangle): ranks below I belong to the shared node,
    # and its instances are drawn in many scenes, not only in the scene whose rows they are
    tris = r.geometry_nodes()[0].mesh.num_triangles
    rank = np.where(gpu["winner"] >= 0, gpu["winner"] // tris, -1)
    scenes_with_shared = int(((rank >= 0) & (rank < ips)).reshape(n, -1).any(axis=1).sum())
    assert scenes_with_shared > n // 2, scenes_with_shared


@pytest.mark.parametrize("kernel", ["warp", "tile"])
def test_shared_node_alone_same_image_in_every_scene(cuda, oracle, kernel):
    """With only the shared node and one camera for all scenes, every scene
    draws the same I instances: all N images are identical and equal the
    oracle's."""
    n, ips = 40, 3
    r, shared, _ = _demo_scene(n, ips, "models/box", raster_kernel=kernel, with_unshared=False, seed=7)
    cmp, gpu, ref = check_parity(r, oracle)
    pix = gpu["pixels"]
    assert (ref["winner"] >= 0).mean() > 0.01, cmp
    assert np.all(pix == pix[:1]), "a shared node must draw the same instances in every scene"


def test_shared_node_plain_method_matches_batched(cuda):
    """The plain per-node method (host-built matrices, one launch per node)
    draws shared nodes with the same semantics."""
    n, ips = 32, 3
    a, a_shared, a_own = _demo_scene(n, ips, "models/box", seed=9)
    b, b_shared, b_own = _demo_scene(n, ips, "models/box", raster_method="plain", seed=9)
    # set_transforms splits the matrices on the node's device (the GPU here, the host for the plain method),
    # where the scale's norm can round differently in the last bit: give both the same node state
    for src, dst in ((a_shared, b_shared), (a_own, b_own)):
        for name in ("pos", "rot3", "scale", "color"):
            getattr(dst, name).copy_(getattr(src, name).cpu())
    pa, da = a.render(return_depth=True)
    pb, db = b.render(return_depth=True)
    assert torch.equal(pa, pb)
    assert torch.equal(da, db)
