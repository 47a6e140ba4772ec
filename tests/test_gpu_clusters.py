"""Cluster culling in the tile kernel (``pbr_mesh_set_clusters``): groups of 32
triangles whose triangles all face away from the eye, or whose projected
bounding sphere holds no pixel centre of the region drawn, are skipped before
setup.  The culled groups hold no triangle that would be drawn, so the output
must be bit-identical with and without clusters: pixels, depth and winner ids,
on the uneven-batching scenes (icosphere-3, cylinder-64 and cubes), with
cameras among the meshes (spheres crossing the near plane), on both region
sizes, on Steering-v0 (icosphere obstacles) and on a textured scene."""
import math

import numpy as np
import pytest
import torch

import pybatchrender_gb300 as pbr
from pybatchrender_gb300 import workloads

pytestmark = pytest.mark.gpu


def _render_all(r):
    out = r.render(return_depth=True, return_winner=True)
    torch.cuda.synchronize()
    return [t.clone() for t in out]


def _assert_same(a, b):
    for x, y in zip(a, b):
        assert torch.equal(x, y)


@pytest.mark.parametrize("threads,seed", [(256, 0), (128, 1), (512, 2)])
def test_uneven_scenes_same_with_and_without_clusters(cuda, threads, seed):
    res = []
    for cull in (True, False):
        r = workloads.uneven(num_scenes=64, res=84, max_instances=128, seed=seed, raster_kernel="tile",
                             raster_threads=threads, cluster_cull=cull)
        res.append(_render_all(r))
    _assert_same(*res)
    assert (res[0][2] >= 0).float().mean() > 0.01


def test_camera_among_meshes_same_with_and_without_clusters(cuda):
    """Cameras inside the cloud of spheres: clusters behind or around the eye,
    spheres crossing the near plane, near-plane clipping of the triangles."""
    res = []
    for cull in (True, False):
        r = workloads.uneven(num_scenes=32, res=84, max_instances=256, seed=5, raster_kernel="tile",
                             cluster_cull=cull)
        g = torch.Generator().manual_seed(6)
        eye = torch.rand((32, 3), generator=g) * 4 - 2
        target = torch.rand((32, 3), generator=g) * 8 - 4
        r._pbr_cam.set_positions_and_lookat(eye.to(cuda), target.to(cuda))
        res.append(_render_all(r))
    _assert_same(*res)


def test_steering_same_with_and_without_clusters(cuda):
    res = []
    for cull in (True, False):
        env = pbr.envs.make("Steering-v0", num_scenes=16, number_of_obstacles=20, cluster_cull=cull,
                            raster_kernel="tile")
        env.reset()
        res.append(_render_all(env._renderer))
    _assert_same(*res)


def test_textured_spheres_same_with_and_without_clusters(cuda):
    from pybatchrender_gb300.renderer import meshes
    rgb = np.random.default_rng(7).integers(0, 256, (16, 16, 3), dtype=np.uint8)
    tex = np.concatenate([rgb, np.full((16, 16, 1), 255, np.uint8)], axis=2)
    res = []
    for cull in (True, False):
        r = pbr.PBRRenderer(num_scenes=8, tile_resolution=(64, 64), raster_kernel="tile", cluster_cull=cull,
                            device="cuda", report_fps=False)
        sphere = meshes.icosphere(3)
        sphere.uvs = (sphere.positions[:, :2] + 0.5).astype(np.float32)
        node = r.add_node(sphere, instances_per_scene=6, texture=tex)
        g = torch.Generator().manual_seed(8)
        node.set_positions(torch.rand((48, 3), generator=g) * 4 - 2)
        node.set_hprs(torch.rand((48, 3), generator=g) * 2 * math.pi)
        node.set_scales(torch.rand(48, generator=g) * 1.5 + 0.5)
        r.add_camera(fov_y_deg=50.0)
        r._pbr_cam.set_positions_and_lookat(torch.tensor([0.0, -7.0, 1.0]), torch.tensor([0.0, 0.0, 0.0]))
        r.add_light()
        r.setup_environment()
        res.append(_render_all(r))
    _assert_same(*res)


def test_triangle_soup_same_with_and_without_clusters(cuda):
    """A mesh whose triangles share no vertex (a triangle soup, 960 vertices):
    looser cluster spheres and cones, the same pixels."""
    from pybatchrender_gb300.renderer import meshes
    ico = meshes.icosphere(2)
    soup = meshes.Mesh(ico.positions[ico.indices.ravel()], ico.normals[ico.indices.ravel()],
                       np.arange(3 * ico.num_triangles, dtype=np.int32).reshape(-1, 3), name="soup")
    res = []
    for cull in (True, False):
        r = pbr.PBRRenderer(num_scenes=8, tile_resolution=(80, 60), raster_kernel="tile", cluster_cull=cull,
                            device="cuda", report_fps=False)
        node = r.add_node(soup.copy(), instances_per_scene=40, model_pivot_relative_point=(0.5, 0.5, 0.5))
        g = torch.Generator().manual_seed(9)
        node.set_positions(torch.rand((320, 3), generator=g) * 6 - 3)
        node.set_hprs(torch.rand((320, 3), generator=g) * 2 * math.pi)
        node.set_colors(torch.rand((320, 4), generator=g))
        r.add_camera(fov_y_deg=50.0)
        r._pbr_cam.set_positions_and_lookat(torch.tensor([0.0, -8.0, 1.0]), torch.tensor([0.0, 0.0, 0.0]))
        r.add_light()
        r.setup_environment()
        res.append(_render_all(r))
    _assert_same(*res)
    assert (res[0][2] >= 0).float().mean() > 0.05


@pytest.mark.parametrize("scenes", ["uneven", "many_cubes"])
def test_pretest_leaves_pixels_unchanged(cuda, scenes):
    """The tile kernel's coverage-and-depth pre-test drops only triangles that
    would not change a pixel: rendering with it forced on and forced off gives
    bit-identical pixels, depth and winners, on dense uneven scenes (where it is
    on by default) and on the many-cubes scenes (where it is off)."""
    res = []
    for mode in ("on", "off"):
        if scenes == "uneven":
            r = workloads.uneven(num_scenes=96, res=84, max_instances=256, seed=11, raster_kernel="tile",
                                 tile_pretest=mode)
        else:
            r = workloads.many_cubes(num_scenes=48, seed=12, raster_kernel="tile", tile_pretest=mode)
        res.append(_render_all(r))
    _assert_same(*res)
    assert (res[0][2] >= 0).float().mean() > 0.05


def test_pretest_leaves_plain_per_node_draws_unchanged(cuda):
    """The per-node plain path (one tile-kernel draw per node against the depth
    and colour buffers of the nodes drawn before, whose keys carry order 0):
    the pre-test forced on and off gives bit-identical pixels and depth on
    dense uneven scenes."""
    res = []
    for mode in ("on", "off"):
        r = workloads.uneven(num_scenes=48, res=84, max_instances=256, seed=13, raster_kernel="tile",
                             raster_method="plain", tile_pretest=mode)
        out, depth = r.render(return_depth=True)
        torch.cuda.synchronize()
        res.append((out.clone(), depth.clone()))
    _assert_same(*res)
    assert (res[0][1] < 1.0).float().mean() > 0.05
