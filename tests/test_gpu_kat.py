"""The known-answer raster scenes of tests/kat_scenes.py on the CUDA kernels
(scene-per-warp and tile): the analytic coverage, depth, winners and colours,
exactly."""
import numpy as np
import pytest
import torch

import pybatchrender_gb300 as pbr
from pybatchrender_gb300.renderer.meshes import Mesh
from tests import kat_scenes as K

pytestmark = pytest.mark.gpu


def _renderer(meshes_colors, kernel, lit=False, n=2):
    r = pbr.PBRRenderer(num_scenes=n, tile_resolution=(K.W, K.H), raster_kernel=kernel)
    for km, col in meshes_colors:
        node = r.add_node(Mesh(km.positions, km.normals, km.indices, name="kat"), 1, shared_across_scenes=True)
        node.set_colors(torch.tensor(col))
    r.add_camera()
    if lit:
        r.add_light(ambient=K.FACE_AMBIENT, dir_dir=(0.0, 0.0, 2.0), dir_col=(1.0, 1.0, 1.0), strength=1.0)
    else:
        r.add_light(strength=0.0)
    r.setup_environment()
    r._pbr_cam.VP_k44.copy_(torch.eye(4).expand(n, 4, 4))  # orthographic: clip = world
    return r


@pytest.mark.parametrize("kernel", ["warp", "tile"])
def test_kat_square_fill_rule_depth_colour(cuda, kernel):
    r = _renderer([(K.screen_mesh(K.SQUARE, K.SQUARE_TRIS), (0.8, 0.4, 0.2, 1.0))], kernel)
    pix, depth, win = r.render(return_depth=True, return_winner=True)
    exp = torch.from_numpy(K.square_expected()).cuda()
    for k in range(2):
        assert torch.equal(win[k] >= 0, exp)
        assert torch.all(depth[k][exp] == 0.625) and torch.all(depth[k][~exp] == 1.0)
        assert torch.all(pix[k, 0][exp] == 204) and torch.all(pix[k, 1][exp] == 102) and torch.all(pix[k, 2][exp] == 51)
        assert torch.all(pix[k][:, ~exp] == 0)


@pytest.mark.parametrize("kernel", ["warp", "tile"])
def test_kat_shared_diagonal_watertight(cuda, kernel):
    cov = []
    for tri in K.SQUARE_TRIS:
        r = _renderer([(K.screen_mesh(K.SQUARE, [tri]), (1.0, 1.0, 1.0, 1.0))], kernel)
        _, _, win = r.render(return_depth=True, return_winner=True)
        cov.append(win[0] >= 0)
    assert not torch.any(cov[0] & cov[1])
    assert torch.equal(cov[0] | cov[1], torch.from_numpy(K.square_expected()).cuda())


@pytest.mark.parametrize("kernel", ["warp", "tile"])
@pytest.mark.parametrize("corners", [[(4.5, 4.5), (12.5, 12.5), (20.5, 20.5)], [(8.6, 20.6), (8.9, 20.6), (8.6, 4.6)],
                                     [(3.2, 3.7), (3.45, 3.7), (3.2, 3.95)]])
def test_kat_degenerate_and_sliver(cuda, kernel, corners):
    r = _renderer([(K.screen_mesh(corners, [(0, 1, 2)]), (1.0, 1.0, 1.0, 1.0))], kernel)
    _, _, win = r.render(return_depth=True, return_winner=True)
    assert not torch.any(win >= 0)


@pytest.mark.parametrize("kernel", ["warp", "tile"])
def test_kat_depth_order_and_ties(cuda, kernel):
    far = K.screen_mesh(K.SQUARE, K.SQUARE_TRIS, z=0.5)
    near = K.screen_mesh(K.SQUARE, K.SQUARE_TRIS, z=-0.5)
    same = K.screen_mesh(K.SQUARE, K.SQUARE_TRIS, z=0.5)
    exp = torch.from_numpy(K.square_expected()).cuda()
    r = _renderer([(far, (1, 0, 0, 1)), (near, (0, 1, 0, 1)), (same, (0, 0, 1, 1))], kernel)
    pix, depth, win = r.render(return_depth=True, return_winner=True)
    assert torch.all(win[0][exp] // 2 == 1) and torch.all(depth[0][exp] == 0.25) and torch.all(pix[0, 1][exp] == 255)
    r = _renderer([(far, (1, 0, 0, 1)), (same, (0, 0, 1, 1))], kernel)
    pix, depth, win = r.render(return_depth=True, return_winner=True)
    assert torch.all(win[0][exp] // 2 == 0) and torch.all(pix[0, 0][exp] == 255)


@pytest.mark.parametrize("kernel", ["warp", "tile"])
def test_kat_back_face_and_lit_face(cuda, kernel):
    r = _renderer([(K.screen_mesh(K.SQUARE, [(0, 2, 1), (0, 3, 2)]), (1.0, 1.0, 1.0, 1.0))], kernel)
    _, _, win = r.render(return_depth=True, return_winner=True)
    assert not torch.any(win >= 0)
    r = _renderer([(K.screen_mesh(K.SQUARE, K.SQUARE_TRIS), K.FACE_COLOR)], kernel, lit=True)
    pix, _, win = r.render(return_depth=True, return_winner=True)
    cov = win[0] >= 0
    assert int(cov.sum()) == 64
    for c in range(3):
        assert torch.all(pix[0, c][cov] == K.FACE_EXPECT[c])


@pytest.mark.parametrize("kernel", ["warp", "tile", "binned"])
def test_kat_soft_coverage(cuda, kernel):
    """The soft known answers of tests/test_oracle_kat.py on each soft kernel:
    half coverage on an edge, full coverage inside, background beyond the cut-off."""
    r = pbr.PBRRenderer(num_scenes=2, tile_resolution=(K.W, K.H), raster_mode="soft", raster_kernel=kernel)
    km = K.screen_mesh(K.SQUARE, K.SQUARE_TRIS)
    node = r.add_node(Mesh(km.positions, km.normals, km.indices, name="kat"), 1, shared_across_scenes=True)
    node.set_colors(torch.tensor((0.8, 0.4, 0.2, 1.0)))
    r.add_camera()
    r.add_light(strength=0.0)
    r.setup_environment()
    r._pbr_cam.VP_k44.copy_(torch.eye(4).expand(2, 4, 4))
    with torch.no_grad():
        out = r.render_soft()
    col = torch.tensor([0.8, 0.4, 0.2], device="cuda")
    for k in range(2):
        assert torch.allclose(out[k, :, 8, 8], 0.5 * col, rtol=0, atol=2e-6)
        assert torch.allclose(out[k, :, 4, 12], 0.5 * col, rtol=0, atol=2e-6)
        assert torch.allclose(out[k, :, 7, 10], col, rtol=0, atol=2e-6)
        assert torch.all(out[k, :, 2, 2] == 0.0) and torch.all(out[k, :, 20, 25] == 0.0)
