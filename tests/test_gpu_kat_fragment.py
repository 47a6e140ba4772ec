"""The fragment-stage and watertightness known answers of
tests/test_oracle_kat.py and tests/test_api_kat_cpu.py on the CUDA raster
kernels (scene-per-warp and tile): texture filtering and orientation,
texel x colour x light, smooth normals, perspective-correct coordinates,
jittered meshes with vertices on pixel centres, and cubes placed through the
public API."""
import math

import numpy as np
import pytest
import torch

import pybatchrender_gb300 as pbr
from pybatchrender_gb300.renderer.meshes import Mesh
from tests import kat_scenes as K
from tests.test_oracle_kat import _jittered_grid

pytestmark = pytest.mark.gpu
KERNELS = ["warp", "tile"]


def _renderer(km, color, kernel, texture=None, lit=None, vp=None, n=2):
    """One shared node of mesh ``km``; ``texture`` in the oracle's layout
    (row 0 at v = 0); ``lit`` = (ambient, direction) or None for unlit."""
    r = pbr.PBRRenderer(num_scenes=n, tile_resolution=(K.W, K.H), raster_kernel=kernel)
    nrm = km.normals / np.linalg.norm(km.normals, axis=1, keepdims=True)
    node = r.add_node(Mesh(km.positions, nrm, km.indices, name="kat", uvs=km.uvs), 1, shared_across_scenes=True)
    node.set_colors(torch.tensor(color))
    if texture is not None:
        node.set_texture(texture[::-1].copy())  # set_texture takes image order (row 0 = top)
    r.add_camera()
    if lit is None:
        r.add_light(strength=0.0)
    else:
        r.add_light(ambient=lit[0], dir_dir=lit[1], dir_col=(1.0, 1.0, 1.0), strength=1.0)
    r.setup_environment()
    v = torch.eye(4) if vp is None else torch.from_numpy(np.asarray(vp, np.float32))
    r._pbr_cam.VP_k44.copy_(v.expand(n, 4, 4))
    return r


def _pixels(r):
    pix, depth, win = r.render(return_depth=True, return_winner=True)
    return pix.cpu().numpy(), depth.cpu().numpy(), win.cpu().numpy()


@pytest.mark.parametrize("kernel", KERNELS)
def test_kat_texture_u_and_v(cuda, kernel):
    quad = K.textured_square([(0, 0), (1, 0), (1, 1), (0, 1)])
    r = _renderer(quad, (1.0, 1.0, 1.0, 1.0), kernel, texture=K.texture([[(0, 0, 0), (200, 100, 40)]]))
    pix, _, win = _pixels(r)
    w1 = np.array([0.5, 0.25, 0.0, 0.25, 0.5, 0.75, 1.0, 0.75])
    for k in range(2):
        assert np.array_equal(win[k] >= 0, K.square_expected())
        for c, full in enumerate((200, 100, 40)):
            assert np.all(pix[k, c, 4:12, 8:16] == np.floor(w1 * full + 0.5).astype(np.uint8)[None, :]), (k, c)
    r = _renderer(quad, (1.0, 1.0, 1.0, 1.0), kernel, texture=K.texture([[(0, 200, 0)], [(200, 0, 0)]]))
    pix, _, _ = _pixels(r)
    w1 = np.array([0.5, 0.75, 1.0, 0.75, 0.5, 0.25, 0.0, 0.25])
    assert np.all(pix[0, 0, 4:12, 8:16] == np.floor(w1 * 200 + 0.5).astype(np.uint8)[:, None])
    assert np.all(pix[0, 1, 4:12, 8:16] == np.floor((1 - w1) * 200 + 0.5).astype(np.uint8)[:, None])


@pytest.mark.parametrize("kernel", KERNELS)
def test_kat_texture_times_colour_and_light(cuda, kernel):
    quad = K.textured_square([(0.5, 0.5)] * 4)
    r = _renderer(quad, K.FACE_COLOR, kernel, texture=K.texture([[(0, 255, 0)]]),
                  lit=(K.FACE_AMBIENT, (0.0, 0.0, 2.0)))
    pix, _, win = _pixels(r)
    cov = win[0] >= 0
    assert cov.sum() == 64
    assert np.all(pix[0, 0][cov] == 0) and np.all(pix[0, 2][cov] == 0)
    assert np.all(pix[0, 1][cov] == K.FACE_EXPECT[1])


@pytest.mark.parametrize("kernel", KERNELS)
def test_kat_smooth_normals(cuda, kernel):
    sq = K.screen_mesh(K.SQUARE, K.SQUARE_TRIS)
    sq.normals = np.array([(-1, 0, 1), (1, 0, 1), (1, 0, 1), (-1, 0, 1)], np.float32)
    r = _renderer(sq, (1.0, 1.0, 1.0, 1.0), kernel, lit=((0.0, 0.0, 0.0), (0.0, 0.0, 1.0)))
    pix, _, _ = _pixels(r)
    t = (np.arange(8, 16) - 8) / 8.0
    expect = np.floor(255.0 / np.sqrt((2 * t - 1) ** 2 + 1) + 0.5).astype(np.uint8)
    for c in range(3):
        assert np.all(pix[0, c, 4:12, 8:16] == expect[None, :]), c


@pytest.mark.parametrize("kernel", KERNELS)
def test_kat_perspective_correct_coordinates(cuda, kernel):
    ramp = K.texture([[(4 * i, 0, 0) for i in range(64)]])
    r = _renderer(K.perspective_quad(), (1.0, 1.0, 1.0, 1.0), kernel, texture=ramp, vp=K.PERSP_VP)
    pix, depth, win = _pixels(r)
    cov = win[0] >= 0
    rows, cols = np.nonzero(cov)
    assert rows.min() == 8 and rows.max() == 23 and cols.min() == 8 and cols.max() == 23
    ndc_x = 2.0 * (np.arange(8, 24) + 0.5) / K.W - 1.0
    u = K.perspective_u(ndc_x)
    value = 256.0 * u - 2.0
    inner = (u * 64 - 0.5 >= 0) & (u * 64 - 0.5 <= 63)
    got = pix[0, 0, 8:24, 8:24].astype(np.float64)
    # FP32 interpolation: within one level of the exact value
    assert np.all(np.abs(got[:, inner] - value[None, inner]) <= 1.0)
    z = K.PERSP_Z0 + (K.PERSP_Z1 - K.PERSP_Z0) * u
    assert np.allclose(depth[0, 8:24, 8:24], (1.0 - 1.0 / z)[None, :], rtol=0, atol=1e-5)


@pytest.mark.parametrize("kernel", KERNELS)
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_kat_jittered_meshes_watertight(cuda, kernel, seed):
    pts, tris = _jittered_grid(seed)
    count = np.zeros((K.H, K.W), np.int32)
    for t in tris:
        r = _renderer(K.screen_mesh([pts[v] for v in t], [(0, 1, 2)]), (1.0, 1.0, 1.0, 1.0), kernel)
        _, _, win = _pixels(r)
        count += (win[0] >= 0).astype(np.int32)
    c = np.arange(K.W) + 0.5
    inside = ((c > 4) & (c < 28))[:, None] & ((c > 4) & (c < 28))[None, :]
    assert count.max() == 1 and np.array_equal(count == 1, inside)


@pytest.mark.parametrize("kernel", KERNELS)
def test_kat_api_cubes(cuda, kernel):
    """The scenes of tests/test_api_kat_cpu.py rendered on the GPU."""
    r = pbr.PBRRenderer(num_scenes=3, tile_resolution=(64, 64), raster_kernel=kernel)
    box = r.add_node("models/box", 1, model_pivot_relative_point=(0.5, 0.5, 0.5))
    cam = r.add_camera(fov_y_deg=40.0, z_near=0.05, z_far=100.0)
    cam.set_positions_and_lookat(torch.tensor([0.0, -8.0, 0.0]), torch.tensor([0.0, 0.0, 0.0]))
    r.add_light(ambient=(0.2, 0.2, 0.2), dir_dir=(0.0, -1.0, 0.0), dir_col=(1.0, 1.0, 1.0), strength=1.0)
    r.setup_environment()
    box.set_positions(torch.tensor([[0.0, 0.0, 0.0], [0.0, 2.5, 0.0], [0.0, 0.0, 0.0]], device="cuda"))
    box.set_hprs(torch.tensor([[0.0, 0.0, 0.0], [0.0, 0.0, 0.0], [math.pi / 4, 0.0, 0.0]], device="cuda"))
    box.set_colors(torch.tensor([K.FACE_COLOR] * 3, device="cuda"))
    pix, _, win = _pixels(r)
    for k, (first, last) in ((0, (26, 37)), (1, (28, 35))):
        expect = np.zeros((64, 64), bool)
        expect[first:last + 1, first:last + 1] = True
        assert np.array_equal(win[k] >= 0, expect), k
        for c in range(3):
            assert np.all(pix[k, c][expect] == K.FACE_EXPECT[c]) and np.all(pix[k, c][~expect] == 0)
    cov = win[2] >= 0
    assert len(np.unique(win[2][cov] // 2)) == 2
    # every covered pixel of the turned cube has colour * (0.2 + cos 45 deg), up to one level on the silhouette
    for c, e in enumerate((93, 139, 185)):
        assert np.abs(pix[2, c][cov].astype(int) - e).max() <= 1
        assert (pix[2, c][cov] == e).mean() > 0.99
