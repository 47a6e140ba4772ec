"""Textured drawing on the GPU (useTexture = 1, shaders/basic.frag:31-32)
against the FP64 oracle, and the plain path of the scene-per-warp kernel with
smooth meshes."""
import numpy as np
import pytest
import torch

import pybatchrender_gb300 as pbr
from pybatchrender_gb300.renderer import meshes
from tests.test_gpu_render import check_parity

pytestmark = pytest.mark.gpu


def _texture(seed: int, h: int, w: int) -> np.ndarray:
    return np.random.default_rng(seed).integers(0, 256, size=(h, w, 3), dtype=np.uint8)


def _quad_mesh() -> meshes.Mesh:
    """A unit quad in the x-z plane facing -y, texture coordinates spanning
    (-0.5, -0.25) .. (1.5, 2.0) so that the repeat wrap is exercised."""
    pos = np.array([[0, 0, 0], [1, 0, 0], [1, 0, 1], [0, 0, 1]], np.float32)
    nrm = np.tile(np.array([[0, -1, 0]], np.float32), (4, 1))
    idx = np.array([[0, 1, 2], [0, 2, 3]], np.int32)
    uv = np.array([[-0.5, -0.25], [1.5, -0.25], [1.5, 2.0], [-0.5, 2.0]], np.float32)
    return meshes.Mesh(pos, nrm, idx, name="quad", uvs=uv)


def _textured_scene(n: int = 48, res=(64, 64), seed: int = 0, **cfg) -> pbr.PBRRenderer:
    g = torch.Generator().manual_seed(seed)
    r = pbr.PBRRenderer(num_scenes=n, tile_resolution=res, **cfg)
    boxes = r.add_node("models/box", 6, model_pivot_relative_point=(0.5, 0.5, 0.5), texture=_texture(seed, 8, 16))
    plain = r.add_node("models/box", 3, model_pivot_relative_point=(0.5, 0.5, 0.5))
    quads = r.add_node(_quad_mesh(), 2, model_pivot_relative_point=(0.5, 0.5, 0.5), texture=_texture(seed + 1, 5, 3))
    spheres = r.add_node("icosphere:1", 2, model_pivot_relative_point=(0.5, 0.5, 0.5),
                         texture=_texture(seed + 2, 4, 4))  # no texture coordinates: samples (0, 0)
    for node in (boxes, plain, quads, spheres):
        B = node.buf_instances
        node.set_positions(torch.rand((B, 3), generator=g) * 6 - 3)
        node.set_hprs(torch.rand((B, 3), generator=g) * 6.3)
        node.set_scales(torch.rand(B, generator=g) * 1.5 + 0.5)
        node.set_colors(torch.cat([torch.rand((B, 3), generator=g) * 0.5 + 0.5, torch.ones((B, 1))], 1))
    r.add_camera(fov_y_deg=50.0)
    r._pbr_cam.set_positions_and_lookat(torch.tensor([0.0, -10.0, 2.0]), torch.tensor([0.0, 0.0, 0.0]))
    r.add_light()
    r.setup_environment()
    return r


@pytest.mark.parametrize("threads", [128, 256])
def test_textured_scene_parity(cuda, oracle, threads):
    r = _textured_scene(raster_threads=threads)
    cmp, gpu, ref = check_parity(r, oracle)
    # the textures are visible: scene 0 alone holds hundreds of distinct colours
    assert np.unique(gpu["pixels"][0].reshape(3, -1), axis=1).shape[1] > 200


def test_textured_near_plane_clipping(cuda, oracle):
    """Camera inside a large textured cube: clipped triangles interpolate the
    texture coordinates at the near plane like the other attributes."""
    r = pbr.PBRRenderer(num_scenes=3, tile_resolution=(64, 64))
    big = r.add_node("models/box", 1, model_pivot_relative_point=(0.5, 0.5, 0.5), model_scale=6.0,
                     texture=_texture(5, 16, 16))
    small = r.add_node("models/box", 3, model_pivot_relative_point=(0.5, 0.5, 0.5), texture=_texture(6, 4, 4))
    big.set_colors(torch.tensor([0.9, 0.8, 1.0, 1.0]))
    small.set_positions(torch.tensor([[0.0, 0.05, 0.0], [0.5, 1.0, 0.2], [-0.3, 2.0, -0.2]]).repeat(3, 1))
    small.set_hprs(torch.rand((9, 3), generator=torch.Generator().manual_seed(7)) * 6)
    r.add_camera()
    r._pbr_cam.set_positions_and_lookat(torch.tensor([[0.0, -0.4, 0.0], [0.2, -0.5, 0.1], [0.0, 0.0, 0.0]]),
                                        torch.tensor([[0.0, 5.0, 0.0], [0.0, 5.0, 1.0], [1.0, 5.0, 0.0]]))
    r.add_light()
    r.setup_environment()
    check_parity(r, oracle, depth_tol=1e-3)


def _plain_parity(r, oracle):
    """The plain path (one draw per node, model matrices built by torch, no
    winner output) against the oracle: colour within 1/255 off the edges."""
    pix, depth = r.render(return_depth=True)
    torch.cuda.synchronize()
    sc, me, no = r.export_scene()
    ref = oracle.render_hard(sc, me, no, want_depth=True, want_winner=True, want_ambiguous=True)
    cmp = oracle.compare_hard({"pixels": pix.cpu().numpy(), "depth": depth.cpu().numpy()}, ref)
    assert cmp["color_max_diff_unambiguous"] <= 1, cmp
    assert cmp["color_within_1"] >= 0.995, cmp
    return pix


def test_textured_plain_path_and_kernel_choice(cuda, oracle):
    a = _textured_scene(n=16, seed=3)
    b = _textured_scene(n=16, seed=3, raster_method="plain")
    pb = _plain_parity(b, oracle)
    assert (a.render() == pb).all(dim=1).float().mean() > 0.99
    # a scene too large for the scene-per-warp kernel is refused when that kernel is forced
    c = _textured_scene(n=4, seed=3, raster_kernel="warp")
    with pytest.raises(RuntimeError):
        c.render()


def _small_textured(kernel, n=256, seed=21):
    """CartPole-sized scenes (two textured boxes and a textured quad): within the
    scene-per-warp kernel's limits."""
    g = torch.Generator().manual_seed(seed)
    r = pbr.PBRRenderer(num_scenes=n, tile_resolution=(64, 64), raster_kernel=kernel)
    a = r.add_node("models/box", 1, model_pivot_relative_point=(0.5, 0.5, 0.5), model_scale=(1.5, 0.8, 0.6),
                   texture=_texture(seed, 6, 10))
    b = r.add_node("models/box", 1, model_pivot_relative_point=(0.5, 0.5, 0.0), model_scale=(0.3, 0.3, 2.0),
                   texture=_texture(seed + 1, 16, 4))
    q = r.add_node(_quad_mesh(), 1, model_pivot_relative_point=(0.5, 0.5, 0.5), model_scale=2.0,
                   texture=_texture(seed + 2, 5, 5))
    for node in (a, b, q):
        node.set_positions(torch.rand((n, 3), generator=g) * 2 - 1)
        node.set_hprs(torch.rand((n, 3), generator=g) * 6.3)
        node.set_colors(torch.cat([torch.rand((n, 3), generator=g) * 0.5 + 0.5, torch.ones((n, 1))], 1))
    r.add_camera(fov_y_deg=45.0)
    r._pbr_cam.set_positions_and_lookat(torch.tensor([0.0, -7.0, 1.0]), torch.tensor([0.0, 0.0, 0.0]))
    r.add_light()
    r.setup_environment()
    return r


def test_small_textured_scenes_both_kernels(cuda, oracle):
    """Textured CartPole-sized scenes: the scene-per-warp kernel draws them (its
    textured instantiation), with the tile kernel's exact output and the
    oracle's parity."""
    w = _small_textured("warp")
    t = _small_textured("tile")
    pw, dw, ww = w.render(return_depth=True, return_winner=True)
    pt, dt, wt = t.render(return_depth=True, return_winner=True)
    assert torch.equal(pw, pt) and torch.equal(dw, dt) and torch.equal(ww, wt)
    # randomly turned quads include near edge-on slivers: window depth to 1e-4
    check_parity(w, oracle, depth_tol=1e-4)
    a = _small_textured("auto")
    assert torch.equal(a.render(), pw)


def test_set_texture_after_setup(cuda, oracle):
    r = _textured_scene(n=8, seed=9)
    before = r.render().clone()
    node = r.geometry_nodes()[0]
    node.set_texture(None)  # untextured: the box's flat colour
    untextured = r.render().clone()
    assert not torch.equal(before, untextured)
    check_parity(r, oracle)
    node.set_texture(_texture(9, 8, 16))
    assert torch.equal(r.render(), before)


def test_warp_kernel_plain_smooth(cuda, oracle):
    """Smooth meshes in the plain (one draw per node) path of the
    scene-per-warp kernel are shaded per pixel like the batched path."""
    def scene(**cfg):
        r = pbr.PBRRenderer(num_scenes=32, tile_resolution=(64, 64), raster_kernel="warp", **cfg)
        g = torch.Generator().manual_seed(12)
        cyl = r.add_node("cylinder:8", 1, model_pivot_relative_point=(0.5, 0.5, 0.5), model_scale=3.0)
        box = r.add_node("models/box", 1, model_pivot_relative_point=(0.5, 0.5, 0.5))
        for node in (cyl, box):
            node.set_positions(torch.rand((32, 3), generator=g) * 2 - 1)
            node.set_hprs(torch.rand((32, 3), generator=g) * 6.3)
            node.set_colors(torch.cat([torch.rand((32, 3), generator=g), torch.ones((32, 1))], 1))
        r.add_camera(fov_y_deg=45.0)
        r._pbr_cam.set_positions_and_lookat(torch.tensor([0.0, -8.0, 1.0]), torch.tensor([0.0, 0.0, 0.0]))
        r.add_light()
        r.setup_environment()
        return r

    a, b = scene(), scene(raster_method="plain")
    pb = _plain_parity(b, oracle)
    assert (a.render() == pb).all(dim=1).float().mean() > 0.99
    # smooth cylinder sides seen nearly edge-on: window depth to 1e-4
    check_parity(a, oracle, depth_tol=1e-4)
