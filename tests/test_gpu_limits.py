"""Size limits and edge sizes on the GPU: large and ragged images, a very
large scene count, and the node-table limit (a clear error, not a fault)."""
import numpy as np
import pytest
import torch

import pybatchrender_gb300 as pbr
from pybatchrender_gb300 import _capi
from tests.test_gpu_render import check_parity

pytestmark = pytest.mark.gpu


def _cubes(n, res, inst=24, seed=0, **cfg):
    r = pbr.PBRRenderer(num_scenes=n, tile_resolution=res, **cfg)
    g = torch.Generator().manual_seed(seed)
    node = r.add_node("models/box", inst, model_pivot_relative_point=(0.5, 0.5, 0.5))
    B = node.buf_instances
    node.set_positions(torch.rand((B, 3), generator=g) * 8 - 4)
    node.set_hprs(torch.rand((B, 3), generator=g) * 6.3)
    node.set_scales(torch.rand(B, generator=g) + 0.3)
    node.set_colors(torch.rand((B, 4), generator=g))
    r.add_camera(fov_y_deg=50.0)
    r._pbr_cam.set_positions_and_lookat(torch.tensor([0.0, -12.0, 1.0]), torch.tensor([0.0, 0.0, 0.0]))
    r.add_light()
    r.setup_environment()
    return r


@pytest.mark.parametrize("res", [(640, 480), (333, 77), (16, 1024)])
def test_large_and_ragged_images(cuda, oracle, res):
    check_parity(_cubes(2, res), oracle)


def test_very_many_scenes(cuda, oracle):
    """65536 scenes of 16 x 16: every scene index and pixel offset in range;
    the first and last 64 scenes against the oracle."""
    n = 65536
    r = _cubes(n, (16, 16), inst=2, seed=3)
    pix, depth, win = r.render(return_depth=True, return_winner=True)
    torch.cuda.synchronize()
    sc, me, no = r.export_scene()
    for k0 in (0, n - 64):
        ref = oracle.render_hard(sc, me, no, k0, k0 + 64, want_depth=True, want_winner=True, want_ambiguous=True)
        gpu = {"pixels": pix[k0:k0 + 64].cpu().numpy(), "winner": win[k0:k0 + 64].cpu().numpy()}
        cmp = oracle.compare_hard(gpu, ref)
        assert cmp["winner_mismatch"] == 0 and cmp["color_max_diff_unambiguous"] <= 1, cmp


def test_node_table_limit_is_an_error(cuda):
    r = pbr.PBRRenderer(num_scenes=2, tile_resolution=(32, 32))
    for _ in range(25):
        r.add_node("models/box", 1)
    r.add_camera()
    with pytest.raises(_capi.PBRError) as e:
        r.setup_environment()
    assert "nodes" in str(e.value)


def test_tile_cull_with_sheared_transforms(cuda, oracle):
    """Instances given as general (sheared, non-uniformly scaled) matrices: the
    tile kernel's instance cull must stay conservative."""
    n, inst = 8, 40
    r = pbr.PBRRenderer(num_scenes=n, tile_resolution=(96, 96), raster_kernel="tile", raster_threads=128)
    node = r.add_node("icosphere:1", inst, model_pivot_relative_point=(0.5, 0.5, 0.5))
    g = torch.Generator().manual_seed(9)
    B = node.buf_instances
    M = torch.eye(4).repeat(B, 1, 1)
    M[:, :3, :3] = torch.eye(3) * 0.6 + (torch.rand((B, 3, 3), generator=g) - 0.5) * 1.2  # shear + stretch
    M[:, :3, 3] = torch.rand((B, 3), generator=g) * 10 - 5
    node.set_transforms(M)
    node.set_colors(torch.rand((B, 4), generator=g))
    r.add_camera(fov_y_deg=60.0)
    r._pbr_cam.set_positions_and_lookat(torch.tensor([0.0, -9.0, 0.0]), torch.tensor([0.0, 0.0, 0.0]))
    r.add_light()
    r.setup_environment()
    check_parity(r, oracle, depth_tol=1e-4)


def test_capi_argument_errors(cuda):
    """Invalid texture, bounds and coordinate arguments are errors with a message."""
    import ctypes
    r = _cubes(2, (32, 32), inst=1)
    lib, ctx = r._lib, r._ctx
    buf = torch.zeros(64, dtype=torch.uint8, device="cuda")
    assert lib.pbr_node_set_texture(ctx, 0, ctypes.c_void_p(buf.data_ptr()), 0, 4) == _capi.PBR_ERR_INVALID
    assert b"texture size" in lib.pbr_last_error(ctx)
    assert lib.pbr_node_set_texture(ctx, 0, ctypes.c_void_p(buf.data_ptr() + 1), 2, 2) == _capi.PBR_ERR_INVALID
    assert lib.pbr_node_set_texture(ctx, 7, ctypes.c_void_p(buf.data_ptr()), 2, 2) == _capi.PBR_ERR_INVALID
    assert lib.pbr_mesh_set_bounds(ctx, 0, 0.0, 0.0, 0.0, -1.0) == _capi.PBR_ERR_INVALID
    assert lib.pbr_mesh_set_bounds(ctx, 0, float("nan"), 0.0, 0.0, 1.0) == _capi.PBR_ERR_INVALID
    assert lib.pbr_mesh_set_uv(ctx, 0, ctypes.c_void_p(buf.data_ptr() + 4)) == _capi.PBR_ERR_INVALID
    assert lib.pbr_mesh_set_uv(ctx, 3, None) == _capi.PBR_ERR_INVALID
    # the context still renders afterwards
    assert r.render().shape == (2, 3, 32, 32)
