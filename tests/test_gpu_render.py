"""Hard-raster parity: the CUDA renderer (through the C ABI) against the FP64
oracle (oracle/raster_ref.c) on the same seeded scenes.

Bar: winner (which triangle covers the pixel, i.e. coverage and
depth order) identical to the oracle except at pixels the oracle flags as
ambiguous (centre within 1e-4 px of an edge of a visible triangle, or two
fragments within 2e-6 in window depth); colour within 1/255 per channel on
>= 99.5 % of all pixels and on every unambiguous pixel; window depth within
1e-5 on unambiguous covered pixels.
"""
import math

import numpy as np
import pytest
import torch

import pybatchrender_gb300 as pbr
from pybatchrender_gb300 import workloads
from pybatchrender_gb300.envs.cartpole import CartPoleConfig, CartPoleRenderer

pytestmark = pytest.mark.gpu


def check_parity(r, oracle, *, depth_tol=1e-5, min_within_1=0.995, **render_kw):
    pix, depth, win = r.render(return_depth=True, return_winner=True, **render_kw)
    torch.cuda.synchronize()
    sc, me, no = r.export_scene()
    ref = oracle.render_hard(sc, me, no, want_depth=True, want_winner=True, want_ambiguous=True)
    gpu = {"pixels": pix.cpu().numpy(), "winner": win.cpu().numpy(), "depth": depth.cpu().numpy()}
    cmp = oracle.compare_hard(gpu, ref)
    assert cmp["winner_mismatch"] == 0, cmp
    assert cmp["color_max_diff_unambiguous"] <= 1, cmp
    assert cmp["color_within_1"] >= min_within_1, cmp
    covered = (ref["winner"] >= 0) & ~ref["ambiguous"]
    if covered.any():
        assert np.abs(gpu["depth"] - ref["depth"])[covered].max() <= depth_tol, cmp
    bg = (ref["winner"] < 0) & ~ref["ambiguous"]
    assert np.all(gpu["depth"][bg] == 1.0)
    return cmp, gpu, ref


def test_cartpole_bench_256_parity(cuda, oracle):
    r = workloads.cartpole_bench(num_scenes=256, res=64, seed=1)
    r._step(workloads.cartpole_states(256, seed=2, device=cuda))
    cmp, gpu, ref = check_parity(r, oracle)
    assert (ref["winner"] >= 0).mean() > 0.002  # the scene is not empty (small objects by design)
    assert cmp["ambiguous"] < 0.01 * cmp["pixels"]


def test_reference_cartpole_scene_parity(cuda, oracle):
    """The reference's own CartPole scene (shared rail, cart, pole)."""
    r = CartPoleRenderer(CartPoleConfig(num_scenes=64))
    g = torch.Generator().manual_seed(3)
    st = torch.zeros((64, 4))
    st[:, 0] = torch.rand(64, generator=g) * 4 - 2
    st[:, 2] = torch.rand(64, generator=g) - 0.5
    r._step(st.to(cuda))
    check_parity(r, oracle)


def test_many_cubes_parity(cuda, oracle):
    r = workloads.many_cubes(num_scenes=16, res=128, instances=64, seed=4)
    check_parity(r, oracle)


@pytest.mark.parametrize("tri_cap", [0, 64])
def test_uneven_mixed_meshes_parity(cuda, oracle, tri_cap):
    """Smooth meshes (perspective-correct normals), per-scene counts, and with
    tri_cap=64 the multi-chunk path."""
    r = workloads.uneven(num_scenes=24, res=84, max_instances=24, seed=5, tri_cap=tri_cap)
    check_parity(r, oracle)


def test_plain_matches_batched(cuda, oracle):
    st = workloads.cartpole_states(64, seed=7, device=cuda)
    a = workloads.cartpole_bench(num_scenes=64, seed=6)
    b = workloads.cartpole_bench(num_scenes=64, seed=6, raster_method="plain")
    a._step(st)
    b._step(st.cpu())
    pa, da = a.render(return_depth=True)
    pb, db = b.render(return_depth=True)
    assert torch.equal(pa, pb)
    assert torch.equal(da, db)


@pytest.mark.parametrize("threads", [128, 256, 512])
@pytest.mark.parametrize("bin_px", [8, 16, 32])
@pytest.mark.parametrize("persistent", [False, True])
def test_launch_configs_bitwise_equal(cuda, threads, bin_px, persistent):
    r = workloads.many_cubes(num_scenes=8, res=96, instances=32, seed=8)
    ref = r.render().clone()
    r.cfg.raster_threads, r.cfg.bin_size, r.cfg.persistent = threads, bin_px, persistent
    r._build_context()
    assert torch.equal(r.render(), ref)


@pytest.mark.parametrize("threads", [224, 448])
def test_warp_kernel_block_sizes_bitwise_equal(cuda, threads):
    """The scene-per-warp kernel in blocks of 7 or 14 warps (one scene per
    warp either way) renders exactly what blocks of 4 warps render, through
    render() and the state-bound step."""
    st = workloads.cartpole_states(300, seed=28, device=cuda)
    a = workloads.cartpole_bench(num_scenes=300, seed=29, raster_kernel="warp", raster_threads=128)
    b = workloads.cartpole_bench(num_scenes=300, seed=29, raster_kernel="warp", raster_threads=threads)
    assert torch.equal(a.step(st).clone(), b.step(st))
    pa, da, wa = a.render(return_depth=True, return_winner=True)
    pb, db, wb = b.render(return_depth=True, return_winner=True)
    assert torch.equal(pa, pb) and torch.equal(da, db) and torch.equal(wa, wb)


def test_deterministic_and_graph_replay(cuda):
    r = workloads.cartpole_bench(num_scenes=128, seed=9, cuda_graph=True)
    st1 = workloads.cartpole_states(128, seed=10, device=cuda)
    st2 = workloads.cartpole_states(128, seed=11, device=cuda)
    e = workloads.cartpole_bench(num_scenes=128, seed=9)
    e._step(st1)
    ref1 = e.render().clone()
    e._step(st2)
    ref2 = e.render().clone()
    out1 = r.step(st1).clone()
    out2 = r.step(st2).clone()
    out1b = r.step(st1).clone()
    assert torch.equal(out1, ref1) and torch.equal(out2, ref2) and torch.equal(out1b, ref1)
    assert not torch.equal(ref1, ref2)


def test_autotune_keeps_output(cuda):
    r = workloads.many_cubes(num_scenes=8, res=64, instances=16, seed=12)
    before = r.render().clone()
    res = r.autotune()
    assert res["threads"] in (128, 256, 512) and res["bin_px"] in (8, 16, 32) and res["ms"] > 0
    assert torch.equal(r.render(), before)


def test_debug_transforms_match_oracle(cuda, oracle):
    r = workloads.many_cubes(num_scenes=4, res=32, instances=8, seed=13)
    node = r.cubes
    got = r.debug_transforms(node).cpu().numpy()
    want = oracle.instance_matrices(dict(node.export(), mesh=0))
    assert np.allclose(got, want, rtol=1e-5, atol=1e-5)
    # set_transforms keeps the reference's rotation / scale / translation split
    M = torch.tensor(want.copy())
    M[:, 0:3, 0:3] *= 1.5
    node.set_transforms(M)
    got2 = r.debug_transforms(node).cpu().numpy()
    assert np.allclose(got2, M.numpy(), rtol=1e-5, atol=1e-5)
    assert node.mode == 1


@pytest.mark.parametrize("channels", [1, 4])
def test_channel_counts(cuda, oracle, channels):
    r = workloads.cartpole_bench(num_scenes=16, seed=14, num_channels=channels)
    r.set_background_color(0.1, 0.2, 0.3, 0.5)
    r._step(workloads.cartpole_states(16, seed=15, device=cuda))
    cmp, gpu, ref = check_parity(r, oracle)
    assert gpu["pixels"].shape[1] == channels


def test_small_and_odd_images(cuda, oracle):
    for res in [(12, 10), (33, 17), (84, 84)]:
        r = pbr.PBRRenderer(num_scenes=5, tile_resolution=res)
        node = r.add_node("icosphere:2", 3, model_pivot_relative_point=(0.5, 0.5, 0.5))
        g = torch.Generator().manual_seed(16)
        node.set_positions(torch.rand((15, 3), generator=g) * 4 - 2)
        node.set_scales(torch.rand(15, generator=g) * 2 + 1)
        node.set_colors(torch.rand((15, 4), generator=g))
        r.add_camera(fov_y_deg=50)
        r._pbr_cam.set_positions_and_lookat([0.0, -9.0, 2.0], [0.0, 0.0, 0.0])
        r.add_light()
        r.setup_environment()
        check_parity(r, oracle)


def test_near_plane_clipping(cuda, oracle):
    """Camera inside a large cube and cubes crossing the near plane."""
    r = pbr.PBRRenderer(num_scenes=3, tile_resolution=(64, 64))
    big = r.add_node("models/box", 1, model_pivot_relative_point=(0.5, 0.5, 0.5), model_scale=6.0)
    small = r.add_node("models/box", 4, model_pivot_relative_point=(0.5, 0.5, 0.5))
    big.set_colors(torch.tensor([0.3, 0.6, 0.9, 1.0]))
    small.set_positions(torch.tensor([[0.0, 0.05, 0.0], [0.5, 1.0, 0.2], [-0.3, 2.0, -0.2], [0.0, -0.2, 0.5]]).repeat(3, 1))
    small.set_hprs(torch.rand((12, 3), generator=torch.Generator().manual_seed(17)) * 6)
    r.add_camera()
    r._pbr_cam.set_positions_and_lookat(torch.tensor([[0.0, -0.4, 0.0], [0.2, -0.5, 0.1], [0.0, 0.0, 0.0]]),
                                        torch.tensor([[0.0, 5.0, 0.0], [0.0, 5.0, 1.0], [1.0, 5.0, 0.0]]))
    r.add_light()
    # two-sided: the big cube is seen from inside, so its back faces are culled like GL does
    r.setup_environment()
    # window depth of near-plane-clipped triangles (vertices far off-screen) is
    # only good to ~1e-3 in FP32; coverage and depth order must still match
    cmp, gpu, ref = check_parity(r, oracle, depth_tol=1e-3)


def test_round_keeps_more_records_than_a_chunk(cuda, oracle):
    """Tile kernel: a round takes min(threads, chunk) source triangles, and
    every triangle of the fan crosses the near plane, so a round keeps two
    records per triangle, more than a chunk holds (256 threads with 256-triangle
    chunks, 512 with 256, 128 with 64).  The round is then placed in two
    halves, in draw order.  Against the oracle and against 256 threads with
    512-triangle chunks, where every round fits whole."""
    from pybatchrender_gb300.renderer import meshes
    # 320 copies of one triangle (two vertices in front of the eye, one behind it), each turned about the
    # vertical axis through (0, 3, 0) and moved along the view axis, so that the copies cross one another
    k = np.arange(320)
    shift = ((k * 37) % 64) * 0.02
    th = 0.15 * ((k * 13) % 7 - 3)
    base = np.array([[-2.0, 0.0, -2.0], [2.0, 0.0, -2.0], [0.0, -6.0, 2.0]])
    pos = np.empty((320, 3, 3), np.float32)
    pos[:, :, 0] = np.cos(th)[:, None] * base[:, 0] - np.sin(th)[:, None] * base[:, 1]
    pos[:, :, 1] = np.sin(th)[:, None] * base[:, 0] + np.cos(th)[:, None] * base[:, 1] + (3.0 + shift)[:, None]
    pos[:, :, 2] = base[:, 2]
    nrm = np.cross(pos[:, 1] - pos[:, 0], pos[:, 2] - pos[:, 0])
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    fan = meshes.Mesh(pos.reshape(-1, 3), np.repeat(nrm, 3, 0), np.arange(960).reshape(-1, 3), name="fan")
    out = []
    for threads, cap in ((256, 512), (256, 256), (512, 256), (128, 64)):
        r = pbr.PBRRenderer(num_scenes=2, tile_resolution=(64, 64), raster_kernel="tile", raster_threads=threads,
                            tri_cap=cap)
        node = r.add_node(fan, 1)
        node.set_colors(torch.tensor([[0.9, 0.5, 0.2, 1.0], [0.2, 0.7, 0.4, 1.0]]))
        r.add_camera()
        r._pbr_cam.set_positions_and_lookat(torch.tensor([[0.0, -0.4, 0.0], [0.1, -0.4, -0.1]]),
                                            torch.tensor([[0.0, 5.0, 0.0], [0.0, 5.0, -0.3]]))
        r.add_light()
        r.setup_environment()
        cmp, gpu, ref = check_parity(r, oracle, depth_tol=1e-3)
        # the fan faces the eye and covers most of the image, with many copies winning somewhere
        assert (ref["winner"] >= 0).mean() > 0.9 and len(np.unique(ref["winner"])) > 10, cmp
        out.append(gpu)
    for other in out[1:]:
        for key in ("pixels", "winner", "depth"):
            assert np.array_equal(out[0][key], other[key])


def test_empty_and_degenerate_inputs(cuda, oracle):
    # no nodes at all: background everywhere
    r = pbr.PBRRenderer(num_scenes=2, tile_resolution=(32, 32))
    r.set_background_color(0.25, 0.5, 0.75)
    r.setup_environment()
    out = r.render()
    assert torch.all(out[:, 0] == 64) and torch.all(out[:, 1] == 128) and torch.all(out[:, 2] == 191)
    # NaN / inf poses and zero scale draw nothing and do not fault
    r = pbr.PBRRenderer(num_scenes=4, tile_resolution=(32, 32))
    n = r.add_node("models/box", 2)
    pos = torch.zeros((8, 3))
    pos[0, 0] = float("nan")
    pos[1, 1] = float("inf")
    n.set_positions(pos)
    sc = torch.ones(8)
    sc[2] = 0.0
    n.set_scales(sc)
    r.add_camera()
    r.setup_environment()
    check_parity(r, oracle)
    # zero active instances
    n.set_active_counts(torch.zeros(4, dtype=torch.int32))
    assert torch.all(r.render() == 0)


def test_env_step_renders(cuda):
    env = pbr.envs.make("CartPole-v0", num_scenes=32)
    td = env.reset()
    assert td["pixels"].shape == (32, 3, 64, 64) and td["pixels"].dtype == torch.uint8
    td["action"] = env.action_spec.rand()
    td = env.step(td)
    assert td["next", "pixels"].shape == (32, 3, 64, 64)
    assert td["next", "pixels"].float().mean() > 0


@pytest.mark.parametrize("kernel", ["warp", "tile"])
def test_cartpole_both_kernels_parity(cuda, oracle, kernel):
    r = workloads.cartpole_bench(num_scenes=96, res=64, seed=21, raster_kernel=kernel)
    r._step(workloads.cartpole_states(96, seed=22, device=cuda))
    check_parity(r, oracle)


def test_warp_and_tile_kernels_bitwise_equal(cuda):
    st = workloads.cartpole_states(200, seed=23, device=cuda)
    # pixels and winners identical; window depth equal up to FMA contraction
    # differences between the two kernel bodies
    outs = []
    for kernel in ("warp", "tile"):
        r = workloads.cartpole_bench(num_scenes=200, res=64, seed=24, raster_kernel=kernel)
        r._step(st)
        outs.append(r.render(return_depth=True, return_winner=True))
    (pa, da, wa), (pb, db, wb) = outs
    assert torch.equal(pa, pb) and torch.equal(wa, wb)
    assert torch.allclose(da, db, rtol=0, atol=1e-6)
    outs = []
    for kernel in ("warp", "tile"):
        r = CartPoleRenderer(CartPoleConfig(num_scenes=40, raster_kernel=kernel))
        r._step(st[:40])
        outs.append(r.render(return_depth=True))
    assert torch.equal(outs[0][0], outs[1][0])
    assert torch.allclose(outs[0][1], outs[1][1], rtol=0, atol=1e-6)


@pytest.mark.parametrize("res", [(48, 20), (16, 16), (96, 40)])
def test_warp_kernel_ragged_bins(cuda, oracle, res):
    """Widths that are multiples of 16 but not of 32, heights not multiple of 16."""
    r = pbr.PBRRenderer(num_scenes=7, tile_resolution=res, raster_kernel="warp")
    node = r.add_node("models/box", 3, model_pivot_relative_point=(0.5, 0.5, 0.5))
    g = torch.Generator().manual_seed(25)
    node.set_positions(torch.rand((21, 3), generator=g) * 3 - 1.5)
    node.set_hprs(torch.rand((21, 3), generator=g) * 6.3)
    node.set_colors(torch.rand((21, 4), generator=g))
    r.add_camera(fov_y_deg=50)
    r._pbr_cam.set_positions_and_lookat([0.0, -7.0, 1.0], [0.0, 0.0, 0.0])
    r.add_light()
    r.set_background_color(0.2, 0.3, 0.4)
    r.setup_environment()
    check_parity(r, oracle)


def test_plain_tile_kernel_matches(cuda):
    st = workloads.cartpole_states(32, seed=26)
    a = workloads.cartpole_bench(num_scenes=32, seed=27, raster_kernel="tile")
    b = workloads.cartpole_bench(num_scenes=32, seed=27, raster_method="plain", raster_kernel="tile")
    a._step(st.to(cuda))
    b._step(st)
    assert torch.equal(a.render(), b.render())


def test_steering_env_renders_and_matches_oracle(cuda, oracle):
    """Steering-v0: reset builds the obstacle spheres, the camera follows the
    player; the rendered scene passes the parity bar against the oracle, and
    a rebuild on the next reset replaces the obstacle node."""
    env = pbr.envs.make("Steering-v0", num_scenes=16, number_of_obstacles=20)
    td = env.reset()
    assert td["pixels"].shape == (16, 3, 64, 64)
    td["action"] = env.action_spec.rand()
    td = env.step(td)
    pix = td["next", "pixels"]
    assert pix.float().mean() > 0
    r = env._renderer
    # Coverage and colour must match exactly; depth is checked per node below.
    cmp, gpu, ref = check_parity(r, oracle, depth_tol=1.0)
    # The 1012-unit rails run from behind the camera (near plane 0.5) to the far
    # plane (1000): their near-clipped vertices carry fp32 rounding of about
    # 1e-4 relative, and close to the near plane the window depth changes by
    # up to ~0.1 per pixel, so rail depths differ from the FP64 oracle by up to
    # a few 1e-3.  Every other node keeps the 1e-5 bar.
    max_tris = max(n.mesh.num_triangles for n in r.geometry_nodes())
    rank = ref["winner"] // max_tris
    covered = (ref["winner"] >= 0) & ~ref["ambiguous"]
    rail = covered & ((rank == 1) | (rank == 2))
    other = covered & ~rail
    derr = np.abs(gpu["depth"] - ref["depth"])
    assert other.any() and rail.any()
    assert derr[other].max() <= 1e-5, (derr[other].max(), np.unique(rank[other & (derr > 1e-5)]))
    assert derr[rail].max() <= 5e-3, derr[rail].max()
    first = env._renderer.sphere_node
    env.reset()
    assert env._renderer.sphere_node is not first and first not in env._renderer.geometry_nodes()


def test_save_batch_snapshots(cuda, tmp_path):
    """save_batch_examples / save_batch_gif on rendered CartPole frames."""
    from pybatchrender_gb300.imagefile import make_grid
    from pybatchrender_gb300.renderer import textures
    from tests.test_imagefile_cpu import _gif_decode

    env = pbr.envs.make("CartPole-v0", num_scenes=9)
    td = env.reset()
    path, data = env.save_batch_examples(pixels=td["pixels"], num=9, scale=2, out_dir=str(tmp_path),
                                         return_bytes=True)
    img = textures.decode_png(data)
    assert np.array_equal(img[..., :3], make_grid(td["pixels"], num=9, scale=2))
    path, data = env.save_batch_gif(num_steps=6, frame_interval=3, num=4, scale=1, out_dir=str(tmp_path),
                                    return_bytes=True)
    frames, delays, loop = _gif_decode(data)
    assert len(frames) == 3 and frames[0].shape == (128, 128, 3) and loop == 0
    assert frames[0].max() > 0
