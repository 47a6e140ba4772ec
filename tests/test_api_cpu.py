"""Host-side API behaviour (CPU only): registry, node/camera/light setters,
error conventions, and that rendering without a CUDA device fails loudly."""
import os
import warnings

import numpy as np
import pytest
import torch

import pybatchrender_gb300 as pbr
from pybatchrender_gb300 import envs, workloads
from pybatchrender_gb300.env import PBREnv, TensorDictLite
from pybatchrender_gb300.envs.cartpole import CartPoleConfig, CartPoleEnv, CartPoleRenderer
from pybatchrender_gb300.renderer import meshes


def test_public_names():
    for name in ("PBRConfig", "PBRRenderer", "PBRNode", "PBRCam", "PBRLight", "PBRShaderContext", "PBREnv", "envs"):
        assert getattr(pbr, name) is not None
    assert pbr.GPUFrameGrabber is None and pbr.CPUFrameGrabber is None


def test_registry():
    assert "CartPole-v0" in envs.list_envs() and envs.is_registered("CartPole-v0")
    env_cls, r_cls, c_cls = envs.get_env_classes("CartPole-v0")
    assert (env_cls, r_cls, c_cls) == (CartPoleEnv, CartPoleRenderer, CartPoleConfig)
    with pytest.raises(ValueError):
        envs.get_env_classes("Nope-v0")
    with pytest.raises(ValueError):
        envs.make("Nope-v0")
    envs.register("Tmp-v0", CartPoleEnv, CartPoleRenderer, CartPoleConfig)
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        envs.register("Tmp-v0", CartPoleEnv, CartPoleRenderer, CartPoleConfig)
        assert any("already registered" in str(x.message) for x in w)
    envs.unregister("Tmp-v0")
    assert not envs.is_registered("Tmp-v0")


def test_rendering_without_cuda_raises():
    r = workloads.cartpole_bench(num_scenes=4, device="cpu")
    with pytest.raises(pbr.RendererUnavailable):
        r.step(workloads.cartpole_states(4, seed=0))
    with pytest.raises(pbr.RendererUnavailable):
        r.render_soft()


def test_node_setter_semantics():
    r = pbr.PBRRenderer(num_scenes=3, device="cpu")
    n = r.add_node("models/box", 2)
    assert n.buf_instances == 6 and n.total_instances == 6
    n.set_positions(torch.tensor([1.0, 2.0, 3.0]))  # a single row broadcasts
    assert torch.equal(n.pos, torch.tensor([[1.0, 2.0, 3.0]]).repeat(6, 1))
    n.set_positions(np.arange(24, dtype=np.float32).reshape(8, 3))  # extra rows are ignored
    assert torch.equal(n.pos, torch.arange(18, dtype=torch.float32).reshape(6, 3))
    n.set_scales(2.5)
    assert torch.all(n.scale == 2.5)
    n.set_hprs(torch.zeros((6, 3)))
    n.set_colors([0.1, 0.2, 0.3, 1.0])
    assert torch.allclose(n.color[3], torch.tensor([0.1, 0.2, 0.3, 1.0]))
    M = n.get_transforms()
    assert torch.allclose(M[:, :3, :3], torch.eye(3).expand(6, 3, 3) * 2.5)
    s = pbr.PBRRenderer(num_scenes=3, device="cpu").add_node("models/box", 2, shared_across_scenes=True)
    assert s.buf_instances == 2
    with pytest.raises(NotImplementedError):
        r.add_node("models/box", 1, backend="loop")
    with pytest.raises(FileNotFoundError):
        r.add_node("models/box", 1, texture="no_such_texture.png")
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        r.add_node("models/box", 1, positions=torch.zeros(3))
        assert any("ignored" in str(x.message) for x in w)
    empty = r.add_node(None, 1)
    empty.set_positions(torch.zeros(3))  # no geometry: a no-op
    assert not empty.has_geometry
    with pytest.raises(NotImplementedError):
        n.reparent_to(empty)


def test_camera_errors_and_light():
    r = pbr.PBRRenderer(num_scenes=4, device="cpu")
    cam = r.add_camera()
    with pytest.raises(ValueError):
        cam.set_eye(torch.zeros((3, 3)))
    with pytest.raises(ValueError):
        cam.set_eye(torch.zeros((4, 2)))
    with pytest.raises(NotImplementedError):
        cam.set_positions(torch.zeros(3), keep_lookat=True)
    cam.set_projection(fov_y_deg=30.0)
    assert cam.P_k44[1, 1] == pytest.approx(1.0 / np.tan(np.radians(15.0)), rel=1e-6)
    light = r.add_light(strength=0.5)
    light.set_ambient((0.3, 0.3, 0.3))
    assert light.ambient == (0.3, 0.3, 0.3) and light.strength == 0.5


def test_meshes_and_baking():
    box = meshes.resolve_model("models/box")
    assert box.num_vertices == 24 and box.num_triangles == 12 and not box.smooth
    assert meshes.cylinder(64).num_triangles == 256 and meshes.icosphere(3).num_triangles == 1280
    b = meshes.bake(box, (0.1, 0.1, 2.0), None, (0.5, 0.5, 0.05))
    lo, hi = b.tight_bounds()
    assert np.allclose(lo, [-0.05, -0.05, -0.1]) and np.allclose(hi, [0.05, 0.05, 1.9])
    a = meshes.bake(box, 0.3, None, None, "absolute")
    assert np.allclose(a.tight_bounds()[1] - a.tight_bounds()[0], 0.3)
    with pytest.raises(ValueError):
        meshes.bake(box, (1.0, 2.0), None, None)
    with pytest.raises(FileNotFoundError):
        meshes.resolve_model("models/teapot")
    assert meshes.resolve_model("models/smiley").num_triangles == 320  # untextured sphere stand-in


def test_env_without_renderer_pixels():
    cfg = CartPoleConfig(num_scenes=8, device="cpu", render=False)
    r = CartPoleRenderer(cfg)
    env = CartPoleEnv(r, cfg)
    td = env.reset()
    assert td["observation"].shape == (8, 4) and "pixels" not in td
    td["action"] = env.action_spec.rand()
    td = env.step(td)
    nxt = td["next"]
    assert nxt["observation"].shape == (8, 4) and nxt["reward"].shape == (8, 1)
    assert nxt["done"].dtype == torch.bool


def test_tensordict_lite_nested_keys():
    td = TensorDictLite({"a": torch.zeros(2)}, batch_size=[2])
    td[("next", "b")] = torch.ones(2)
    assert torch.equal(td["next", "b"], torch.ones(2)) and td.get("missing") is None


def test_atlas_roundtrip():
    r = pbr.PBRRenderer(num_scenes=5, tile_resolution=(8, 6), device="cpu")
    pix = torch.randint(0, 255, (5, 3, 6, 8), dtype=torch.uint8)
    atlas = r.to_atlas(pix)
    assert atlas.shape == (2 * 6, 3 * 8, 3)
    assert torch.equal(r._rearrange_img(atlas), pix)


def test_bind_state_validation():
    r = workloads.cartpole_bench(num_scenes=4, res=32, device="cpu")
    assert {(b[1], b[2]) for b in r._state_bindings} == {(0, 0), (4, 2)}
    r.bind_state(r.cart, "y", 1)
    assert (r.cart, 1, 1) in r._state_bindings
    r.bind_state(r.cart, "y", 3)  # rebinding replaces
    assert (r.cart, 1, 1) not in r._state_bindings and (r.cart, 1, 3) in r._state_bindings
    with pytest.raises(KeyError):
        r.bind_state(r.cart, "w", 0)
    with pytest.raises(ValueError):
        r.bind_state(r.cart, 6, 0)
    with pytest.raises(ValueError):
        r.bind_state(r.cart, "x", -1)
    # no CUDA context: the fused path is never taken
    assert r._bound_state((torch.zeros(4, 4),), {}) is None


def test_steering_env_dynamics_cpu():
    """Steering-v0 without pixels: obstacle layout, forward motion, passages
    speed the player up, a collision outside the grace period is penalised."""
    env = envs.make("Steering-v0", num_scenes=4, device="cpu", render=False, number_of_obstacles=5,
                    distance_to_first_obstacle=2.0, obstacle_y_spacing=3.0)
    td = env.reset()
    obs = td["observation"]
    assert obs.shape == (4, 6)
    ob = env._obstacles
    assert ob.shape == (4, 5, 4)
    assert torch.allclose(ob[0, :, 1], torch.tensor([2.0, 5.0, 8.0, 11.0, 14.0]))
    assert set(ob[:, :, 0].unique().tolist()) <= set(float(v) for v in range(-11, 12, 2))
    # put every player on the first obstacle's lane: the first passage is a hit
    env._player_x = ob[:, 0, 0].clone()
    td = pbr.env.TensorDict({"observation": env._get_observation(), "action": torch.zeros(4, 1),
                             "step_count": torch.zeros(4, dtype=torch.long)}, batch_size=[4])
    y0 = env._player_y.clone()
    nxt = env._step(td)
    assert torch.allclose(env._player_y, y0 + 96.0 / 60.0)  # speed_initial * tau, one step
    assert (nxt["reward"] == 0.0).all()  # y = 1.6: the first obstacle (y = 2) is not passed yet
    nxt = env._step(pbr.env.TensorDict({"observation": nxt["observation"], "action": torch.zeros(4, 1),
                                        "step_count": nxt["step_count"]}, batch_size=[4]))
    assert (nxt["reward"] == -1.0).all() and (nxt["observation"][:, 3] == 1.0).all()  # hit, grace active
    assert torch.allclose(env._forward_speed, torch.full((4,), 96.0 + 0.072 - 6.12))
    # a second hit inside the grace period is not penalised
    env._player_x = ob[:, 1, 0].clone()
    for _ in range(2):
        nxt = env._step(pbr.env.TensorDict({"observation": nxt["observation"], "action": torch.zeros(4, 1),
                                            "step_count": nxt["step_count"]}, batch_size=[4]))
    assert (nxt["reward"] == 0.0).all()
    a = env.action_spec.rand()
    assert a.shape == (4, 1) and (a.abs() <= 327.68).all()


def test_template_env_runs_cpu():
    """The template environment works as shipped (no pixels on the CPU)."""
    from pybatchrender_gb300.envs._template import MyEnv, MyEnvConfig, MyEnvRenderer
    envs.register("Template-v0", MyEnv, MyEnvRenderer, MyEnvConfig)
    try:
        env = envs.make("Template-v0", num_scenes=6, device="cpu", render=False, max_steps=5)
        td = env.reset()
        for _ in range(6):
            td["action"] = env.action_spec.rand()
            td = env.step(td)["next"]
        assert td["observation"].shape == (6, 2) and td["reward"].shape == (6, 1)
        assert int(td["step_count"].max()) < 5  # max_steps reached once: every scene was reset
    finally:
        envs.unregister("Template-v0")


def test_manual_camera_control_headless():
    r = pbr.PBRRenderer(num_scenes=2, device="cpu")
    cam = r.add_camera()
    r.enable_camera_control()  # no window: warns and switches the option off
    assert r.cfg.manual_camera_control is False
    eye0 = cam.get_eye().reshape(-1, 3).clone()
    r.set_key("w", True)
    r.set_key("a", True)
    r.update_camera(dt=0.1)
    eye1 = cam.get_eye().reshape(-1, 3)
    assert torch.allclose(eye1 - eye0, torch.tensor([[-2.5, 2.5, 0.0]]).expand(2, 3))


def test_report_fps_prints(capsys):
    r = pbr.PBRRenderer(num_scenes=10, device="cpu", report_fps_interval=0.0)
    r.report_fps()
    r.report_fps()
    out = capsys.readouterr().out
    assert out.startswith("FPS: ")
    q = pbr.PBRRenderer(num_scenes=10, device="cpu", report_fps=False)
    q.step(return_pixels=False)
    assert capsys.readouterr().out == ""


def test_mesh_clusters_bound_their_triangles():
    """Mesh.clusters(): each group of 32 consecutive triangles lies inside its
    bounding sphere, and every (non-degenerate) geometric face normal of the
    group lies inside its normal cone."""
    import numpy as np
    from pybatchrender_gb300.renderer import meshes
    for m in (meshes.icosphere(3), meshes.icosphere(2), meshes.cylinder(64), meshes.unit_cube()):
        cl = m.clusters().astype(np.float64)
        assert cl.shape == ((m.num_triangles + 31) // 32, 8)
        p = m.positions.astype(np.float64)
        f = m.indices
        fn = np.cross(p[f[:, 1]] - p[f[:, 0]], p[f[:, 2]] - p[f[:, 0]])
        for c in range(cl.shape[0]):
            sl = slice(32 * c, min(32 * (c + 1), m.num_triangles))
            pts = p[f[sl].ravel()]
            assert np.linalg.norm(pts - cl[c, :3], axis=1).max() <= cl[c, 3]
            if cl[c, 7] > 0:
                n = fn[sl] / np.linalg.norm(fn[sl], axis=1, keepdims=True)
                assert (n @ cl[c, 4:7]).min() >= cl[c, 7]

