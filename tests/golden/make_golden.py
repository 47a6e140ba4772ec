"""Generate the golden fixtures of this directory from the reference itself.

Runs the reference's unmodified Python scene code (imported from a reference
checkout whose path is given on the command line or in ``PBR_REFERENCE_DIR``)
under the stand-ins of ``stub_panda3d.py`` and records what it would upload to
OpenGL.  The fixtures pin everything before
rasterisation: baked vertices, per-instance model matrices and colours,
per-scene view-projection matrices, tile rectangles, shader uniforms and the
``PBRConfig`` resolution bookkeeping.  ``ref_env_dynamics.npz`` records
trajectories of the reference's CartPole and Steering environments
(observations, rewards, done flags and step counters) from seeded inputs, and
``ref_steering_scene.npz`` the Steering renderer's node buffers and cameras;
``ref_config_defaults.json`` holds the default of every configuration field
``ref_grid_frames.npz`` the snapshot grids of ``PBREnv._make_grid_frame`` and
``ref_defaults_scene.npz`` a scene built with every node, camera and light
argument left at its default.  ``ref_model_assets.npz`` holds the model files
the reference ships (``pybatchrender/models/cone.egg``, the Steering rails'
``pybatchrender/models/cylinder/scene.gltf`` with its ``scene.bin`` and
licence) byte for byte, with facts read from them independently of this
package's loaders: vertex and triangle counts and position bounds.  The
cylinder is "Cylinder" by username7777777
(https://sketchfab.com/3d-models/cylinder-679440db551840d2b4586e790228a12c),
licensed under CC-BY-4.0 (http://creativecommons.org/licenses/by/4.0/); the
cone is part of the reference (MIT licence, copyright 2025 Evgenii Rudakov
and contributors).  Usage (from the repository root):

    python tests/golden/make_golden.py /path/to/reference
    PBR_REFERENCE_DIR=/path/to/reference python tests/golden/make_golden.py
"""
from __future__ import annotations

import contextlib
import io
import json
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import scenes  # noqa: E402
import stub_panda3d  # noqa: E402


def import_reference(path: str):
    stub_panda3d.install()
    sys.path.insert(0, path)
    with contextlib.redirect_stdout(io.StringIO()):
        import pybatchrender  # noqa: F401
        import pybatchrender.envs.cartpole as cp  # noqa: F401
    return sys.modules["pybatchrender"], sys.modules["pybatchrender.envs.cartpole"]


def node_record(node, prefix: str) -> dict:
    B = node.buf_instances
    mats = node.matbuf.array((B, 4, 4)).transpose(0, 2, 1)  # column-packed -> row-major
    out = {f"{prefix}_M": mats, f"{prefix}_color": node.colbuf.array((B, 4)),
           f"{prefix}_verts": node.np.verts.astype(np.float32)}
    for k, v in node.np.shader_inputs.items():
        if isinstance(v, (int, float, tuple, list)):
            out[f"{prefix}_in_{k}"] = np.asarray(v, np.float64)
    return out


def camera_record(cam, N: int) -> dict:
    vp = cam.viewbuf.array((N, 4, 4)).transpose(0, 2, 1)
    return {"VP": vp, "tiles": cam.tilebuf.array((N, 4)), "P": cam.P_k44.numpy()}


def _jsonable(v):
    if isinstance(v, (tuple, list)):
        return [_jsonable(x) for x in v]
    if isinstance(v, (bool, int, float, str)) or v is None:
        return v
    return repr(v)


def cartpole_trajectory(cp, B: int = 64, T: int = 60) -> dict:
    """The reference's CartPoleEnv._step (no rendering, no auto-reset) from
    seeded states and actions: dynamics, termination (including the step
    limit) and reward."""
    env = cp.CartPoleEnv(renderer=None, cfg=cp.CartPoleConfig(num_scenes=B, device="cpu", render=False,
                                                               auto_reset=False))
    g = torch.Generator().manual_seed(11)
    u = lambda lo, hi: torch.rand(B, generator=g) * (hi - lo) + lo  # noqa: E731
    obs = torch.stack([u(-2.6, 2.6), u(-2.0, 2.0), u(-0.25, 0.25), u(-2.0, 2.0)], dim=-1)
    sc = torch.randint(0, 520, (B,), generator=g)
    actions = torch.randint(0, 2, (T, B), generator=g)
    rec = {"cp_obs0": obs.numpy(), "cp_sc0": sc.numpy(), "cp_actions": actions.numpy()}
    outs = {"observation": [], "reward": [], "done": [], "step_count": []}
    for t in range(T):
        td = env._step({"observation": obs, "step_count": sc, "action": actions[t]})
        for k in outs:
            outs[k].append(td[k].numpy())
        obs, sc = td["observation"], td["step_count"]
    rec.update({f"cp_{k}": np.stack(v) for k, v in outs.items()})
    return rec


def steering_trajectory(B: int = 32, T: int = 200) -> dict:
    """The reference's SteeringEnv._step (no rendering, no auto-reset) from a
    seeded world: 20 obstacles, a 300-step limit, continuous steering."""
    st = sys.modules["pybatchrender.envs.steering"]
    cfg = st.SteeringConfig(num_scenes=B, device="cpu", render=False, auto_reset=False, number_of_obstacles=20,
                            max_steps=300)
    env = st.SteeringEnv(renderer=None, cfg=cfg)
    g = torch.Generator().manual_seed(12)
    n = env.number_of_obstacles
    xs = torch.tensor(env.obstacle_x_positions, dtype=torch.float32)
    obstacles = torch.zeros(B, n, 4)
    obstacles[:, :, 0] = xs[torch.randint(0, len(xs), (B, n), generator=g)]
    obstacles[:, :, 1] = torch.arange(n, dtype=torch.float32) * env.obstacle_y_spacing + env.distance_to_first_obstacle
    obstacles[:, :, 2] = (torch.rand(B, n, generator=g) < env.prob_gold).float()
    obstacles[:, :, 3] = (torch.rand(B, n, generator=g) < env.prob_cone).float()
    player_x = torch.rand(B, generator=g) * (env.x_max - env.x_min) + env.x_min
    sc = torch.randint(0, 300, (B,), generator=g)
    actions = (torch.rand(T, B, 1, generator=g) * 2 - 1) * env.action_high
    rec = {"st_obstacles": obstacles.numpy(), "st_player_x0": player_x.numpy(), "st_sc0": sc.numpy(),
           "st_actions": actions.numpy()}
    env._obstacles = obstacles.clone()
    env._player_x = player_x.clone()
    env._player_y = torch.zeros(B)
    env._prev_player_x = torch.zeros(B)
    env._prev_player_y = torch.zeros(B)
    env._forward_speed = torch.full((B,), env.speed_initial)
    env._grace_remaining = torch.zeros(B)
    env._next_obstacle_idx = torch.zeros(B, dtype=torch.long)
    obs = env._get_observation()
    rec["st_obs0"] = obs.numpy()
    outs = {"observation": [], "reward": [], "done": [], "step_count": []}
    grace, idx = [], []
    for t in range(T):
        td = env._step({"observation": obs, "step_count": sc, "action": actions[t]})
        for k in outs:
            outs[k].append(td[k].numpy())
        grace.append(env._grace_remaining.numpy().copy())
        idx.append(env._next_obstacle_idx.numpy().copy())
        obs, sc = td["observation"], td["step_count"]
    rec.update({f"st_{k}": np.stack(v) for k, v in outs.items()})
    rec["st_grace"], rec["st_next_idx"] = np.stack(grace), np.stack(idx)
    return rec


def steering_scene(B: int = 8, n: int = 20) -> dict:
    """The reference's SteeringRenderer: build_obstacles on a seeded world,
    then two _step calls (the second with grace flags set).  Models other
    than the box load as the stand-in box: the instance matrices, colours
    and cameras recorded here do not depend on the mesh."""
    st = sys.modules["pybatchrender.envs.steering"]
    load_model = stub_panda3d.Loader.loadModel

    def any_model(self, path):
        try:
            return load_model(self, path)
        except FileNotFoundError:
            return stub_panda3d.NodePath(os.path.basename(str(path)), stub_panda3d._unit_box())
    stub_panda3d.Loader.loadModel = any_model
    try:
        r = st.SteeringRenderer(st.SteeringConfig(num_scenes=B, device="cpu"))
        g = torch.Generator().manual_seed(13)
        xs = torch.tensor(r.cfg.obstacle_x_position, dtype=torch.float32)
        obstacles = torch.zeros(B, n, 4)
        obstacles[:, :, 0] = xs[torch.randint(0, len(xs), (B, n), generator=g)]
        obstacles[:, :, 1] = torch.arange(n, dtype=torch.float32) * 12.0 + 6.0
        obstacles[:, :, 2] = (torch.rand(B, n, generator=g) < 0.3).float()
        r.build_obstacles(obstacles)
        rec = {"obstacles": obstacles.numpy()}
        for step in range(2):
            state = torch.rand(B, 6, generator=g) * torch.tensor([20.0, 300.0, 100.0, 1.0, 20.0, 300.0]) \
                - torch.tensor([10.0, 0.0, 0.0, 0.0, 10.0, 0.0])
            state[:, 3] = (state[:, 3] > 0.5).float() if step else 0.0
            r._step(state)
            rec[f"state{step}"] = state.numpy()
            for name, node in (("player", r.player_node), ("left", r.left_border), ("right", r.right_border),
                               ("sphere", r.sphere_node)):
                for k, v in node_record(node, f"s{step}_{name}").items():
                    if not k.endswith("_verts"):
                        rec[k] = v
            rec.update({f"s{step}_{k}": v for k, v in camera_record(r._pbr_cam, B).items()})
    finally:
        stub_panda3d.Loader.loadModel = load_model
    return rec


GRID_CASES = [  # (pixel batch shape, float pixels, indices, num)
    ((7, 3, 5, 4), False, None, 16),
    ((9, 3, 4, 6), False, [6, -1, 2, 100, 0], 3),
    ((5, 1, 3, 3), True, None, 4),
    ((2, 3, 3, 4, 4), False, [5, 1], 16),
    ((3, 4, 2, 2), False, None, 0),
]


def grid_frames(env_cls) -> dict:
    """The reference's PBREnv._make_grid_frame (scale 1: no PIL involved) on
    seeded pixel batches of GRID_CASES."""
    g = torch.Generator().manual_seed(14)
    rec = {}
    for i, (shape, as_float, indices, num) in enumerate(GRID_CASES):
        if as_float:
            pix = torch.rand(shape, generator=g) * 400.0 - 50.0
        else:
            pix = torch.randint(0, 256, shape, generator=g, dtype=torch.uint8)
        rec[f"pixels{i}"] = pix.numpy()
        rec[f"grid{i}"] = env_cls._make_grid_frame(None, pix, indices, num, 1)
    return rec


def model_assets(ref_path: str) -> dict:
    """The reference's model files, byte for byte, and facts about them read
    straight from the files: the egg's <Vertex> and <Polygon> entries (each
    polygon's vertex count, so the triangle count of a fan triangulation), and
    the glTF's accessor counts and the POSITION accessor's declared bounds."""
    import re
    models = os.path.join(ref_path, "pybatchrender", "models")
    rec = {}
    with open(os.path.join(models, "cone.egg"), "rb") as f:
        egg = f.read()
    rec["cone_egg"] = np.frombuffer(egg, np.uint8)
    text = egg.decode()
    rec["cone_vertices"] = len(re.findall(r"<Vertex>", text))
    polys = re.findall(r"<Polygon>\s*\{(.*?)<VertexRef>\s*\{([^}]*)\}", text, flags=re.S)
    sizes = [len(re.sub(r"<Ref>.*", "", refs, flags=re.S).split()) for _, refs in polys]
    rec["cone_polygon_sizes"] = np.asarray(sizes, np.int32)
    rec["cone_triangles"] = int(sum(n - 2 for n in sizes))
    cyl = os.path.join(models, "cylinder")
    for name, key in (("scene.gltf", "cylinder_gltf"), ("scene.bin", "cylinder_bin"),
                      ("license.txt", "cylinder_license")):
        with open(os.path.join(cyl, name), "rb") as f:
            rec[key] = np.frombuffer(f.read(), np.uint8)
    doc = json.loads(bytes(rec["cylinder_gltf"]).decode())
    prim = doc["meshes"][0]["primitives"][0]
    pos = doc["accessors"][prim["attributes"]["POSITION"]]
    rec["cylinder_vertices"] = int(pos["count"])
    rec["cylinder_triangles"] = int(doc["accessors"][prim["indices"]]["count"]) // 3
    rec["cylinder_pos_min"] = np.asarray(pos["min"], np.float64)
    rec["cylinder_pos_max"] = np.asarray(pos["max"], np.float64)
    return rec


def main(ref_path: str) -> None:
    np.savez_compressed(os.path.join(HERE, "ref_model_assets.npz"), **model_assets(ref_path))
    pbr, cp = import_reference(ref_path)
    np.savez_compressed(os.path.join(HERE, "ref_grid_frames.npz"), **grid_frames(pbr.PBREnv))
    with contextlib.redirect_stdout(io.StringIO()):
        import pybatchrender.envs.steering  # noqa: F401
        rec = cartpole_trajectory(cp)
        rec.update(steering_trajectory())
        np.savez_compressed(os.path.join(HERE, "ref_env_dynamics.npz"), **rec)
        np.savez_compressed(os.path.join(HERE, "ref_steering_scene.npz"), **steering_scene())
    with contextlib.redirect_stdout(io.StringIO()):
        for N, keep in ((5, None), (64, None), (4098, 16)):
            r = cp.CartPoleRenderer(cp.CartPoleConfig(num_scenes=N))
            st = scenes.cartpole_states(N, seed=N)
            r._step(st)
            rec = {"state": st.numpy(), "N": N, "tiles_cfg": np.asarray(r.cfg.tiles),
                   "window": np.asarray(r.cfg.window_resolution)}
            for name in ("rail", "cart", "pole"):
                rec.update(node_record(getattr(r, name), name))
            rec.update(camera_record(r._pbr_cam, N))
            if keep:  # store the first and last `keep` scenes only
                sel = np.r_[0:keep, N - keep:N]
                for k in list(rec):
                    if isinstance(rec[k], np.ndarray) and rec[k].ndim >= 1 and rec[k].shape[0] == N and k != "state":
                        rec[k] = rec[k][sel]
                rec["sel"] = sel
            np.savez_compressed(os.path.join(HERE, f"ref_cartpole_N{N}.npz"), **rec)

        r, snaps = scenes.api_scene(pbr)
        rec = {}
        for name, node in zip("abc", r.nodes_abc):
            rec.update(node_record(node, name))
            rec[f"{name}_shared_ips"] = np.asarray(node.instances_per_scene)
        rec.update(camera_record(r._pbr_cam, r.num_scenes))
        for label, vp in snaps:
            rec[f"snap_{label}"] = vp.numpy()
        light = r._pbr_light
        rec["light"] = np.asarray(light.ambient + light.dir_dir + light.dir_col + (light.strength,), np.float64)
        np.savez_compressed(os.path.join(HERE, "ref_api_scene.npz"), **rec)

        d = scenes.defaults_scene(pbr)
        rec = node_record(d.box, "box")
        rec.update(camera_record(d._pbr_cam, d.num_scenes))
        light = d._pbr_light
        rec["light"] = np.asarray(light.ambient + light.dir_dir + light.dir_col + (light.strength,), np.float64)
        cam = d._pbr_cam
        rec["cam_params"] = np.asarray([cam.fov_y_deg, cam.z_near, cam.z_far], np.float64)
        np.savez_compressed(os.path.join(HERE, "ref_defaults_scene.npz"), **rec)

    defaults = {}
    import dataclasses
    import pybatchrender.envs.steering as st
    for name, cls in (("PBRConfig", pbr.PBRConfig), ("CartPoleConfig", cp.CartPoleConfig),
                      ("SteeringConfig", st.SteeringConfig)):
        defaults[name] = {f.name: _jsonable(getattr(cls(device="cpu"), f.name)) for f in dataclasses.fields(cls)}
    with open(os.path.join(HERE, "ref_config_defaults.json"), "w") as f:
        json.dump(defaults, f, indent=1, sort_keys=True)

    cases = []
    for kw in scenes.CONFIG_CASES:
        try:
            c = pbr.PBRConfig(device="cpu", **kw)
            cases.append({"kwargs": {k: list(v) if isinstance(v, tuple) else v for k, v in kw.items()},
                          "tiles": list(c.tiles), "tile_resolution": list(c.tile_resolution),
                          "window_resolution": list(c.window_resolution), "num_scenes": c.num_scenes,
                          "batch_inner_dim": c.batch_inner_dim})
        except Exception as e:  # the reference's own error conventions
            cases.append({"kwargs": {k: list(v) if isinstance(v, tuple) else v for k, v in kw.items()},
                          "error": type(e).__name__})
    with open(os.path.join(HERE, "ref_config_cases.json"), "w") as f:
        json.dump(cases, f, indent=1)


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PBR_REFERENCE_DIR")
    if not ref:
        sys.exit("usage: make_golden.py <reference checkout> (or set PBR_REFERENCE_DIR)")
    main(ref)
