"""Generate the golden fixtures of this directory from the reference itself.

Runs the reference's unmodified Python scene code (imported from the reference
checkout at ``/root/reference``) under the stand-ins of ``stub_panda3d.py`` and
records what it would upload to OpenGL.  The fixtures pin everything before
rasterisation: baked vertices, per-instance model matrices and colours,
per-scene view-projection matrices, tile rectangles, shader uniforms and the
``PBRConfig`` resolution bookkeeping.  Usage (from the repository root):

    python tests/golden/make_golden.py [/path/to/reference]
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


def main(ref_path: str) -> None:
    pbr, cp = import_reference(ref_path)
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
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
