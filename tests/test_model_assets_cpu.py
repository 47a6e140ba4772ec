"""The model files the reference ships -- ``models/cone.egg`` and the Steering
rails' ``models/cylinder/scene.gltf`` (+ ``scene.bin``) -- loaded by this
package's loaders from the recorded bytes, found through the model search path
(``PBR_MODEL_PATH``) as the reference's Steering renderer finds them in its
package directory (``envs/steering/renderer.py:89-108``).  The counts and
bounds they must have are read from the files themselves by the fixture
generator, independently of the loaders."""
import os
import re

import numpy as np
import pytest

from pybatchrender_gb300.renderer import meshes
from tests import model_assets


@pytest.fixture
def model_dir(tmp_path, monkeypatch):
    d = model_assets.unpack(str(tmp_path))
    monkeypatch.setenv(meshes.MODEL_PATH_ENV, d)
    return d


def test_cylinder_gltf_loads_with_its_counts_and_bounds(model_dir):
    f = model_assets.facts()
    m = meshes.resolve_model("models/cylinder/scene.gltf")
    assert (m.num_vertices, m.num_triangles) == (int(f["cylinder_vertices"]), int(f["cylinder_triangles"])) == (226, 320)
    assert m.indices.min() >= 0 and m.indices.max() < m.num_vertices
    assert np.allclose(np.linalg.norm(m.normals, axis=1), 1.0, atol=1e-6)
    # the file is Y-up and its node matrices keep the cylinder's axis along Y; Panda3D's Z-up frame maps
    # glTF (x, y, z) to (x, -z, y)
    lo, hi = m.tight_bounds()
    gmin, gmax = f["cylinder_pos_min"], f["cylinder_pos_max"]
    assert np.allclose(lo, [gmin[0], -gmax[2], gmin[1]], atol=1e-4), lo
    assert np.allclose(hi, [gmax[0], -gmin[2], gmax[1]], atol=1e-4), hi
    # the extension may be left out, as with Panda3D's loader
    assert meshes.resolve_model("models/cylinder/scene").num_triangles == 320


def test_cone_egg_loads_with_its_counts_and_positions(model_dir):
    f = model_assets.facts()
    m = meshes.resolve_model("models/cone.egg")
    assert m.num_triangles == int(f["cone_triangles"]) == 62
    text = f["cone_egg"].tobytes().decode()
    # every loaded vertex is one of the file's <Vertex> positions (a polygon's vertices are copied per polygon)
    pool = np.array([[float(v) for v in blk.split()[:3]]
                     for blk in re.findall(r"<Vertex>\s*\d+\s*\{([^<]*)", text)], np.float32)
    assert len(pool) == int(f["cone_vertices"])
    d = np.abs(m.positions[:, None, :] - pool[None, :, :]).max(axis=2).min(axis=1)
    assert d.max() <= 1e-6
    lo, hi = m.tight_bounds()
    assert np.allclose(lo, pool.min(axis=0)) and np.allclose(hi, pool.max(axis=0))
    # every polygon's winding is kept: the triangle normals of the fan agree with the file's normals
    p = m.positions[m.indices]
    fn = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0])
    vn = m.normals[m.indices].sum(axis=1)
    assert np.all((fn * vn).sum(axis=1) > 0)


def test_model_files_not_found_fall_back_to_stand_ins(monkeypatch):
    monkeypatch.delenv(meshes.MODEL_PATH_ENV, raising=False)
    assert meshes.resolve_model("models/cylinder/scene.gltf").num_triangles == 256
    with pytest.raises(FileNotFoundError):
        meshes.resolve_model("models/no_such_model.egg")


def test_steering_rails_use_the_reference_rail_model(model_dir):
    """``SteeringConfig.border_model`` is the reference's ``models/cylinder/scene.gltf``;
    with the file on the model search path the rails are that mesh."""
    from pybatchrender_gb300.envs.steering import SteeringConfig, SteeringRenderer
    cfg = SteeringConfig(num_scenes=4, device="cpu")
    assert cfg.border_model == "models/cylinder/scene.gltf"
    r = SteeringRenderer(cfg)
    assert r.left_border.mesh.num_triangles == 320 and r.right_border.mesh.num_triangles == 320
    # absolute model scale: the rail spans rail_dimensions
    lo, hi = r.left_border.mesh.tight_bounds()
    assert np.allclose(hi - lo, cfg.rail_dimensions, rtol=1e-5)


@pytest.mark.skipif(not os.environ.get("PBR_REFERENCE_DIR"), reason="PBR_REFERENCE_DIR not set")
def test_fixture_bytes_equal_the_reference_files():
    f = model_assets.facts()
    base = os.path.join(os.environ["PBR_REFERENCE_DIR"], "pybatchrender", "models")
    for rel, key in (("cone.egg", "cone_egg"), ("cylinder/scene.gltf", "cylinder_gltf"),
                     ("cylinder/scene.bin", "cylinder_bin")):
        with open(os.path.join(base, rel), "rb") as fh:
            assert fh.read() == f[key].tobytes(), rel
