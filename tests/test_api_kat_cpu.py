"""Known answers through the public API on the CPU: unit cubes placed with
``add_node`` / ``add_camera`` / ``add_light`` exactly as a user would, exported
with ``export_scene`` and rasterised by the FP64 oracle.  The expected images
follow from the camera model alone (GL perspective, fov 40 degrees, eye
(0, -8, 0) looking at the origin, 64 x 64): a face of half-size 0.5 at
distance d spans 32 +- 0.5 / (d tan 20 deg) * 32 pixels, the faces turned
away from the eye are culled, and a flat face's colour is
colour * (ambient + n.l)."""
import math

import numpy as np
import pytest
import torch

import pybatchrender_gb300 as pbr
from tests import kat_scenes as K

T = math.tan(math.radians(20.0))
COLOR = (0.4, 0.6, 0.8, 1.0)


def _expected_span(d: float) -> tuple[int, int]:
    """First and last pixel column (or row) whose centre lies inside the
    face seen at distance d."""
    half = 0.5 / (d * T) * 32.0
    lo, hi = 32.0 - half, 32.0 + half
    first, last = math.ceil(lo - 0.5), math.floor(hi - 0.5)
    assert min(first + 0.5 - lo, hi - (last + 0.5)) > 1e-3  # no centre near an edge
    return first, last


@pytest.fixture(scope="module")
def cubes():
    r = pbr.PBRRenderer(num_scenes=3, tile_resolution=(64, 64), device="cpu")
    box = r.add_node("models/box", 1, model_pivot_relative_point=(0.5, 0.5, 0.5))
    cam = r.add_camera(fov_y_deg=40.0, z_near=0.05, z_far=100.0)
    cam.set_positions_and_lookat(torch.tensor([0.0, -8.0, 0.0]), torch.tensor([0.0, 0.0, 0.0]))
    r.add_light(ambient=(0.2, 0.2, 0.2), dir_dir=(0.0, -1.0, 0.0), dir_col=(1.0, 1.0, 1.0), strength=1.0)
    r.setup_environment()
    # scene 0: the cube at the origin; scene 1: 2.5 farther away; scene 2: turned 45 degrees about z
    box.set_positions(torch.tensor([[0.0, 0.0, 0.0], [0.0, 2.5, 0.0], [0.0, 0.0, 0.0]]))
    box.set_hprs(torch.tensor([[0.0, 0.0, 0.0], [0.0, 0.0, 0.0], [math.pi / 4, 0.0, 0.0]]))
    box.set_colors(torch.tensor([COLOR] * 3))
    return r.export_scene()


def test_front_face_square_and_colour(oracle, cubes):
    ref = oracle.render_hard(*cubes, want_winner=True, want_depth=True, want_ambiguous=True)
    for k, d in ((0, 7.5), (1, 10.0)):
        first, last = _expected_span(d)
        expect = np.zeros((64, 64), bool)
        expect[first:last + 1, first:last + 1] = True
        cov = ref["winner"][k] >= 0
        assert np.array_equal(cov, expect), k
        # the only centres within 1e-4 px of an edge lie on the face's shared diagonal (row + column = 63)
        rows, cols = np.nonzero(ref["ambiguous"][k])
        assert len(rows) == last - first + 1 and np.all(rows + cols == 63)
        for c in range(3):
            assert np.all(ref["pixels"][k][c][cov] == K.FACE_EXPECT[c])
            assert np.all(ref["pixels"][k][c][~cov] == 0)
        # GL window depth of the plane y = -0.5 at eye distance d
        zn, zf = 0.05, 100.0
        z_ndc = (zf + zn) / (zf - zn) - 2.0 * zf * zn / ((zf - zn) * d)
        assert np.allclose(ref["depth"][k][cov], 0.5 * z_ndc + 0.5, rtol=0, atol=2e-6)
    assert _expected_span(7.5) == (26, 37) and _expected_span(10.0) == (28, 35)


def test_turned_cube_shows_two_faces_lit_at_45_degrees(oracle, cubes):
    """Heading 45 degrees: the -y and the +x face both face the eye and both
    make 45 degrees with the light, so every covered pixel has the colour
    colour * (0.2 + cos 45 deg)."""
    ref = oracle.render_hard(*cubes, want_winner=True, want_ambiguous=True)
    win = ref["winner"][2]
    cov = win >= 0
    faces = np.unique(win[cov] // 2)  # two triangles per face
    assert len(faces) == 2
    ndl = math.cos(math.pi / 4)
    expect = [K.unorm8(np.float32(c) * (0.2 + ndl)) for c in COLOR[:3]]
    assert expect == [93, 139, 185]
    ok = cov & ~ref["ambiguous"][2]
    for c in range(3):
        assert np.all(ref["pixels"][2][c][ok] == expect[c])
    # the turned cube is wider than the front face alone: its silhouette spans the diagonal 0.5 * sqrt(2)
    cols = np.nonzero(cov.any(axis=0))[0]
    assert cols.max() - cols.min() + 1 > 12


def _floor_coverage(ndc_x, ndc_y, t, aspect, X, Y):
    """Analytic coverage of the floor quad |x| <= X, |y| <= Y, z = -1 seen
    from the origin looking along +y (up +z): the pixel ray
    d = (ndc_x t aspect, 1, ndc_y t) hits the floor at s = -1 / d_z."""
    dz = ndc_y * t
    with np.errstate(divide="ignore", invalid="ignore"):
        s = np.where(dz < 0, -1.0 / dz, np.inf)
    hx, hy = s * ndc_x * t * aspect, s
    return (dz < 0) & (np.abs(hx) <= X) & (hy <= Y)


def test_floor_through_the_near_plane(oracle):
    """A floor quad that reaches 20 units behind the camera (its far half is
    behind the eye, w < 0): near-plane clipping keeps exactly the pixels
    whose rays hit the quad in front of the camera; without clipping the
    vertices behind the eye would project to the wrong side of the image."""
    from pybatchrender_gb300.renderer.meshes import Mesh
    X, Y, res = 3.0, 20.0, 64
    r = pbr.PBRRenderer(num_scenes=1, tile_resolution=(res, res), device="cpu")
    pts = np.array([(-X, -Y, -1.0), (X, -Y, -1.0), (X, Y, -1.0), (-X, Y, -1.0)], np.float32)
    floor = r.add_node(Mesh(pts, np.tile([0.0, 0.0, 1.0], (4, 1)), [(0, 1, 2), (0, 2, 3)], name="floor"), 1)
    floor.set_colors(torch.tensor([[0.4, 0.6, 0.8, 1.0]]))
    cam = r.add_camera(fov_y_deg=60.0, z_near=0.05, z_far=100.0)
    cam.set_positions_and_lookat(torch.tensor([0.0, 0.0, 0.0]), torch.tensor([0.0, 1.0, 0.0]))
    r.add_light(strength=0.0)
    r.setup_environment()
    ref = oracle.render_hard(*r.export_scene(), want_winner=True, want_ambiguous=True)
    cov = ref["winner"][0] >= 0
    c = (np.arange(res) + 0.5) / res * 2 - 1
    nx, ny = c[None, :], -c[:, None]
    t = math.tan(math.radians(30.0))
    expect = _floor_coverage(nx, ny, t, 1.0, X, Y)
    # centres within 1e-3 px of the quad's outline are left out (the rule there is the fill rule's, tested elsewhere)
    e = 2e-3 / res
    stable = np.ones_like(expect)
    for dx, dy in ((e, 0), (-e, 0), (0, e), (0, -e)):
        stable &= _floor_coverage(nx + dx, ny + dy, t, 1.0, X, Y) == expect
    assert stable.mean() > 0.95
    assert np.array_equal(cov[stable], expect[stable])
    assert expect.sum() > 500 and not cov[: res // 2].any()  # the whole upper half (above the horizon) is empty
