"""Known-answer tests that pin the oracle's raster rules (CPU): the top-left
fill rule on edges through pixel centres, watertight shared edges (every
centre on a shared edge belongs to exactly one triangle), degenerate and
sliver triangles that cover no centre, exact window depth, back-face culling
and an analytically shaded face."""
import numpy as np
import pytest

from tests import kat_scenes as K


def _render(oracle, scene, meshes, nodes):
    return oracle.render_hard(scene, meshes, nodes, want_depth=True, want_winner=True, want_ambiguous=True)


def test_top_left_rule_square(oracle):
    mesh = K.screen_mesh(K.SQUARE, K.SQUARE_TRIS)
    ref = _render(oracle, K.scene(), [mesh], [K.node(0)])
    cov = ref["winner"][0] >= 0
    assert np.array_equal(cov, K.square_expected())
    # unlit: the colour is the instance colour
    px = ref["pixels"][0][:, cov]
    assert np.all(px[0] == K.unorm8(np.float32(0.8))) and np.all(px[1] == 102) and np.all(px[2] == 51)
    assert np.all(ref["depth"][0][cov] == 0.625) and np.all(ref["depth"][0][~cov] == 1.0)


def test_shared_diagonal_is_watertight(oracle):
    """Each half of the square alone: the two coverages are disjoint and their
    union is the square; the 7 centres on the diagonal go to one side only."""
    a = K.screen_mesh(K.SQUARE, [K.SQUARE_TRIS[0]])
    b = K.screen_mesh(K.SQUARE, [K.SQUARE_TRIS[1]])
    ca = _render(oracle, K.scene(), [a], [K.node(0)])["winner"][0] >= 0
    cb = _render(oracle, K.scene(), [b], [K.node(0)])["winner"][0] >= 0
    assert not np.any(ca & cb)
    assert np.array_equal(ca | cb, K.square_expected())
    diag = [(9 + i, 11 - i) for i in range(7)]  # (column, row) with centres on the diagonal
    assert sum(int(ca[r, c]) for c, r in diag) + sum(int(cb[r, c]) for c, r in diag) == 7


@pytest.mark.parametrize("corners", [
    [(4.5, 4.5), (12.5, 12.5), (20.5, 20.5)],        # collinear: zero area
    [(8.6, 20.6), (8.9, 20.6), (8.6, 4.6)],          # sliver between two columns of centres
    [(3.2, 3.7), (3.45, 3.7), (3.2, 3.95)],          # smaller than a pixel, no centre inside
])
def test_degenerate_and_sliver_cover_nothing(oracle, corners):
    mesh = K.screen_mesh(corners, [(0, 1, 2)])
    ref = _render(oracle, K.scene(), [mesh], [K.node(0)])
    assert not np.any(ref["winner"][0] >= 0)


def test_back_face_is_culled(oracle):
    mesh = K.screen_mesh(K.SQUARE, [(0, 2, 1), (0, 3, 2)])  # clockwise (y up): facing away
    ref = _render(oracle, K.scene(), [mesh], [K.node(0)])
    assert not np.any(ref["winner"][0] >= 0)


def test_nearer_triangle_wins_and_ties_keep_draw_order(oracle):
    near = K.screen_mesh(K.SQUARE, K.SQUARE_TRIS, z=-0.5)
    far = K.screen_mesh(K.SQUARE, K.SQUARE_TRIS, z=0.5)
    same = K.screen_mesh(K.SQUARE, K.SQUARE_TRIS, z=0.5)
    ref = _render(oracle, K.scene(), [far, near, same], [K.node(0), K.node(1, color=(0, 1, 0, 1)), K.node(2)])
    cov = K.square_expected()
    # winner id = rank * max_tris + triangle: rank 1 (the nearer node) everywhere in the square
    assert np.all(ref["winner"][0][cov] // 2 == 1)
    assert np.all(ref["depth"][0][cov] == 0.25)
    ref2 = _render(oracle, K.scene(), [far, same], [K.node(0), K.node(1)])
    assert np.all(ref2["winner"][0][cov] // 2 == 0)  # equal depth: the earlier drawn node keeps the pixel


def test_lit_face_colour(oracle):
    """A unit square facing the light head-on: colour * (ambient + 1 * light colour)."""
    mesh = K.screen_mesh(K.SQUARE, K.SQUARE_TRIS)
    sc = K.scene(strength=1.0, ambient=K.FACE_AMBIENT, ldir=(0.0, 0.0, 2.0), lcol=(1.0, 1.0, 1.0))
    ref = _render(oracle, sc, [mesh], [K.node(0, color=K.FACE_COLOR)])
    cov = ref["winner"][0] >= 0
    assert cov.sum() == 64
    for c in range(3):
        assert np.all(ref["pixels"][0][c][cov] == K.FACE_EXPECT[c])
    assert K.FACE_EXPECT == (122, 184, 245)


def test_soft_coverage_known_answers(oracle):
    """Soft mode on the square (sigma = 0.5 / (2 ln 9) px, coverage cut off 16
    sigma outside a triangle): a centre on one edge and far from the others is
    half covered (sigmoid(0) = 1/2), a centre well inside is fully covered,
    a centre beyond the cut-off sees only the background."""
    mesh = K.screen_mesh(K.SQUARE, K.SQUARE_TRIS)
    out = oracle.render_soft(K.scene(), [mesh], [K.node(0)], out_dtype=np.float64)[0]
    col = np.array([0.8, 0.4, 0.2], np.float32).astype(np.float64)
    assert np.allclose(out[:, 8, 8], 0.5 * col, rtol=0, atol=1e-7)     # (8.5, 8.5): on the left edge
    assert np.allclose(out[:, 4, 12], 0.5 * col, rtol=0, atol=1e-7)    # (12.5, 4.5): on the top edge
    assert np.allclose(out[:, 7, 10], col, rtol=0, atol=1e-6)          # 2 px or more from every edge
    assert np.all(out[:, 2, 2] == 0.0) and np.all(out[:, 20, 25] == 0.0)  # beyond the cut-off
