"""Known-answer tests that pin the oracle's raster rules (CPU): the top-left
fill rule on edges through pixel centres, watertight shared edges (every
centre on a shared edge belongs to exactly one triangle), degenerate and
sliver triangles that cover no centre, exact window depth, back-face culling,
an analytically shaded face, GL_LINEAR + GL_REPEAT texture sampling with
row 0 at v = 0, per-fragment renormalised smooth normals and
perspective-correct texture coordinates."""
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


def test_texture_bilinear_repeat_along_u(oracle):
    """A 2 x 1 texture (texel 0 black, texel 1 = 200) stretched over the
    square with u = 0 .. 1 left to right.  Pixel column c samples
    u = (c - 8) / 8, i.e. texel x = 2u - 0.5; GL_LINEAR with GL_REPEAT blends
    texel 1 into the left half-texel and the right half-texel wraps to texel 0."""
    mesh = K.textured_square([(0, 0), (1, 0), (1, 1), (0, 1)])
    nd = K.node(0, color=(1.0, 1.0, 1.0, 1.0))
    nd["texture"] = K.texture([[(0, 0, 0), (200, 100, 40)]])
    ref = _render(oracle, K.scene(), [mesh], [nd])
    cov = ref["winner"][0] >= 0
    assert np.array_equal(cov, K.square_expected())
    # texel x = -0.5, -0.25, 0, 0.25, 0.5, 0.75, 1, 1.25 -> weight of texel 1
    w1 = np.array([0.5, 0.25, 0.0, 0.25, 0.5, 0.75, 1.0, 0.75])
    for c, full in enumerate((200, 100, 40)):
        expect = np.floor(w1 * full + 0.5).astype(np.uint8)
        assert np.all(ref["pixels"][0][c][4:12, 8:16] == expect[None, :]), c


def test_texture_row_zero_is_at_the_bottom(oracle):
    """A 1 x 2 texture: row 0 (v = 0) is drawn at the bottom of the square.
    Pixel row r samples v = (12 - r) / 8, texel y = 2v - 0.5."""
    mesh = K.textured_square([(0, 0), (1, 0), (1, 1), (0, 1)])
    nd = K.node(0, color=(1.0, 1.0, 1.0, 1.0))
    nd["texture"] = K.texture([[(0, 200, 0)], [(200, 0, 0)]])
    ref = _render(oracle, K.scene(), [mesh], [nd])
    # rows 4..11: texel y = 1.5, 1.25, 1, 0.75, 0.5, 0.25, 0, -0.25 -> weight of row 1
    w1 = np.array([0.5, 0.75, 1.0, 0.75, 0.5, 0.25, 0.0, 0.25])
    red = np.floor(w1 * 200 + 0.5).astype(np.uint8)
    green = np.floor((1 - w1) * 200 + 0.5).astype(np.uint8)
    assert np.all(ref["pixels"][0][0][4:12, 8:16] == red[:, None])
    assert np.all(ref["pixels"][0][1][4:12, 8:16] == green[:, None])
    assert np.all(ref["pixels"][0][2][4:12, 8:16] == 0)


def test_texture_colour_is_modulated_by_instance_colour_and_light(oracle):
    """Texel colour times instance colour times (ambient + n.l light)."""
    mesh = K.textured_square([(0.5, 0.5)] * 4)  # one uv: the texel centre of a 1 x 1 texture
    nd = K.node(0, color=K.FACE_COLOR)
    nd["texture"] = K.texture([[(255, 255, 255)]])
    sc = K.scene(strength=1.0, ambient=K.FACE_AMBIENT, ldir=(0.0, 0.0, 2.0), lcol=(1.0, 1.0, 1.0))
    ref = _render(oracle, sc, [mesh], [nd])
    cov = ref["winner"][0] >= 0
    for c in range(3):
        assert np.all(ref["pixels"][0][c][cov] == K.FACE_EXPECT[c])
    nd["texture"] = K.texture([[(0, 255, 0)]])
    ref = _render(oracle, sc, [mesh], [nd])
    assert np.all(ref["pixels"][0][0][cov] == 0) and np.all(ref["pixels"][0][2][cov] == 0)
    assert np.all(ref["pixels"][0][1][cov] == K.FACE_EXPECT[1])


def test_smooth_normals_are_interpolated_and_renormalised(oracle):
    """Vertex normals (-1, 0, 1) on the left corners and (1, 0, 1) on the
    right: at pixel column c the fragment normal is (2t - 1, 0, 1) up to
    scale with t = (c - 8) / 8, so n.l = 1 / sqrt((2t - 1)^2 + 1) for a
    light along +z (per-fragment renormalisation, not a lerp of n.l)."""
    mesh = K.screen_mesh(K.SQUARE, K.SQUARE_TRIS)
    mesh.normals = np.array([(-1, 0, 1), (1, 0, 1), (1, 0, 1), (-1, 0, 1)], np.float32)
    sc = K.scene(strength=1.0, ambient=(0.0, 0.0, 0.0), ldir=(0.0, 0.0, 1.0), lcol=(1.0, 1.0, 1.0))
    ref = _render(oracle, sc, [mesh], [K.node(0, color=(1.0, 1.0, 1.0, 1.0))])
    t = (np.arange(8, 16) - 8) / 8.0
    ndl = 1.0 / np.sqrt((2 * t - 1) ** 2 + 1)
    expect = np.floor(ndl * 255 + 0.5)
    assert np.all(np.abs(ndl * 255 + 0.5 - np.round(ndl * 255 + 0.5)) > 1e-3)  # no value sits on a rounding tie
    for c in range(3):
        assert np.all(ref["pixels"][0][c][4:12, 8:16] == expect.astype(np.uint8)[None, :])
    # per-vertex n.l interpolated linearly would give 1/sqrt(2) at both edges and in between
    assert expect[4] == 255 and expect[0] == 180


def test_perspective_correct_texture_coordinates(oracle):
    """A quad whose right edge is twice as far as its left, textured with a
    64-texel ramp (texel i = 4 i): the sampled value at NDC x is
    256 u - 2 with u the perspective-correct coordinate, which differs from
    the screen-affine one by up to 43 levels in the middle of the quad."""
    mesh = K.perspective_quad()
    nd = K.node(0, color=(1.0, 1.0, 1.0, 1.0))
    ramp = [[(4 * i, 0, 0) for i in range(64)]]
    nd["texture"] = K.texture(ramp)
    ref = _render(oracle, K.scene(vp=K.PERSP_VP), [mesh], [nd])
    cov = ref["winner"][0] >= 0
    rows, cols = np.nonzero(cov)
    assert rows.min() == 8 and rows.max() == 23 and cols.min() == 8 and cols.max() == 23
    ndc_x = 2.0 * (np.arange(8, 24) + 0.5) / K.W - 1.0
    u = K.perspective_u(ndc_x)
    value = 256.0 * u - 2.0
    inner = (u * 64 - 0.5 >= 0) & (u * 64 - 0.5 <= 63)  # away from the repeat seam
    got = ref["pixels"][0][0][8:24, 8:24].astype(np.float64)
    assert np.all(np.abs(got[:, inner] - value[None, inner]) <= 0.5 + 1e-6)
    affine = 256.0 * (ndc_x + 0.5) - 2.0
    assert np.max(np.abs(affine - value)[inner]) > 40
    # window depth is the plane's: 0.5 (1 - 2 / z) + 0.5 with z = z0 + (z1 - z0) u
    z = K.PERSP_Z0 + (K.PERSP_Z1 - K.PERSP_Z0) * u
    assert np.allclose(ref["depth"][0][8:24, 8:24], (1.0 - 1.0 / z)[None, :], rtol=0, atol=1e-6)


def _jittered_grid(seed: int, cells: int = 4, size: float = 6.0, origin: float = 4.0):
    """A cells x cells grid of quads (two triangles each, counter-clockwise in
    GL's y-up window space) whose interior vertices are moved onto pixel
    centres (offsets of +-0.5 or +-1.5 px), so that each is a centre shared by
    up to six triangles and many shared edges run exactly through further
    centres.  Returns screen points [(sx, sy)] and triangles."""
    rng = np.random.default_rng(seed)
    n = cells + 1
    pts = []
    for j in range(n):
        for i in range(n):
            sx, sy = origin + i * size, origin + j * size
            if 0 < i < cells and 0 < j < cells:
                sx += rng.integers(-2, 2) + 0.5
                sy += rng.integers(-2, 2) + 0.5
            pts.append((sx, sy))
    tris = []
    for j in range(cells):
        for i in range(cells):
            a, b, c, d = j * n + i, j * n + i + 1, (j + 1) * n + i + 1, (j + 1) * n + i
            # screen y grows downwards, so (a, d, c) / (a, c, b) wind counter-clockwise with y up
            tris += [(a, d, c), (a, c, b)] if (i + j) % 2 == 0 else [(a, d, b), (b, d, c)]
    return pts, tris


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_shared_edges_are_watertight_on_jittered_meshes(oracle, seed):
    """Every triangle of a jittered grid rendered on its own: no pixel centre
    is covered twice and every centre strictly inside the grid is covered
    once, although edges run through centres at arbitrary slopes."""
    pts, tris = _jittered_grid(seed)
    count = np.zeros((K.H, K.W), np.int32)
    for t in tris:
        p = np.array([pts[v] for v in t])
        area = (p[1, 0] - p[0, 0]) * (p[2, 1] - p[0, 1]) - (p[2, 0] - p[0, 0]) * (p[1, 1] - p[0, 1])
        assert area < 0  # front-facing (counter-clockwise with y up)
        mesh = K.screen_mesh([pts[v] for v in t], [(0, 1, 2)])
        count += (_render(oracle, K.scene(), [mesh], [K.node(0)])["winner"][0] >= 0).astype(np.int32)
    assert count.max() == 1
    # the grid's outer boundary is the square [4, 28]^2: centres strictly inside it are covered
    c = np.arange(K.W) + 0.5
    inside = ((c > 4) & (c < 28))[:, None] & ((c > 4) & (c < 28))[None, :]
    assert np.all(count[inside] == 1)
    # on the boundary the top-left rule takes the left (x = 4) and top (y = 4) edges only; no centre lies on
    # them here (centres are at .5), so coverage is exactly the interior
    assert np.array_equal(count == 1, inside)
    # the meshes put centres on shared edges and vertices: count them to show the test exercises the tie rule
    on_edge = set()
    for t in tris:
        p = np.array([pts[v] for v in t])
        for k in range(3):
            (x0, y0), (x1, y1) = p[k], p[(k + 1) % 3]
            for y in range(K.H):
                for x in range(K.W):
                    px, py = x + 0.5, y + 0.5
                    cross = (x1 - x0) * (py - y0) - (y1 - y0) * (px - x0)
                    if cross == 0 and min(x0, x1) <= px <= max(x0, x1) and min(y0, y1) <= py <= max(y0, y1):
                        on_edge.add((x, y))
    assert len(on_edge) >= 40
