"""State-bound pose components (``PBRRenderer.bind_state``): the env step as
one raster launch.  The fused step must give exactly the pixels of the
explicit ``_step`` copies + render, leave the node tensors holding the copied
values, and reject inconsistent bindings through the C ABI."""
import ctypes

import pytest
import torch

from pybatchrender_gb300 import _capi, workloads
from pybatchrender_gb300.envs.cartpole import CartPoleConfig, CartPoleRenderer

pytestmark = pytest.mark.gpu


def _pair(n, **kw):
    fused = workloads.cartpole_bench(num_scenes=n, res=64, seed=5, device="cuda", **kw)
    plain = workloads.cartpole_bench(num_scenes=n, res=64, seed=5, device="cuda", **kw)
    plain._state_bindings = []  # falls back to _step + render
    return fused, plain


@pytest.mark.parametrize("kw", [{}, {"cuda_graph": True}, {"raster_kernel": "tile"}, {"return_depth": True}])
def test_fused_step_matches_step_copies(cuda, kw):
    n = 96
    fused, plain = _pair(n, **kw)
    for seed in (7, 8, 9):
        st = workloads.cartpole_states(n, seed=seed, device=cuda)
        a, b = fused.step(st), plain.step(st)
        if isinstance(a, tuple):
            assert torch.equal(a[1], b[1])
            a, b = a[0], b[0]
        assert torch.equal(a, b)
        # the node tensors hold what _step would have copied
        assert torch.equal(fused.cart.pos[:, 0], st[:, 0])
        assert torch.equal(fused.pole.pos[:, 0], st[:, 0])
        assert torch.equal(fused.pole.hpr[:, 1], st[:, 2])
        assert torch.equal(fused.cart.pos, plain.cart.pos)
        assert torch.equal(fused.pole.hpr, plain.pole.hpr)


def test_fused_step_falls_back(cuda):
    """A CPU state or a non-float32 state go through _step."""
    n = 32
    fused, plain = _pair(n)
    st = workloads.cartpole_states(n, seed=11, device=cuda)
    for arg in (st.cpu(), st.double()):
        assert fused._bound_state((arg,), {}) is None
        assert torch.equal(fused.step(arg), plain.step(arg))


def test_cartpole_env_renderer_fused(cuda):
    cfg = CartPoleConfig(num_scenes=16, tile_resolution=(64, 64), report_fps=False)
    r = CartPoleRenderer(cfg)
    st = workloads.cartpole_states(16, seed=12, device=cuda)
    assert r._bound_state((st,), {}) is not None
    a = r.step(st).clone()
    r2 = CartPoleRenderer(cfg)
    r2._state_bindings = []
    assert torch.equal(a, r2.step(st))
    # fewer rows than scenes: _step pads with the last row (renderer.py of the reference env)
    short = st[:13]
    assert r._bound_state((short,), {}) is None
    assert torch.equal(r.step(short), r2.step(short))


def test_state_source_validation(cuda):
    r = workloads.cartpole_bench(num_scenes=8, res=32, seed=0, device="cuda")
    lib, ctx = r._lib, r._ctx
    st = torch.zeros((8, 4), device=cuda)
    out = torch.empty((8, 3, 32, 32), dtype=torch.uint8, device=cuda)
    bad = [(st, 8, 2, 4),   # pole pitch is bound to column 2 of a 2-column state
           (st, 4, 4, 4),   # 8 scenes need 8 rows
           (st, 8, 4, 3)]   # row stride below the column count
    for t, rows, cols, stride in bad:
        rc = lib.pbr_render_state(ctx, _capi.ptr(t), rows, cols, stride, _capi.ptr(out), None, None, None)
        assert rc == _capi.PBR_ERR_INVALID, lib.pbr_last_error(ctx)
    assert lib.pbr_node_bind_state(ctx, 0, 6, 0) == _capi.PBR_ERR_INVALID
    assert lib.pbr_render_state(ctx, _capi.ptr(st), 8, 4, 4, _capi.ptr(out), None, None, None) == 0
    torch.cuda.synchronize()
