"""The headline configuration at its full size, on the launch the benchmark
times: 4096 CartPole bench scenes at 64x64 RGB, rendered by ``step(state)``
-- the state-bound scene-per-warp launch that writes pixels only (no winner
ids, no depth) -- with the autotuned launch configuration.

Every scene of the batch is checked against the FP64 oracle with the parity
bar of test_gpu_render.py.  The winner ids and depths come from a second
render of the same state (``return_winner=True``, ``return_depth=True``),
whose pixels must equal the timed launch's bit for bit."""
import numpy as np
import pytest
import torch

from pybatchrender_gb300 import workloads

pytestmark = pytest.mark.gpu


def test_headline_4096_state_bound_parity(cuda, oracle, measured):
    n, res = 4096, 64
    r = workloads.cartpole_bench(num_scenes=n, res=res, seed=0, device="cuda", cuda_graph=True)
    tuned = r.autotune()
    st = workloads.cartpole_states(n, seed=100, device=cuda)
    assert r._bound_state((st,), {}) is not None, "step(state) must take the state-bound launch"
    pix = r.step(st).clone()
    pix2, depth, win = r.render(return_depth=True, return_winner=True)
    torch.cuda.synchronize()
    assert torch.equal(pix, pix2), "the timed launch and the winner launch disagree"
    sc, me, no = r.export_scene()
    ref = oracle.render_hard(sc, me, no, want_depth=True, want_winner=True, want_ambiguous=True, nthreads=8)
    gpu = {"pixels": pix.cpu().numpy(), "winner": win.cpu().numpy(), "depth": depth.cpu().numpy()}
    cmp = oracle.compare_hard(gpu, ref)
    print("headline 4096x64x64 (launch", tuned, "):", cmp)
    assert cmp["winner_mismatch"] == 0, cmp
    assert cmp["color_max_diff_unambiguous"] <= 1, cmp
    assert cmp["color_within_1"] >= 0.995, cmp
    covered = (ref["winner"] >= 0) & ~ref["ambiguous"]
    derr = float(np.abs(gpu["depth"] - ref["depth"])[covered].max())
    measured("oracle comparison of 4096 scenes", dict(cmp, depth_max_err=f"{derr:.2e}"))
    assert derr <= 1e-5, cmp
    bg = (ref["winner"] < 0) & ~ref["ambiguous"]
    assert np.all(gpu["depth"][bg] == 1.0)
    # every scene draws its cart and pole: the first, last and busiest scenes are covered
    per_scene = (ref["winner"] >= 0).reshape(n, -1).sum(axis=1)
    assert per_scene[0] > 0 and per_scene[-1] > 0 and per_scene.max() > 0
    assert per_scene.min() > 0, int(np.argmin(per_scene))
